"""Engine-level restatements on top of the C oracle — TEST INFRASTRUCTURE ONLY
(imported by tests/ and bench.py's CPU-baseline leg, never by the product).

traceback / traceback_from_end: src/search/engine.rs:1328-1445.
"""
from . import oracle as orc


def traceback_from_end(q, s, bias, mat, go, ge, want, limit, band_pad, max_dir_bytes, ctr):
    """engine.rs:1403-1445 -> (alignment, exact) or None."""
    m, n = len(q), len(s)
    scope = limit if limit is not None else (-m, n)
    sc, qe, se, cells = orc.banded_score(q, s, bias, mat, go, ge, scope[0], scope[1])
    ctr["banded_cells"] += cells
    if sc <= 0:
        return None
    ctr["end_anchored"] += 1
    target = max(sc, want)
    d_end = se - qe
    pad = max(band_pad, 4)
    while True:
        lo = max(d_end - pad, scope[0])
        hi = min(d_end + pad, scope[1])
        covers = lo <= scope[0] and hi >= scope[1]
        ctr["tracebacks"] += 1
        try:
            al = orc.banded_align(q, s, bias, mat, go, ge, lo, hi, max_dir_bytes, target)
        except MemoryError:
            return None
        if al is not None:
            ctr["banded_cells"] += al["cells"]
            if al["score"] >= target or covers:
                return al, al["score"] >= want
        elif covers:
            return None
        ctr["band_widenings"] += 1
        pad *= 2


def traceback(q, s, bias, mat, go, ge, d_min, d_max, want, limit, full, band_pad, max_dir_bytes, ctr):
    """engine.rs:1328-1393 for one region: d_min/d_max relative to the window
    start, limit = plan band or None, full = exhaustive or region best == 0.
    Returns (alignment, exact) or None."""
    m, n = len(q), len(s)
    pad = max(band_pad, 4)
    best = None
    while True:
        if full:
            lo, hi = -m, n
        else:
            lo, hi = d_min - pad, d_max + pad
        covers = lo <= -(m - 1) and hi >= n - 1
        if limit is not None:
            lo, hi = max(lo, limit[0]), min(hi, limit[1])
            covers = covers or (lo <= limit[0] and hi >= limit[1])
        ctr["tracebacks"] += 1
        try:
            al = orc.banded_align(q, s, bias, mat, go, ge, lo, hi, max_dir_bytes, want)
        except MemoryError:
            found = traceback_from_end(q, s, bias, mat, go, ge, want, limit, band_pad, max_dir_bytes, ctr)
            if found is not None:
                return found
            ctr["band_capped"] += 1
            return None if best is None else (best, False)
        if al is not None:
            ctr["banded_cells"] += al["cells"]
            done = al["score"] >= want or covers
            best = al
            if done:
                return best, best["score"] >= want
        elif covers:
            return None
        ctr["band_widenings"] += 1
        pad *= 2


def new_counters():
    return {"tracebacks": 0, "band_widenings": 0, "end_anchored": 0, "band_capped": 0, "banded_cells": 0}


# ---------------------------------------------------------------------------
# End-to-end restatement of one scan-schedule batch (engine.rs / scan.rs),
# driving the C oracle for every compute step.  The f64 statistics and the
# composition bias are the host modules saber_gb300.stats / saber_gb300.bias
# (host arithmetic of the reference, not part of the GPU path).
# ---------------------------------------------------------------------------
import math  # noqa: E402

import numpy as np  # noqa: E402


def _clip(lo, hi, m, n):
    return max(lo, -(m - 1)), min(hi, n - 1)


def plan_windows(regions, qlen, slen, hsp_threshold, window_slack, score_band, exhaustive):
    """engine.rs:1247-1324 (score_band > 0 branch and window-only plans)."""
    def window(dmin, dmax, sl):
        lo = min(max(dmin - window_slack, 0), sl)
        hi = max(min(qlen + dmax + window_slack, sl), lo)
        return (0, sl) if (hi - lo) * 4 >= sl * 3 else (lo, hi)

    groups = {}
    for i, r in enumerate(regions):
        groups.setdefault(r[0], []).append(i)
    span = {i: (r[1], r[2]) for i, r in enumerate(regions)}
    for idx in groups.values():
        top = max(regions[i][3] for i in idx)
        strong = max(2 * hsp_threshold, top // 4)
        chosen = sorted((i for i in idx if regions[i][3] >= strong),
                        key=lambda i: (regions[i][1], regions[i][2], i))
        k = 0
        while k < len(chosen):
            lo, hi = regions[chosen[k]][1], regions[chosen[k]][2]
            e = k + 1
            while e < len(chosen) and regions[chosen[e]][1] - hi <= 1024:
                hi = max(hi, regions[chosen[e]][2])
                e += 1
            for i in chosen[k:e]:
                span[i] = (lo, hi)
            k = e
    plans = []
    for i, (s, dmin, dmax, best) in enumerate(regions):
        sl = int(slen[s])
        lo, hi = window(dmin, dmax, sl)
        if exhaustive or best == 0 or score_band <= 0:
            plans.append((lo, hi, None))
            continue
        a, b = span[i]
        lo2 = min(max(a - score_band, 0), sl)
        hi2 = max(min(qlen + b + score_band, sl), lo2)
        n = hi2 - lo2
        blo, bhi = _clip(a - score_band - lo2, b + score_band - lo2, qlen, n)
        covers = blo <= -(qlen - 1) and bhi >= n - 1
        plans.append((lo2, hi2, None if (n == 0 or covers) else (blo, bhi)))
    return plans


def _rust_e(x):
    mant, ex = ("%.2e" % x).split("e")
    return mant + "e" + str(int(ex))


def m8_line(qid, sid, h):
    """output.rs:20-52"""
    e = h["evalue"]
    es = "inf" if not math.isfinite(e) else "0.0" if e == 0.0 else ("%.3f" % e if 0.001 <= e < 10.0 else _rust_e(e))
    ident = 0.0 if h["columns"] == 0 else 100.0 * h["matches"] / h["columns"]
    return "\t".join([qid, sid, "%.2f" % ident, str(h["columns"]), str(h["mismatches"]), str(h["gap_opens"]),
                      str(h["q_start"]), str(h["q_end"]), str(h["s_start"]), str(h["s_end"]), es,
                      "%.1f" % h["bitscore"]])


def search_batch(db_codes, db_offsets, q_codes, q_offsets, params, matrix, go, ge, kp, scan_params, db_mask=None,
                 q_mask=None, is_protein=True, stats_size=None, threads=1):
    """Hits per query (lists of dicts in report order) for one batch.
    stats_size: (database length, sequences) of the statistics when they are
    not the residues and subjects (translated databases, driver.rs:575-583).
    threads: host threads of the scan and of the banded scores (every window
    is scored on its own, so the hits do not depend on it)."""
    from saber_gb300.bias import composition_bias
    from saber_gb300.gpu import JOB_DTYPE
    from saber_gb300.stats import SearchStatistics
    P = params
    slen = np.diff(np.asarray(db_offsets, np.int64))
    soff = np.asarray(db_offsets, np.int64)
    nsub = slen.size
    stats = SearchStatistics(kp, *(stats_size or (int(len(db_codes)), nsub)), P.evalue_model)
    nq = len(q_offsets) - 1
    e_reg = max(P.evalue, 10.0)
    if P.ref_db_residues > 0 and stats.db_length > P.ref_db_residues:
        e_reg = e_reg * (stats.db_length / P.ref_db_residues)
    preps = []
    for qi in range(nq):
        q = np.asarray(q_codes[q_offsets[qi]:q_offsets[qi + 1]])
        b = composition_bias(q, matrix) if (P.comp_bias and is_protein) else np.zeros(len(q), np.int8)
        qs = stats.for_query(max(len(q), 1))
        floor = qs.min_score(P.evalue, P.min_bitscore)
        rfloor = floor if (e_reg == P.evalue and P.min_bitscore is None) else qs.min_score(e_reg, None)
        thr = P.hsp_threshold
        if P.hsp_floor_fraction > 0.0 and rfloor > 0:
            thr = max(P.hsp_threshold, int(min(math.ceil(rfloor * P.hsp_floor_fraction), float(2 ** 31 - 1))))
        preps.append((q, b, qs, floor, rfloor, thr))
    bias = np.concatenate([p[1] for p in preps]) if nq else np.zeros(0, np.int8)
    regs_q = [[] for _ in range(nq)]
    if P.exhaustive:
        for qi in range(nq):
            if len(preps[qi][0]):
                regs_q[qi] = [(s, -len(preps[qi][0]), int(slen[s]), 0) for s in range(nsub)]
    elif nq and nsub:
        rthr = np.array([p[5] for p in preps], np.int32)
        regs, _ = orc.scan_regions(db_codes, db_offsets, db_mask, q_codes, q_offsets, bias, q_mask, rthr, matrix,
                                   scan_params, threads=threads)
        for r in regs:
            regs_q[int(r["query"])].append((int(r["subject"]), int(r["d_min"]), int(r["d_max"]), int(r["best"])))
    # score_windows (engine.rs:1021-1099) for every query: the first stage
    # (the full window, the region's narrow band, or the plan band), then the
    # plan band for the narrow scores that pass the prefilter threshold
    wn, fb = P.score_prefilter_band, P.score_band
    plans_q, jobs1, jobs2, where2 = [], [], [], []
    for qi in range(nq):
        q, b, qs, floor, rfloor, _ = preps[qi]
        m = len(q)
        regs = regs_q[qi] if m else []
        plans = plan_windows(regs, m, slen, P.hsp_threshold, P.window_slack, P.score_band, P.exhaustive)
        plans_q.append(plans)
        for (s, dmin, dmax, best), (lo, hi, band) in zip(regs, plans):
            n = hi - lo
            if band is None:
                jobs1.append((qi, s, soff[s] + lo, n, -m, n, 0))
            elif 0 < wn < fb:
                nlo, nhi = _clip(dmin - wn - lo, dmax + wn - lo, m, n)
                jobs1.append((qi, s, soff[s] + lo, n, nlo, nhi, 1))
            else:
                jobs1.append((qi, s, soff[s] + lo, n, band[0], band[1], 0))
    j1 = np.array(jobs1, JOB_DTYPE) if jobs1 else np.zeros(0, JOB_DTYPE)
    sc1 = orc.score_band_jobs(db_codes, q_codes, q_offsets, bias, j1, matrix, go, ge, threads)[0] if j1.size \
        else np.zeros(0, np.int32)
    k = 0
    for qi in range(nq):
        qs, rfloor = preps[qi][2], preps[qi][4]
        for (s, dmin, dmax, best), (lo, hi, band) in zip(regs_q[qi] if len(preps[qi][0]) else [], plans_q[qi]):
            if j1[k]["flags"] == 1:
                thr = P.score_prefilter_frac * qs.floor_lower_bound(e_reg, None, int(slen[s]), rfloor)
                if not float(sc1[k]) < thr:
                    jobs2.append((qi, s, soff[s] + lo, hi - lo, band[0], band[1], 0))
                    where2.append(k)
            k += 1
    scores_all = sc1.copy()
    if jobs2:
        sc2 = orc.score_band_jobs(db_codes, q_codes, q_offsets, bias, np.array(jobs2, JOB_DTYPE), matrix, go, ge,
                                  threads)[0]
        scores_all[np.array(where2, np.int64)] = sc2
    out = []
    k = 0
    for qi in range(nq):
        q, b, qs, floor, rfloor, _ = preps[qi]
        m = len(q)
        regs = regs_q[qi] if m else []
        bo = b if np.any(b != 0) else None
        plans = plans_q[qi]
        scores = [int(x) for x in scores_all[k:k + len(regs)]]
        k += len(regs)
        # finish, engine.rs:1127-1221
        ecut = P.evalue if (P.evalue > 0 and math.isfinite(P.evalue)) else math.inf
        order = []
        for i, (s, dmin, dmax, best) in enumerate(regs):
            sc = scores[i]
            if qs.model == "database":
                if sc >= floor:
                    order.append((qs.evalue(sc), i))
                continue
            if sc <= 0 or (P.min_bitscore is not None and qs.bitscore(sc) < P.min_bitscore):
                continue
            n = int(slen[s])
            if qs.evalue_in(sc, qs.space_lower_bound(n)) > ecut:
                continue
            e = qs.evalue_for(sc, n)
            if e <= ecut:
                order.append((e, i))
        order.sort(key=lambda t: (t[0], -scores[t[1]], -regs[t[1]][3], regs[t[1]][0], regs[t[1]][1], regs[t[1]][2]))
        hits, per, rep = [], {}, 0
        for _, i in order:
            s, dmin, dmax, best = regs[i]
            if rep >= P.max_target_seqs and s not in per:
                break
            cnt = per.get(s, 0)
            if cnt >= P.max_hsps:
                continue
            lo, hi, band = plans[i]
            sfull = np.asarray(db_codes[db_offsets[s]:db_offsets[s + 1]])
            sub = sfull[lo:hi]
            ctr = new_counters()
            tbres = traceback(q, sub, bo, matrix, go, ge, dmin - lo, dmax - lo, scores[i], band,
                              P.exhaustive or best == 0, P.band_pad, P.traceback_max_bytes, ctr)
            if tbres is None:
                continue
            al, exact = tbres
            h = _make_hit(q, sfull, s, lo, al, exact, qs, matrix, is_protein)
            if cnt > 0 and any(x["subject"] == s and x["q_start"] <= h["q_end"] and h["q_start"] <= x["q_end"]
                               and x["s_start"] <= h["s_end"] and h["s_start"] <= x["s_end"] for x in hits):
                continue
            passes = (h["score"] >= floor) if qs.model == "database" else \
                (h["evalue"] <= ecut and (P.min_bitscore is None or h["bitscore"] >= P.min_bitscore))
            ident = 0.0 if h["columns"] == 0 else 100.0 * h["matches"] / h["columns"]
            qcov = 100.0 * (h["q_end"] + 1 - h["q_start"]) / h["q_len"] if h["q_len"] else 0.0
            scov = 100.0 * (h["s_end"] + 1 - h["s_start"]) / h["s_len"] if h["s_len"] else 0.0
            if ident < P.min_identity or qcov < P.min_query_cover or scov < P.min_subject_cover or not passes:
                continue
            if cnt == 0:
                rep += 1
            per[s] = cnt + 1
            hits.append(h)
        hits.sort(key=lambda x: (x["evalue"], -x["score"], x["subject"], x["s_start"]))
        out.append(hits)
    return out


def _make_hit(q, sfull, subject, s_off, al, exact, qs, matrix, is_protein):
    """engine.rs:1447-1530"""
    s = sfull[s_off:]
    i, j = al["q_start"], al["s_start"]
    mt = mm = ps = go_ = gc = 0
    lim = 20 if is_protein else 4
    for op, l in al["ops"]:
        if op == "M":
            for _ in range(l):
                a, b = int(q[i]), int(s[j])
                ident = a == b and a < lim
                mt += ident
                mm += not ident
                ps += ident or matrix[a if a < 24 else 22][b if b < 24 else 22] > 0
                i += 1
                j += 1
        elif op == "I":
            go_ += 1
            gc += l
            i += l
        else:
            go_ += 1
            gc += l
            j += l
    return dict(subject=subject, score=al["score"], bitscore=qs.bitscore(al["score"]),
                evalue=qs.evalue_for(al["score"], len(sfull)), q_start=al["q_start"] + 1, q_end=al["q_end"],
                s_start=al["s_start"] + s_off + 1, s_end=al["s_end"] + s_off, columns=sum(l for _, l in al["ops"]),
                matches=mt, mismatches=mm, positives=ps, gap_opens=go_, gap_columns=gc, q_len=len(q),
                s_len=len(sfull), ops=al["ops"], exact=exact)


def finish_record_nx(frame_hits, max_target_seqs, max_hsps):
    """finish_record for nx (driver.rs:481-501): frame_hits = hit lists of the
    record's frames 0..5; returns (frame, hit) pairs after the merge (stable
    sort by score descending, subject, frame; then max_hsps per subject and
    max_target_seqs subjects)."""
    import functools
    flat = []
    for f in range(6):
        for h in frame_hits[f]:
            flat.append((f, h))

    def cmp(a, b):
        if a[1]["score"] != b[1]["score"]:
            return -1 if a[1]["score"] > b[1]["score"] else 1
        if a[1]["subject"] != b[1]["subject"]:
            return -1 if a[1]["subject"] < b[1]["subject"] else 1
        return (a[0] > b[0]) - (a[0] < b[0])
    flat.sort(key=functools.cmp_to_key(cmp))
    count, out, nsubj = {}, [], 0
    for f, h in flat:
        c = count.setdefault(h["subject"], 0)
        if c >= max_hsps or (c == 0 and nsubj >= max_target_seqs):
            continue
        if c == 0:
            nsubj += 1
        count[h["subject"]] = c + 1
        out.append((f, h))
    return out


def frame_nt_range(frame, p_start, p_end, nt_len):
    """protein_to_nt (translation.rs:323-337) and frame_label (:316-318)."""
    if frame < 3:
        return frame + 3 * p_start - 2, frame + 3 * p_end, frame + 1
    off = frame - 3
    return nt_len - (off + 3 * p_start - 2) + 1, nt_len - (off + 3 * p_end) + 1, -(off + 1)
