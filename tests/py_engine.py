"""The engine stages of one search batch written in Python over the same
device calls as the library's C++ host engine (saber_gpu_search) — TEST
INFRASTRUCTURE: tests hold the C++ engine to this readable restatement, hit
for hit and m8 row for m8 row.

It restates, on top of a saber_gb300.search.Searcher (database, parameters,
statistics and device handle): query preparation (composition bias,
statistics and floors, engine.rs:714-786), the GPU scan, plan_windows
(engine.rs:1223-1324), two-stage banded scoring (score_windows,
engine.rs:1021-1099), finish with E-values and the widening traceback
(engine.rs:1127-1221, 1328-1445) and make_hit (engine.rs:1447-1530).
"""
import math

import numpy as np

from saber_gb300.bias import composition_bias
from saber_gb300.gpu import JOB_DTYPE, TB_JOB_DTYPE
from saber_gb300.search import I32_MAX, Hit

REGION_FLOOR_EVALUE = 10.0   # engine.rs:518
BAND_SCORE_MIN_CELLS = 1 << 20  # engine.rs:401
BAND_COST_RATIO = 12            # engine.rs:402
BAND_BRIDGE = 1024              # engine.rs:404


class _Prep:
    """QueryPrep (engine.rs:497-510)."""
    __slots__ = ("bias", "has_bias", "qstats", "floor", "region_floor", "region_thr")


def _band_clip(lo, hi, m, n):
    return max(lo, -(m - 1)), min(hi, n - 1)


def _band_covers(lo, hi, m, n):
    return lo <= -(m - 1) and hi >= n - 1


def _band_width(lo, hi):
    return max(hi - lo + 1, 0)


def _overlaps(a, b):
    """engine.rs:2415-2417"""
    return a["q_start"] <= b["q_end"] and b["q_start"] <= a["q_end"] and a["s_start"] <= b["s_end"] and \
        b["s_start"] <= a["s_end"]


class PyEngine:
    """search(q_codes, q_offsets, q_mask) of a Searcher's batch with every
    engine step in Python; device calls go through the searcher's handle."""

    def __init__(self, searcher):
        self.se = searcher

    def __getattr__(self, name):
        return getattr(self.se, name)

    # ---- query preparation (engine.rs:714-786) ----
    def region_evalue(self):
        e = max(self.p.evalue, REGION_FLOOR_EVALUE)
        r = self.p.ref_db_residues
        if r > 0 and self.stats.db_length > r:
            return e * (self.stats.db_length / r)
        return e

    def prepare(self, q):
        pr = _Prep()
        if self.p.comp_bias and self.is_protein:
            pr.bias = composition_bias(q, self.matrix)
        else:
            pr.bias = np.zeros(len(q), np.int8)
        pr.has_bias = bool(np.any(pr.bias != 0))
        pr.qstats = self.stats.for_query(max(len(q), 1))
        pr.floor = pr.qstats.min_score(self.p.evalue, self.p.min_bitscore)
        re_ = self.region_evalue()
        if re_ == self.p.evalue and self.p.min_bitscore is None:
            pr.region_floor = pr.floor
        else:
            pr.region_floor = pr.qstats.min_score(re_, None)
        f = self.p.hsp_floor_fraction
        if f > 0.0 and pr.region_floor > 0:
            pr.region_thr = max(self.p.hsp_threshold, int(min(math.ceil(pr.region_floor * f), float(I32_MAX))))
        else:
            pr.region_thr = self.p.hsp_threshold
        return pr


    # ---- plan_windows (engine.rs:1223-1324) ----
    def window(self, d_min, d_max, subject, qlen):
        sl = int(self.slen[subject])
        slack = self.p.window_slack
        lo = min(max(d_min - slack, 0), sl)
        hi = max(min(qlen + d_max + slack, sl), lo)
        if (hi - lo) * 4 >= sl * 3:
            return 0, sl
        return lo, hi

    def plan_windows(self, regions, qlen):
        """regions: list of (subject, d_min, d_max, best) -> list of (lo, hi, band or None)."""
        by_subject = {}
        for i, r in enumerate(regions):
            by_subject.setdefault(r[0], []).append(i)
        span = [(r[1], r[2]) for r in regions]
        for idx in by_subject.values():
            top = max(regions[i][3] for i in idx)
            strong = max(2 * self.p.hsp_threshold, int(top / 4) if top >= 0 else -((-top) // 4))
            idx = [i for i in idx if regions[i][3] >= strong]
            idx.sort(key=lambda i: (regions[i][1], regions[i][2], i))
            start = 0
            while start < len(idx):
                lo, hi = regions[idx[start]][1], regions[idx[start]][2]
                end = start + 1
                while end < len(idx) and regions[idx[end]][1] - hi <= BAND_BRIDGE:
                    hi = max(hi, regions[idx[end]][2])
                    end += 1
                lo = min(lo, regions[idx[start]][1])
                for i in idx[start:end]:
                    span[i] = (lo, hi)
                start = end
        plans = []
        for ri, (s, dmin0, dmax0, best) in enumerate(regions):
            lo, hi = self.window(dmin0, dmax0, s, qlen)
            own = (lo, hi, None)
            if self.p.exhaustive or best == 0 or self.p.window_slack >= (2 ** 63 - 1) // 8:
                plans.append(own)
                continue
            if self.p.score_band > 0:
                w = self.p.score_band
                dmin, dmax = span[ri]
                sl = int(self.slen[s])
                lo2 = min(max(dmin - w, 0), sl)
                hi2 = max(min(qlen + dmax + w, sl), lo2)
                n = hi2 - lo2
                blo, bhi = _band_clip(dmin - w - lo2, dmax + w - lo2, qlen, n)
                if n == 0 or _band_covers(blo, bhi, qlen, n):
                    plans.append((lo2, hi2, None))
                else:
                    plans.append((lo2, hi2, (blo, bhi)))
                continue
            if qlen * (hi - lo) < BAND_SCORE_MIN_CELLS:
                plans.append(own)
                continue
            dmin, dmax = span[ri]
            ulo, uhi = self.window(dmin, dmax, s, qlen)
            n = uhi - ulo
            blo, bhi = _band_clip(dmin - ulo - self.p.window_slack, dmax - ulo + self.p.window_slack, qlen, n)
            if _band_covers(blo, bhi, qlen, n):
                plans.append(own)
                continue
            rows = min(qlen, n + _band_width(blo, bhi))
            rect = qlen * n
            if _band_width(blo, bhi) * rows * BAND_COST_RATIO < rect:
                plans.append((ulo, uhi, (blo, bhi)))
            else:
                plans.append(own)
        return plans


    # ---- the same batch with the engine steps in Python (cross-check) ----
    def search(self, q_codes, q_offsets, q_mask=None):
        """Hits of every query of the batch: list (per query) of Hit, in report order."""
        q_codes = np.ascontiguousarray(q_codes, dtype=np.uint8)
        q_offsets = np.ascontiguousarray(q_offsets, dtype=np.uint64)
        nq = q_offsets.size - 1
        qlens = np.diff(q_offsets.astype(np.int64))
        q_mask, n_masked = self.query_mask(q_codes, q_offsets, q_mask)
        preps = [self.prepare(q_codes[q_offsets[i]:q_offsets[i + 1]]) for i in range(nq)]
        bias = np.concatenate([p.bias for p in preps]) if nq else np.zeros(0, np.int8)
        self.dev.load_queries(q_codes, q_offsets, bias)
        ctr = {"queries": nq, "query_residues_masked": n_masked}
        # candidate regions (engine.rs:1014-1019 for the exhaustive preset)
        per_q = [[] for _ in range(nq)]
        if self.p.exhaustive:
            for qi in range(nq):
                if qlens[qi] > 0 and self.nsub > 0:
                    per_q[qi] = [(s, -int(qlens[qi]), int(self.slen[s]), 0) for s in range(self.nsub)]
        elif nq and self.nsub:
            rthr = np.array([p.region_thr for p in preps], np.int32)
            regs, st = self.dev.scan(self.scan_params, q_mask, rthr)
            ctr.update({k: v for k, v in st.items()})
            for r in regs:
                per_q[int(r["query"])].append((int(r["subject"]), int(r["d_min"]), int(r["d_max"]), int(r["best"])))
        for qi in range(nq):
            if qlens[qi] == 0:
                per_q[qi] = []
        plans = [self.plan_windows(per_q[qi], int(qlens[qi])) for qi in range(nq)]
        scores = self.score_windows(preps, per_q, plans, qlens, ctr)
        out = self.finish(q_codes, q_offsets, preps, per_q, plans, scores, ctr)
        self.counters = ctr
        return out

    # ---- score_windows (engine.rs:1021-1099), batched over the queries ----
    def _jobs(self, items):
        jobs = np.zeros(len(items), JOB_DTYPE)
        if items:
            a = np.array(items, dtype=np.int64)
            jobs["query"] = a[:, 0]
            jobs["subject"] = a[:, 1]
            jobs["win_begin"] = self.db_offsets[a[:, 1]].astype(np.int64) + a[:, 2]
            jobs["win_len"] = a[:, 3] - a[:, 2]
            jobs["band_lo"] = np.clip(a[:, 4], -(2 ** 31), I32_MAX)
            jobs["band_hi"] = np.clip(a[:, 5], -(2 ** 31), I32_MAX)
        return jobs

    def score_windows(self, preps, per_q, plans, qlens, ctr):
        scores = [np.zeros(len(r), np.int64) for r in per_q]
        wn, full_band = self.p.score_prefilter_band, self.p.score_band
        stage1, stage1_ref = [], []
        for qi, regs in enumerate(per_q):
            m = int(qlens[qi])
            for ri, (s, dmin, dmax, best) in enumerate(regs):
                lo, hi, band = plans[qi][ri]
                n = hi - lo
                if band is None:
                    stage1.append((qi, s, lo, hi, -m, n))  # Band::full(m, n)
                    stage1_ref.append((qi, ri, "full"))
                elif 0 < wn < full_band:
                    blo, bhi = _band_clip(dmin - wn - lo, dmax + wn - lo, m, n)
                    stage1.append((qi, s, lo, hi, blo, bhi))
                    stage1_ref.append((qi, ri, "narrow"))
                else:
                    stage1.append((qi, s, lo, hi, band[0], band[1]))
                    stage1_ref.append((qi, ri, "band"))
        sc1 = self._score(stage1, ctr)
        stage2, stage2_ref = [], []
        re_ = self.region_evalue()
        n_banded = n_rescored = 0
        for k, (qi, ri, kind) in enumerate(stage1_ref):
            if kind != "narrow":
                scores[qi][ri] = int(sc1[k])
                n_banded += kind == "band"
                continue
            n_banded += 1
            s = per_q[qi][ri][0]
            pr = preps[qi]
            thr = self.p.score_prefilter_frac * pr.qstats.floor_lower_bound(re_, None, int(self.slen[s]),
                                                                             pr.region_floor)
            if float(sc1[k]) >= thr:
                lo, hi, band = plans[qi][ri]
                stage2.append((qi, s, lo, hi, band[0], band[1]))
                stage2_ref.append((qi, ri))
            else:
                scores[qi][ri] = int(sc1[k])
        sc2 = self._score(stage2, ctr)
        for k, (qi, ri) in enumerate(stage2_ref):
            scores[qi][ri] = int(sc2[k])
        ctr["band_scored_regions"] = ctr.get("band_scored_regions", 0) + n_banded
        ctr["band_rescored"] = ctr.get("band_rescored", 0) + len(stage2)
        return scores

    def _score(self, items, ctr):
        if not items:
            return np.zeros(0, np.int32)
        jobs = self._jobs(items)
        sc, st = self.dev.score_band_jobs(jobs)
        ctr["banded_cells"] = ctr.get("banded_cells", 0) + st["banded_cells"]
        ctr["score_launches"] = ctr.get("score_launches", 0) + 1
        return sc

    # ---- finish (engine.rs:1127-1221) ----
    def finish(self, q_codes, q_offsets, preps, per_q, plans, scores, ctr):
        p = self.p
        ecut = p.evalue if (p.evalue > 0.0 and math.isfinite(p.evalue)) else math.inf
        orders = []
        for qi, regs in enumerate(per_q):
            qs = preps[qi].qstats
            order = []
            for i, (s, dmin, dmax, best) in enumerate(regs):
                sc = int(scores[qi][i])
                if qs.model == "database":
                    if sc >= preps[qi].floor:
                        order.append((qs.evalue(sc), i))
                    continue
                if sc <= 0 or (p.min_bitscore is not None and qs.bitscore(sc) < p.min_bitscore):
                    continue
                n = int(self.slen[s])
                if qs.evalue_in(sc, qs.space_lower_bound(n)) > ecut:
                    continue
                e = qs.evalue_for(sc, n)
                if e <= ecut:
                    order.append((e, i))
            regs_ = regs
            sc_ = scores[qi]
            order.sort(key=lambda t: (t[0], -int(sc_[t[1]]), -regs_[t[1]][3], regs_[t[1]][0], regs_[t[1]][1],
                                      regs_[t[1]][2]))
            orders.append(order)
        # speculative batched tracebacks: the next chunk of candidates of every
        # unfinished query per round (a traceback depends only on its region)
        tb = {}
        state = [dict(pos=0, out=[], per_subject={}, reported=0, done=len(orders[qi]) == 0) for qi in range(len(orders))]
        chunk = max(4, 2 * p.max_target_seqs * p.max_hsps)
        tstats = {}
        while True:
            need = []
            for qi, stt in enumerate(state):
                if stt["done"]:
                    continue
                k = stt["pos"]
                for _, ri in orders[qi][k:k + chunk]:
                    if (qi, ri) not in tb:
                        need.append((qi, ri))
            if need:
                res, st = self._traceback(need, per_q, plans, scores, preps, q_offsets)
                for key, r in zip(need, res):
                    tb[key] = r
                for k_, v in st.items():
                    tstats[k_] = tstats.get(k_, 0) + v
            progress = False
            for qi, stt in enumerate(state):
                if stt["done"]:
                    continue
                progress |= self._finish_steps(qi, stt, orders[qi], per_q[qi], plans[qi], tb, preps[qi], q_codes,
                                               q_offsets, ecut)
            if all(s["done"] for s in state):
                break
            if not need and not progress:
                break
        for k_, v in tstats.items():
            ctr["tb_" + k_] = v
        out = []
        for stt in state:
            hits = stt["out"]
            hits.sort(key=lambda h: (h["evalue"], -h["score"], h["subject"], h["s_start"]))
            out.append(hits)
        ctr["alignments"] = sum(len(h) for h in out)
        return out

    def _finish_steps(self, qi, stt, order, regs, plans, tb, prep, q_codes, q_offsets, ecut):
        p = self.p
        moved = False
        while stt["pos"] < len(order):
            _, ri = order[stt["pos"]]
            s, dmin, dmax, best = regs[ri]
            if stt["reported"] >= p.max_target_seqs and s not in stt["per_subject"]:
                stt["done"] = True
                return True
            cnt = stt["per_subject"].get(s, 0)
            if cnt >= p.max_hsps:
                stt["pos"] += 1
                moved = True
                continue
            if (qi, ri) not in tb:
                return moved
            stt["pos"] += 1
            moved = True
            al = tb[(qi, ri)]
            if al is None:
                continue
            lo = plans[ri][0]
            hit = self.make_hit(q_codes[q_offsets[qi]:q_offsets[qi + 1]], s, lo, al, prep.qstats)
            if cnt > 0 and any(h["subject"] == hit["subject"] and _overlaps(h, hit) for h in stt["out"]):
                continue
            if prep.qstats.model == "database":
                passes = hit["score"] >= prep.floor
            else:
                passes = hit["evalue"] <= ecut and (p.min_bitscore is None or hit["bitscore"] >= p.min_bitscore)
            if (hit.identity() < p.min_identity or hit.query_cover() < p.min_query_cover
                    or hit.subject_cover() < p.min_subject_cover or not passes):
                continue
            if cnt == 0:
                stt["reported"] += 1
            stt["per_subject"][s] = cnt + 1
            stt["out"].append(hit)
        stt["done"] = True
        return True

    def _traceback(self, need, per_q, plans, scores, preps, q_offsets):
        jobs = np.zeros(len(need), TB_JOB_DTYPE)
        for k, (qi, ri) in enumerate(need):
            s, dmin, dmax, best = per_q[qi][ri]
            lo, hi, band = plans[qi][ri]
            full = self.p.exhaustive or best == 0
            jobs[k] = (qi, s, int(self.db_offsets[s]) + lo, hi - lo, dmin - lo, dmax - lo,
                       band[0] if band else 0, band[1] if band else 0, int(scores[qi][ri]),
                       (1 if full else 0) | (2 if band else 0), 0)
        res, st = self.dev.traceback(jobs, self.p.band_pad, self.p.traceback_max_bytes)
        return res, st

    # ---- make_hit (engine.rs:1447-1530) ----
    def make_hit(self, q, subject, s_off, al, qs):
        s_full = self.db_codes[self.db_offsets[subject]:self.db_offsets[subject + 1]]
        s = s_full[s_off:]
        i, j = al["q_start"], al["s_start"]
        matches = mism = pos = gopen = gcols = 0
        M = self.matrix
        lim = 20 if self.is_protein else 4
        for op, l in al["ops"]:
            if op == "M":
                a = q[i:i + l].astype(np.int64)
                b = s[j:j + l].astype(np.int64)
                ident = (a == b) & (a < lim)
                sc = M[np.where(a < 24, a, 22), np.where(b < 24, b, 22)]  # code_index (alphabet.rs:39)
                posit = ident | (sc > 0)
                nid = int(ident.sum())
                matches += nid
                mism += l - nid
                pos += int(posit.sum())
                i += l
                j += l
            elif op == "I":
                gopen += 1
                gcols += l
                i += l
            else:
                gopen += 1
                gcols += l
                j += l
        score = al["score"]
        cols = sum(l for _, l in al["ops"])
        return Hit(subject=subject, score=score, bitscore=qs.bitscore(score), evalue=qs.evalue_for(score, s_full.size),
                   q_start=al["q_start"] + 1, q_end=al["q_end"], s_start=al["s_start"] + s_off + 1,
                   s_end=al["s_end"] + s_off, columns=cols, matches=matches, mismatches=mism, positives=pos,
                   gap_opens=gopen, gap_columns=gcols, q_len=len(q), s_len=int(s_full.size), ops=al["ops"],
                   exact=al["status"] == 1)
