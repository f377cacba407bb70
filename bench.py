"""Benchmark of the banded Smith-Waterman scoring stage (SW scoring-stage
microbench): 1,000,000 banded candidate regions from synthetic protein data
of 2,000 queries x 200,000 subjects (log-normal lengths, BLOSUM62 background,
10 % planted homologs), band half-widths 8-128, BLOSUM62 with gap open 11 /
extend 1, per-position query bias.  Metric: GCUPS (in-band cells counted as
the reference counts them / second), every score bit-exact.

One JSON line on rank 0.  `value`: device-resident jobs and scores (whole
pipeline: classify, sort, pair, packed int16 kernel, int32 kernel), L2
flushed between steps.  `e2e`: the same call through the C ABI with pinned
host buffers (job upload and score download inside the timed region).
`--impl reference` times the CPU oracle (the reference algorithm restated in
C, all host threads) on bounded samples of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "banded SW GCUPS (bit-exact)"
ALGO_OPS_PER_CELL = 11  # E: 2 sub + max, F: 2 sub + max, H: add + 3 max, best: max


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--jobs", type=int, default=1_000_000)
    ap.add_argument("--queries", type=int, default=2000)
    ap.add_argument("--subjects", type=int, default=200_000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample size (seconds of work)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--strip-rows", type=int, default=16, help="rows per strip of the int16 kernel (8 or 16)")
    ap.add_argument("--no-autotune", action="store_true", help="keep --strip-rows and the default pairing")
    ap.add_argument("--no-search", action="store_true", help="skip the batched-search / learned-triage lines")
    ap.add_argument("--search-only", action="store_true",
                    help="only the batched-search section (printed as its own JSON line)")
    ap.add_argument("--no-triage", action="store_true", help="search section without the learned triage")
    ap.add_argument("--no-pool", action="store_true", help="search section without the two-batches-in-flight lines")
    ap.add_argument("--no-masking", action="store_true", help="search section without the tantan masking line")
    ap.add_argument("--search-queries", type=int, default=2000)
    ap.add_argument("--search-subjects", type=int, default=500_000)
    ap.add_argument("--nn-search", action="store_true",
                    help="only the blastn (nn) batched search: DNA queries of 1-10 kb vs a synthetic genome-scale "
                         "database (its own JSON line)")
    ap.add_argument("--translated", action="store_true",
                    help="only the translated searches (nx, pn) and the six-frame translation (its own JSON line)")
    ap.add_argument("--no-translated", action="store_true", help="skip the translated-search lines")
    ap.add_argument("--tr-records", type=int, default=1000, help="nx DNA query records / pn protein queries")
    ap.add_argument("--tr-subjects", type=int, default=100_000, help="nx protein subjects / pn DNA sequences")
    ap.add_argument("--nn-queries", type=int, default=2000)
    ap.add_argument("--nn-bases", type=float, default=500e6, help="database size in bases (subjects of 1-10 kb)")
    ap.add_argument("--long-steps", type=int, default=0,
                    help="scoring: one-lane sweeps longer than this go to the warp-per-job kernel (0: library default)")
    return ap.parse_args()


def workload(seed, nq, ns, nj):
    from saber_gb300 import synth
    qs, ss, planted = synth.protein_db(seed, nq, ns)
    bias = synth.query_bias(seed + 1, qs)
    jobs = synth.band_jobs(seed + 2, qs, ss, planted, nj)
    return qs, ss, planted, bias, jobs


def config_dict(a, world):
    return {"workload": "sw-scoring-microbench: %d banded regions, %d queries x %d subjects, half-widths 8-128, "
                        "BLOSUM62 11/1, query bias" % (a.jobs, a.queries, a.subjects),
            "jobs_per_gpu": a.jobs, "queries": a.queries, "subjects": a.subjects, "seed": a.seed,
            "l2": "flushed between timed steps (512 MB write)", "parallelism": "replicas x%d" % world}


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None
        self.lines = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(qs, ss, bias, jobs, matrix, seconds):
    """The oracle port on all host cores over a bounded sample of the jobs."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    n = min(jobs.size, 4000)
    t0 = time.perf_counter()
    _, cells = orc.score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, jobs[:n], matrix, 11, 1, threads)
    dt = time.perf_counter() - t0
    rate = cells / max(dt, 1e-9)
    want_cells = rate * seconds
    per_job = cells / max(n, 1)
    n2 = int(min(jobs.size, max(n, want_cells / max(per_job, 1))))
    t0 = time.perf_counter()
    _, cells = orc.score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, jobs[:n2], matrix, 11, 1, threads)
    dt = time.perf_counter() - t0
    return {"value": round(cells / dt / 1e9, 3), "unit": "GCUPS", "cores": threads, "kind": "port",
            "sample": "first %d of the %d jobs (%.3g cells, %.1f s), scalar C oracle (banded.rs restatement), "
                      "%d threads" % (n2, jobs.size, cells, dt, threads)}


def run_reference(a, rank, world):
    if rank != 0:
        return
    from saber_gb300.scoring import matrix
    from oracle import oracle as orc
    qs, ss, planted, bias, jobs = workload(a.seed, a.queries, a.subjects, a.jobs)
    mat = matrix("BLOSUM62")
    threads = os.cpu_count() or 1
    per_step = 30000
    rng = np.random.default_rng(a.seed + 9)
    tot_cells, tot_t = 0, 0.0
    for step in range(a.warmup + a.steps):
        sel = jobs[rng.integers(0, jobs.size, size=min(per_step, jobs.size))]
        t0 = time.perf_counter()
        _, cells = orc.score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, sel, mat, 11, 1, threads)
        dt = time.perf_counter() - t0
        if step >= a.warmup:
            tot_cells += cells
            tot_t += dt
    v = tot_cells / tot_t / 1e9
    out = {"metric": METRIC, "impl": "reference", "value": round(v, 3), "unit": "GCUPS", "n_gpus": world,
           "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(tot_t / a.steps * 1e3, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic", "config": config_dict(a, world),
           "cpu_baseline": {"value": round(v, 3), "unit": "GCUPS", "cores": threads, "kind": "port",
                            "sample": "%d random jobs per step of the same workload, scalar C restatement of "
                                      "banded_score (the reference is Rust; no cargo here)" % per_step},
           "e2e": {"value": round(v, 3), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_search(a, dev):
    """Batched full search (config-2 style data: 50 % background, 25 % planted
    homologs at 30-60 % identity, 25 % reversed decoys; the database at the
    config's 150 M residues, fewer queries than its 11,000 to keep the run
    short) through the C ABI's batch engine, plain and with the learned
    triage; the triage network is trained on the GPU on a separately seeded
    database from labels of the plain search."""
    from saber_gb300 import synth
    from saber_gb300 import triage as tr
    from saber_gb300.search import Searcher, SearchParams
    triage = not a.no_triage
    t0 = t1 = t2 = time.perf_counter()
    if triage:
        qa, sa, _ = synth.protein_db(a.seed + 501, max(a.search_queries // 2, 1), max(a.search_subjects * 2 // 5, 1),
                                     reversed_frac=0.25, identity_range=(0.3, 0.6))
        se = Searcher(dev, sa.codes, sa.offsets, SearchParams("default", masking="none"))
        rows, y, _ = tr.collect(se, qa.codes, qa.offsets)
        t1 = time.perf_counter()
        model, st = tr.train(dev, rows, y, seed=a.seed + 1)
        t2 = time.perf_counter()
        thr = tr.threshold_for_recall(dev.triage_predict(model, rows), y, recall=0.999, margin=0.5)
    qb, sb, _ = synth.protein_db(a.seed + 502, a.search_queries, a.search_subjects, reversed_frac=0.25,
                                 identity_range=(0.3, 0.6))
    if a.long_steps:
        dev.long_steps = a.long_steps
    se2 = Searcher(dev, sb.codes, sb.offsets, SearchParams("default", masking="none"))
    cpar = se2.cparams()

    def call():
        # the C ABI's batch search (host buffers in, hit records out)
        return dev.search(cpar, se2.db_codes, se2.db_offsets, qb.codes, qb.offsets)

    call()  # warm: database state, scratch sizes

    def timed(reps=3):
        ts, out = [], None
        for _ in range(reps):
            t = time.perf_counter()
            out = call()
            ts.append(time.perf_counter() - t)
        return out[0], float(np.median(ts)), out[2]

    def keyset(hits):
        return {(int(r["query"]), int(r["subject"]), int(r["score"]), int(r["q_start"]), int(r["q_end"]),
                 int(r["s_start"]), int(r["s_end"]), float(r["evalue"])) for r in hits}

    plain, tp, cp = timed()
    nq = a.search_queries
    stages = ("t_scan_ms", "t_triage_ms", "t_plan_ms", "t_score_ms", "t_finish_ms", "t_total_ms",
              "t_score_calls_ms", "t_score_device_ms", "t_finish_tb_ms")
    out = {
        "workload": "batched search, default preset: %d synthetic queries vs %d subjects (%d residues; 50%% "
                    "background, 25%% planted 30-60%% identity, 25%% reversed), BLOSUM62 11/1, E<=10, -k 10"
                    % (nq, a.search_subjects, int(sb.codes.size)),
        "unit": "queries/s", "timing": "median of 3 calls, host wall clock around saber_gpu_search (query "
                                        "codes in, hit records out)",
        "plain": {"value": round(nq / tp, 1), "hits": int(len(plain)), "regions": cp["regions"],
                  "banded_cells": cp["banded_cells"], "stages_ms": {k: round(cp[k], 1) for k in stages},
                  # the scan stage as database bytes (1 per residue) per second; it is bound by
                  # the L1 data pipe and issue (seed-table lookups), not by HBM
                  "scan_db_gb_per_s": round(int(sb.codes.size) / (cp["t_scan_ms"] * 1e-3) / 1e9, 2)
                  if cp["t_scan_ms"] > 0 else None,
                  "score_device_gcups": round(cp["banded_cells"] / (cp["t_score_device_ms"] * 1e-3) / 1e9, 1)
                  if cp["t_score_device_ms"] > 0 else None},
    }
    # two batches in flight (SearchPool: two handles, host stages of one batch
    # overlapping device stages of the other); the second batch is another
    # 2,000 seeded queries of the same model
    from saber_gb300.search import SearchPool
    qc, _, _ = synth.protein_db(a.seed + 503, a.search_queries, 1, reversed_frac=0.25, identity_range=(0.3, 0.6))
    batches = [(qb.codes, qb.offsets), (qc.codes, qc.offsets)]
    pool = None if a.no_pool else SearchPool(sb.codes, sb.offsets, SearchParams("default", masking="none"), slots=2)

    def pooled(reps=3):
        pool.raw_batches(batches)
        ts, res = [], None
        for _ in range(reps):
            t = time.perf_counter()
            res = pool.raw_batches(batches)
            ts.append(time.perf_counter() - t)
        return res, float(np.median(ts))

    nq2 = sum(len(b[1]) - 1 for b in batches)
    if not a.no_masking:
        out["masking"] = run_masking(a, dev, sb, qb)
    if not a.no_pool:
        pres, pt = pooled()
        out["plain"]["two_batches_in_flight"] = {
            "value": round(nq2 / pt, 1), "queries": nq2,
            "same_hits_as_single_handle": bool(keyset(pres[0][0]) == keyset(plain))}
    if not triage:
        return out
    if not a.no_pool:
        for se_ in pool.searchers:
            se_.dev.set_triage(model, thr)
        tres, tpt = pooled()
        for se_ in pool.searchers:
            se_.dev.set_triage(None)
    dev.set_triage(model, thr)
    try:
        call()
        tri, tt, ct = timed()
    finally:
        dev.set_triage(None)
    kp_, kt_ = keyset(plain), keyset(tri)
    total, kept = len(kp_), len(kp_ & kt_)
    out.update({
        "triage": {"value": round(nq / tt, 1), "regions_scored": ct["regions"], "regions_dropped": ct["triage_dropped"],
                   "banded_cells": ct["banded_cells"], "hits_kept": kept, "hits_plain": total,
                   "kept_frac": round(kept / max(total, 1), 5), "lost_hit_rate": round(1 - kept / max(total, 1), 5),
                   "threshold": round(thr, 4), "stages_ms": {k: round(ct[k], 1) for k in stages}},
        "speedup": round(tp / tt, 3),
        "training": {"regions": int(y.size), "positives": int(y.sum()), "steps": st["steps"],
                     "final_loss": round(st["final_loss"], 5), "pos_weight": round(st["pos_weight"], 2),
                     "collect_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 2),
                     "data": "separately seeded database (%d queries x %d subjects)" % (len(qa.offsets) - 1,
                                                                                          len(sa.offsets) - 1)},
    })
    if not a.no_pool:
        out["triage"]["two_batches_in_flight"] = {"value": round(nq2 / tpt, 1), "queries": nq2,
                                                  "same_hits_as_single_handle": bool(keyset(tres[0][0]) == kt_)}
    return out


def run_masking(a, dev, sb, qb):
    """Tantan seed masking (masking.rs) on the GPU: the search's database
    masked on the device (saber_gpu_tantan_mask_db, as the reference's scan
    database recomputes it) and the query batch through the C ABI with host
    buffers; the oracle's scalar C restatement on one host core over a
    bounded sample of the queries is the CPU baseline, and the GPU masks of
    that sample must equal the oracle's."""
    from oracle import oracle as orc
    from saber_gb300 import masking, scoring
    P = masking.TantanParams()
    b62 = scoring.matrix("BLOSUM62")

    def med(f, reps=3):
        f()
        ts, r = [], None
        for _ in range(reps):
            t = time.perf_counter()
            r = f()
            ts.append(time.perf_counter() - t)
        return r, float(np.median(ts))

    (n_db, lam), tdb = med(lambda: dev.tantan_mask_db(P, b62))
    dev.load_db_mask(None)
    (qm, _, n_q, _), tq = med(lambda: dev.tantan_mask(P, b62, qb.codes, qb.offsets))
    # CPU sample: whole queries until about cpu_seconds / 4 of oracle work
    t0, k = time.perf_counter(), 0
    offs = qb.offsets.astype(np.int64)
    budget = max(a.cpu_seconds / 4, 0.5)
    parts = []
    while k < len(offs) - 1 and time.perf_counter() - t0 < budget:
        k1 = min(k + 64, len(offs) - 1)
        parts.append(orc.tantan_mask(qb.codes[offs[k]:offs[k1]], offs[k:k1 + 1] - offs[k], b62)[0])
        k = k1
    tc = time.perf_counter() - t0
    om = np.concatenate(parts)
    nres_db, nres_q = int(sb.codes.size), int(qb.codes.size)
    return {
        "workload": "tantan protein defaults (r 0.005, e 0.05, W 50, d 0.9, BLOSUM62, lambda %.17g), posterior >= "
                    "0.5" % lam,
        "unit": "residues/s", "timing": "median of 3 calls, host wall clock",
        "database": {"residues": nres_db, "subjects": int(len(sb.offsets) - 1), "masked": n_db,
                     "ms": round(tdb * 1e3, 2), "value": round(nres_db / tdb, 1)},
        "queries": {"residues": nres_q, "queries": int(len(qb.offsets) - 1), "masked": n_q,
                    "ms": round(tq * 1e3, 2), "value": round(nres_q / tq, 1),
                    "e2e": "host codes in, host mask out"},
        "cpu_baseline": {"value": round(int(offs[k]) / tc, 1), "unit": "residues/s", "cores": 1, "kind": "port",
                         "sample": "first %d queries (%d residues, %.1f s), oracle scalar C restatement of "
                                   "masking.rs compute_body" % (k, int(offs[k]), tc)},
        "gpu_equals_oracle_on_sample": bool(np.array_equal(qm[:offs[k]], om)),
    }


def run_nn_search(a, local_rank):
    """blastn (nn) batched search: DNA queries of 1-10 kb (uniform ACGT)
    against a database of 1-10 kb subjects, 10 % of them planted homologs at
    80-95 % identity with indels at 0.01 per base; +2/-3 with SABER gaps 7/2,
    one contiguous 11-mer shape, no window filter, E <= 10, -k 10; through
    the C ABI batch engine, median of 2 calls after a warm-up."""
    from saber_gb300 import Device, synth
    from saber_gb300.search import Searcher, SearchParams
    dev = Device(local_rank)
    if a.long_steps:
        dev.long_steps = a.long_steps
    nsub = max(1, int(a.nn_bases / 5500))
    t0 = time.perf_counter()
    qs, ss, _ = synth.dna_db(a.seed + 700, a.nn_queries, nsub)
    t1 = time.perf_counter()
    se = Searcher(dev, ss.codes, ss.offsets, SearchParams.nucleotide(), gap_open=7, gap_extend=2,
                  nucleotide=(2, -3))
    cpar = se.cparams()

    def call():
        return dev.search(cpar, se.db_codes, se.db_offsets, qs.codes, qs.offsets)

    call()
    ts, out = [], None
    for _ in range(2):
        t = time.perf_counter()
        out = call()
        ts.append(time.perf_counter() - t)
    tp = float(np.median(ts))
    st = out[2]
    keys = ("seed_positions", "hits", "ungapped_extensions", "extensions_avoided", "xdrop_steps", "hsps",
            "regions", "banded_cells", "tb_tracebacks")
    print(json.dumps({"metric": "batched nn search queries/s", "nn": {
        "workload": "blastn (nn) batched search: %d DNA queries (%d bases) vs %d subjects (%d bases; 10%% planted "
                    "80-95%% identity homologs, indels 0.01), +2/-3, gaps 7/2, 11-mers, E<=10, -k 10"
                    % (len(qs.offsets) - 1, int(qs.codes.size), nsub, int(ss.codes.size)),
        "unit": "queries/s", "value": round((len(qs.offsets) - 1) / tp, 1), "s_per_search": round(tp, 3),
        "hits": int(len(out[0])), "counters": {k: int(st[k]) for k in keys if k in st},
        "stages_ms": {k: round(v, 1) for k, v in st.items() if k.startswith("t_")},
        "score_device_gcups": round(st["banded_cells"] / (st["t_score_device_ms"] * 1e-3) / 1e9, 1)
        if st.get("t_score_device_ms", 0) > 0 else None,
        "data_gen_s": round(t1 - t0, 1), "long_steps": dev.long_steps,
        "timing": "median of 2 calls, host wall clock around saber_gpu_search"}}),
        flush=True)


def run_translated(a, dev):
    """Translated searches through the library's host buffers, default
    preset, tantan on both sides: nx (DNA query records, six frames each,
    merged per record, against a protein database) and pn (protein queries
    against a DNA database stored as six frames per sequence), each on a
    seeded workload whose DNA side is back-translated proteins with random
    flanks, half on the minus strand.  The six-frame translation of the pn
    database is timed alone (kernel through the C ABI, host buffers) with
    the oracle's scalar C on one host core as its CPU baseline."""
    from oracle import oracle as orc
    from saber_gb300 import synth
    from saber_gb300.search import SearchParams
    from saber_gb300.translated import BlastxSearcher, TblastnSearcher
    from saber_gb300.translation import codon_table

    def med(f, reps=3):
        f()
        ts, r = [], None
        for _ in range(reps):
            t = time.perf_counter()
            r = f()
            ts.append(time.perf_counter() - t)
        return r, float(np.median(ts))

    out = {"metric": "translated search queries/s", "unit": "queries/s",
           "timing": "median of 3 calls, host wall clock (sequences in, merged results out)"}
    dna_q, ps, _ = synth.translated_db(a.seed + 601, a.tr_records, a.tr_subjects, "nx", planted_frac=0.1)
    bx = BlastxSearcher(dev, ps.codes, ps.offsets, SearchParams("default"))
    res, t = med(lambda: bx.search(dna_q.codes, dna_q.offsets))
    c = bx.counters
    out["nx"] = {"workload": "%d DNA query records (%d nt) x six frames vs %d protein subjects (%d residues)"
                 % (len(dna_q), int(dna_q.codes.size), len(ps), int(ps.codes.size)),
                 "value": round(len(dna_q) / t, 1), "ms": round(t * 1e3, 1),
                 "hits": int(sum(len(r) for r in res)), "regions": int(c.get("regions", 0)),
                 "frames_with_hits": sorted({h["query_frame"] for r in res for h in r})}
    pq, dna_s, _ = synth.translated_db(a.seed + 602, a.tr_records, a.tr_subjects, "pn", planted_frac=0.1)
    t0 = time.perf_counter()
    tn = TblastnSearcher(dev, dna_s.codes, dna_s.offsets, SearchParams("default"))
    tload = time.perf_counter() - t0
    res, t = med(lambda: tn.search(pq.codes, pq.offsets))
    c = tn.counters
    out["pn"] = {"workload": "%d protein queries vs %d DNA sequences (%d nt, %d frame residues)"
                 % (len(pq), len(dna_s), int(dna_s.codes.size), int(tn.se.db_codes.size)),
                 "value": round(len(pq) / t, 1), "ms": round(t * 1e3, 1), "database_setup_s": round(tload, 2),
                 "hits": int(sum(len(r) for r in res)), "regions": int(c.get("regions", 0)),
                 "frames_with_hits": sorted({h["subject_frame"] for r in res for h in r})}
    aa = codon_table()
    (tc, to), tt = med(lambda: dev.translate6(dna_s.codes, dna_s.offsets, aa))
    k = min(len(dna_s), 2000)
    t0 = time.perf_counter()
    oc, oo = orc.translate6(dna_s.codes[:int(dna_s.offsets[k])], dna_s.offsets[:k + 1], aa)
    tcpu = time.perf_counter() - t0
    nt_bytes = int(dna_s.codes.size)
    out["translate6"] = {
        "workload": "six frames of %d DNA sequences (%d nt -> %d residues)" % (len(dna_s), nt_bytes, int(tc.size)),
        "unit": "nt/s", "value": round(nt_bytes / tt, 1), "ms": round(tt * 1e3, 2),
        "e2e": "host nucleotides in, host frames out",
        "equals_oracle_on_sample": bool(np.array_equal(tc[:int(to[6 * k])], oc)),
        "cpu_baseline": {"value": round(int(dna_s.offsets[k]) / tcpu, 1), "unit": "nt/s", "cores": 1,
                         "kind": "port", "sample": "first %d sequences (%d nt), oracle scalar C restatement of "
                                                   "translate_codes" % (k, int(dna_s.offsets[k]))}}
    return out


def run_search_only(a, local_rank):
    from saber_gb300 import Device
    dev = Device(local_rank)
    print(json.dumps({"metric": "batched search queries/s", "search": run_search(a, dev)}), flush=True)


def run_ours(a, rank, world, local_rank):
    import torch
    from saber_gb300 import Device
    from saber_gb300.gpu import JOB_DTYPE
    from saber_gb300.scoring import matrix
    from saber_gb300.replicas import rank_seed, whole_job
    torch.cuda.set_device(local_rank)
    seed = rank_seed(a.seed, rank)
    qs, ss, planted, bias, jobs = workload(seed, a.queries, a.subjects, a.jobs)
    mat = matrix("BLOSUM62")
    dev = Device(local_rank)
    dev.strip_rows = a.strip_rows
    dev.set_scheme(mat, 11, 1)
    dev.load_db(ss.codes, ss.offsets)
    dev.load_queries(qs.codes, qs.offsets, bias)
    stream = torch.cuda.ExternalStream(dev.stream, device=local_rank)
    d_jobs = torch.from_numpy(jobs.view(np.uint8).copy()).to("cuda:%d" % local_rank)
    d_scores = torch.empty(jobs.size, dtype=torch.int32, device="cuda:%d" % local_rank)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda:%d" % local_rank)
    dpx_peak, i32_peak = dev.probe_int_peak()

    def step_dev():
        return dev.score_band_jobs_dev(d_jobs.data_ptr(), jobs.size, d_scores.data_ptr())

    for _ in range(a.warmup):
        step_dev()
    torch.cuda.synchronize()
    tuned = None
    if not a.no_autotune:
        from saber_gb300.tune import autotune_scoring
        tuned = autotune_scoring(dev, d_jobs, d_scores)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(local_rank)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    tot_ms, fast_ms, cells, fast_cells, launches, lib_launches, rescored = 0.0, 0.0, 0, 0, 0, 0, 0
    for _ in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        torch.cuda.synchronize()
        ev0.record(stream)
        st = step_dev()
        ev1.record(stream)
        ev1.synchronize()
        tot_ms += ev0.elapsed_time(ev1)
        fast_ms += st["t_fast_ms"]
        cells += st["banded_cells"]
        fast_cells += st["fast_cells"]
        launches += st["kernel_launches"]
        lib_launches += st["library_launches"]
        rescored += st["i16_rescored"]
    torch.cuda.synchronize()
    clk = clocks.stop()
    all_cells, max_ms = whole_job(cells, tot_ms, world)
    value = all_cells / (max_ms * 1e-3) / 1e9

    # end to end: pinned host jobs in, scores out, through the C ABI
    h_jobs = torch.from_numpy(jobs.view(np.uint8).copy()).pin_memory()
    h_scores = torch.empty(jobs.size, dtype=torch.int32).pin_memory()
    for _ in range(max(1, a.warmup)):
        dev.score_band_jobs_ptr(h_jobs.data_ptr(), jobs.size, h_scores.data_ptr())
    e2e_s = 0.0
    for _ in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev.score_band_jobs_ptr(h_jobs.data_ptr(), jobs.size, h_scores.data_ptr())
        e2e_s += time.perf_counter() - t0
    _, max_e2e_s = whole_job(cells, e2e_s, world)
    e2e = all_cells / max_e2e_s / 1e9
    same = bool(np.array_equal(h_scores.numpy(), d_scores.cpu().numpy()))

    if rank != 0:
        return
    fast_s = fast_ms * 1e-3
    achieved = fast_cells * ALGO_OPS_PER_CELL / fast_s / 1e12 if fast_s > 0 else None
    peak = dpx_peak * 2 / 1e12
    cfg = config_dict(a, world)
    cfg["strip_rows"] = dev.strip_rows
    cfg["pair_steps"] = dev.pair_steps
    if tuned is not None:
        cfg["autotune"] = tuned["candidates"]
    out = {"metric": METRIC, "value": round(value, 2), "unit": "GCUPS", "n_gpus": world, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": round(tot_ms / a.steps, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int16 (int32 rescore)", "data": "synthetic",
           "config": cfg,
           "e2e": {"value": round(e2e, 2), "unit": "GCUPS", "h2d_bytes_per_step": int(jobs.nbytes),
                   "d2h_bytes_per_step": int(jobs.size * 4), "matches_device_path": same},
           "roofline": {"bound": "int", "kernel": "k_band_fast",
                        "achieved": round(achieved, 3) if achieved else None, "peak": round(peak, 3),
                        "unit": "Tops/s", "frac": round(achieved / peak, 3) if achieved else None,
                        "traffic": None,
                        "basis": "11 algorithmic int ops per in-band cell; peak = measured DPX s16x2 "
                                 "lane-instructions/s x 2 (probe kernel, this run)",
                        "fast_kernel_gcups": round(fast_cells / fast_s / 1e9, 2) if fast_s > 0 else None,
                        "fast_share_of_step": round(fast_ms / tot_ms, 3) if tot_ms else None,
                        "int32_max_lane_ops_per_s": i32_peak},
           "clocks": clk, "gpu_launches": int(launches),
           "library_launches": int(lib_launches), "i16_rescored": int(rescored),
           "cells_per_step": int(cells // max(a.steps, 1))}
    if not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(qs, ss, bias, jobs, mat, a.cpu_seconds)
    # the search and translated sections run at N = 1 only (the other ranks
    # would wait at the barrier meanwhile)
    if not a.no_search and world == 1:
        out["search"] = run_search(a, dev)
    if not a.no_translated and world == 1:
        out["translated"] = run_translated(a, dev)
    print(json.dumps(out), flush=True)


def main():
    a = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        torch.distributed.init_process_group("gloo")
    if a.impl == "reference":
        run_reference(a, rank, world)
    elif a.nn_search:
        if rank == 0:
            run_nn_search(a, local_rank)
    elif a.translated:
        if rank == 0:
            from saber_gb300 import Device
            print(json.dumps(run_translated(a, Device(local_rank))), flush=True)
    elif a.search_only:
        if rank == 0:
            run_search_only(a, local_rank)
    else:
        run_ours(a, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
