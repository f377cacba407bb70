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
K_BAND_FAST_DRAM_BYTES = 1.73e9 + 2.34e9  # dram__bytes_read.sum + dram__bytes_write.sum, one launch (int8 profile)


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
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle checks of the microbench scores")
    ap.add_argument("--no-config0", action="store_true", help="skip the 64 x 20,000 blastp search and its oracle check")
    ap.add_argument("--parity-queries", type=int, default=100,
                    help="batched search: queries whose hits are checked against the oracle pipeline")
    ap.add_argument("--strip-rows", type=int, default=16, help="rows per strip of the int16 kernel (8 or 16)")
    ap.add_argument("--no-autotune", action="store_true", help="keep --strip-rows and the default pairing")
    ap.add_argument("--no-search", action="store_true", help="skip the batched-search / learned-triage lines")
    ap.add_argument("--search-only", action="store_true",
                    help="only the batched-search section (printed as its own JSON line)")
    ap.add_argument("--no-triage", action="store_true", help="search section without the learned triage")
    ap.add_argument("--triage-recall", type=float, default=0.998,
                    help="share of the held-out positive regions the triage threshold keeps")
    ap.add_argument("--triage-margin", type=float, default=0.0, help="logits below that threshold point")
    ap.add_argument("--no-pool", action="store_true", help="search section without the two-batches-in-flight lines")
    ap.add_argument("--no-masking", action="store_true", help="search section without the tantan masking line")
    ap.add_argument("--search-queries", type=int, default=11000)
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
    ap.add_argument("--nn-parity-queries", type=int, default=10,
                    help="blastn: queries whose hits are checked against the oracle pipeline")
    ap.add_argument("--no-nn", action="store_true", help="skip the blastn (nn) batched-search section")
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


def simd_whole_workload(qs, ss, bias, jobs, matrix, min_seconds, max_runs=5):
    """The SIMD-class restatement of the reference's CPU scoring (oracle/
    simd_band.cpp) over the whole workload on all host cores: one warm run,
    then timed runs until min_seconds have passed (at most max_runs).
    Returns (scores, GCUPS of the median run, counters, run seconds, threads)."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    scores, ct = orc.simd_score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, jobs, matrix, 11, 1, threads)
    ts = []
    while len(ts) < max_runs and (not ts or sum(ts) < min_seconds):
        t0 = time.perf_counter()
        orc.simd_score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, jobs, matrix, 11, 1, threads)
        ts.append(time.perf_counter() - t0)
    dt = float(np.median(ts))
    return scores, ct["cells"] / dt / 1e9, ct, ts, threads


def cpu_baseline(qs, ss, bias, jobs, matrix, seconds):
    """The reference's CPU scoring restated with its vector kernels (score_banded_many: 32-lane
    8-bit batches, 16-bit rows, 32-bit re-runs; NEON on the aarch64 host) over all the jobs."""
    scores, gcups, ct, ts, threads = simd_whole_workload(qs, ss, bias, jobs, matrix, seconds)
    out = {"value": round(gcups, 3), "unit": "GCUPS", "cores": threads, "kind": "port",
           "per_core_gcups": round(gcups / threads, 3),
           "reference_recorded_per_thread_gcups": "3.4-4.2 (16-bit), 12.8 (8-bit batches), AVX2 at 2.8 GHz",
           "sample": "all %d jobs (%.3g cells) per run, median of %d runs (%.2f s each), SIMD-class restatement of "
                     "score_banded_many (band_simd8.rs batch_u8 + banded_simd.rs banded_avx2_16 + 32-bit re-run) "
                     "on %d threads; %d jobs through 8-bit batches (%d re-scored), %d in 16 bits, %d re-run in 32 bits"
                     % (jobs.size, ct["cells"], len(ts), float(np.median(ts)), threads, ct["u8_jobs"],
                        ct["u8_overflows"], ct["i16_jobs"], ct["i32_jobs"])}
    return out, scores


def parity_config1(qs, ss, bias, jobs, matrix, gpu_scores, simd_scores):
    """Every GPU score of the microbench against the scalar oracle (banded_score_scalar,
    banded.rs:134-224), all jobs, all host threads."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    want, cells = orc.score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, jobs, matrix, 11, 1, threads)
    dt = time.perf_counter() - t0
    bad = np.nonzero(gpu_scores != want)[0]
    return {"config": "sw-scoring-microbench", "jobs": int(jobs.size), "cells": int(cells),
            "oracle": "scalar C restatement of banded_score_scalar, every job (%.1f s on %d threads)" % (dt, threads),
            "mismatches": int(bad.size), "first_mismatches": [int(x) for x in bad[:5]],
            "simd_baseline_mismatches": int(np.count_nonzero(simd_scores != want)) if simd_scores is not None
            else None}


def run_reference(a, rank, world):
    """The reference arm: the reference's CPU scoring restated with its vector
    kernels (oracle/simd_band.cpp; the reference itself is Rust and cannot be
    built here) over the whole microbench workload each step, all host threads."""
    if rank != 0:
        return
    from saber_gb300.scoring import matrix
    from oracle import oracle as orc
    qs, ss, planted, bias, jobs = workload(a.seed, a.queries, a.subjects, a.jobs)
    mat = matrix("BLOSUM62")
    threads = os.cpu_count() or 1
    tot_cells, tot_t = 0, 0.0
    ct = None
    for step in range(a.warmup + a.steps):
        t0 = time.perf_counter()
        _, ct = orc.simd_score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, jobs, mat, 11, 1, threads)
        dt = time.perf_counter() - t0
        if step >= a.warmup:
            tot_cells += ct["cells"]
            tot_t += dt
    v = tot_cells / tot_t / 1e9
    out = {"metric": METRIC, "impl": "reference", "value": round(v, 3), "unit": "GCUPS", "n_gpus": world,
           "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(tot_t / a.steps * 1e3, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8 / i16 (i32 re-run)",
           "data": "synthetic", "config": config_dict(a, world),
           "cpu_baseline": {"value": round(v, 3), "unit": "GCUPS", "cores": threads, "kind": "port",
                            "per_core_gcups": round(v / threads, 3),
                            "sample": "all %d jobs of the workload every step; SIMD-class restatement of "
                                      "score_banded_many (band_simd8.rs batch_u8, banded_simd.rs banded_avx2_16, "
                                      "32-bit re-run) on NEON; the reference is Rust and cannot be built here "
                                      "(no cargo)" % jobs.size},
           "e2e": {"value": round(v, 3), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_config0(a, dev):
    """blastp (pp), default preset, plain method: 64 synthetic queries against
    20,000 subjects, seed 0 (log-normal lengths, background residues, 10 %
    planted homologs at about 40 % identity), BLOSUM62 11/1, E <= 10, -k 10,
    tantan masking of the database (once, at load) and of the queries (every
    call) on the GPU, through Searcher.search (host query codes in, hits out).
    Parity: every m8 row must equal the oracle pipeline's (tantan masks by
    oracle/tantan.c, scan, scores and tracebacks by the C oracle, statistics
    and m8 formatting restated in Python), which is also the CPU baseline
    (query masking + search, all host threads)."""
    from oracle import engine as oeng
    from oracle import oracle as orc
    from saber_gb300 import synth
    from saber_gb300.search import Searcher, SearchParams, m8_row
    from saber_gb300.stats import gapped_protein
    qs, ss, _ = synth.protein_db(0, 64, 20000)
    se = Searcher(dev, ss.codes, ss.offsets, SearchParams("default"))
    se.search(qs.codes, qs.offsets)
    ts, hits = [], None
    for _ in range(5):
        t0 = time.perf_counter()
        hits = se.search(qs.codes, qs.offsets)
        ts.append(time.perf_counter() - t0)
    tg = float(np.median(ts))
    got = [m8_row("q%d" % qi, "s%d" % h["subject"], h) for qi, hl in enumerate(hits) for h in hl]
    threads = os.cpu_count() or 1
    dbm = orc.tantan_mask(ss.codes, ss.offsets, se.matrix)[0]
    t0 = time.perf_counter()
    qm = orc.tantan_mask(qs.codes, qs.offsets, se.matrix)[0]
    want_h = oeng.search_batch(ss.codes, ss.offsets, qs.codes, qs.offsets, se.p, se.matrix, 11, 1,
                               gapped_protein("BLOSUM62", 11, 1), se.scan_params, dbm, qm, threads=threads)
    tc = time.perf_counter() - t0
    want = [oeng.m8_line("q%d" % qi, "s%d" % h["subject"], h) for qi, hl in enumerate(want_h) for h in hl]
    diff = sum(1 for x, y in zip(got, want) if x != y) + abs(len(got) - len(want))
    nq = len(qs)
    return {"workload": "blastp default preset, plain: %d queries (%d residues) vs %d subjects (%d residues), seed 0, "
                        "tantan on both sides" % (nq, int(qs.codes.size), len(ss), int(ss.codes.size)),
            "unit": "queries/s", "value": round(nq / tg, 1), "ms": round(tg * 1e3, 2),
            "timing": "median of 5 calls of Searcher.search (query masking, scan, scores, tracebacks, hits)",
            "hits": len(got), "database_residues_masked": int(se.db_residues_masked),
            "cpu_baseline": {"value": round(nq / tc, 2), "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": "the whole batch (%.1f s): oracle pipeline (tantan, scan, banded scores, "
                                       "tracebacks in C on %d threads; engine steps in Python)" % (tc, threads)},
            "parity": {"config": "blastp 64 x 20,000, seed 0", "m8_rows": len(got), "oracle_m8_rows": len(want),
                       "mismatching_rows": int(diff), "m8_identical": got == want}}


def run_search(a, dev):
    """Batched full search and learned triage on the batched-search workload:
    a.search_queries (default 11,000) synthetic queries against a.search_subjects
    (default 500,000) subjects, about 150 M residues (50 % background, 25 %
    planted homologs at 30-60 % identity, 25 % reversed decoys), default preset
    with masking none (the oracle legs then see the same seeds), through the C
    ABI's batch engine (saber_gpu_search: query codes in, hit records out).

    plain: the whole query set as one batch, and as two half batches in
    flight on two handles (SearchPool).  parity: the first a.parity_queries
    queries' hits from the whole-batch call against the oracle pipeline on
    those queries and the whole database (m8 rows), which also gives the CPU
    queries/s.  triage: the MLP trained on the GPU from plain-search labels of
    a separately seeded database of the same size, its threshold calibrated on
    the labels of other queries (held out from training), then the same
    batches with the triage installed: hits kept with identical scores and
    E-values, regions and cells saved, queries/s."""
    from oracle import engine as oeng
    from saber_gb300 import synth
    from saber_gb300 import triage as tr
    from saber_gb300.search import Searcher, SearchParams, SearchPool, hits_from_records, m8_row
    from saber_gb300.stats import gapped_protein
    triage = not a.no_triage
    nq = a.search_queries
    P = SearchParams("default", masking="none")
    out = {}
    if triage:
        tc0 = time.perf_counter()
        ntr, ncal = max(nq // 2, 1), max(nq // 5, 1)
        qa, sa, _ = synth.protein_db(a.seed + 501, ntr + ncal, a.search_subjects, reversed_frac=0.25,
                                     identity_range=(0.3, 0.6))
        offs = qa.offsets.astype(np.int64)
        se = Searcher(dev, sa.codes, sa.offsets, P)
        rows, y, _ = tr.collect(se, qa.codes[:offs[ntr]], offs[:ntr + 1])
        rows_c, y_c, _ = tr.collect(se, qa.codes[offs[ntr]:], offs[ntr:] - offs[ntr])
        tc1 = time.perf_counter()
        # all positives and a seeded sample of the negatives (at most 3 M rows)
        rng = np.random.default_rng(a.seed + 7)
        neg = np.nonzero(y == 0)[0]
        keep_neg = neg if neg.size + int(y.sum()) <= 3_000_000 else \
            np.sort(rng.choice(neg, 3_000_000 - int(y.sum()), replace=False))
        sel = np.sort(np.concatenate([np.nonzero(y > 0)[0], keep_neg]))
        model, st = tr.train(dev, rows[sel], y[sel], seed=a.seed + 1)
        tc2 = time.perf_counter()
        z_c = dev.triage_predict(model, rows_c)
        thr = tr.threshold_for_recall(z_c, y_c, recall=a.triage_recall, margin=a.triage_margin)
        cal = {"regions": int(y_c.size), "positives": int(y_c.sum()),
               "positives_kept": int(np.count_nonzero(z_c[y_c > 0] >= thr)),
               "regions_dropped_frac": round(float(np.mean(z_c < thr)), 5),
               "recall_target": a.triage_recall, "margin": a.triage_margin,
               # the held-out trade-off: regions dropped at other recall targets (no margin)
               "curve": [{"recall": r, "threshold": round(t_, 4), "regions_dropped_frac": round(float(np.mean(z_c < t_)), 5)}
                         for r in (0.99, 0.995, 0.996, 0.997, 0.998, 0.999)
                         for t_ in [tr.threshold_for_recall(z_c, y_c, recall=r, margin=0.0)]]}
        del rows, rows_c
    qb, sb, _ = synth.protein_db(a.seed + 502, nq, a.search_subjects, reversed_frac=0.25, identity_range=(0.3, 0.6))
    if a.long_steps:
        dev.long_steps = a.long_steps
    se2 = Searcher(dev, sb.codes, sb.offsets, P)
    cpar = se2.cparams()

    def call():
        return dev.search(cpar, se2.db_codes, se2.db_offsets, qb.codes, qb.offsets)

    call()  # warm: database state, scratch sizes

    def timed(reps=3):
        ts, res = [], None
        for _ in range(reps):
            t = time.perf_counter()
            res = call()
            ts.append(time.perf_counter() - t)
        return res, float(np.median(ts))

    def keyset(hits, qoff=0):
        return {(int(r["query"]) + qoff, int(r["subject"]), int(r["score"]), int(r["q_start"]), int(r["q_end"]),
                 int(r["s_start"]), int(r["s_end"]), float(r["evalue"])) for r in hits}

    plain, tp = timed()
    cp = plain[2]
    stages = ("t_scan_ms", "t_triage_ms", "t_plan_ms", "t_score_ms", "t_finish_ms", "t_total_ms",
              "t_score_calls_ms", "t_score_device_ms", "t_finish_tb_ms", "t_score_build_ms", "t_score_stage2_ms",
              "t_finish_order_ms")
    out.update({
        "workload": "batched search, default preset: %d synthetic queries vs %d subjects (%d residues; 50%% "
                    "background, 25%% planted 30-60%% identity, 25%% reversed), BLOSUM62 11/1, E<=10, -k 10"
                    % (nq, a.search_subjects, int(sb.codes.size)),
        "unit": "queries/s", "timing": "median of 3 calls, host wall clock around saber_gpu_search (query "
                                        "codes in, hit records out)",
        "plain": {"value": round(nq / tp, 1), "hits": int(len(plain[0])), "regions": cp["regions"],
                  "banded_cells": cp["banded_cells"], "stages_ms": {k: round(cp[k], 1) for k in stages},
                  "counters": {k: int(cp[k]) for k in ("seed_positions", "hits", "hits_filtered",
                                                       "ungapped_extensions", "xdrop_steps", "hsps") if k in cp},
                  # the scan stage as database bytes (1 per residue) per second; it is bound by
                  # the L1 data pipe and issue (seed-table lookups), not by HBM
                  "scan_db_gb_per_s": round(int(sb.codes.size) / (cp["t_scan_ms"] * 1e-3) / 1e9, 2)
                  if cp["t_scan_ms"] > 0 else None,
                  "score_device_gcups": round(cp["banded_cells"] / (cp["t_score_device_ms"] * 1e-3) / 1e9, 1)
                  if cp["t_score_device_ms"] > 0 else None},
    })
    # parity sample: the first queries' hits of the whole-batch call against the oracle pipeline
    k = min(a.parity_queries, nq)
    if k > 0:
        threads = os.cpu_count() or 1
        qo = qb.offsets.astype(np.int64)
        got_h = hits_from_records(plain[0], plain[1], nq, queries=k)
        t0 = time.perf_counter()
        want_h = oeng.search_batch(sb.codes, sb.offsets, qb.codes[:qo[k]], qo[:k + 1], P, se2.matrix, 11, 1,
                                   gapped_protein("BLOSUM62", 11, 1), se2.scan_params, None, None, threads=threads)
        tc = time.perf_counter() - t0
        got = [m8_row("q%d" % qi, "s%d" % h["subject"], h) for qi, hl in enumerate(got_h) for h in hl]
        want = [oeng.m8_line("q%d" % qi, "s%d" % h["subject"], h) for qi, hl in enumerate(want_h) for h in hl]
        diff = sum(1 for x, y_ in zip(got, want) if x != y_) + abs(len(got) - len(want))
        out["parity"] = {"config": "batched search, first %d of %d queries against the whole database" % (k, nq),
                         "m8_rows": len(got), "oracle_m8_rows": len(want), "mismatching_rows": int(diff),
                         "m8_identical": got == want}
        out["cpu_baseline"] = {"value": round(k / tc, 2), "unit": "queries/s", "cores": threads, "kind": "port",
                               "sample": "first %d queries against the whole database (%.1f s): oracle pipeline "
                                         "(scan, banded scores and tracebacks in C on %d threads, engine steps "
                                         "in Python)" % (k, tc, threads)}
    # two half batches in flight on two handles
    qo = qb.offsets.astype(np.int64)
    h = nq // 2
    batches = [(qb.codes[:qo[h]], qo[:h + 1]), (qb.codes[qo[h]:], qo[h:] - qo[h])]
    pool = None if a.no_pool else SearchPool(sb.codes, sb.offsets, P, slots=2)

    def pooled(reps=3):
        pool.raw_batches(batches)
        ts, res = [], None
        for _ in range(reps):
            t = time.perf_counter()
            res = pool.raw_batches(batches)
            ts.append(time.perf_counter() - t)
        return res, float(np.median(ts))

    def pooled_keys(res):
        return keyset(res[0][0]) | keyset(res[1][0], h)

    if not a.no_masking:
        out["masking"] = run_masking(a, dev, sb, qb)
    tpp = None
    if pool is not None:
        pres, tpp = pooled()
        out["plain"]["two_batches_in_flight"] = {
            "value": round(nq / tpp, 1), "queries": nq, "batches": 2,
            "same_hits_as_whole_batch": bool(pooled_keys(pres) == keyset(plain[0]))}
    if not triage:
        return out
    tpt = None
    if pool is not None:
        for se_ in pool.searchers:
            se_.dev.set_triage(model, thr)
        tres, tpt = pooled()
        for se_ in pool.searchers:
            se_.dev.set_triage(None)
    dev.set_triage(model, thr)
    try:
        call()
        tri, tt = timed()
    finally:
        dev.set_triage(None)
    ct = tri[2]
    kp_, kt_ = keyset(plain[0]), keyset(tri[0])
    total, kept = len(kp_), len(kp_ & kt_)
    out.update({
        "triage": {"value": round(nq / tt, 1), "regions_scored": ct["regions"], "regions_dropped": ct["triage_dropped"],
                   "banded_cells": ct["banded_cells"], "hits_kept": kept, "hits_plain": total,
                   "kept_frac": round(kept / max(total, 1), 5), "lost_hit_rate": round(1 - kept / max(total, 1), 5),
                   "extra_hits": len(kt_ - kp_), "threshold": round(thr, 4), "calibration": cal,
                   "stages_ms": {k_: round(ct[k_], 1) for k_ in stages}},
        "speedup": round(tp / tt, 3),
        "training": {"regions": int(y.size), "positives": int(y.sum()), "rows_trained": int(sel.size),
                     "steps": st["steps"], "final_loss": round(st["final_loss"], 5),
                     "pos_weight": round(st["pos_weight"], 2), "collect_s": round(tc1 - tc0, 1),
                     "train_s": round(tc2 - tc1, 2),
                     "data": "separately seeded database (%d subjects, %d residues): %d training queries, %d "
                             "held-out calibration queries" % (len(sa), int(sa.codes.size), ntr, ncal)},
    })
    if tpt is not None:
        out["triage"]["two_batches_in_flight"] = {"value": round(nq / tpt, 1), "queries": nq, "batches": 2,
                                                  "same_hits_as_whole_batch": bool(pooled_keys(tres) == kt_)}
        out["speedup_two_batches_in_flight"] = round(tpp / tpt, 3)
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


def run_nn(a, local_rank):
    """blastn (nn) batched search: a.nn_queries DNA queries of 1-10 kb
    (uniform ACGT) against about a.nn_bases bases of 1-10 kb subjects, 10 % of
    them planted homologs at 80-95 % identity with indels at 0.01 per base;
    +2/-3 with SABER gaps 7/2, one contiguous 11-mer shape, no window filter,
    E <= 10, -k 10; through the C ABI batch engine (query codes in, hit
    records out), median of 2 calls after a warm-up, on a handle of its own
    (closed afterwards).  Parity: the first a.nn_parity_queries queries' hits
    of the whole-batch call against the oracle pipeline on those queries and
    the whole database (m8 rows), which also gives the CPU queries/s."""
    from oracle import engine as oeng
    from saber_gb300 import Device, synth
    from saber_gb300.search import Searcher, SearchParams, hits_from_records, m8_row
    from saber_gb300.stats import gapped_nucleotide
    nsub = max(1, int(a.nn_bases / 5500))
    t0 = time.perf_counter()
    qs, ss, _ = synth.dna_db(a.seed + 700, a.nn_queries, nsub)
    t1 = time.perf_counter()
    P = SearchParams.nucleotide()
    with Device(local_rank) as dev:
        if a.long_steps:
            dev.long_steps = a.long_steps
        se = Searcher(dev, ss.codes, ss.offsets, P, gap_open=7, gap_extend=2, nucleotide=(2, -3))
        cpar = se.cparams()

        def call():
            return dev.search(cpar, se.db_codes, se.db_offsets, qs.codes, qs.offsets)

        call()
        ts, res = [], None
        for _ in range(2):
            t = time.perf_counter()
            res = call()
            ts.append(time.perf_counter() - t)
        tp = float(np.median(ts))
        st = res[2]
        nq = len(qs.offsets) - 1
        keys = ("seed_positions", "hits", "ungapped_extensions", "extensions_avoided", "xdrop_steps", "hsps",
                "regions", "banded_cells", "tb_tracebacks")
        out = {
            "workload": "blastn (nn) batched search: %d DNA queries (%d bases) vs %d subjects (%d bases; 10%% planted "
                        "80-95%% identity homologs, indels 0.01), +2/-3, gaps 7/2, 11-mers, E<=10, -k 10"
                        % (nq, int(qs.codes.size), nsub, int(ss.codes.size)),
            "unit": "queries/s", "value": round(nq / tp, 1), "s_per_search": round(tp, 3),
            "hits": int(len(res[0])), "counters": {k: int(st[k]) for k in keys if k in st},
            "stages_ms": {k: round(v, 1) for k, v in st.items() if k.startswith("t_")},
            "score_device_gcups": round(st["banded_cells"] / (st["t_score_device_ms"] * 1e-3) / 1e9, 1)
            if st.get("t_score_device_ms", 0) > 0 else None,
            "data_gen_s": round(t1 - t0, 1), "long_steps": dev.long_steps,
            "timing": "median of 2 calls, host wall clock around saber_gpu_search"}
        k = min(a.nn_parity_queries, nq)
        if k > 0:
            threads = os.cpu_count() or 1
            qo = qs.offsets.astype(np.int64)
            got_h = hits_from_records(res[0], res[1], nq, queries=k)
            t0 = time.perf_counter()
            want_h = oeng.search_batch(ss.codes, ss.offsets, qs.codes[:qo[k]], qo[:k + 1], P, se.matrix, 7, 2,
                                       gapped_nucleotide(2, -3, 7, 2), se.scan_params, None, None, is_protein=False,
                                       threads=threads)
            tc = time.perf_counter() - t0
            got = [m8_row("q%d" % qi, "s%d" % h["subject"], h) for qi, hl in enumerate(got_h) for h in hl]
            want = [oeng.m8_line("q%d" % qi, "s%d" % h["subject"], h) for qi, hl in enumerate(want_h) for h in hl]
            diff = sum(1 for x, y in zip(got, want) if x != y) + abs(len(got) - len(want))
            out["parity"] = {"config": "blastn, first %d of %d queries against the whole database" % (k, nq),
                             "m8_rows": len(got), "oracle_m8_rows": len(want), "mismatching_rows": int(diff),
                             "m8_identical": got == want}
            out["cpu_baseline"] = {"value": round(k / tc, 3), "unit": "queries/s", "cores": threads, "kind": "port",
                                   "sample": "first %d queries against the whole database (%.1f s): oracle pipeline "
                                             "(scan, banded scores and tracebacks in C on %d threads, engine steps "
                                             "in Python)" % (k, tc, threads)}
    return out


def run_nn_search(a, local_rank):
    print(json.dumps({"metric": "batched nn search queries/s", "nn": run_nn(a, local_rank)}), flush=True)


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
    pipe_rates = dev.probe_pipe_rates()

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
    prof8 = 0
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
        prof8 = int(st["prof8"])
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
    cfg["long_steps"] = dev.long_steps
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
                        # DRAM bytes (read + write) of one k_band_fast<16> launch on this workload, from one
                        # ncu capture of the same command (profiles/k_band_fast16_traffic_1M.md)
                        "traffic": K_BAND_FAST_DRAM_BYTES if a.jobs == 1_000_000 and a.seed == 0 else None,
                        "traffic_unit": "bytes per launch",
                        # jobs, scores, the database, the query profiles (25 codes x 1 or 2 bytes per residue)
                        "algorithmic_bytes": int(jobs.nbytes + jobs.size * 4 + ss.codes.size
                                                 + (25 if prof8 else 50) * qs.codes.size),
                        "profile": "int8" if prof8 else "int16",
                        "basis": "11 algorithmic int ops per in-band cell; peak = measured DPX s16x2 "
                                 "lane-instructions/s x 2 (probe kernel, this run)",
                        "fast_kernel_gcups": round(fast_cells / fast_s / 1e9, 2) if fast_s > 0 else None,
                        "fast_share_of_step": round(fast_ms / tot_ms, 3) if tot_ms else None,
                        "int32_max_lane_ops_per_s": i32_peak,
                        # the packed cell pair (two cells): 3 DPX + 1 prmt + 0.5 vimax3 on the ALU pipe, 2 vadd2
                        # on the FMA pipe; each instruction's measured rate (alone, and add-max beside vadd2)
                        "cell_pair_instructions": {"alu_pipe": 4.5, "fma_pipe": 2.0},
                        "pipe_rates_lane_instr_per_s": {k: round(v, -8) for k, v in pipe_rates.items()}},
           "clocks": clk, "gpu_launches": int(launches),
           "library_launches": int(lib_launches), "i16_rescored": int(rescored),
           "cells_per_step": int(cells // max(a.steps, 1))}
    simd_scores = None
    if not a.no_cpu_baseline:
        out["cpu_baseline"], simd_scores = cpu_baseline(qs, ss, bias, jobs, mat, a.cpu_seconds)
    if not a.no_parity:
        out["parity"] = {"sw_microbench": parity_config1(qs, ss, bias, jobs, mat, d_scores.cpu().numpy(),
                                                         simd_scores)}
    if not a.no_config0 and world == 1:
        out["blastp_64x20000"] = run_config0(a, dev)
        if "parity" in out:
            out["parity"]["blastp_64x20000"] = out["blastp_64x20000"]["parity"]
    # the search and translated sections run at N = 1 only (the other ranks
    # would wait at the barrier meanwhile)
    if not a.no_search and world == 1:
        out["search"] = run_search(a, dev)
        if "parity" in out and "parity" in out["search"]:
            out["parity"]["batched_search_sample"] = out["search"]["parity"]
    if not a.no_translated and world == 1:
        out["translated"] = run_translated(a, dev)
    if not a.no_nn and world == 1:
        dev.close()
        out["blastn_2000x500M"] = run_nn(a, local_rank)
        if "parity" in out and "parity" in out["blastn_2000x500M"]:
            out["parity"]["blastn_sample"] = out["blastn_2000x500M"]["parity"]
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
