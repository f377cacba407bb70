"""GPU parity tests of the banded traceback (banded_align_until + walk) and of
the widening traceback driver: alignments (score, coordinates, CIGAR runs,
cells) bit-exact against the oracle."""
import numpy as np
import pytest

from oracle import engine as oeng
from oracle import oracle as orc
from saber_gb300 import synth
from saber_gb300.gpu import ALIGN_JOB_DTYPE, TB_JOB_DTYPE
from saber_gb300.scoring import matrix
from tests.refgen import Lcg, mutate, rand_seq

pytestmark = pytest.mark.gpu
B62 = matrix("BLOSUM62")


def _same(a, b):
    if a is None or b is None:
        return a is None and b is None
    return all(a[k] == b[k] for k in ("score", "q_start", "q_end", "s_start", "s_end", "ops", "cells"))


def test_align_matches_oracle_on_reference_cases(dev):
    """banded.rs:645-671 cases (LCG 2024): five gap schemes, with and without
    bias, random/related pairs, bands (lo, hi), full and offset."""
    r = Lcg(2024)
    for t in range(240):
        go, ge = [(11, 1), (10, 2), (6, 3), (15, 1), (8, 8)][t % 5]
        la = 1 + r.next(700 if t % 7 == 0 else 220)
        a = rand_seq(r, la)
        lb = 1 + r.next(220)
        b = mutate(r, a) if t % 2 == 0 else rand_seq(r, lb)
        bias = np.array([r.next(9) - 4 for _ in range(len(a))], np.int8)
        bo = bias if t % 3 == 0 else None
        lo = -r.next(60)
        hi = r.next(60) + (300 if t % 5 == 0 else 0)
        dev.set_scheme(B62, go, ge)
        for band in [(lo, hi), (-len(a), len(b)), (5, 40)]:
            want = orc.banded_align(a, b, bo, B62, go, ge, band[0], band[1])
            got = dev.banded_align_one(a, bo, b, band[0], band[1])
            assert _same(got, want), (t, band, got, want)


def test_stop_at_gives_same_alignment_fewer_cells(dev):
    # banded.rs:733-755 (LCG 5)
    r = Lcg(5)
    dev.set_scheme(B62, 11, 1)
    for _ in range(60):
        la = 20 + r.next(300)
        a = rand_seq(r, la)
        b = np.concatenate([rand_seq(r, 40), mutate(r, a[:la // 2]), rand_seq(r, 40)])
        full = orc.banded_align(a, b, None, B62, 11, 1, 0, 90)
        if full is None:
            assert dev.banded_align_one(a, None, b, 0, 90) is None
            continue
        early_o = orc.banded_align(a, b, None, B62, 11, 1, 0, 90, stop_at=full["score"])
        early_g = dev.banded_align_one(a, None, b, 0, 90, stop_at=full["score"])
        assert _same(early_g, early_o)


def test_long_w_and_memory_cap(dev):
    # banded.rs:716-731 (44 000) and banded.rs:757-765 (cap -> error)
    dev.set_scheme(B62, 11, 1)
    a = np.full(4000, 17, np.uint8)
    got = dev.banded_align_one(a, None, a, -20, 20)
    want = orc.banded_align(a, a, None, B62, 11, 1, -20, 20)
    assert got["score"] == 44000 and _same(got, want)
    b = np.full(1000, 17, np.uint8)
    with pytest.raises(MemoryError):
        dev.banded_align_one(b, None, b, -500, 500, max_dir_bytes=1000)


def _tb_workload(seed, nq, ns, nj):
    qs, ss, planted = synth.protein_db(seed, nq, ns)
    bias = synth.query_bias(seed + 1, qs)
    jobs = synth.band_jobs(seed + 2, qs, ss, planted, nj, half_min=4, half_max=64, related_frac=0.6)
    return qs, ss, bias, jobs


@pytest.mark.parametrize("gaps", [(11, 1), (10, 2), (6, 3), (15, 1), (8, 8)])
def test_batched_align_matches_oracle(dev, gaps):
    """Direction bytes, best cell and CIGAR of the warp-per-job kernel (E by
    a warp max-scan) against the oracle, including stop_at early exits."""
    go, ge = gaps
    qs, ss, bias, jobs = _tb_workload(41 + go, 12, 400, 300)
    dev.set_scheme(B62, go, ge)
    dev.load_db(ss.codes, ss.offsets)
    dev.load_queries(qs.codes, qs.offsets, bias)
    aj = np.zeros(jobs.size, ALIGN_JOB_DTYPE)
    for f in ("query", "subject", "win_begin", "win_len", "band_lo", "band_hi"):
        aj[f] = jobs[f]
    aj["stop_at"] = 2 ** 31 - 1
    aj["stop_at"][::5] = 60
    got = dev.banded_align(aj)
    for t, j in enumerate(jobs):
        q = qs.seq(j["query"])
        qb = bias[qs.offsets[j["query"]]:qs.offsets[j["query"] + 1]]
        s = ss.codes[j["win_begin"]:j["win_begin"] + j["win_len"]]
        want = orc.banded_align(q, s, qb, B62, go, ge, int(j["band_lo"]), int(j["band_hi"]),
                                stop_at=int(aj["stop_at"][t]))
        assert _same(got[t], want), (t, gaps)


def test_widening_traceback_driver_matches_oracle(dev):
    """Engine::traceback + traceback_from_end (engine.rs:1328-1445): regions
    with narrow diagonal spans, want = the exact score of the plan band,
    limits, full-band regions, and a byte cap small enough to force the
    end-anchored fallback on some."""
    qs, ss, bias, jobs = _tb_workload(51, 10, 300, 240)
    dev.set_scheme(B62, 11, 1)
    dev.load_db(ss.codes, ss.offsets)
    dev.load_queries(qs.codes, qs.offsets, bias)
    rng = np.random.default_rng(3)
    tb = np.zeros(jobs.size, TB_JOB_DTYPE)
    cases = []
    for t, j in enumerate(jobs):
        q = qs.seq(j["query"])
        qb = bias[qs.offsets[j["query"]]:qs.offsets[j["query"] + 1]]
        s = ss.codes[j["win_begin"]:j["win_begin"] + j["win_len"]]
        center = (int(j["band_lo"]) + int(j["band_hi"])) // 2
        d_min = center - int(rng.integers(0, 4))
        d_max = center + int(rng.integers(0, 4))
        has_limit = t % 3 != 0
        limit = (int(j["band_lo"]), int(j["band_hi"])) if has_limit else None
        full = t % 17 == 0
        scope = limit if limit is not None else (-len(q), len(s))
        want = orc.banded_score(q, s, qb, B62, 11, 1, scope[0], scope[1])[0]
        tb[t] = (j["query"], j["subject"], j["win_begin"], j["win_len"], d_min, d_max,
                 limit[0] if limit else 0, limit[1] if limit else 0, want, (1 if full else 0) | (2 if limit else 0), 0)
        cases.append((q, qb, s, d_min, d_max, want, limit, full))
    for cap in (32 << 20, 6000):
        got, st = dev.traceback(tb, band_pad=16, max_dir_bytes=cap)
        ctr = oeng.new_counters()
        for t, (q, qb, s, d_min, d_max, want, limit, full) in enumerate(cases):
            w = oeng.traceback(q, s, qb, B62, 11, 1, d_min, d_max, want, limit, full, 16, cap, ctr)
            g = got[t]
            if w is None:
                assert g is None, t
                continue
            al, exact = w
            assert g is not None and g["status"] == (1 if exact else 2), (t, g, w)
            for k in ("score", "q_start", "q_end", "s_start", "s_end", "ops"):
                assert g[k] == al[k], (t, k, g[k], al[k])
        for k in ("tracebacks", "band_widenings", "end_anchored", "band_capped", "banded_cells"):
            assert st[k] == ctr[k], (cap, k, st[k], ctr[k])
