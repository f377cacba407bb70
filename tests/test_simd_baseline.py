"""CPU tests: the SIMD-class restatement of the reference's CPU scoring
(oracle/simd_band.cpp: score_banded_many with batch_u8, banded_avx2_16 and
the 32-bit re-run) gives the scalar oracle's scores on the same jobs.  It is
the CPU baseline and the reference arm of bench.py, so its scores must be
the reference's."""
import numpy as np
import pytest

from oracle import oracle as orc
from saber_gb300 import synth
from saber_gb300.gpu import JOB_DTYPE
from saber_gb300.scoring import matrix, nucleotide

B62 = matrix("BLOSUM62")


def _both(res, qc, qo, bias, jobs, mat, go, ge):
    want, cells = orc.score_band_jobs(res, qc, qo, bias, jobs, mat, go, ge, threads=4)
    got, ct = orc.simd_score_band_jobs(res, qc, qo, bias, jobs, mat, go, ge, threads=4)
    assert np.array_equal(got, want), np.nonzero(got != want)[0][:10]
    assert ct["cells"] == cells
    return ct


@pytest.mark.parametrize("with_bias", [True, False])
def test_microbench_style_jobs(with_bias):
    qs, ss, planted = synth.protein_db(11, 30, 800)
    bias = synth.query_bias(12, qs) if with_bias else None
    jobs = synth.band_jobs(13, qs, ss, planted, 3000)
    ct = _both(ss.codes, qs.codes, qs.offsets, bias, jobs, B62, 11, 1)
    # every path of score_banded_many ran: 8-bit lanes, their overflows, 16 bits
    assert ct["u8_jobs"] > 0 and ct["u8_overflows"] > 0 and ct["i16_jobs"] > 0


@pytest.mark.parametrize("name,go,ge", [("BLOSUM45", 15, 2), ("PAM30", 9, 1), ("BLOSUM80", 10, 10)])
def test_other_schemes(name, go, ge):
    qs, ss, planted = synth.protein_db(21, 12, 300)
    bias = synth.query_bias(22, qs, levels=(-3, 0, 2))
    jobs = synth.band_jobs(23, qs, ss, planted, 800, half_min=2, half_max=90)
    _both(ss.codes, qs.codes, qs.offsets, bias, jobs, matrix(name), go, ge)


def test_large_bias_takes_the_exact_kernels():
    # a bias range that breaks the 8-bit offset rule (pmax >= 128) sends every job to 16 bits
    qs, ss, planted = synth.protein_db(31, 6, 100)
    bias = synth.query_bias(32, qs, levels=(-120, 0, 120))
    jobs = synth.band_jobs(33, qs, ss, planted, 300)
    ct = _both(ss.codes, qs.codes, qs.offsets, bias, jobs, B62, 11, 1)
    assert ct["u8_jobs"] == 0


def _jobs(rows):
    j = np.zeros(len(rows), JOB_DTYPE)
    for t, (q, b, n, lo, hi) in enumerate(rows):
        j[t] = (q, 0, b, n, lo, hi, 0)
    return j


def test_known_answers_and_edges():
    # banded.rs:716-731 (W x 4000 in [-20, 20] = 44 000: past the 16-bit limit, re-run in 32 bits),
    # band_simd8.rs:454-468 (300 W in [-5, 5] = 3300: an 8-bit lane overflow), and empty jobs
    w4000 = np.full(4000, 17, np.uint8)
    w300 = np.full(300, 17, np.uint8)
    qc = np.concatenate([w4000, w300])
    qo = np.array([0, 4000, 4300], np.uint64)
    res = np.concatenate([w4000, w300, np.full(64, 22, np.uint8)])
    jobs = _jobs([(0, 0, 4000, -20, 20), (1, 4000, 300, -5, 5), (1, 4000, 300, 5, -5), (1, 4000, 0, -5, 5),
                  (1, 4000, 300, 400, 500), (1, 4000, 300, -900, -400), (1, 4000, 1, 0, 0)])
    want, _ = orc.score_band_jobs(res, qc, qo, None, jobs, B62, 11, 1)
    got, ct = orc.simd_score_band_jobs(res, qc, qo, None, jobs, B62, 11, 1)
    assert list(got) == list(want)
    assert got[0] == 44000 and got[1] == 3300
    assert ct["i32_jobs"] == 1 and ct["u8_overflows"] >= 1


def test_nucleotide_scoring():
    qs, ss, _ = synth.dna_db(41, 4, 30, qlen=(200, 600), slen=(200, 900))
    rng = np.random.default_rng(42)
    rows = []
    for _ in range(400):
        q = int(rng.integers(0, len(qs)))
        s = int(rng.integers(0, len(ss)))
        b, e = int(ss.offsets[s]), int(ss.offsets[s + 1])
        n = int(rng.integers(1, e - b + 1))
        d = int(rng.integers(-200, 200))
        h = int(rng.integers(0, 150))
        rows.append((q, b, n, d - h, d + h))
    _both(ss.codes, qs.codes, qs.offsets, None, _jobs(rows), nucleotide(2, -3), 7, 2)
