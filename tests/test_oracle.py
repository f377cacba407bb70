"""CPU tests: the oracle against the reference's known answers and golden
vectors, and the reference's own banded-kernel properties (regenerated with
the reference tests' LCG)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from saber_gb300.scoring import encode_protein, matrix, nucleotide
from tests.refgen import Lcg, mutate, rand_seq

HERE = os.path.dirname(os.path.abspath(__file__))
B62 = matrix("BLOSUM62")


def test_known_answers_reference_rs():
    # reference.rs:127-134: WAGNER self score 37 at (6, 6)
    q = encode_protein("WAGNER")
    assert orc.sw_reference(q, q, B62, None, 11, 1) == (37, 6, 6)
    # reference.rs:136-146: 4 W pairs, 3 query residues vs gaps, 4 W pairs
    q = encode_protein("WWWWAAAWWWW")
    s = encode_protein("WWWWWWWW")
    assert orc.score_alignment(q, s, 0, 0, [("M", 4), ("I", 3), ("M", 4)], B62, None, 11, 1) == (75, 11, 8)


def test_known_answer_long_w_band():
    # banded.rs:716-731: W x 4000 in band [-20, 20] scores 44 000
    a = np.full(4000, 17, np.uint8)
    al = orc.banded_align(a, a, None, B62, 11, 1, -20, 20)
    assert al["score"] == 44000
    assert orc.banded_score(a, a, None, B62, 11, 1, -20, 20)[0] == 44000


def test_known_answer_nucleotide():
    # gpu/mod.rs:177-182: ACGTACGTAC vs itself -> 20, vs acgtnnacgt -> 8 (+2/-3, 7/2)
    nt = nucleotide(2, -3)
    enc = {"A": 0, "C": 1, "G": 2, "T": 3}
    q = np.array([enc[c] for c in "ACGTACGTAC"], np.uint8)
    s2 = np.array([enc.get(c.upper(), 4) for c in "acgtnnacgt"], np.uint8)
    assert orc.sw_reference(q, q, nt, None, 7, 2)[0] == 20
    assert orc.sw_reference(q, s2, nt, None, 7, 2)[0] == 8


def test_known_answer_overflow_lane():
    # band_simd8.rs:454-468: 300 W in band [-5, 5] scores 3300
    q = np.full(300, 17, np.uint8)
    assert orc.banded_score(q, q, None, B62, 11, 1, -5, 5)[0] == 3300


def _golden():
    with open(os.path.join(HERE, "golden", "sw_vectors.json")) as f:
        return json.load(f)["cases"]


def _case_matrix(c):
    return nucleotide(2, -3) if c["matrix"] == "NT_2_-3" else matrix(c["matrix"])


def test_oracle_matches_reference_kernel_vectors():
    """Full-window SW of the oracle == the reference's CUDA kernel source run on
    the host (examples/gpu_vectors.rs cases; tests/golden/make_golden.py)."""
    n = 0
    for c in _golden():
        mat = _case_matrix(c)
        q = np.array(c["query"], np.uint8)
        bias = None if c["bias"] is None else np.array(c["bias"], np.int8)
        for w, want in zip(c["windows"], c["expected"]):
            s = np.array(w, np.uint8)
            if len(q) <= 1000 and len(s) <= 1000:
                assert orc.sw_reference(q, s, mat, bias, c["gap_open"], c["gap_extend"])[0] == want
            full = orc.banded_score(q, s, bias, mat, c["gap_open"], c["gap_extend"], -len(q), len(s))
            assert full[0] == want
            n += 1
    assert n == 437


def test_full_band_equals_reference_on_random_and_related_pairs():
    # banded.rs:565-596
    r = Lcg(42)
    for t in range(300):
        la = 1 + r.next(160)
        a = rand_seq(r, la)
        lb = 1 + r.next(160)
        b = mutate(r, a) if t % 2 == 0 else rand_seq(r, lb)
        bias = np.array([r.next(7) - 3 for _ in range(len(a))], np.int8)
        bo = bias if t % 3 == 0 else None
        rs, ri, rj = orc.sw_reference(a, b, B62, bo, 11, 1)
        bs = orc.banded_score(a, b, bo, B62, 11, 1, -len(a), len(b))
        assert bs[0] == rs
        if rs > 0:
            assert (bs[1], bs[2]) == (ri, rj)
        al = orc.banded_align(a, b, bo, B62, 11, 1, -len(a), len(b))
        if rs == 0:
            assert al is None
            continue
        assert al["score"] == rs
        rescored = orc.score_alignment(a, b, al["q_start"], al["s_start"], al["ops"], B62, bo, 11, 1)
        assert rescored == (rs, al["q_end"], al["s_end"])


def test_band_never_exceeds_full_and_columns_stay_in_band():
    # banded.rs:598-628
    r = Lcg(7)
    for _ in range(60):
        la = 50 + r.next(200)
        a = rand_seq(r, la)
        b = mutate(r, a)
        rs = orc.sw_reference(a, b, B62, None, 11, 1)[0]
        for half in (2, 8, 32):
            bs = orc.banded_score(a, b, None, B62, 11, 1, -half, half)
            assert bs[0] <= rs
            al = orc.banded_align(a, b, None, B62, 11, 1, -half, half)
            if al is None:
                continue
            assert al["score"] == bs[0]
            assert orc.score_alignment(a, b, al["q_start"], al["s_start"], al["ops"], B62, None, 11, 1)[0] == bs[0]
            i, j = al["q_start"], al["s_start"]
            for op, ln in al["ops"]:
                for _ in range(ln):
                    assert -half <= j - i <= half
                    if op == "M":
                        i += 1
                        j += 1
                    elif op == "I":
                        i += 1
                    else:
                        j += 1


def test_shifted_diagonal_needs_band_on_that_diagonal():
    # banded.rs:630-643
    core = encode_protein("MKVLAAGIVGHHWWPQRSTVYCCMKDEFGHIKLMNPQRSTVWY")
    subj = np.concatenate([np.zeros(300, np.uint8), core])
    rs = orc.sw_reference(core, subj, B62, None, 11, 1)[0]
    near = orc.banded_score(core, subj, None, B62, 11, 1, -10, 10)[0]
    assert near < rs // 2
    assert orc.banded_score(core, subj, None, B62, 11, 1, 290, 310)[0] == rs


def test_stopping_at_known_score_gives_same_alignment():
    # banded.rs:733-755
    r = Lcg(5)
    saved = 0
    for _ in range(80):
        la = 20 + r.next(300)
        a = rand_seq(r, la)
        b = np.concatenate([rand_seq(r, 40), mutate(r, a[:la // 2]), rand_seq(r, 40)])
        full = orc.banded_align(a, b, None, B62, 11, 1, 0, 90)
        if full is None:
            continue
        early = orc.banded_align(a, b, None, B62, 11, 1, 0, 90, stop_at=full["score"])
        for k in ("score", "q_start", "q_end", "s_start", "s_end", "ops"):
            assert early[k] == full[k]
        assert early["cells"] <= full["cells"]
        saved += full["cells"] - early["cells"]
    assert saved > 0


def test_traceback_respects_memory_cap():
    # banded.rs:757-765
    a = np.full(1000, 17, np.uint8)
    with pytest.raises(MemoryError):
        orc.banded_align(a, a, None, B62, 11, 1, -500, 500, max_dir_bytes=1000)


def test_ungapped_xdrop_basic():
    # engine.rs:2460-2494: identical W runs extend to the ends
    a = np.full(50, 17, np.uint8)
    sc, lo, hi = orc.ungapped_xdrop(a, a, 10, 10, B62, None, 20)
    assert (sc, lo, hi) == (550, 0, 50)


def test_batched_jobs_equal_single_calls():
    from saber_gb300 import synth
    qs, ss, planted = synth.protein_db(3, 8, 60)
    jobs = synth.band_jobs(4, qs, ss, planted, 200)
    bias = synth.query_bias(5, qs)
    got, cells = orc.score_band_jobs(ss.codes, qs.codes, qs.offsets, bias, jobs, B62, 11, 1, threads=4)
    tot = 0
    for t, j in enumerate(jobs):
        q = qs.seq(j["query"])
        qb = bias[qs.offsets[j["query"]]:qs.offsets[j["query"] + 1]]
        s = ss.codes[j["win_begin"]:j["win_begin"] + j["win_len"]]
        r = orc.banded_score(q, s, qb, B62, 11, 1, int(j["band_lo"]), int(j["band_hi"]))
        assert got[t] == r[0]
        tot += r[3]
    assert cells == tot
