"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the saber_gb300 package.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


class BandScore(ctypes.Structure):
    _fields_ = [("score", ctypes.c_int32), ("q_end", ctypes.c_uint64), ("s_end", ctypes.c_uint64),
                ("cells", ctypes.c_uint64)]


class Alignment(ctypes.Structure):
    _fields_ = [("score", ctypes.c_int32), ("q_start", ctypes.c_uint64), ("q_end", ctypes.c_uint64),
                ("s_start", ctypes.c_uint64), ("s_end", ctypes.c_uint64), ("cells", ctypes.c_uint64),
                ("n_ops", ctypes.c_uint32)]


class Scheme(ctypes.Structure):
    _fields_ = [("matrix", ctypes.c_void_p), ("gap_open", ctypes.c_int32), ("gap_extend", ctypes.c_int32)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.check_call(["make", "-s", "-C", HERE, "all"])
        _lib = ctypes.CDLL(LIB)
        P, U64, I64, I32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int32
        _lib.orc_sw_reference.restype = I64
        _lib.orc_sw_reference.argtypes = [P, U64, P, U64, P, P, I64, I64, P, P]
        _lib.orc_score_alignment.restype = ctypes.c_int
        _lib.orc_score_alignment.argtypes = [P, U64, P, U64, U64, U64, P, P, ctypes.c_uint32, P, P, I64, I64,
                                             P, P, P]
        _lib.orc_banded_score.restype = None
        _lib.orc_banded_score.argtypes = [P, U64, P, U64, P, Scheme, I64, I64, P]
        _lib.orc_banded_align.restype = ctypes.c_int
        _lib.orc_banded_align.argtypes = [P, U64, P, U64, P, Scheme, I64, I64, U64, I32, P, P, P,
                                          ctypes.c_uint32]
        _lib.orc_ungapped_xdrop.restype = I32
        _lib.orc_ungapped_xdrop.argtypes = [P, U64, P, U64, U64, U64, P, P, I32, P, P]
        _lib.orc_score_band_jobs.restype = ctypes.c_int
        _lib.orc_score_band_jobs.argtypes = [P, P, P, P, P, U64, P, I32, I32, P, ctypes.c_int, P]
    return _lib


def _a(x, dt):
    return np.ascontiguousarray(x, dtype=dt)


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data) if a.size else ctypes.c_void_p(
        np.zeros(1, a.dtype).ctypes.data)


class _Keep:
    pass


def _scheme(matrix, go, ge, keep):
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    keep.m = m
    return Scheme(m.ctypes.data, int(go), int(ge))


def sw_reference(q, s, matrix, bias, go, ge):
    """reference.rs:15-52 -> (score, q_end, s_end)"""
    q, s = _a(q, np.uint8), _a(s, np.uint8)
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    b = None if bias is None else _a(bias, np.int8)
    qe, se = ctypes.c_uint64(), ctypes.c_uint64()
    sc = lib().orc_sw_reference(_p(q), q.size, _p(s), s.size, _p(m), _p(b) if b is not None else None, go, ge,
                                ctypes.byref(qe), ctypes.byref(se))
    return int(sc), int(qe.value), int(se.value)


def score_alignment(q, s, q_start, s_start, ops, matrix, bias, go, ge):
    """reference.rs:58-103 -> (score, q_end, s_end) or None"""
    q, s = _a(q, np.uint8), _a(s, np.uint8)
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    b = None if bias is None else _a(bias, np.int8)
    o = _a([ord(op) if isinstance(op, str) else op for op, _ in ops], np.uint8)
    ln = _a([l for _, l in ops], np.uint32)
    sc, qe, se = ctypes.c_int64(), ctypes.c_uint64(), ctypes.c_uint64()
    rc = lib().orc_score_alignment(_p(q), q.size, _p(s), s.size, q_start, s_start, _p(o), _p(ln), len(ops), _p(m),
                                   _p(b) if b is not None else None, go, ge, ctypes.byref(sc), ctypes.byref(qe),
                                   ctypes.byref(se))
    if rc != 0:
        return None
    return int(sc.value), int(qe.value), int(se.value)


def banded_score(q, s, bias, matrix, go, ge, lo, hi):
    """banded.rs:134-224 -> (score, q_end, s_end, cells)"""
    q, s = _a(q, np.uint8), _a(s, np.uint8)
    b = None if bias is None else _a(bias, np.int8)
    k = _Keep()
    sc = _scheme(matrix, go, ge, k)
    out = BandScore()
    lib().orc_banded_score(_p(q), q.size, _p(s), s.size, _p(b) if b is not None else None, sc, int(lo), int(hi),
                           ctypes.byref(out))
    return out.score, int(out.q_end), int(out.s_end), int(out.cells)


def banded_align(q, s, bias, matrix, go, ge, lo, hi, max_dir_bytes=1 << 62, stop_at=2 ** 31 - 1):
    """banded.rs:227-403 (+ stop_at) -> dict or None; raises MemoryError on the byte cap."""
    q, s = _a(q, np.uint8), _a(s, np.uint8)
    b = None if bias is None else _a(bias, np.int8)
    k = _Keep()
    sc = _scheme(matrix, go, ge, k)
    out = Alignment()
    cap = q.size + s.size + 2
    ops = np.zeros(cap, np.uint8)
    lens = np.zeros(cap, np.uint32)
    rc = lib().orc_banded_align(_p(q), q.size, _p(s), s.size, _p(b) if b is not None else None, sc, int(lo),
                                int(hi), int(max_dir_bytes), int(stop_at), ctypes.byref(out), _p(ops), _p(lens),
                                cap)
    if rc == -2:
        raise MemoryError("direction matrix over the cap")
    if rc == 0:
        return None
    n = out.n_ops
    return dict(score=out.score, q_start=int(out.q_start), q_end=int(out.q_end), s_start=int(out.s_start),
                s_end=int(out.s_end), cells=int(out.cells),
                ops=[(chr(ops[i]), int(lens[i])) for i in range(n)])


def ungapped_xdrop(q, s, qp, sp, matrix, bias, x):
    q, s = _a(q, np.uint8), _a(s, np.uint8)
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    b = None if bias is None else _a(bias, np.int8)
    lo, hi = ctypes.c_uint64(), ctypes.c_uint64()
    sc = lib().orc_ungapped_xdrop(_p(q), q.size, _p(s), s.size, qp, sp, _p(m), _p(b) if b is not None else None,
                                  x, ctypes.byref(lo), ctypes.byref(hi))
    return int(sc), int(lo.value), int(hi.value)


def score_band_jobs(residues, qcodes, qoffs, qbias, jobs, matrix, go, ge, threads=1):
    """Scores of JOB_DTYPE jobs with `threads` POSIX threads -> (scores, cells)."""
    res = _a(residues, np.uint8)
    qc = _a(qcodes, np.uint8)
    qo = _a(qoffs, np.uint64)
    qb = None if qbias is None else _a(qbias, np.int8)
    jb = np.ascontiguousarray(jobs)
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    out = np.zeros(jb.size, np.int32)
    cells = ctypes.c_uint64()
    lib().orc_score_band_jobs(_p(res), _p(qc), _p(qo), _p(qb) if qb is not None else None, _p(jb), jb.size, _p(m),
                              int(go), int(ge), _p(out), int(threads), ctypes.byref(cells))
    return out, int(cells.value)
