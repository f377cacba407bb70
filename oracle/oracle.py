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
        _lib.orc_simd_score_band_jobs.restype = ctypes.c_int
        _lib.orc_simd_score_band_jobs.argtypes = [P, P, P, P, P, U64, P, I32, I32, P, ctypes.c_int, P]
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


class SimdCounters(ctypes.Structure):
    _fields_ = [("cells", ctypes.c_uint64), ("u8_jobs", ctypes.c_uint64), ("u8_overflows", ctypes.c_uint64),
                ("i16_jobs", ctypes.c_uint64), ("i32_jobs", ctypes.c_uint64)]


def simd_score_band_jobs(residues, qcodes, qoffs, qbias, jobs, matrix, go, ge, threads=1):
    """The SIMD-class restatement of score_banded_many (simd_band.cpp): the
    same jobs and scores as score_band_jobs -> (scores, counters dict)."""
    res = _a(residues, np.uint8)
    qc = _a(qcodes, np.uint8)
    qo = _a(qoffs, np.uint64)
    qb = None if qbias is None else _a(qbias, np.int8)
    jb = np.ascontiguousarray(jobs)
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    out = np.zeros(jb.size, np.int32)
    ct = SimdCounters()
    lib().orc_simd_score_band_jobs(_p(res), _p(qc), _p(qo), _p(qb) if qb is not None else None, _p(jb), jb.size,
                                   _p(m), int(go), int(ge), _p(out), int(threads), ctypes.byref(ct))
    return out, {k: int(getattr(ct, k)) for k, _ in SimdCounters._fields_}


class ScanParams(ctypes.Structure):
    _fields_ = [("alpha_map", ctypes.c_uint8 * 24), ("alpha_size", ctypes.c_uint32), ("nshapes", ctypes.c_uint32),
                ("shape_span", ctypes.c_uint32 * 32), ("shape_weight", ctypes.c_uint32 * 32),
                ("shape_off", (ctypes.c_uint16 * 16) * 32), ("hit_filter_min_ids", ctypes.c_uint32),
                ("hit_filter_exact_weight", ctypes.c_uint32), ("hsp_threshold", ctypes.c_int32),
                ("x_drop", ctypes.c_int32), ("window_slack", ctypes.c_int32),
                ("max_regions_per_subject", ctypes.c_uint32), ("max_candidates", ctypes.c_uint32),
                ("seed_max_occ", ctypes.c_uint64), ("ref_db_residues", ctypes.c_uint64), ("db_length", ctypes.c_uint64)]


class ScanCounters(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "seed_positions", "seeds_frequent_skipped", "hits", "hits_filtered", "ungapped_extensions",
        "extensions_avoided", "xdrop_steps", "hsps", "regions", "regions_weak_dropped", "regions_dropped_by_cap")]


REGION_DTYPE = np.dtype([("query", "<u4"), ("subject", "<u4"), ("d_min", "<i4"), ("d_max", "<i4"), ("best", "<i4")])


def make_scan_params(alpha_map, alpha_size, shapes, min_ids=27, exact_weight=2, hsp_threshold=40, x_drop=20,
                     window_slack=64, max_regions_per_subject=4, max_candidates=5000, seed_max_occ=0,
                     ref_db_residues=40_000_000, db_length=0):
    p = ScanParams()
    for i in range(24):
        p.alpha_map[i] = int(alpha_map[i])
    p.alpha_size = int(alpha_size)
    p.nshapes = len(shapes)
    for si, sh in enumerate(shapes):
        offs = [i for i, ch in enumerate(sh) if ch == "1"]
        p.shape_span[si] = len(sh)
        p.shape_weight[si] = len(offs)
        for k, o in enumerate(offs):
            p.shape_off[si][k] = o
    p.hit_filter_min_ids = min_ids
    p.hit_filter_exact_weight = exact_weight
    p.hsp_threshold = hsp_threshold
    p.x_drop = x_drop
    p.window_slack = window_slack
    p.max_regions_per_subject = max_regions_per_subject
    p.max_candidates = max_candidates
    p.seed_max_occ = seed_max_occ
    p.ref_db_residues = ref_db_residues
    p.db_length = db_length
    return p


def scan_regions(res, soffs, db_mask, qcodes, qoffs, qbias, q_mask, region_thr, matrix, params, out_cap=None,
                 threads=1):
    """Engine::search_scan's candidate regions for one batch -> (REGION_DTYPE array, counters dict);
    `threads` host threads (the result does not depend on it)."""
    L = lib()
    f = L.orc_scan_regions_mt
    f.restype = ctypes.c_int64
    P = ctypes.c_void_p
    f.argtypes = [P, P, ctypes.c_uint64, P, P, P, ctypes.c_uint32, P, P, P, P, P, P, ctypes.c_uint64, P,
                  ctypes.c_int]
    res = _a(res, np.uint8)
    so = _a(soffs, np.uint64)
    dm = None if db_mask is None else _a(db_mask, np.uint8)
    qc = _a(qcodes, np.uint8)
    qo = _a(qoffs, np.uint64)
    qb = None if qbias is None else _a(qbias, np.int8)
    qm = None if q_mask is None else _a(q_mask, np.uint8)
    rt = None if region_thr is None else _a(region_thr, np.int32)
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    cap = out_cap or max(1024, (qo.size - 1) * params.max_candidates)
    out = np.zeros(cap, REGION_DTYPE)
    ctr = ScanCounters()
    n = f(_p(res), _p(so), so.size - 1, _p(dm) if dm is not None else None, _p(qc), _p(qo), qo.size - 1,
          _p(qb) if qb is not None else None, _p(qm) if qm is not None else None,
          _p(rt) if rt is not None else None, _p(m), ctypes.byref(params), _p(out), cap, ctypes.byref(ctr),
          int(threads))
    if n < 0:
        raise MemoryError("region buffer too small")
    return out[:n].copy(), {k: int(getattr(ctr, k)) for k, _ in ctr._fields_}


class TantanParams(ctypes.Structure):
    """TantanParams (masking.rs:36-49) with tantan's protein defaults."""
    _fields_ = [("repeat_start", ctypes.c_double), ("repeat_end", ctypes.c_double), ("max_period", ctypes.c_uint32),
                ("decay", ctypes.c_double), ("min_prob", ctypes.c_double)]

    def __init__(self, repeat_start=0.005, repeat_end=0.05, max_period=50, decay=0.9, min_prob=0.5):
        super().__init__(repeat_start, repeat_end, max_period, decay, min_prob)


def tantan_lambda(matrix):
    """implied_lambda (masking.rs:531-583); NaN when no root exists."""
    f = lib().orc_tantan_lambda
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_void_p]
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    return float(f(_p(m)))


def tantan_tables(matrix, params=None, lam=0.0):
    """Tantan::with_params (masking.rs:162-179) -> (lambda, lr float32[24][32], b2f float32[W])."""
    p = params or TantanParams()
    f = lib().orc_tantan_tables
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    lr = np.zeros(24 * 32, np.float32)
    b2f = np.zeros(max(1, p.max_period), np.float32)
    lam = f(_p(m), ctypes.byref(p), float(lam), _p(lr), _p(b2f))
    return float(lam), lr.reshape(24, 32), b2f


def tantan_mask(codes, offsets, matrix, params=None, lam=0.0):
    """Tantan::mask (masking.rs:191-196) over a batch -> (mask bool array, posteriors float32, masked count)."""
    p = params or TantanParams()
    f = lib().orc_tantan_mask
    f.restype = ctypes.c_int64
    P = ctypes.c_void_p
    f.argtypes = [P, P, ctypes.c_uint64, P, P, ctypes.c_double, P, P]
    c = _a(codes, np.uint8)
    o = _a(offsets, np.uint64)
    m = _a(np.asarray(matrix).reshape(576), np.int32)
    n = int(o[-1]) if o.size else 0
    mask = np.zeros(max(n, 1), np.uint8)
    probs = np.zeros(max(n, 1), np.float32)
    k = f(_p(c), _p(o), max(o.size - 1, 0), _p(m), ctypes.byref(p), float(lam), _p(mask), _p(probs))
    if k < 0:
        raise MemoryError("oracle tantan allocation")
    return mask[:n].astype(bool), probs[:n], int(k)


def translate6(nt, nt_offsets, aa64):
    """Six frames of every sequence (translate_codes, translation.rs:277-299)
    -> (protein codes, offsets[6 * nseq + 1]); subject 6 * s + f is frame f of s."""
    f = lib().orc_translate_codes
    f.restype = ctypes.c_size_t
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p]
    nt = _a(nt, np.uint8)
    offs = np.asarray(nt_offsets, np.int64)
    aa = _a(aa64, np.uint8)
    parts, lens = [], []
    for s in range(offs.size - 1):
        seq = np.ascontiguousarray(nt[offs[s]:offs[s + 1]])
        for fr in range(6):
            out = np.zeros(max(seq.size // 3 + 1, 1), np.uint8)
            k = f(_p(seq), seq.size, fr, _p(aa), _p(out))
            parts.append(out[:k])
            lens.append(k)
    codes = np.concatenate(parts) if parts else np.zeros(0, np.uint8)
    return codes, np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
