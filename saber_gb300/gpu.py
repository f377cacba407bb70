"""ctypes binding of libsaber_gb300.so (the C ABI in include/saber_gpu.h).

Host-side mirror of the reference's scoring interfaces:

* :class:`CudaBackend` — ``ScoreBackend`` (src/gpu/mod.rs:45-59): ``name()``
  and ``score_windows(query, bias, windows, matrix, gaps)``;
* :func:`score_banded_many` — ``band_simd8::score_banded_many``
  (src/algorithm/band_simd8.rs:78-185): one query, many banded windows;
* :class:`Device` — the batched device path: a resident database and query
  set, and :meth:`Device.score_band_jobs` over a whole query batch.

There is no CPU fallback: without the compiled library every call raises.
"""
import ctypes
import os

import numpy as np

from . import _build

_LIB = None

JOB_DTYPE = np.dtype([
    ("query", "<u4"), ("subject", "<u4"), ("win_begin", "<u8"), ("win_len", "<u4"),
    ("band_lo", "<i4"), ("band_hi", "<i4"), ("flags", "<u4"),
])
assert JOB_DTYPE.itemsize == 32


class SaberGpuError(RuntimeError):
    """A call of the C ABI returned an error status."""


ALIGN_JOB_DTYPE = np.dtype([
    ("query", "<u4"), ("subject", "<u4"), ("win_begin", "<u8"), ("win_len", "<u4"),
    ("band_lo", "<i4"), ("band_hi", "<i4"), ("stop_at", "<i4")])
TB_JOB_DTYPE = np.dtype([
    ("query", "<u4"), ("subject", "<u4"), ("win_begin", "<u8"), ("win_len", "<u4"),
    ("d_min", "<i4"), ("d_max", "<i4"), ("limit_lo", "<i4"), ("limit_hi", "<i4"), ("want", "<i4"),
    ("flags", "<u4"), ("reserved", "<u4")])
assert ALIGN_JOB_DTYPE.itemsize == 32 and TB_JOB_DTYPE.itemsize == 48


class Alignment(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("score", ctypes.c_int32), ("q_start", ctypes.c_uint32),
                ("q_end", ctypes.c_uint32), ("s_start", ctypes.c_uint32), ("s_end", ctypes.c_uint32),
                ("n_ops", ctypes.c_uint32), ("ops_offset", ctypes.c_uint32), ("cells", ctypes.c_uint64)]


class TracebackStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("tracebacks", "band_widenings", "end_anchored", "band_capped",
                                                 "banded_cells", "launches")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


def _alignment_dict(a, ops):
    runs = [(chr(ops[a.ops_offset + k] & 0xFF), int(ops[a.ops_offset + k] >> 8)) for k in range(a.n_ops)]
    return dict(status=int(a.status), score=int(a.score), q_start=int(a.q_start), q_end=int(a.q_end),
                s_start=int(a.s_start), s_end=int(a.s_end), cells=int(a.cells), ops=runs)


class ScanParams(ctypes.Structure):
    """saber_scan_params (include/saber_gpu.h)."""
    _fields_ = [("alpha_map", ctypes.c_uint8 * 24), ("alpha_size", ctypes.c_uint32), ("nshapes", ctypes.c_uint32),
                ("shape_span", ctypes.c_uint32 * 32), ("shape_weight", ctypes.c_uint32 * 32),
                ("shape_off", (ctypes.c_uint16 * 16) * 32), ("hit_filter_min_ids", ctypes.c_uint32),
                ("hit_filter_exact_weight", ctypes.c_uint32), ("hsp_threshold", ctypes.c_int32),
                ("x_drop", ctypes.c_int32), ("window_slack", ctypes.c_int32),
                ("max_regions_per_subject", ctypes.c_uint32), ("max_candidates", ctypes.c_uint32),
                ("seed_max_occ", ctypes.c_uint64), ("ref_db_residues", ctypes.c_uint64), ("db_length", ctypes.c_uint64)]


class ScanStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "seed_positions", "seeds_frequent_skipped", "hits", "hits_filtered", "ungapped_extensions",
        "extensions_avoided", "xdrop_steps", "hsps", "regions", "regions_weak_dropped", "regions_dropped_by_cap")] + [
        (n, ctypes.c_double) for n in ("t_tables_ms", "t_scan_ms", "t_visit_ms", "t_regions_ms")]

    def as_dict(self):
        return {n: (float(getattr(self, n)) if n.startswith("t_") else int(getattr(self, n))) for n, _ in self._fields_}


class SearchParamsC(ctypes.Structure):
    """saber_search_params (include/saber_gpu.h)."""
    _fields_ = [("evalue", ctypes.c_double), ("min_bitscore", ctypes.c_double),
                ("max_target_seqs", ctypes.c_uint32), ("max_hsps", ctypes.c_uint32),
                ("min_identity", ctypes.c_double), ("min_query_cover", ctypes.c_double),
                ("min_subject_cover", ctypes.c_double), ("hsp_threshold", ctypes.c_int32),
                ("hsp_floor_fraction", ctypes.c_double), ("band_pad", ctypes.c_int32),
                ("window_slack", ctypes.c_int32), ("score_band", ctypes.c_int32),
                ("score_prefilter_band", ctypes.c_int32), ("score_prefilter_frac", ctypes.c_double),
                ("comp_bias", ctypes.c_uint32), ("exhaustive", ctypes.c_uint32),
                ("traceback_max_bytes", ctypes.c_uint64), ("ref_db_residues", ctypes.c_uint64),
                ("evalue_model", ctypes.c_uint32), ("is_protein", ctypes.c_uint32),
                ("lambda_", ctypes.c_double), ("k", ctypes.c_double), ("h", ctypes.c_double),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("even_scores_only", ctypes.c_uint32), ("pad_", ctypes.c_uint32), ("scan", ScanParams),
                ("stats_num_seqs", ctypes.c_uint64)]


class SearchStats(ctypes.Structure):
    """saber_search_stats (include/saber_gpu.h)."""
    _fields_ = [("scan", ScanStats), ("traceback", TracebackStats)] + [
        (n, ctypes.c_uint64) for n in ("regions", "triage_dropped", "band_scored_regions", "band_rescored",
                                       "banded_cells", "score_launches", "alignments")] + [
        (n, ctypes.c_double) for n in ("t_prep_ms", "t_scan_ms", "t_triage_ms", "t_plan_ms", "t_score_ms",
                                       "t_finish_ms", "t_total_ms", "t_score_calls_ms", "t_score_device_ms",
                                       "t_finish_tb_ms", "t_score_prep_ms", "t_score_fast_ms", "t_score_generic_ms",
                                       "t_score_build_ms", "t_score_stage2_ms", "t_finish_order_ms")]

    def as_dict(self):
        d = {}
        d.update({("scan_" + k if k.startswith("t_") else k): v for k, v in self.scan.as_dict().items()})
        d.update({"tb_" + k: v for k, v in self.traceback.as_dict().items()})
        for n, t in self._fields_[2:]:
            v = getattr(self, n)
            d[n] = float(v) if n.startswith("t_") else int(v)
        return d


class TriageTrainCfg(ctypes.Structure):
    """saber_triage_train_cfg (include/saber_gpu.h)."""
    _fields_ = [("epochs", ctypes.c_uint32), ("batch", ctypes.c_uint32), ("lr", ctypes.c_float),
                ("pos_weight", ctypes.c_float), ("weight_decay", ctypes.c_float), ("pad_", ctypes.c_uint32),
                ("seed", ctypes.c_uint64)]


class TriageTrainStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("final_loss", ctypes.c_double)]


TRIAGE_MODEL_FLOATS = 74561
TRIAGE_ROW_FLOATS = 32

# saber_hit
HIT_DTYPE = np.dtype([("query", "<u4"), ("subject", "<u4"), ("score", "<i4"), ("exact", "<u4"),
                      ("evalue", "<f8"), ("bitscore", "<f8"), ("q_start", "<u4"), ("q_end", "<u4"),
                      ("s_start", "<u4"), ("s_end", "<u4"), ("columns", "<u4"), ("matches", "<u4"),
                      ("mismatches", "<u4"), ("positives", "<u4"), ("gap_opens", "<u4"), ("gap_columns", "<u4"),
                      ("q_len", "<u4"), ("s_len", "<u4"), ("n_ops", "<u4"), ("pad_", "<u4"), ("ops_offset", "<u8")])
assert HIT_DTYPE.itemsize == 96


REGION_DTYPE = np.dtype([("query", "<u4"), ("subject", "<u4"), ("d_min", "<i4"), ("d_max", "<i4"), ("best", "<i4")])


def scan_params(alpha_map, alpha_size, shapes, min_ids=27, exact_weight=2, hsp_threshold=40, x_drop=20,
                window_slack=64, max_regions_per_subject=4, max_candidates=5000, seed_max_occ=0,
                ref_db_residues=40_000_000, db_length=0):
    """Fill saber_scan_params from shape patterns ("11110111", ...)."""
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


class ScoreStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "jobs", "banded_cells", "fast_cells", "fast_jobs", "generic_jobs", "i16_rescored", "empty_jobs",
        "kernel_launches", "library_launches")] + [
        (n, ctypes.c_double) for n in ("t_prep_ms", "t_fast_ms", "t_generic_ms")] + [("prof8", ctypes.c_uint64)]

    def as_dict(self):
        return {n: (float(getattr(self, n)) if n.startswith("t_") else int(getattr(self, n)))
                for n, _ in self._fields_}


def lib_path():
    return _build.LIB


def load_library():
    """Load libsaber_gb300.so; raises if it has not been built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        raise SaberGpuError("libsaber_gb300.so is not built (%s); run "
                            "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    lib = ctypes.CDLL(path)
    P, U32, U64, I32, I64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int64
    sig = {
        "saber_gpu_open": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(P)]),
        "saber_gpu_close": (ctypes.c_int, [P]),
        "saber_gpu_last_error": (ctypes.c_char_p, [P]),
        "saber_gpu_stream": (P, [P]),
        "saber_gpu_set_scheme": (ctypes.c_int, [P, P, I32, I32]),
        "saber_gpu_load_db": (ctypes.c_int, [P, P, U64, P, U64]),
        "saber_gpu_load_queries": (ctypes.c_int, [P, P, P, P, U32]),
        "saber_gpu_score_band_jobs": (ctypes.c_int, [P, P, U64, P, P]),
        "saber_gpu_score_band_jobs_dev": (ctypes.c_int, [P, P, U64, P, P]),
        "saber_gpu_score_banded_many": (ctypes.c_int, [P, P, U32, P, P, P, P, P, U64, P]),
        "saber_gpu_score_windows": (ctypes.c_int, [P, P, U32, P, P, P, U32, P, I32, I32, P]),
        "saber_band_cells": (U64, [U64, U64, I64, I64]),
        "saber_gpu_probe_int_peak": (ctypes.c_int, [P, P, P]),
        "saber_gpu_probe_pipe_rates": (ctypes.c_int, [P, P]),
        "saber_gpu_set_strip_rows": (ctypes.c_int, [P, I32]),
        "saber_gpu_banded_align": (ctypes.c_int, [P, P, U64, U64, P, P, U64]),
        "saber_gpu_banded_align_one": (ctypes.c_int, [P, P, U32, P, P, U32, I64, I64, U64, I32, P, P, U64]),
        "saber_gpu_traceback": (ctypes.c_int, [P, P, U64, I32, U64, P, P, U64, P]),
        "saber_gpu_load_db_mask": (ctypes.c_int, [P, P, U64]),
        "saber_gpu_scan": (ctypes.c_int, [P, P, P, P, P, U64, P, P]),
        "saber_gpu_get_strip_rows": (I32, [P]),
        "saber_gpu_set_pair_steps": (ctypes.c_int, [P, U32]),
        "saber_gpu_set_graphs": (ctypes.c_int, [P, I32]),
        "saber_gpu_get_graphs": (I32, [P]),
        "saber_gpu_graph_captures": (U64, [P]),
        "saber_gpu_search": (ctypes.c_int, [P, P, P, P, U64, P, P, U32, P, P, U64, P, P, U64, P, P]),
        "saber_gpu_triage_grads": (ctypes.c_int, [P, P, P, P, U32, ctypes.c_float, P, P]),
        "saber_gpu_triage_train": (ctypes.c_int, [P, P, P, P, U64, P, P]),
        "saber_gpu_triage_predict": (ctypes.c_int, [P, P, P, U64, P]),
        "saber_gpu_set_triage": (ctypes.c_int, [P, P, ctypes.c_float]),
        "saber_gpu_collect_regions": (ctypes.c_int, [P, I32]),
        "saber_gpu_collected_regions": (ctypes.c_int, [P, P, P, P, U64, P]),
        "saber_gpu_get_pair_steps": (U32, [P]),
        "saber_gpu_set_scan_table_bytes": (ctypes.c_int, [P, U64]),
        "saber_gpu_set_long_steps": (ctypes.c_int, [P, U32]),
        "saber_gpu_get_long_steps": (U32, [P]),
        "saber_gpu_get_scan_table_bytes": (U64, [P]),
        "saber_gpu_score_band_jobs_noalloc": (ctypes.c_int, [P, P, U64, I32, P]),
        "saber_tantan_implied_lambda": (ctypes.c_double, [P]),
        "saber_gpu_tantan_mask": (ctypes.c_int, [P, P, P, P, P, U64, P, P, P, P]),
        "saber_gpu_tantan_mask_db": (ctypes.c_int, [P, P, P, P, P]),
        "saber_gpu_translate6": (ctypes.c_int, [P, P, P, U64, P, P, U64, P]),
        "saber_gpu_load_db_mask_runs": (ctypes.c_int, [P, P, U64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def band_cells(m, n, lo, hi):
    """In-band cells of one job (reference counting; host-only)."""
    return int(load_library().saber_band_cells(int(m), int(n), int(lo), int(hi)))


def _flat_matrix(matrix):
    mat = np.ascontiguousarray(np.asarray(matrix, dtype=np.int32).reshape(576))
    return mat


class Device:
    """One handle of the C ABI: a CUDA stream plus device-resident data."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.saber_gpu_open(int(device), ctypes.byref(h))
        if rc != 0:
            raise SaberGpuError("saber_gpu_open(%d) failed with status %d" % (device, rc))
        self.h = h
        self._keep = {}

    def close(self):
        if self.h:
            self.lib.saber_gpu_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            msg = self.lib.saber_gpu_last_error(self.h)
            raise SaberGpuError("%s failed (%d): %s" % (what, rc, msg.decode() if msg else ""))

    @property
    def stream(self):
        return self.lib.saber_gpu_stream(self.h)

    def set_scheme(self, matrix, gap_open, gap_extend):
        mat = _flat_matrix(matrix)
        self._check(self.lib.saber_gpu_set_scheme(self.h, _ptr(mat), int(gap_open), int(gap_extend)),
                    "set_scheme")

    def load_db(self, residues, offsets):
        res = np.ascontiguousarray(residues, dtype=np.uint8)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        self._check(self.lib.saber_gpu_load_db(self.h, _ptr(res), res.size, _ptr(off), off.size - 1), "load_db")

    def load_queries(self, codes, offsets, bias=None):
        c = np.ascontiguousarray(codes, dtype=np.uint8)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        b = None if bias is None else np.ascontiguousarray(bias, dtype=np.int8)
        self._check(self.lib.saber_gpu_load_queries(self.h, _ptr(c), _ptr(off), _ptr(b), off.size - 1),
                    "load_queries")

    def score_band_jobs(self, jobs, out=None):
        """Scores of host jobs (structured JOB_DTYPE array); host in, host out."""
        jobs = np.ascontiguousarray(jobs, dtype=JOB_DTYPE)
        if out is None:
            out = np.empty(jobs.size, dtype=np.int32)
        st = ScoreStats()
        self._check(self.lib.saber_gpu_score_band_jobs(self.h, _ptr(jobs), jobs.size, _ptr(out), ctypes.byref(st)),
                    "score_band_jobs")
        return out, st.as_dict()

    def score_band_jobs_ptr(self, jobs_ptr, njobs, scores_ptr):
        """Host-buffer call with raw host pointers (e.g. pinned torch tensors)."""
        st = ScoreStats()
        self._check(self.lib.saber_gpu_score_band_jobs(self.h, ctypes.c_void_p(jobs_ptr), int(njobs),
                                                       ctypes.c_void_p(scores_ptr), ctypes.byref(st)),
                    "score_band_jobs")
        return st.as_dict()

    def score_band_jobs_dev(self, d_jobs_ptr, njobs, d_scores_ptr):
        """Device-resident variant: raw device pointers (e.g. torch tensors' data_ptr())."""
        st = ScoreStats()
        self._check(self.lib.saber_gpu_score_band_jobs_dev(self.h, ctypes.c_void_p(d_jobs_ptr), int(njobs),
                                                           ctypes.c_void_p(d_scores_ptr), ctypes.byref(st)),
                    "score_band_jobs_dev")
        return st.as_dict()

    def score_band_jobs_noalloc(self, d_jobs_ptr, njobs, max_band_width, d_scores_ptr):
        """Allocation-free scoring of device-resident jobs: the call allocates no
        device memory (its scratch is a fixed 16 MiB array in the library).  It
        runs on the handle's stream and returns once the scores are written;
        the jobs must be written before the call."""
        self._check(self.lib.saber_gpu_score_band_jobs_noalloc(self.h, ctypes.c_void_p(d_jobs_ptr), int(njobs),
                                                               int(max_band_width), ctypes.c_void_p(d_scores_ptr)),
                    "score_band_jobs_noalloc")

    def banded_align_one(self, query, bias, subject, lo, hi, max_dir_bytes=1 << 62, stop_at=2 ** 31 - 1):
        """banded_align_until for one pair -> dict (status 1), None (status 0) or MemoryError (cap)."""
        q = np.ascontiguousarray(query, dtype=np.uint8)
        sj = np.ascontiguousarray(subject, dtype=np.uint8)
        b = None if bias is None else np.ascontiguousarray(bias, dtype=np.int8)
        cap = q.size + sj.size + 2
        ops = np.zeros(cap, np.uint32)
        out = Alignment()
        self._check(self.lib.saber_gpu_banded_align_one(
            self.h, _ptr(q) if q.size else None, q.size, _ptr(b), _ptr(sj) if sj.size else None, sj.size, int(lo),
            int(hi), int(max_dir_bytes), int(stop_at), ctypes.byref(out), _ptr(ops), cap), "banded_align_one")
        if out.status == -5:
            raise MemoryError("direction matrix over the cap")
        if out.status == 0:
            return None
        return _alignment_dict(out, ops)

    def banded_align(self, jobs, max_dir_bytes=1 << 62):
        """Batched banded_align_until over ALIGN_JOB_DTYPE jobs -> list of dicts / None / 'cap'."""
        jobs = np.ascontiguousarray(jobs, dtype=ALIGN_JOB_DTYPE)
        out = (Alignment * max(1, jobs.size))()
        cap = int(np.sum(jobs["win_len"].astype(np.int64))) + 64 * jobs.size + 64
        ops = np.zeros(cap, np.uint32)
        self._check(self.lib.saber_gpu_banded_align(self.h, _ptr(jobs), jobs.size, int(max_dir_bytes), out,
                                                    _ptr(ops), cap), "banded_align")
        res = []
        for t in range(jobs.size):
            a = out[t]
            res.append("cap" if a.status == -5 else None if a.status == 0 else _alignment_dict(a, ops))
        return res

    def traceback(self, jobs, band_pad=16, max_dir_bytes=32 << 20):
        """Widening band traceback of TB_JOB_DTYPE regions -> (list of dicts or None, stats)."""
        jobs = np.ascontiguousarray(jobs, dtype=TB_JOB_DTYPE)
        out = (Alignment * max(1, jobs.size))()
        cap = int(np.sum(jobs["win_len"].astype(np.int64))) + 4096 * jobs.size + 64
        ops = np.zeros(cap, np.uint32)
        st = TracebackStats()
        self._check(self.lib.saber_gpu_traceback(self.h, _ptr(jobs), jobs.size, int(band_pad), int(max_dir_bytes),
                                                 out, _ptr(ops), cap, ctypes.byref(st)), "traceback")
        res = [None if out[t].status == 0 else _alignment_dict(out[t], ops) for t in range(jobs.size)]
        return res, st.as_dict()

    def load_db_mask(self, mask):
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        self._check(self.lib.saber_gpu_load_db_mask(self.h, _ptr(m), 0 if m is None else m.size), "load_db_mask")

    def load_db_mask_runs(self, runs):
        """Seed mask of the loaded database from half-open (start, end) runs, expanded on the device."""
        r = np.ascontiguousarray(np.asarray(runs, np.uint64).reshape(-1, 2))
        self._check(self.lib.saber_gpu_load_db_mask_runs(self.h, _ptr(r) if r.size else None, r.shape[0]),
                    "load_db_mask_runs")

    def tantan_mask(self, params, matrix, codes, offsets, want_probs=False):
        """Tantan seed mask of a batch of sequences -> (mask bool array, posteriors or None, masked, lambda)."""
        c = np.ascontiguousarray(codes, dtype=np.uint8)
        o = np.ascontiguousarray(offsets, dtype=np.uint64)
        m = np.ascontiguousarray(np.asarray(matrix).reshape(576), dtype=np.int32)
        n = int(o[-1]) if o.size else 0
        mask = np.zeros(max(n, 1), np.uint8)
        probs = np.zeros(max(n, 1), np.float32) if want_probs else None
        nm, lam = ctypes.c_uint64(), ctypes.c_double()
        self._check(self.lib.saber_gpu_tantan_mask(self.h, ctypes.byref(params), _ptr(m), _ptr(c), _ptr(o),
                                                   max(o.size - 1, 0), _ptr(mask), _ptr(probs), ctypes.byref(nm),
                                                   ctypes.byref(lam)), "tantan_mask")
        return mask[:n].astype(bool), None if probs is None else probs[:n], int(nm.value), float(lam.value)

    def tantan_mask_db(self, params, matrix):
        """Mask the loaded database on the device and install it as its seed mask -> (masked, lambda)."""
        m = np.ascontiguousarray(np.asarray(matrix).reshape(576), dtype=np.int32)
        nm, lam = ctypes.c_uint64(), ctypes.c_double()
        self._check(self.lib.saber_gpu_tantan_mask_db(self.h, ctypes.byref(params), _ptr(m), ctypes.byref(nm),
                                                      ctypes.byref(lam)), "tantan_mask_db")
        return int(nm.value), float(lam.value)

    def translate6(self, nt, nt_offsets, codon64):
        """Six frames of every nucleotide sequence -> (protein codes, offsets[6 * nseq + 1])."""
        x = np.ascontiguousarray(nt, dtype=np.uint8)
        o = np.ascontiguousarray(nt_offsets, dtype=np.uint64)
        aa = np.ascontiguousarray(codon64, dtype=np.uint8)
        nseq = max(o.size - 1, 0)
        total = int(o[-1] - o[0]) if o.size else 0
        out = np.zeros(max(2 * total + 6, 1), np.uint8)
        offs = np.zeros(6 * nseq + 1, np.uint64)
        self._check(self.lib.saber_gpu_translate6(self.h, _ptr(x) if x.size else None, _ptr(o), nseq, _ptr(aa),
                                                  _ptr(out), out.size, _ptr(offs)), "translate6")
        return out[:int(offs[-1])].copy(), offs

    def scan(self, params, q_mask=None, region_thr=None, out_cap=None):
        """Candidate regions of the loaded query set (REGION_DTYPE, ordered by query and region order)."""
        qm = None if q_mask is None else np.ascontiguousarray(q_mask, dtype=np.uint8)
        rt = None if region_thr is None else np.ascontiguousarray(region_thr, dtype=np.int32)
        cap = out_cap or 1 << 20
        for _ in range(4):
            out = np.zeros(cap, REGION_DTYPE)
            n = ctypes.c_uint64()
            st = ScanStats()
            rc = self.lib.saber_gpu_scan(self.h, ctypes.byref(params), _ptr(qm), _ptr(rt), _ptr(out), cap,
                                         ctypes.byref(n), ctypes.byref(st))
            if rc == 0:
                return out[:n.value].copy(), st.as_dict()
            if n.value > cap:
                cap = int(n.value)
                continue
            self._check(rc, "scan")
        self._check(rc, "scan")

    def search(self, cparams, db_codes, db_offsets, q_codes, q_offsets, q_mask=None):
        """saber_gpu_search: (HIT_DTYPE array ordered by query, ops uint32 array, stats dict)."""
        db = np.ascontiguousarray(db_codes, dtype=np.uint8)
        do = np.ascontiguousarray(db_offsets, dtype=np.uint64)
        qc = np.ascontiguousarray(q_codes, dtype=np.uint8)
        qo = np.ascontiguousarray(q_offsets, dtype=np.uint64)
        qm = None if q_mask is None else np.ascontiguousarray(q_mask, dtype=np.uint8)
        hcap, ocap = 1 << 16, 1 << 20
        for _ in range(3):
            hits = np.zeros(hcap, HIT_DTYPE)
            ops = np.zeros(ocap, np.uint32)
            nh, no = ctypes.c_uint64(), ctypes.c_uint64()
            st = SearchStats()
            rc = self.lib.saber_gpu_search(self.h, ctypes.byref(cparams), _ptr(db), _ptr(do), do.size - 1, _ptr(qc),
                                           _ptr(qo), qo.size - 1, _ptr(qm), _ptr(hits), hcap, ctypes.byref(nh),
                                           _ptr(ops), ocap, ctypes.byref(no), ctypes.byref(st))
            if rc == 0:
                return hits[:nh.value].copy(), ops[:no.value].copy(), st.as_dict()
            if rc == -5 and (nh.value > hcap or no.value > ocap):  # SABER_ERR_CAP
                hcap, ocap = max(hcap, int(nh.value)), max(ocap, int(no.value))
                continue
            self._check(rc, "search")
        self._check(rc, "search")

    # ---- learned triage ----
    def triage_grads(self, model, rows, labels, pos_weight=1.0):
        """(gradients in the model layout, loss) of one forward + backward pass."""
        m = np.ascontiguousarray(model, dtype=np.float32)
        x = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, TRIAGE_ROW_FLOATS)
        y = np.ascontiguousarray(labels, dtype=np.uint8)
        g = np.zeros(TRIAGE_MODEL_FLOATS, np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.saber_gpu_triage_grads(self.h, _ptr(m), _ptr(x), _ptr(y), x.shape[0],
                                                    float(pos_weight), _ptr(g), ctypes.byref(loss)), "triage_grads")
        return g, loss.value

    def triage_train(self, model, rows, labels, epochs=8, batch=1024, lr=1e-3, pos_weight=1.0, weight_decay=0.0,
                     seed=0):
        """Adam training on the GPU; returns (trained model, stats)."""
        m = np.ascontiguousarray(model, dtype=np.float32).copy()
        x = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, TRIAGE_ROW_FLOATS)
        y = np.ascontiguousarray(labels, dtype=np.uint8)
        cfg = TriageTrainCfg(epochs=epochs, batch=batch, lr=lr, pos_weight=pos_weight, weight_decay=weight_decay,
                             seed=seed)
        st = TriageTrainStats()
        self._check(self.lib.saber_gpu_triage_train(self.h, _ptr(m), _ptr(x), _ptr(y), x.shape[0], ctypes.byref(cfg),
                                                    ctypes.byref(st)), "triage_train")
        return m, {"steps": int(st.steps), "final_loss": float(st.final_loss)}

    def triage_predict(self, model, rows):
        m = np.ascontiguousarray(model, dtype=np.float32)
        x = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, TRIAGE_ROW_FLOATS)
        out = np.zeros(x.shape[0], np.float32)
        self._check(self.lib.saber_gpu_triage_predict(self.h, _ptr(m), _ptr(x), x.shape[0], _ptr(out)),
                    "triage_predict")
        return out

    def set_triage(self, model, threshold=0.0):
        m = None if model is None else np.ascontiguousarray(model, dtype=np.float32)
        self._check(self.lib.saber_gpu_set_triage(self.h, _ptr(m), float(threshold)), "set_triage")

    def collect_regions(self, on=True):
        self._check(self.lib.saber_gpu_collect_regions(self.h, 1 if on else 0), "collect_regions")

    def collected_regions(self):
        """(feature rows n x 32, labels, logits) of the regions of the last search."""
        n = ctypes.c_uint64()
        self.lib.saber_gpu_collected_regions(self.h, None, None, None, 0, ctypes.byref(n))
        k = int(n.value)
        rows = np.zeros((k, TRIAGE_ROW_FLOATS), np.float32)
        y = np.zeros(k, np.uint8)
        z = np.zeros(k, np.float32)
        self._check(self.lib.saber_gpu_collected_regions(self.h, _ptr(rows), _ptr(y), _ptr(z), k, ctypes.byref(n)),
                    "collected_regions")
        return rows, y, z

    @property
    def strip_rows(self):
        return int(self.lib.saber_gpu_get_strip_rows(self.h))

    @strip_rows.setter
    def strip_rows(self, r):
        self._check(self.lib.saber_gpu_set_strip_rows(self.h, int(r)), "set_strip_rows")

    @property
    def graphs(self):
        """Captured scoring graphs on (default) or off."""
        return bool(self.lib.saber_gpu_get_graphs(self.h))

    @graphs.setter
    def graphs(self, on):
        self._check(self.lib.saber_gpu_set_graphs(self.h, 1 if on else 0), "set_graphs")

    @property
    def graph_captures(self):
        return int(self.lib.saber_gpu_graph_captures(self.h))

    @property
    def pair_steps(self):
        """Paired-strip threshold in column steps (0xFFFFFFFF: never pair)."""
        return int(self.lib.saber_gpu_get_pair_steps(self.h))

    @pair_steps.setter
    def pair_steps(self, v):
        self._check(self.lib.saber_gpu_set_pair_steps(self.h, int(v) & 0xFFFFFFFF), "set_pair_steps")

    @property
    def long_steps(self):
        """Lane-sweep length (column steps) above which a job goes to the warp-per-job kernel."""
        return int(self.lib.saber_gpu_get_long_steps(self.h))

    @long_steps.setter
    def long_steps(self, v):
        self._check(self.lib.saber_gpu_set_long_steps(self.h, int(v) & 0xFFFFFFFF), "set_long_steps")

    @property
    def scan_table_bytes(self):
        """Seed-table bytes per database pass of the scan (shapes split into passes)."""
        return int(self.lib.saber_gpu_get_scan_table_bytes(self.h))

    @scan_table_bytes.setter
    def scan_table_bytes(self, v):
        self._check(self.lib.saber_gpu_set_scan_table_bytes(self.h, int(v)), "set_scan_table_bytes")

    def probe_int_peak(self):
        """(DPX s16x2 lane-instructions/s, int32 max lane-instructions/s) of this GPU."""
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.saber_gpu_probe_int_peak(self.h, ctypes.byref(a), ctypes.byref(b)), "probe_int_peak")
        return a.value, b.value

    PIPE_OPS = ("viaddmax_s16x2", "vimax3_s16x2_relu", "vadd2", "prmt", "viaddmax_s16x2 + vadd2")

    def probe_pipe_rates(self):
        """Lane-instructions/s of the packed cell's instructions, each alone, and a
        fused add-max chain beside a packed-add chain (dict by PIPE_OPS name)."""
        r = (ctypes.c_double * 5)()
        self._check(self.lib.saber_gpu_probe_pipe_rates(self.h, r), "probe_pipe_rates")
        return dict(zip(self.PIPE_OPS, list(r)))

    def score_banded_many(self, query, bias, subjects, bands):
        """One query against banded windows: list of (window codes, (lo, hi))."""
        q = np.ascontiguousarray(query, dtype=np.uint8)
        b = None if bias is None else np.ascontiguousarray(bias, dtype=np.int8)
        wins = [np.asarray(s, dtype=np.uint8) for s in subjects]
        offs = np.zeros(len(wins) + 1, dtype=np.uint64)
        offs[1:] = np.cumsum([w.size for w in wins]) if wins else []
        cat = np.concatenate(wins) if wins and offs[-1] > 0 else np.zeros(1, np.uint8)
        lo = np.ascontiguousarray([x[0] for x in bands], dtype=np.int64)
        hi = np.ascontiguousarray([x[1] for x in bands], dtype=np.int64)
        out = np.empty(len(wins), dtype=np.int32)
        self._check(self.lib.saber_gpu_score_banded_many(self.h, _ptr(q), q.size, _ptr(b), _ptr(cat), _ptr(offs),
                                                         _ptr(lo), _ptr(hi), len(wins), _ptr(out)),
                    "score_banded_many")
        return out

    def score_windows(self, query, bias, windows, matrix, gap_open, gap_extend):
        q = np.ascontiguousarray(query, dtype=np.uint8)
        b = None if bias is None else np.ascontiguousarray(bias, dtype=np.int8)
        wins = [np.asarray(s, dtype=np.uint8) for s in windows]
        offs = np.zeros(len(wins) + 1, dtype=np.uint64)
        if wins:
            offs[1:] = np.cumsum([w.size for w in wins])
        cat = np.concatenate(wins) if wins and offs[-1] > 0 else np.zeros(1, np.uint8)
        mat = _flat_matrix(matrix)
        out = np.empty(len(wins), dtype=np.int32)
        self._check(self.lib.saber_gpu_score_windows(self.h, _ptr(q), q.size, _ptr(b), _ptr(cat), _ptr(offs),
                                                     len(wins), _ptr(mat), int(gap_open), int(gap_extend),
                                                     _ptr(out)), "score_windows")
        return out


class CudaBackend:
    """The reference's ``ScoreBackend`` (src/gpu/mod.rs:45-59) on the GB300 library.

    ``score_windows`` returns exact int32 scores in input order or raises
    :class:`SaberGpuError`; it never returns a saturated score.  Calls are
    serialised per handle by the library (as src/gpu/cuda.rs:144 does with a
    mutex)."""

    def __init__(self, device=0):
        self.dev = Device(device)

    def name(self):
        return "cuda-gb300"

    def score_windows(self, query, bias, windows, matrix, gaps):
        go, ge = gaps
        return self.dev.score_windows(query, bias, windows, matrix, go, ge)


def score_banded_many(dev, query, bias, jobs, scheme):
    """``score_banded_many(query, bias, jobs, scheme)`` (band_simd8.rs:78): jobs
    are (subject window, (lo, hi)) pairs, scheme is (matrix, gap_open, gap_extend)."""
    matrix, go, ge = scheme
    dev.set_scheme(matrix, go, ge)
    return dev.score_banded_many(query, bias, [j[0] for j in jobs], [j[1] for j in jobs])
