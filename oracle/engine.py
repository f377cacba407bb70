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
