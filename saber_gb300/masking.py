"""Tantan seed masking (masking.rs), computed on the GPU.

Masked residues are excluded from seed formation on the query and the
database side; the residues themselves are kept for extension, alignment and
output, so masking only removes seeds (masking.rs:1-9).  The posteriors come
from the CUDA kernel of libsaber_gb300 (tantan.cu) and equal the reference's
f32 scalar body bit for bit.

    t = Tantan.protein(dev)                 # BLOSUM62, tantan's protein defaults
    mask, n = t.mask(codes, offsets)        # Tantan::mask (masking.rs:191)
    probs = t.repeat_probs(codes, offsets)  # Tantan::repeat_probs (masking.rs:184)
    t.mask_database()                       # scan.rs:1078-1123, on the loaded database
"""
import ctypes

import numpy as np

from . import scoring


class TantanParams(ctypes.Structure):
    """TantanParams (masking.rs:36-49) laid out as saber_tantan_params; lambda <= 0 = implied by the matrix."""
    _fields_ = [("repeat_start", ctypes.c_double), ("repeat_end", ctypes.c_double), ("max_period", ctypes.c_uint32),
                ("pad_", ctypes.c_uint32), ("decay", ctypes.c_double), ("min_prob", ctypes.c_double),
                ("lambda_", ctypes.c_double)]

    def __init__(self, repeat_start=0.005, repeat_end=0.05, max_period=50, decay=0.9, min_prob=0.5, lambda_=0.0):
        super().__init__(repeat_start, repeat_end, max_period, 0, decay, min_prob, lambda_)


class MaskingMode:
    """MaskingMode (masking.rs:54-80): "tantan" or "none"."""
    NONE = "none"
    TANTAN = "tantan"

    @staticmethod
    def parse(s):
        v = str(s).lower()
        if v in ("none", "0", "off", "no"):
            return MaskingMode.NONE
        if v in ("tantan", "1", "on", "yes"):
            return MaskingMode.TANTAN
        raise ValueError("unknown masking mode '%s' (expected tantan|none)" % v)


def implied_lambda(matrix):
    """implied_lambda (masking.rs:531-583) of a 24x24 matrix; NaN when no root exists."""
    from .gpu import load_library
    m = np.ascontiguousarray(np.asarray(matrix).reshape(576), dtype=np.int32)
    return float(load_library().saber_tantan_implied_lambda(ctypes.c_void_p(m.ctypes.data)))


class Tantan:
    """Reusable tantan masker on one device handle (Tantan, masking.rs:90-200)."""

    def __init__(self, dev, matrix=None, params=None, lam=None):
        self.dev = dev
        self.matrix = np.ascontiguousarray(scoring.matrix("BLOSUM62") if matrix is None else matrix, np.int32)
        self.params = params or TantanParams()
        if lam is not None:
            self.params.lambda_ = float(lam)
        self._lambda = None

    @classmethod
    def protein(cls, dev, matrix=None):
        """tantan's protein defaults (`tantan -p`) for the given matrix (BLOSUM62 by default)."""
        return cls(dev, matrix)

    @property
    def lambda_(self):
        if self._lambda is None:
            self._lambda = self.params.lambda_ if self.params.lambda_ > 0 else implied_lambda(self.matrix)
            if np.isnan(self._lambda):
                self._lambda = 0.3176
        return self._lambda

    def mask(self, codes, offsets):
        """Boolean seed mask of every residue and the number masked."""
        m, _, n, lam = self.dev.tantan_mask(self.params, self.matrix, codes, offsets)
        self._lambda = lam
        return m, n

    def repeat_probs(self, codes, offsets):
        """Posterior repeat probability (float32) of every residue."""
        _, p, _, lam = self.dev.tantan_mask(self.params, self.matrix, codes, offsets, want_probs=True)
        self._lambda = lam
        return p

    def mask_database(self):
        """Mask the handle's loaded database on the device and install it as the seed mask; returns the count."""
        n, lam = self.dev.tantan_mask_db(self.params, self.matrix)
        self._lambda = lam
        return n


def mask_runs(mask, offsets):
    """Half-open (start, end) runs of masked residues, in database coordinates (scan.rs:1100-1115)."""
    m = np.asarray(mask, bool).astype(np.int8)
    if m.size == 0:
        return np.zeros((0, 2), np.uint64)
    d = np.diff(np.concatenate([[0], m, [0]]))
    starts = np.flatnonzero(d == 1)
    ends = np.flatnonzero(d == -1)
    # runs never cross a subject boundary: split them there
    bounds = np.asarray(offsets, np.int64)[1:-1]
    out = []
    for a, b in zip(starts, ends):
        cuts = bounds[(bounds > a) & (bounds < b)]
        prev = a
        for c in cuts:
            out.append((prev, c))
            prev = c
        out.append((prev, b))
    return np.asarray(out, np.uint64).reshape(-1, 2)
