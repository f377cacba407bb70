"""Input generators of the reference's own unit tests, restated so the same
cases are regenerated here (test infrastructure)."""
import numpy as np

MASK64 = 0xFFFFFFFFFFFFFFFF


class Lcg:
    """banded.rs:530-536, band_simd8.rs:395-401: 64-bit LCG, (s >> 33) % m."""

    def __init__(self, seed):
        self.s = seed

    def next(self, m):
        self.s = (self.s * 6364136223846793005 + 1442695040888963407) & MASK64
        return (self.s >> 33) % m


def rand_seq(r, n):
    """banded.rs:538-540"""
    return np.array([r.next(24) for _ in range(n)], dtype=np.uint8)


def mutate(r, s):
    """banded.rs:542-563"""
    out = []
    i = 0
    while i < len(s):
        x = r.next(100)
        if x < 6:
            for _ in range(1 + r.next(12)):
                out.append(r.next(20))
        elif x < 12:
            i += 1 + r.next(10)
            continue
        elif x < 45:
            out.append(r.next(20))
        else:
            out.append(int(s[i]))
        i += 1
    return np.array(out, dtype=np.uint8)
