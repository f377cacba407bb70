"""Composition-bias correction of a query (Hauser et al. per-position
correction as src/scoring/bias.rs:64-122 computes it; host-side f64)."""
import numpy as np

from .synth import ROBINSON_PER_1000

BIAS_WINDOW_HALF = 20


def background_scores(m):
    """bias.rs:69-76: sum_a p_a S(r, a), summed in alphabet order."""
    s = 0.0
    for v in ROBINSON_PER_1000:
        s += float(v)
    p = [float(v) / s for v in ROBINSON_PER_1000]
    out = []
    for r in range(20):
        acc = 0.0
        for a in range(20):
            acc += p[a] * float(m[r][a])
        out.append(acc)
    return out


def composition_bias(query, m):
    """int8 correction per position (bias.rs:80-122)."""
    q = np.asarray(query, dtype=np.int64)
    n = q.size
    out = np.zeros(n, dtype=np.int8)
    if n < 2:
        return out
    m = np.asarray(m, dtype=np.int64)
    bg = background_scores(m)
    cols = m[:20][:, np.minimum(q, 23)]          # S(r, q_j) for r < 20
    csum = np.concatenate([np.zeros((20, 1), np.int64), np.cumsum(cols, axis=1)], axis=1)
    half = BIAS_WINDOW_HALF
    for i in range(n):
        r = int(q[i])
        if r >= 20:
            continue
        hi = min(i + half + 1, n)
        lo = max(i - half, 0)
        w = hi - lo
        if w < 2:
            continue
        acc = int(csum[r, hi] - csum[r, lo])
        own = int(m[r][r])
        neigh = float(acc - own) / float(w - 1)
        f = bg[r] - neigh
        v = int(f - 0.5) if f < 0.0 else int(f + 0.5)
        out[i] = max(-127, min(127, v))
    return out
