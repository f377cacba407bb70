"""Seeded synthetic workloads (no external data is used).

* :func:`protein_db` — queries and subjects with log-normal lengths (median
  250, sigma 0.6, clipped), residues iid from the Robinson & Robinson (1991)
  background frequencies (the table the reference carries for its
  composition bias, src/scoring/bias.rs:30-53), and a fraction of subjects
  planted as homologs of random queries: substitutions drawn from the
  BLOSUM62 target frequencies p_a p_b exp(lambda_u S_ab) (lambda_u = 0.3176,
  src/scoring/stats.rs:145) mixed with identity to reach the requested
  identity, indels at a per-residue rate with geometric lengths.
* :func:`band_jobs` — banded scoring jobs shaped like the reference's region
  windows (src/search/engine.rs:1223-1234,1288-1302): a diagonal d0, a band
  half-width h, the subject window [d0 - h, m + d0 + h) clipped to the
  subject, the band [d0 - h, d0 + h] in window coordinates.  A share of the
  jobs sit on the planted homolog's true diagonal, the rest are random
  (query, subject, diagonal) triples.
"""
import numpy as np

from .gpu import JOB_DTYPE
from .scoring import matrix as _matrix

ROBINSON_PER_1000 = np.array([
    78.05, 51.29, 44.87, 53.64, 19.25, 42.64, 62.95, 73.77, 21.99, 51.42,
    90.19, 57.44, 22.43, 38.56, 52.03, 71.20, 58.41, 13.30, 32.16, 64.41])
BACKGROUND = ROBINSON_PER_1000 / ROBINSON_PER_1000.sum()
LAMBDA_U = 0.3176


def _lengths(rng, n, median=250.0, sigma=0.6, lo=30, hi=1500):
    x = rng.lognormal(np.log(median), sigma, size=n)
    return np.clip(np.rint(x), lo, hi).astype(np.int64)


def _target_conditional():
    s = _matrix("BLOSUM62")[:20, :20].astype(np.float64)
    t = BACKGROUND[:, None] * BACKGROUND[None, :] * np.exp(LAMBDA_U * s)
    cond = t / t.sum(axis=1, keepdims=True)          # P(b | a)
    return cond


class ProteinSet:
    """Concatenated sequences: codes (uint8) and offsets (uint64, n + 1)."""

    def __init__(self, codes, offsets):
        self.codes = codes
        self.offsets = offsets

    def __len__(self):
        return self.offsets.size - 1

    def seq(self, i):
        return self.codes[self.offsets[i]:self.offsets[i + 1]]

    def lengths(self):
        return np.diff(self.offsets).astype(np.int64)


def _concat(seqs):
    lens = np.array([len(s) for s in seqs], dtype=np.uint64)
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum(lens)
    codes = np.concatenate(seqs).astype(np.uint8) if len(seqs) else np.zeros(0, np.uint8)
    return ProteinSet(codes, off)


def mutate(rng, seq, identity, indel_rate, cond=None):
    """Planted homolog of `seq`: substitutions at the target identity plus indels."""
    if cond is None:
        cond = _target_conditional()
    p_self = float(np.sum(BACKGROUND * np.diag(cond)))
    keep = max(0.0, (identity - p_self) / (1.0 - p_self))
    out = seq.copy()
    sub = rng.random(seq.size) >= keep
    if sub.any():
        # inverse-CDF draw from P(b | a) per substituted position
        cdf = np.cumsum(cond, axis=1)
        a = np.minimum(seq[sub], 19)
        u = rng.random(a.size)
        out[sub] = (u[:, None] > cdf[a]).sum(axis=1).astype(np.uint8)
    if indel_rate <= 0:
        return out
    pieces = []
    pos = 0
    n = out.size
    events = np.flatnonzero(rng.random(n) < indel_rate)
    for e in events:
        if e < pos:
            continue
        pieces.append(out[pos:e])
        ln = int(rng.geometric(1.0 / 3.0))
        if rng.random() < 0.5:
            pieces.append(rng.choice(20, size=ln, p=BACKGROUND).astype(np.uint8))
            pos = e
        else:
            pos = min(n, e + ln)
    pieces.append(out[pos:])
    return np.concatenate(pieces).astype(np.uint8)


def protein_db(seed, n_queries, n_subjects, planted_frac=0.10, identity=0.40, indel_rate=0.02,
               max_len=1500, reversed_frac=0.0, identity_range=None):
    """Queries, subjects and the planted (subject -> query, diagonal offset) map.

    Returns (queries, subjects, planted) with planted an int64 array of the
    query index each subject was derived from (-1 for background/decoys)."""
    rng = np.random.default_rng(seed)
    qlen = _lengths(rng, n_queries, hi=max_len)
    qs = [rng.choice(20, size=int(l), p=BACKGROUND).astype(np.uint8) for l in qlen]
    slen = _lengths(rng, n_subjects, hi=max_len)
    cond = _target_conditional()
    planted = np.full(n_subjects, -1, dtype=np.int64)
    n_pl = int(round(planted_frac * n_subjects))
    pl_idx = rng.choice(n_subjects, size=n_pl, replace=False) if n_pl else np.zeros(0, np.int64)
    planted[pl_idx] = rng.integers(0, n_queries, size=n_pl)
    n_rev = int(round(reversed_frac * n_subjects))
    free = np.flatnonzero(planted < 0)
    rev_idx = rng.choice(free, size=min(n_rev, free.size), replace=False) if n_rev else np.zeros(0, np.int64)
    is_rev = np.zeros(n_subjects, dtype=bool)
    is_rev[rev_idx] = True
    total_bg = int(slen[planted < 0].sum())
    bg = rng.choice(20, size=total_bg, p=BACKGROUND).astype(np.uint8)
    subs = []
    bpos = 0
    for s in range(n_subjects):
        q = planted[s]
        if q >= 0:
            ident = identity if identity_range is None else rng.uniform(*identity_range)
            subs.append(mutate(rng, qs[q], ident, indel_rate, cond)[:max(30, max_len)])
        else:
            l = int(slen[s])
            seq = bg[bpos:bpos + l]
            bpos += l
            if is_rev[s]:
                src = qs[int(rng.integers(0, n_queries))]
                seq = src[::-1].copy()
            subs.append(seq)
    return _concat(qs), _concat(subs), planted


def query_bias(seed, queries, levels=(-1, 0, 1)):
    """Per-position int8 bias values for the queries (a stand-in for the
    composition-bias correction; the kernels only add it per column)."""
    rng = np.random.default_rng(seed)
    return rng.choice(np.asarray(levels, dtype=np.int8), size=queries.codes.size)


def band_jobs(seed, queries, subjects, planted, n_jobs, half_min=8, half_max=128, related_frac=0.25,
              win_min=30, win_max=2000):
    """Banded region jobs (JOB_DTYPE) over `subjects` for `queries`."""
    rng = np.random.default_rng(seed)
    qlen = queries.lengths()
    slen = subjects.lengths()
    soff = subjects.offsets.astype(np.int64)
    jobs = np.zeros(n_jobs, dtype=JOB_DTYPE)
    related = np.flatnonzero(planted >= 0)
    n_rel = int(round(related_frac * n_jobs)) if related.size else 0
    subj = np.empty(n_jobs, dtype=np.int64)
    qry = np.empty(n_jobs, dtype=np.int64)
    d0 = np.empty(n_jobs, dtype=np.int64)
    if n_rel:
        subj[:n_rel] = related[rng.integers(0, related.size, size=n_rel)]
        qry[:n_rel] = planted[subj[:n_rel]]
        d0[:n_rel] = rng.integers(-3, 4, size=n_rel)   # near the homolog's main diagonal
    nr = n_jobs - n_rel
    subj[n_rel:] = rng.integers(0, slen.size, size=nr)
    qry[n_rel:] = rng.integers(0, qlen.size, size=nr)
    m = qlen[qry]
    sl = slen[subj]
    d0[n_rel:] = (rng.random(nr) * (m[n_rel:] + sl[n_rel:] - 1)).astype(np.int64) - (m[n_rel:] - 1)
    h = rng.integers(half_min, half_max + 1, size=n_jobs)
    wlo = np.clip(d0 - h, 0, sl)
    whi = np.clip(m + d0 + h, wlo, sl)
    # widen short windows to win_min where the subject allows, cap at win_max
    short = (whi - wlo) < win_min
    whi = np.where(short, np.minimum(sl, wlo + win_min), whi)
    wlo = np.where(short & ((whi - wlo) < win_min), np.maximum(0, whi - win_min), wlo)
    whi = np.minimum(whi, wlo + win_max)
    jobs["query"] = qry
    jobs["subject"] = subj
    jobs["win_begin"] = soff[subj] + wlo
    jobs["win_len"] = whi - wlo
    jobs["band_lo"] = d0 - h - wlo
    jobs["band_hi"] = d0 + h - wlo
    perm = rng.permutation(n_jobs)
    return jobs[perm]


def dna_db(seed, n_queries, n_subjects, qlen=(1000, 10000), slen=(1000, 10000), planted_frac=0.10,
           identity_range=(0.80, 0.95), indel_rate=0.01):
    """Nucleotide queries and subjects, codes 0..3 = A, C, G, T, uniform
    (GC 0.5); a fraction of subjects are planted homologs of a random query
    (substitutions and indels at the given rates, embedded in background)."""
    rng = np.random.default_rng(seed)
    ql = rng.integers(qlen[0], qlen[1] + 1, size=n_queries)
    qs = [rng.integers(0, 4, size=int(l)).astype(np.uint8) for l in ql]
    sl = rng.integers(slen[0], slen[1] + 1, size=n_subjects)
    planted = np.full(n_subjects, -1, dtype=np.int64)
    n_pl = int(round(planted_frac * n_subjects))
    pl_idx = rng.choice(n_subjects, size=n_pl, replace=False) if n_pl else np.zeros(0, np.int64)
    planted[pl_idx] = rng.integers(0, n_queries, size=n_pl)
    subs = []
    for s in range(n_subjects):
        q = planted[s]
        bg = rng.integers(0, 4, size=int(sl[s])).astype(np.uint8)
        if q >= 0:
            src = qs[q]
            a = int(rng.integers(0, max(1, src.size // 2)))
            b = int(rng.integers(a + min(200, src.size - a), src.size + 1))
            seg = src[a:b].copy()
            ident = rng.uniform(*identity_range)
            sub = rng.random(seg.size) > ident
            seg[sub] = (seg[sub] + rng.integers(1, 4, size=int(sub.sum()))) % 4
            # indel events at rate indel_rate per position: a deletion skips,
            # an insertion adds, geometric(1/3) bases (mean 3)
            ev = np.flatnonzero(rng.random(seg.size) < indel_rate)
            is_del = rng.random(ev.size) < 0.5
            klen = rng.geometric(1.0 / 3.0, size=ev.size)
            out = []
            prev = 0
            for e, d, k in zip(ev.tolist(), is_del.tolist(), klen.tolist()):
                if e < prev:
                    continue  # inside a deleted stretch
                out.append(seg[prev:e])
                if d:
                    prev = e + k
                else:
                    out.append(rng.integers(0, 4, size=k).astype(np.uint8))
                    prev = e
            out.append(seg[prev:])
            body = np.concatenate(out) if out else np.zeros(0, np.uint8)
            cut = int(rng.integers(0, bg.size + 1))
            bg = np.concatenate([bg[:cut], body, bg[cut:]]).astype(np.uint8)
        subs.append(bg)
    return _concat(qs), _concat(subs), planted


def back_translate(rng, protein, n_frac=0.0):
    """DNA codes (0..3 = A, C, G, T; 4 = N) encoding a protein with random
    synonymous codons of the standard code; X and residues without a codon
    (B, Z) become NNN, and a fraction n_frac of bases is set to N."""
    from .translation import codon_table
    ct = codon_table("standard")
    table = np.full((256, 6), -1, np.int64)  # codons per protein code
    count = np.zeros(256, np.int64)
    for idx, aa in enumerate(ct.tolist()):
        table[aa, count[aa]] = idx
        count[aa] += 1
    p = np.asarray(protein, np.uint8)
    k = np.floor(rng.random(p.size) * np.maximum(count[p], 1)).astype(np.int64)
    c = table[p, k]
    out = np.full((p.size, 3), 4, np.uint8)
    ok = c >= 0
    out[ok, 0] = c[ok] // 16
    out[ok, 1] = (c[ok] // 4) % 4
    out[ok, 2] = c[ok] % 4
    dna = out.reshape(-1)
    if n_frac > 0:
        dna[rng.random(dna.size) < n_frac] = 4
    return dna


def reverse_complement(dna):
    """Reverse complement of DNA codes (N stays N)."""
    d = np.asarray(dna, np.uint8)[::-1]
    return np.where(d > 3, d, 3 - d).astype(np.uint8)


def translated_db(seed, n_queries, n_subjects, mode, flank=(0, 300), **kw):
    """A protein workload (protein_db) with one side as DNA: mode "nx" turns
    the queries into DNA, "pn" the subjects; each DNA sequence is the
    back-translated protein between random flanks, on the minus strand for
    half of them (so hits come from all six frames)."""
    qs, ss, planted = protein_db(seed, n_queries, n_subjects, **kw)
    rng = np.random.default_rng(seed + 7)
    side = qs if mode == "nx" else ss
    seqs = []
    for i in range(len(side)):
        body = back_translate(rng, side.seq(i), n_frac=0.002)
        left = rng.integers(0, 4, size=int(rng.integers(flank[0], flank[1] + 1))).astype(np.uint8)
        right = rng.integers(0, 4, size=int(rng.integers(flank[0], flank[1] + 1))).astype(np.uint8)
        dna = np.concatenate([left, body, right])
        seqs.append(reverse_complement(dna) if rng.random() < 0.5 else dna)
    dna = _concat(seqs)
    return (dna, ss, planted) if mode == "nx" else (qs, dna, planted)
