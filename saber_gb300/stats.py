"""Gapped Karlin-Altschul statistics, host-side f64 (src/scoring/stats.rs).

The NCBI blast_stat.c tables are package data (data/karlin.json); the
length adjustment is BLAST_ComputeLengthAdjustment as stats.rs:458-520 ports
it, and every E-value, bit score and score floor follows stats.rs:523-760
operation by operation (math.log / math.exp / math.sqrt are the platform
libm, as Rust's f64 methods are).
"""
import json
import math
import os

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "karlin.json")
_T = None
LN_2 = math.log(2.0)


def _tables():
    global _T
    if _T is None:
        with open(_DATA) as f:
            _T = json.load(f)
    return _T


class KarlinParams:
    """stats.rs:277-310"""

    def __init__(self, row, calibrated=True, even=False):
        _, _, lam, k, h, alpha, beta = row
        self.lambda_ = lam
        self.k = k
        self.log_k = math.log(k)
        self.h = h
        self.alpha = alpha
        self.alpha_d_lambda = alpha / lam
        self.beta = beta
        self.calibrated = calibrated
        self.even_scores_only = even


def gapped_protein(matrix_name, gap_open, gap_extend):
    """stats.rs:351-396: table row of (existence = open - extend, extension)."""
    t = _tables()["protein"][matrix_name.upper()]
    a, b = gap_open - gap_extend, gap_extend
    for r in t["gapped"]:
        if r[0] == a and r[1] == b:
            return KarlinParams(r)
    raise ValueError("no published gapped parameters for %s with SABER gaps %d/%d" % (matrix_name, gap_open,
                                                                                       gap_extend))


def gapped_nucleotide(reward, penalty, gap_open, gap_extend):
    """stats.rs:398-443"""
    a, b = gap_open - gap_extend, gap_extend
    for t in _tables()["nucleotide"]:
        if t["reward"] == reward and t["penalty"] == penalty:
            for r in t["rows"]:
                if r[0] == a and r[1] == b:
                    return KarlinParams(r, even=t["even_only"])
    raise ValueError("no published gapped parameters for nucleotide %d/%d gaps %d/%d" % (reward, penalty, gap_open,
                                                                                         gap_extend))


def compute_length_adjustment(k, log_k, alpha_d_lambda, beta, query_length, db_length, db_num_seqs):
    """BLAST_ComputeLengthAdjustment (stats.rs:458-520) -> (adjustment, converged)."""
    m = float(query_length)
    n = float(db_length)
    nn = float(db_num_seqs)
    ell_min = 0.0
    converged = False
    ell_next = 0.0
    a = nn
    mb = m * nn + n
    c = n * m - max(m, n) / k
    if c < 0.0:
        return 0, False
    ell_max = 2.0 * c / (mb + math.sqrt(mb * mb - 4.0 * a * c))
    for i in range(1, 21):
        ell = ell_next
        ss = (m - ell) * (n - nn * ell)
        ell_bar = alpha_d_lambda * (log_k + math.log(ss)) + beta
        if ell_bar >= ell:
            ell_min = ell
            if ell_bar - ell_min <= 1.0:
                converged = True
                break
            if ell_min == ell_max:
                break
        else:
            ell_max = ell
        if ell_min <= ell_bar <= ell_max:
            ell_next = ell_bar
        else:
            ell_next = ell_max if i == 1 else (ell_min + ell_max) / 2.0
    if converged:
        adj = int(ell_min)
        ell = math.ceil(ell_min)
        if ell <= ell_max:
            ss = (m - ell) * (n - nn * ell)
            if alpha_d_lambda * (log_k + math.log(ss)) + beta >= ell:
                adj = int(ell)
        return adj, True
    return int(ell_min), False


class SearchStatistics:
    """stats.rs:581-645 (model: 'per-subject' or 'database')."""

    def __init__(self, params, db_length, db_num_seqs, model="per-subject"):
        self.params = params
        self.db_length = max(int(db_length), 1)
        self.db_num_seqs = max(int(db_num_seqs), 1)
        self.model = model

    def for_query(self, query_len):
        p = self.params
        m = max(int(query_len), 1)
        adj, _ = compute_length_adjustment(p.k, p.log_k, p.alpha_d_lambda, p.beta, m, self.db_length,
                                           self.db_num_seqs)
        min_q = int(math.ceil(1.0 / p.k))
        if m - adj < min_q:
            adj = max(m - min_q, 0)
        eff_q = max(float(m - adj), 1.0)
        eff_db = max(float(self.db_length) - float(self.db_num_seqs) * float(adj), 1.0)
        return QueryStatistics(p, adj, eff_q, eff_db, self.model, m, float(self.db_num_seqs))


class QueryStatistics:
    """stats.rs:646-760"""

    def __init__(self, p, adj, eff_q, eff_db, model, query_len, num_seqs):
        self.lambda_ = p.lambda_
        self.k = p.k
        self.log_k = p.log_k
        self.length_adjustment = adj
        self.eff_query_len = eff_q
        self.eff_db_len = eff_db
        self.search_space = eff_q * eff_db
        self.even_scores_only = p.even_scores_only
        self.model = model
        self.query_len = query_len
        self.num_seqs = num_seqs
        self.alpha_d_lambda = p.alpha_d_lambda
        self.beta = p.beta

    def adj_score(self, raw):
        return float(raw - 1 if self.even_scores_only and raw % 2 != 0 else raw)

    def space_for(self, subject_len):
        if self.model == "database":
            return self.search_space
        m = max(self.query_len, 1)
        n = max(int(subject_len), 1)
        adj, _ = compute_length_adjustment(self.k, self.log_k, self.alpha_d_lambda, self.beta, m, n, 1)
        min_l = int(math.ceil(1.0 / self.k))
        adj = max(min(min(adj, max(m - min_l, 0)), max(n - min_l, 0)), 0)
        return self.num_seqs * float(max(m - adj, 1)) * float(max(n - adj, 1))

    def space_lower_bound(self, subject_len):
        if self.model == "database":
            return self.search_space
        m = float(max(self.query_len, 1))
        n = float(max(int(subject_len), 1))
        up = math.ceil(max(self.alpha_d_lambda * (self.log_k + math.log(m * n)) + self.beta, 0.0))
        return self.num_seqs * max(m - up, 1.0) * max(n - up, 1.0)

    def floor_lower_bound(self, evalue_cut, min_bits, subject_len, db_floor):
        if self.model == "database":
            return float(db_floor)
        f = 1.0
        if evalue_cut > 0.0 and math.isfinite(evalue_cut):
            f = max(f, math.log(self.k * self.space_lower_bound(subject_len) / evalue_cut) / self.lambda_)
        if min_bits is not None:
            f = max(f, (min_bits * LN_2 + self.log_k) / self.lambda_)
        if self.even_scores_only:
            f -= 1.0
        return f

    def evalue_for(self, raw, subject_len):
        return self.evalue_in(raw, self.space_for(subject_len))

    def evalue_in(self, raw, space):
        if raw <= 0:
            return math.inf
        s = self.adj_score(raw)
        e = self.k * space * math.exp(-self.lambda_ * s)
        return 2.2250738585072014e-308 if e == 0.0 else e

    def evalue(self, raw):
        if raw <= 0:
            return math.inf
        s = self.adj_score(raw)
        e = self.k * self.search_space * math.exp(-self.lambda_ * s)
        return 2.2250738585072014e-308 if e == 0.0 else e

    def bitscore(self, raw):
        if raw <= 0:
            return 0.0
        return (self.lambda_ * self.adj_score(raw) - self.log_k) / LN_2

    def min_score(self, evalue_cut, min_bits):
        floor = 1.0
        if evalue_cut > 0.0 and math.isfinite(evalue_cut):
            floor = max(floor, math.log((self.k * self.search_space) / evalue_cut) / self.lambda_)
        if min_bits is not None:
            floor = max(floor, (min_bits * LN_2 + self.log_k) / self.lambda_)
        if not math.isfinite(floor):
            return 1
        s = int(max(math.ceil(floor), 1.0))
        while s > 1 and self._passes(s - 1, evalue_cut, min_bits):
            s -= 1
        while not self._passes(s, evalue_cut, min_bits) and s < (2 ** 63 - 1) // 2:
            s += 1
        return s

    def _passes(self, s, evalue_cut, min_bits):
        return self.evalue(s) <= evalue_cut and (min_bits is None or self.bitscore(s) >= min_bits)
