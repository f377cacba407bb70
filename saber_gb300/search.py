"""Batched protein / nucleotide search on the GB300 library.

The search API above the library's batch engine (saber_gpu_search, which
restates Engine::search_scan, src/search/engine/scan.rs:1261-1497, and the
shared Engine stages of src/search/engine.rs: query preparation, the GPU scan,
plan_windows, two-stage banded scoring, finish with E-values and the widening
traceback, make_hit), the search parameters and presets, hit records and BLAST
m8 rows (src/io/output.rs:20-52), and a pool of handles that keeps several
query batches in flight.

Every scoring, scan and traceback step runs on the GPU through the C ABI,
batched over the whole query batch; the host keeps the f64 statistics and
the bookkeeping, as the reference keeps them on its host.
"""
import math

import numpy as np

from . import presets as _presets
from .gpu import SearchParamsC, scan_params
from .masking import MaskingMode, Tantan
from .scoring import ALPHABET, matrix as _matrix, nucleotide as _nt_matrix
from .stats import SearchStatistics, gapped_nucleotide, gapped_protein

REF_DB_RESIDUES = 40_000_000  # engine.rs:522
I32_MAX = 2 ** 31 - 1


class SearchParams:
    """SearchParams (engine.rs:60-201) with the CLI defaults (src/bin/main.rs:494-538)."""

    def __init__(self, preset="default", **kw):
        (alpha, shapes, ids, kx, thr, cand, floor_frac, score_band, pre_band, exhaustive) = _presets.PRESETS[preset]
        self.preset = preset
        self.alphabet = alpha
        self.shapes = list(shapes)
        self.evalue = 10.0
        self.min_bitscore = None
        self.max_target_seqs = 10
        self.max_hsps = 1
        self.min_identity = 0.0
        self.min_query_cover = 0.0
        self.min_subject_cover = 0.0
        self.hsp_threshold = thr
        self.hsp_floor_fraction = floor_frac
        self.x_drop_ungapped = 20
        self.hit_filter_min_ids = ids
        self.hit_filter_exact_weight = kx
        self.band_pad = 16
        self.window_slack = 64
        self.score_band = score_band
        self.score_prefilter_band = pre_band
        self.score_prefilter_frac = 0.75
        self.max_candidates = cand
        self.max_regions_per_subject = 4
        self.seed_max_occ = 0
        self.comp_bias = True
        self.traceback_max_bytes = 32 << 20
        self.exhaustive = exhaustive
        self.ref_db_residues = REF_DB_RESIDUES
        self.evalue_model = "per-subject"
        # tantan seed masking of the queries and the database (--masking,
        # src/bin/main.rs:299-302, 472-517): the reference's default
        self.masking = MaskingMode.TANTAN
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(k)
            setattr(self, k, v)

    @classmethod
    def nucleotide(cls, k=11, **kw):
        """blastn (nn) mode (src/bin/main.rs:473-545, driver.rs:111-129,
        344-360): one contiguous k-mer shape over ACGT, no window filter, no
        composition bias, the default preset's other settings.  Use with
        Searcher(..., nucleotide=(2, -3), gap_open=7, gap_extend=2)."""
        p = cls("default")
        p.preset = "nn"
        p.alphabet = "acgt"
        p.shapes = ["1" * k]
        p.hit_filter_min_ids = 0
        p.comp_bias = False
        for key, v in kw.items():
            if not hasattr(p, key):
                raise AttributeError(key)
            setattr(p, key, v)
        return p


class Hit(dict):
    """One reported alignment (Hit, engine.rs:310-357), 1-based inclusive coordinates."""

    def identity(self):
        return 0.0 if self["columns"] == 0 else 100.0 * self["matches"] / self["columns"]

    def query_cover(self):
        return 0.0 if self["q_len"] == 0 else 100.0 * (self["q_end"] + 1 - self["q_start"]) / self["q_len"]

    def subject_cover(self):
        return 0.0 if self["s_len"] == 0 else 100.0 * (self["s_end"] + 1 - self["s_start"]) / self["s_len"]

    def cigar(self):
        return "".join("%d%s" % (l, op) for op, l in self["ops"])


def _rust_exp(e, prec):
    """Rust's `{:.Ne}`: mantissa with N decimals, exponent without sign padding."""
    m, x = ("%.*e" % (prec, e)).split("e")
    return "%se%d" % (m, int(x))


def format_evalue(e):
    """format_evalue (output.rs:38-52)."""
    if not math.isfinite(e):
        return "inf"
    if e == 0.0:
        return "0.0"
    if 0.001 <= e < 10.0:
        return "%.3f" % e
    return _rust_exp(e, 2)


def m8_row(query_id, subject_id, h):
    """write_m8_row (output.rs:20-36)."""
    return "%s\t%s\t%.2f\t%d\t%d\t%d\t%d\t%d\t%d\t%d\t%s\t%.1f" % (
        query_id, subject_id, h.identity(), h["columns"], h["mismatches"], h["gap_opens"], h["q_start"],
        h["q_end"], h["s_start"], h["s_end"], format_evalue(h["evalue"]), h["bitscore"])


def hits_from_records(hits, ops, nq, queries=None):
    """Hit lists per query from saber_gpu_search's hit records and operation
    runs; `queries` (optional): only the queries below that index."""
    out = [[] for _ in range(nq if queries is None else min(nq, queries))]
    for r in hits:
        qi = int(r["query"])
        if qi >= len(out):
            continue
        o, n = int(r["ops_offset"]), int(r["n_ops"])
        runs = [(chr(int(w) & 0xFF), int(w) >> 8) for w in ops[o:o + n]]
        out[qi].append(Hit(
            subject=int(r["subject"]), score=int(r["score"]), bitscore=float(r["bitscore"]),
            evalue=float(r["evalue"]), q_start=int(r["q_start"]), q_end=int(r["q_end"]),
            s_start=int(r["s_start"]), s_end=int(r["s_end"]), columns=int(r["columns"]),
            matches=int(r["matches"]), mismatches=int(r["mismatches"]), positives=int(r["positives"]),
            gap_opens=int(r["gap_opens"]), gap_columns=int(r["gap_columns"]), q_len=int(r["q_len"]),
            s_len=int(r["s_len"]), ops=runs, exact=bool(r["exact"])))
    return out



class Searcher:
    """A database resident on the GPU and the search configuration; search()
    runs one batch of queries end to end."""

    def __init__(self, dev, db_codes, db_offsets, params=None, matrix_name="BLOSUM62", gap_open=11, gap_extend=1,
                 db_mask=None, nucleotide=None, stats_size=None, db_mask_runs=None):
        """stats_size: (database length, sequences) of the statistics when they
        are not the loaded residues and subjects (a translated database:
        nucleotides / 3 and nucleotide sequences, driver.rs:575-583).
        db_mask_runs: the database seed mask as half-open runs (a SABERIDX
        file's "maskruns"), expanded on the device."""
        self.dev = dev
        self.p = params or SearchParams()
        self.is_protein = nucleotide is None
        self.matrix = _matrix(matrix_name) if self.is_protein else _nt_matrix(*nucleotide)
        self.go, self.ge = gap_open, gap_extend
        self.db_codes = np.ascontiguousarray(db_codes, dtype=np.uint8)
        self.db_offsets = np.ascontiguousarray(db_offsets, dtype=np.uint64)
        self.nsub = self.db_offsets.size - 1
        self.slen = np.diff(self.db_offsets.astype(np.int64))
        kp = gapped_protein(matrix_name, gap_open, gap_extend) if self.is_protein else \
            gapped_nucleotide(nucleotide[0], nucleotide[1], gap_open, gap_extend)
        self.karlin = kp
        self.stats_size = stats_size
        db_len, db_seqs = stats_size if stats_size else (int(self.db_codes.size), self.nsub)
        self.stats = SearchStatistics(kp, db_len, db_seqs, self.p.evalue_model)
        dev.set_scheme(self.matrix, gap_open, gap_extend)
        dev.load_db(self.db_codes, self.db_offsets)
        # seed masks: tantan on both sides for protein searches unless masking
        # is "none" (engine.rs:575-577; scan.rs:1078-1123); an explicit db_mask
        # replaces the database's
        masking = MaskingMode.parse(self.p.masking) if self.is_protein else MaskingMode.NONE
        self.tantan = Tantan.protein(dev) if masking == MaskingMode.TANTAN else None
        self.db_residues_masked = 0
        if db_mask_runs is not None:
            dev.load_db_mask_runs(db_mask_runs)
        elif db_mask is not None or self.tantan is None:
            dev.load_db_mask(db_mask)
        else:
            self.db_residues_masked = self.tantan.mask_database()
        if self.p.alphabet == "murphy10":
            amap, asz = _presets.alphabet_map()
        elif self.is_protein:
            amap, asz = _presets.full_alphabet()
        else:
            amap, asz = [i if i < 4 else 255 for i in range(24)], 4
        self.scan_params = scan_params(
            amap, asz, self.p.shapes, min_ids=self.p.hit_filter_min_ids, exact_weight=self.p.hit_filter_exact_weight,
            hsp_threshold=self.p.hsp_threshold, x_drop=self.p.x_drop_ungapped, window_slack=self.p.window_slack,
            max_regions_per_subject=self.p.max_regions_per_subject, max_candidates=min(self.p.max_candidates, I32_MAX),
            seed_max_occ=self.p.seed_max_occ, ref_db_residues=self.p.ref_db_residues,
            db_length=self.stats.db_length if stats_size else int(self.db_codes.size))
        self.counters = {}

    @classmethod
    def from_index(cls, dev, index, params=None, **kw):
        """A searcher over a SABERIDX database (saber_gb300.index.SeedIndex):
        its residues, offsets and stored mask runs, and for a translated
        database its statistics sizes (run_with_index, driver.rs:615+)."""
        if index.is_translated:
            kw.setdefault("stats_size", index.stats_size())
        return cls(dev, index.residues, index.subject_offsets, params, db_mask_runs=index.mask_runs, **kw)

    def query_mask(self, q_codes, q_offsets, q_mask=None):
        """The batch's query seed mask (Engine::prepare, engine.rs:769-775):
        the caller's, else tantan's when masking is on, else none."""
        if q_mask is not None:
            m = np.ascontiguousarray(q_mask, dtype=np.uint8)
            return m, int(np.count_nonzero(m))
        if self.tantan is None or int(q_offsets[-1]) == 0:
            return None, 0
        m, n = self.tantan.mask(q_codes, q_offsets)
        return m.view(np.uint8), n

    # ---- the batch, through the library's host engine (saber_gpu_search) ----
    def cparams(self):
        """saber_search_params of this configuration."""
        p, kp = self.p, self.karlin
        c = SearchParamsC()
        c.evalue = p.evalue
        c.min_bitscore = math.nan if p.min_bitscore is None else p.min_bitscore
        c.max_target_seqs, c.max_hsps = p.max_target_seqs, p.max_hsps
        c.min_identity, c.min_query_cover, c.min_subject_cover = p.min_identity, p.min_query_cover, \
            p.min_subject_cover
        c.hsp_threshold, c.hsp_floor_fraction = p.hsp_threshold, p.hsp_floor_fraction
        c.band_pad, c.window_slack = p.band_pad, min(p.window_slack, I32_MAX)
        c.score_band, c.score_prefilter_band = p.score_band, p.score_prefilter_band
        c.score_prefilter_frac = p.score_prefilter_frac
        c.comp_bias, c.exhaustive = int(bool(p.comp_bias)), int(bool(p.exhaustive))
        c.traceback_max_bytes, c.ref_db_residues = p.traceback_max_bytes, p.ref_db_residues
        c.evalue_model = 1 if p.evalue_model == "database" else 0
        c.is_protein = int(self.is_protein)
        c.lambda_, c.k, c.h, c.alpha, c.beta = kp.lambda_, kp.k, kp.h, kp.alpha, kp.beta
        c.even_scores_only = int(bool(kp.even_scores_only))
        c.scan = self.scan_params
        c.stats_num_seqs = self.stats.db_num_seqs if self.stats_size else 0
        return c

    def search(self, q_codes, q_offsets, q_mask=None):
        """Hits of every query of the batch: list (per query) of Hit, in report order."""
        q_offsets = np.ascontiguousarray(q_offsets, dtype=np.uint64)
        nq = q_offsets.size - 1
        q_mask, n_masked = self.query_mask(q_codes, q_offsets, q_mask)
        hits, ops, st = self.dev.search(self.cparams(), self.db_codes, self.db_offsets, q_codes, q_offsets, q_mask)
        st["query_residues_masked"] = n_masked
        st["queries"] = nq
        self.counters = st
        return hits_from_records(hits, ops, nq)

def decode_protein(codes):
    return bytes(ALPHABET[c] if c < 24 else ord("X") for c in codes).decode()


class SearchPool:
    """Several query batches in flight on one GPU: one handle (stream,
    scratch, resident database) per slot, batches dealt to the slots round
    robin and searched from one host thread per slot, so that one batch's
    host stages (plans, E-values, hit construction) overlap another's device
    stages.  Each batch's hits are those of Searcher.search on it alone."""

    def __init__(self, db_codes, db_offsets, params=None, slots=2, device=0, triage=None, **kw):
        from .gpu import Device
        self.searchers = [Searcher(Device(device), db_codes, db_offsets, params, **kw) for _ in range(slots)]
        if triage is not None:
            for se in self.searchers:
                se.dev.set_triage(*triage)

    def raw_batches(self, batches):
        """dev.search results (hits, ops, stats) of each (q_codes, q_offsets) batch, in order."""
        import threading
        out = [None] * len(batches)
        err = []

        def work(slot):
            se = self.searchers[slot]
            cp = se.cparams()
            try:
                for b in range(slot, len(batches), len(self.searchers)):
                    qc, qo = batches[b][0], batches[b][1]
                    out[b] = se.dev.search(cp, se.db_codes, se.db_offsets, qc, qo)
            except Exception as e:  # re-raised in the caller's thread
                err.append(e)

        threads = [threading.Thread(target=work, args=(s,)) for s in range(len(self.searchers))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if err:
            raise err[0]
        return out
