"""End-to-end GPU parity of one search batch (scan -> regions -> plans ->
two-stage banded scoring -> E-values -> widening traceback -> hits -> m8):
identical hit lists and m8 rows to the oracle pipeline on the same data."""
import numpy as np
import pytest

from oracle import engine as oeng
from saber_gb300 import synth
from saber_gb300.gpu import scan_params
from saber_gb300.search import Searcher, SearchParams, m8_row
from saber_gb300.stats import gapped_protein
from tests.py_engine import PyEngine

pytestmark = pytest.mark.gpu
KEYS = ("subject", "score", "q_start", "q_end", "s_start", "s_end", "columns", "matches", "mismatches", "positives",
        "gap_opens", "gap_columns", "ops", "exact")


def _compare(got, want):
    assert len(got) == len(want)
    for qi, (g, w) in enumerate(zip(got, want)):
        assert len(g) == len(w), (qi, len(g), len(w))
        for a, b in zip(g, w):
            for k in KEYS:
                assert a[k] == b[k], (qi, k, a[k], b[k])
            assert a["evalue"] == b["evalue"] and a["bitscore"] == b["bitscore"]
            assert m8_row("q%d" % qi, "s%d" % a["subject"], a) == oeng.m8_line("q%d" % qi, "s%d" % b["subject"], b)


def _case(dev, preset, seed, nq, ns, masks=True, **kw):
    qs, ss, planted = synth.protein_db(seed, nq, ns)
    rng = np.random.default_rng(seed + 1)
    db_mask = (rng.random(ss.codes.size) < 0.02).astype(np.uint8) if masks else None
    q_mask = (rng.random(qs.codes.size) < 0.03).astype(np.uint8) if masks else None
    if not masks:
        kw.setdefault("masking", "none")
    P = SearchParams(preset, **kw)
    se = Searcher(dev, ss.codes, ss.offsets, P, db_mask=db_mask)
    got = se.search(qs.codes, qs.offsets, q_mask)
    want = oeng.search_batch(ss.codes, ss.offsets, qs.codes, qs.offsets, P, se.matrix, 11, 1,
                             gapped_protein("BLOSUM62", 11, 1), se.scan_params, db_mask, q_mask)
    return got, want, se


def test_search_default_preset_matches_oracle(dev):
    got, want, se = _case(dev, "default", 123, 12, 700)
    assert sum(len(h) for h in want) > 0
    _compare(got, want)


def test_search_variants_match_oracle(dev):
    got, want, _ = _case(dev, "fast", 5, 8, 500, masks=False, max_target_seqs=3, max_hsps=2)
    _compare(got, want)
    got, want, _ = _case(dev, "default", 6, 8, 500, evalue_model="database", evalue=1e-3)
    _compare(got, want)


@pytest.mark.parametrize("preset,kw", [("default", {}), ("fast", {}), ("sensitive", {"max_target_seqs": 25}),
                                       ("exhaustive", {}), ("default", {"comp_bias": False, "min_bitscore": 30.0}),
                                       ("default", {"min_identity": 35.0, "max_hsps": 3})])
def test_native_engine_matches_python_engine(dev, preset, kw):
    """The library's host engine (saber_gpu_search) against the same stages
    written in Python over the same device calls: identical hits and m8 rows."""
    qs, ss, planted = synth.protein_db(77, 16 if preset == "exhaustive" else 30, 500 if preset == "exhaustive" else 1500)
    se = Searcher(dev, ss.codes, ss.offsets, SearchParams(preset, **kw))
    got = se.search(qs.codes, qs.offsets)
    want = PyEngine(se).search(qs.codes, qs.offsets)
    assert sum(len(h) for h in want) > 0
    _compare(got, want)


def test_nucleotide_search_matches_oracle(dev):
    """blastn (nn) mode: contiguous 11-mers over ACGT, +2/-3 with SABER gaps
    7/2 (BLAST 5/2), even-score E-values; hits and m8 rows identical to the
    oracle pipeline on planted 80-95 % identity homologs."""
    from saber_gb300.stats import gapped_nucleotide
    qs, ss, planted = synth.dna_db(71, 10, 120, qlen=(800, 3000), slen=(1000, 5000))
    P = SearchParams.nucleotide()
    se = Searcher(dev, ss.codes, ss.offsets, P, gap_open=7, gap_extend=2, nucleotide=(2, -3))
    got = se.search(qs.codes, qs.offsets)
    want = oeng.search_batch(ss.codes, ss.offsets, qs.codes, qs.offsets, P, se.matrix, 7, 2,
                             gapped_nucleotide(2, -3, 7, 2), se.scan_params, None, None, is_protein=False)
    assert sum(len(h) for h in want) >= 5
    _compare(got, want)
    assert [len(h) for h in got] == [len(h) for h in PyEngine(se).search(qs.codes, qs.offsets)]


@pytest.mark.gpu
def test_search_pool_matches_single_handle(dev):
    """Batches searched concurrently on a pool of handles give each batch the
    hits of a plain search of that batch alone."""
    from saber_gb300.search import Searcher, SearchPool, SearchParams
    qa, sa, _ = synth.protein_db(91, 40, 3000, reversed_frac=0.25, identity_range=(0.3, 0.6))
    qb, _, _ = synth.protein_db(92, 30, 1, reversed_frac=0.25, identity_range=(0.3, 0.6))
    batches = [(qa.codes, qa.offsets), (qb.codes, qb.offsets), (qa.codes, qa.offsets)]
    pool = SearchPool(sa.codes, sa.offsets, SearchParams("default"), slots=2)
    got = pool.raw_batches(batches)
    se = Searcher(dev, sa.codes, sa.offsets, SearchParams("default"))
    for (qc, qo), (hits, ops, st) in zip(batches, got):
        want, wops, _ = dev.search(se.cparams(), se.db_codes, se.db_offsets, qc, qo)
        assert np.array_equal(hits, want) and np.array_equal(ops, wops)
    assert sum(len(h) for h, _, _ in got) > 0
