"""GPU parity of the scan schedule (seed tables, database scan, window filter,
coverage + X-drop, regions, caps): the candidate regions and the work
counters equal the oracle's restatement of Engine::search_scan."""
import numpy as np
import pytest

from oracle import oracle as orc
from saber_gb300 import presets, synth
from saber_gb300.gpu import scan_params
from saber_gb300.scoring import matrix

pytestmark = pytest.mark.gpu
B62 = matrix("BLOSUM62")
COUNTERS = ("seed_positions", "seeds_frequent_skipped", "hits", "hits_filtered", "ungapped_extensions",
            "extensions_avoided", "xdrop_steps", "hsps", "regions", "regions_weak_dropped", "regions_dropped_by_cap")


def _run(dev, qs, ss, bias, db_mask, q_mask, region_thr, shapes, alpha, **kw):
    amap, asz = alpha
    gp = scan_params(amap, asz, shapes, db_length=int(ss.codes.size), **kw)
    op = orc.make_scan_params(amap, asz, shapes, db_length=int(ss.codes.size), **kw)
    dev.set_scheme(B62, 11, 1)
    dev.load_db(ss.codes, ss.offsets)
    dev.load_db_mask(db_mask)
    dev.load_queries(qs.codes, qs.offsets, bias)
    got, gst = dev.scan(gp, q_mask, region_thr)
    want, ost = orc.scan_regions(ss.codes, ss.offsets, db_mask, qs.codes, qs.offsets, bias, q_mask, region_thr, B62, op)
    return got, gst, want, ost


def _check(got, gst, want, ost):
    assert got.size == want.size, (got.size, want.size)
    for f in ("query", "subject", "d_min", "d_max", "best"):
        assert np.array_equal(got[f], want[f]), f
    for k in COUNTERS:
        assert gst[k] == ost[k], (k, gst[k], ost[k])


@pytest.mark.parametrize("preset", ["default", "very-fast", "sensitive"])
def test_scan_regions_match_oracle(dev, preset):
    qs, ss, planted = synth.protein_db(7, 16, 1500)
    bias = synth.query_bias(8, qs)
    rng = np.random.default_rng(9)
    q_mask = (rng.random(qs.codes.size) < 0.05).astype(np.uint8)
    db_mask = (rng.random(ss.codes.size) < 0.03).astype(np.uint8)
    region_thr = rng.integers(40, 70, size=len(qs)).astype(np.int32)
    _, shapes, ids, kx, thr, cand, _, _, _, _ = presets.PRESETS[preset]
    got, gst, want, ost = _run(dev, qs, ss, bias, db_mask, q_mask, region_thr, shapes, presets.alphabet_map(),
                               min_ids=ids, exact_weight=kx, hsp_threshold=thr, max_candidates=cand)
    assert want.size > 0
    _check(got, gst, want, ost)


@pytest.mark.parametrize("per_subject", [2, 9])
def test_scan_caps_and_no_filter(dev, per_subject):
    """Small frequent-seed cap, no window filter, tiny per-subject and
    per-query region caps, full 20-letter alphabet with contiguous seeds.
    Per-subject caps up to 4 keep the top list in registers, larger ones in
    local memory."""
    qs, ss, planted = synth.protein_db(17, 10, 800)
    got, gst, want, ost = _run(dev, qs, ss, None, None, None, None, ["1111", "11011"], presets.full_alphabet(),
                               min_ids=0, exact_weight=0, seed_max_occ=6, max_regions_per_subject=per_subject,
                               max_candidates=7)
    assert ost["seeds_frequent_skipped"] > 0 and ost["regions_dropped_by_cap"] > 0
    _check(got, gst, want, ost)


def test_scan_with_empty_and_tiny_sequences(dev):
    """Subjects and queries of length 0 and 1-7 beside long ones (many
    sequences start inside one 256-position block of the owner tables, and
    long ones span several blocks): regions and counters still equal the
    oracle's."""
    from saber_gb300.synth import ProteinSet
    qs, ss, _ = synth.protein_db(27, 12, 600)
    rng = np.random.default_rng(28)

    def splice(seqs, n_tiny):
        parts = [seqs.seq(i) for i in range(len(seqs))]
        for _ in range(n_tiny):
            k = int(rng.integers(0, len(parts) + 1))
            parts.insert(k, rng.integers(0, 20, size=int(rng.integers(0, 8))).astype(np.uint8))
        parts.append(np.concatenate([seqs.seq(0)] * 12))  # one sequence over several blocks
        offs = np.zeros(len(parts) + 1, np.uint64)
        offs[1:] = np.cumsum([p.size for p in parts])
        return ProteinSet(np.concatenate(parts).astype(np.uint8), offs)

    q2, s2 = splice(qs, 6), splice(ss, 400)
    assert np.any(np.diff(s2.offsets.astype(np.int64)) == 0)
    got, gst, want, ost = _run(dev, q2, s2, None, None, None, None, presets.DS16, presets.alphabet_map(),
                               min_ids=27, exact_weight=2)
    assert want.size > 0
    _check(got, gst, want, ost)


def test_scan_filter_with_the_full_alphabet(dev):
    """The window filter with the 20-letter alphabet (too many letters for
    the combined one-byte codes: separate letter and full-code records)."""
    qs, ss, planted = synth.protein_db(37, 12, 900)
    bias = synth.query_bias(38, qs)
    got, gst, want, ost = _run(dev, qs, ss, bias, None, None, None, ["1111", "11011", "110101"],
                               presets.full_alphabet(), min_ids=27, exact_weight=2)
    assert want.size > 0 and ost["hits_filtered"] > 0
    _check(got, gst, want, ost)
