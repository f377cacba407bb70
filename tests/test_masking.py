"""Tantan seed masking (masking.rs).

CPU: the oracle restatement is pinned to the reference's published lambda of
BLOSUM62 and to the behaviour its own tests check (masking.rs:628-706,
tests/cli.rs:118-133); the library's host lambda equals the oracle's.
GPU: the CUDA posteriors equal the oracle's bit for bit on the reference's
test sequence families (masking.rs:661-700: random residues of many lengths,
mutated periodic repeats of periods 1-60, a homopolymer, a 3-periodic run),
for the default 50 repeat states and other state counts; and a search with
tantan on both sides equals the oracle engine's with the oracle's masks."""
import numpy as np
import pytest

from oracle import oracle as orc
from saber_gb300 import masking, scoring

B62 = scoring.matrix("BLOSUM62")
# bench/results/v1.2.0/masking_f32_vs_f64.txt: "f32: lambda = 0.32403216734804396"
REF_LAMBDA_B62 = 0.32403216734804396


def _xorshift(seed=0x9E3779B97F4A7C15):
    x = seed
    mask = (1 << 64) - 1

    def rnd():
        nonlocal x
        x ^= (x << 13) & mask
        x ^= x >> 7
        x ^= (x << 17) & mask
        return x
    return rnd


def reference_test_sequences():
    """The sequence families of masking.rs:661-683, from the same xorshift generator."""
    rnd = _xorshift()
    seqs = []
    for n in (0, 1, 2, 3, 7, 8, 9, 48, 49, 50, 51, 56, 57, 300, 2000):
        seqs.append([rnd() % 24 for _ in range(n)])
    for period in range(1, 61):
        unit = [rnd() % 20 for _ in range(period)]
        s = [rnd() % 20 for _ in range(40)]
        for k in range(max(400 // period, 3) * period):
            s.append(rnd() % 20 if rnd() % 10 == 0 else unit[k % period])
        s.extend(rnd() % 20 for _ in range(40))
        seqs.append(s)
    seqs.append([5] * 1000)
    seqs.append([(0, 7, 15)[i % 3] for i in range(1500)])
    codes = np.array([c for s in seqs for c in s], np.uint8)
    offs = np.concatenate([[0], np.cumsum([len(s) for s in seqs])]).astype(np.uint64)
    return codes, offs


def test_oracle_lambda_is_the_reference_value():
    assert orc.tantan_lambda(B62) == REF_LAMBDA_B62


def test_library_lambda_equals_oracle_for_every_matrix():
    for name in ("BLOSUM45", "BLOSUM50", "BLOSUM62", "BLOSUM80", "BLOSUM90", "PAM30", "PAM70", "PAM250"):
        m = scoring.matrix(name)
        a, b = masking.implied_lambda(m), orc.tantan_lambda(m)
        assert (np.isnan(a) and np.isnan(b)) or a == b, (name, a, b)
    assert masking.implied_lambda(B62) == REF_LAMBDA_B62


def test_oracle_masks_repeats_not_diverse_sequence():
    """masking.rs:640-660: a poly-Q run is masked, a diverse head is not."""
    head = ("MSTNPKPQRKTKRNTNRRPQDVKFPGGGQIVGGVYLLPRRGPRLGVRATRKTSERSQPRGRRQPIPKARRPEGRTWAQPGYPWPLYGNEGCGWAGWLL"
            "SPRGSRPSWGPTDPRRRSRNLGKVIDTLTCGFADLMGYIPLVGAPLGGAARALAHGVRVLEDGVNYATGNLPGCSFSIFLLALLSCLTVPASA")
    s = head + "Q" * 30 + "MKVLAAGIVALLLAAGCSSSKEETTEEKPAEEAPKAEEKPAEEAPK"
    c = scoring.encode_protein(s)
    mask, probs, n = orc.tantan_mask(c, np.array([0, c.size], np.uint64), B62)
    assert mask[len(head):len(head) + 30].sum() >= 25
    assert mask[:60].sum() <= 6
    assert n == int(mask.sum())


def test_oracle_masks_low_complexity_queries():
    """tests/cli.rs:118-133: more than 900 of the 980 residues of a poly-Q
    query and a PEST-repeat query are masked."""
    c = np.concatenate([scoring.encode_protein("Q" * 500), scoring.encode_protein("PESTPEST" * 60)])
    _, _, n = orc.tantan_mask(c, np.array([0, 500, 980], np.uint64), B62)
    assert n > 900


def test_oracle_probabilities_in_unit_interval():
    """masking.rs:701-706."""
    c = scoring.encode_protein("AAAAAAAAAAPPPPPPPPGSGSGSGSGSGSMKVLHHHHHHHHHH")
    _, p, _ = orc.tantan_mask(c, np.array([0, c.size], np.uint64), B62)
    assert np.all((p >= 0.0) & (p <= 1.0001))


def test_mask_runs_split_at_subject_boundaries():
    mask = np.array([0, 1, 1, 1, 0, 1, 1, 0, 0, 1], bool)
    offs = np.array([0, 3, 6, 10])
    runs = masking.mask_runs(mask, offs)
    assert runs.tolist() == [[1, 3], [3, 4], [5, 6], [6, 7], [9, 10]]
    assert masking.MaskingMode.parse("on") == "tantan" and masking.MaskingMode.parse("off") == "none"
    with pytest.raises(ValueError):
        masking.MaskingMode.parse("dust")


@pytest.mark.gpu
@pytest.mark.parametrize("max_period", [50, 20, 64, 33, 7, 1])
def test_gpu_posteriors_bit_identical_to_oracle(dev, max_period):
    codes, offs = reference_test_sequences()
    P = masking.TantanParams(max_period=max_period)
    OP = orc.TantanParams(max_period=max_period)
    m, p, n, lam = dev.tantan_mask(P, B62, codes, offs, want_probs=True)
    wm, wp, wn = orc.tantan_mask(codes, offs, B62, OP)
    assert lam == REF_LAMBDA_B62
    assert p.view(np.uint32).tolist() == wp.view(np.uint32).tolist()
    assert np.array_equal(m, wm) and n == wn
    if max_period == 50:
        assert codes.size > 20000 and n > 1000


@pytest.mark.gpu
def test_gpu_mask_other_matrices_and_parameters(dev):
    rng = np.random.default_rng(3)
    lens = rng.integers(0, 900, 120)
    lens[:3] = [0, 1, 5000]
    codes = rng.integers(0, 24, int(lens.sum())).astype(np.uint8)
    # low-complexity stretches
    for s in range(0, codes.size - 200, 997):
        codes[s:s + 60] = codes[s]
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    for name, kw in (("BLOSUM45", {}), ("PAM30", {"decay": 1.0}), ("BLOSUM80", {"min_prob": 0.2}),
                     ("BLOSUM62", {"lambda_": 0.25, "repeat_start": 0.02, "repeat_end": 0.1})):
        mat = scoring.matrix(name)
        okw = {k: v for k, v in kw.items() if k != "lambda_"}
        m, p, n, lam = dev.tantan_mask(masking.TantanParams(**kw), mat, codes, offs, want_probs=True)
        wm, wp, wn = orc.tantan_mask(codes, offs, mat, orc.TantanParams(**okw), kw.get("lambda_", 0.0))
        assert p.view(np.uint32).tolist() == wp.view(np.uint32).tolist(), name
        assert np.array_equal(m, wm) and n == wn, name


@pytest.mark.gpu
def test_gpu_mask_masks_low_complexity_queries(dev):
    t = masking.Tantan.protein(dev)
    c = np.concatenate([scoring.encode_protein("Q" * 500), scoring.encode_protein("PESTPEST" * 60)])
    mask, n = t.mask(c, np.array([0, 500, 980], np.uint64))
    assert n > 900 and int(mask.sum()) == n
    assert t.lambda_ == REF_LAMBDA_B62


@pytest.mark.gpu
def test_search_with_tantan_matches_oracle_engine(dev):
    """Tantan on both sides (the reference's default): the GPU masks the
    database on the device and the queries per batch; the oracle engine gets
    the oracle's masks."""
    from oracle import engine as oeng
    from saber_gb300 import synth
    from saber_gb300.search import Searcher, SearchParams
    from saber_gb300.stats import gapped_protein
    from tests.test_search_gpu import _compare
    qs, ss, _ = synth.protein_db(41, 12, 900)
    # low-complexity stretches in a third of the queries and subjects
    rng = np.random.default_rng(9)
    for codes, offs in ((qs.codes, qs.offsets), (ss.codes, ss.offsets)):
        for i in range(0, len(offs) - 1, 3):
            a, b = int(offs[i]), int(offs[i + 1])
            if b - a > 80:
                s = a + int(rng.integers(0, b - a - 60))
                codes[s:s + 40] = rng.integers(0, 20)
    P = SearchParams("default")
    assert P.masking == "tantan"
    se = Searcher(dev, ss.codes, ss.offsets, P)
    got = se.search(qs.codes, qs.offsets)
    dbm, _, dn = orc.tantan_mask(ss.codes, ss.offsets, B62)
    qm, _, qn = orc.tantan_mask(qs.codes, qs.offsets, B62)
    assert se.db_residues_masked == dn and se.counters["query_residues_masked"] == qn and dn > 0 and qn > 0
    want = oeng.search_batch(ss.codes, ss.offsets, qs.codes, qs.offsets, P, se.matrix, 11, 1,
                             gapped_protein("BLOSUM62", 11, 1), se.scan_params, dbm.view(np.uint8),
                             qm.view(np.uint8))
    assert sum(len(h) for h in want) > 0
    _compare(got, want)
    # the python engine over the same device calls sees the same masks
    from tests.py_engine import PyEngine
    _compare(PyEngine(se).search(qs.codes, qs.offsets), want)


@pytest.mark.gpu
def test_gpu_mask_across_launches_and_odd_codes(dev):
    """Two 5 M-residue sequences exceed one launch's 8 M scratch rows (the
    batch is cut into launches, longest first); codes above 23 are clamped
    to 23 as the reference does; an empty batch and empty sequences."""
    rng = np.random.default_rng(11)
    lens = np.array([5_000_000, 0, 37, 5_000_000, 0], np.int64)
    codes = rng.integers(0, 20, int(lens.sum())).astype(np.uint8)
    for s in range(0, codes.size - 500, 250_000):
        codes[s:s + 300] = np.tile(rng.integers(0, 20, 7).astype(np.uint8), 43)[:300]
    codes[5_000_000:5_000_037] = np.array([24, 30, 255] * 12 + [23], np.uint8)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    m, p, n, _ = dev.tantan_mask(masking.TantanParams(), B62, codes, offs, want_probs=True)
    wm, wp, wn = orc.tantan_mask(codes, offs, B62)
    assert np.array_equal(p.view(np.uint32), wp.view(np.uint32))
    assert np.array_equal(m, wm) and n == wn and n > 0
    m0, p0, n0, _ = dev.tantan_mask(masking.TantanParams(), B62, np.zeros(0, np.uint8), np.zeros(1, np.uint64))
    assert m0.size == 0 and n0 == 0
