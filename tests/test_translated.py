"""Translated modes (translation.rs, driver.rs:387-503): six-frame
translation, coordinates, and nx / pn searches.

CPU: the reference's translation known answers (translation.rs:340-420)
hold for the oracle and the codon tables; the oracle's six frames equal a
codon-string translation of the strand and its reverse complement.
GPU: the CUDA translation equals the oracle byte for byte for every genetic
code; nx and pn searches equal the oracle engine run over the oracle's
frames, with the oracle's frame merge and coordinate mapping."""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle import engine as oeng
from saber_gb300 import synth, translation as T

ALPHA = "ARNDCQEGHILKMFPSTWYVBZX*"
STANDARD_TCAG = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG"


def _frames(seq, code="standard"):
    nt = T.encode_nucleotide(seq)
    c, o = orc.translate6(nt, [0, nt.size], T.codon_table(code))
    return ["".join(ALPHA[x] for x in c[o[f]:o[f + 1]]) for f in range(6)]


def _string_translate(seq):
    code = {a + b + c: STANDARD_TCAG[16 * "TCAG".index(a) + 4 * "TCAG".index(b) + "TCAG".index(c)]
            for a in "TCAG" for b in "TCAG" for c in "TCAG"}
    return "".join(code.get(seq[i:i + 3], "X") for i in range(0, len(seq) - 2, 3))


def test_known_answers():
    """translation.rs:371-420."""
    assert _frames("ATG")[0] == "M"
    assert _frames("ATGTAAGCT")[0] == "M*A"
    assert _frames("ATN")[0] == "X"
    assert _frames("TGA")[0] == "*" and _frames("TGA", "vertebrate")[0] == "W"
    assert _frames("ATGTAGTGG", "archaeal")[0] == "M*W" == _frames("ATGTAGTGG", "bacterial")[0]
    assert _frames("ATGTAGTGG", "15")[0] == "MQW"
    assert T.parse_genetic_code("11") == "bacterial" and T.parse_genetic_code("standard") == "standard"
    with pytest.raises(ValueError):
        T.parse_genetic_code("martian")
    assert len(_frames("ATGCCCGGGTTTAAA")) == 6


def test_coordinates():
    """translation.rs:354-363."""
    assert T.protein_to_nt(1, 1, 1, 30) == (2, 4)
    assert T.protein_to_nt(3, 1, 1, 30) == (30, 28)
    assert T.protein_to_nt(4, 2, 3, 30) == (26, 21)
    assert T.frame_label(0) == 1 and T.frame_label(5) == -3
    for f in range(6):
        for ps, pe, n in ((1, 1, 30), (2, 7, 31), (3, 9, 32)):
            a, b, lab = oeng.frame_nt_range(f, ps, pe, n)
            assert (a, b) == T.protein_to_nt(f, ps, pe, n) and lab == T.frame_label(f)


def test_six_frames_match_codon_strings():
    """translation.rs:341-352: the table-driven frames equal a codon-string
    translation of the strand and of its reverse complement."""
    seq = "ATGGCGTTTAAACCCGGGTTTAAATAGCGNATGCATGCTAGCTAGGATCCAAGCTTGAATTC"
    rc = seq[::-1].translate(str.maketrans("ACGTN", "TGCAN"))
    fr = _frames(seq)
    for f in range(3):
        assert fr[f] == _string_translate(seq[f:])
        assert fr[3 + f] == _string_translate(rc[f:])
    for n in range(0, 8):
        assert [len(x) for x in _frames("A" * n)] == T.frame_lengths(n)


@pytest.mark.gpu
@pytest.mark.parametrize("code", ["standard", "vertebrate", "yeast", "mold", "invertebrate", "ciliate",
                                  "echinoderm", "bacterial", "alt-yeast", "archaeal", "blepharisma"])
def test_gpu_translation_equals_oracle(dev, code):
    rng = np.random.default_rng(len(code))
    lens = rng.integers(0, 60, 200)
    lens[:4] = [0, 1, 2, 3]
    lens[-2:] = [5000, 3001]
    nt = rng.integers(0, 4, int(lens.sum())).astype(np.uint8)
    nt[rng.random(nt.size) < 0.02] = 4
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    aa = T.codon_table(code)
    got, goffs = dev.translate6(nt, offs, aa)
    want, woffs = orc.translate6(nt, offs, aa)
    assert np.array_equal(goffs, woffs) and np.array_equal(got, want)


def _compare_results(got, want_pairs):
    assert len(got) == len(want_pairs)
    keys = ("subject", "score", "evalue", "bitscore", "q_start", "q_end", "s_start", "s_end", "columns",
            "matches", "mismatches", "gap_opens", "ops")
    for g, w in zip(got, want_pairs):
        for k in keys:
            assert g[k] == w[k], (k, g[k], w[k])


@pytest.mark.gpu
def test_blastx_matches_oracle(dev):
    from saber_gb300.search import SearchParams
    from saber_gb300.stats import gapped_protein
    from saber_gb300.translated import BlastxSearcher, m8_row
    dna, ss, _ = synth.translated_db(21, 10, 600, "nx", planted_frac=0.3)
    P = SearchParams("default", masking="none", max_target_seqs=5, max_hsps=2)
    bx = BlastxSearcher(dev, ss.codes, ss.offsets, P)
    got = bx.search(dna.codes, dna.offsets)
    fc, fo = orc.translate6(dna.codes, dna.offsets, T.codon_table())
    frame_hits = oeng.search_batch(ss.codes, ss.offsets, fc, fo, P, bx.se.matrix, 11, 1,
                                   gapped_protein("BLOSUM62", 11, 1), bx.se.scan_params)
    total = 0
    frames_seen = set()
    for r in range(len(dna)):
        nl = int(dna.offsets[r + 1] - dna.offsets[r])
        kept = oeng.finish_record_nx(frame_hits[6 * r:6 * r + 6], P.max_target_seqs, P.max_hsps)
        want = []
        for f, h in kept:
            w = dict(h)
            w["q_start"], w["q_end"], lab = oeng.frame_nt_range(f, h["q_start"], h["q_end"], nl)
            want.append(w)
            frames_seen.add(lab)
        _compare_results(got[r], want)
        for g, (f, _) in zip(got[r], kept):
            assert g["query_frame"] == T.frame_label(f)
            assert m8_row("q%d" % r, "s%d" % g["subject"], g).split("\t")[0] == "q%d|frame%+d" % (r, T.frame_label(f))
        total += len(want)
    assert total > 0 and any(l < 0 for l in frames_seen) and any(l > 0 for l in frames_seen)


@pytest.mark.gpu
def test_tblastn_matches_oracle(dev):
    from saber_gb300.search import SearchParams
    from saber_gb300.stats import gapped_protein
    from saber_gb300.translated import TblastnSearcher
    qs, dna, _ = synth.translated_db(22, 12, 500, "pn", planted_frac=0.3)
    P = SearchParams("default")
    tn = TblastnSearcher(dev, dna.codes, dna.offsets, P)
    got = tn.search(qs.codes, qs.offsets)
    fc, fo = orc.translate6(dna.codes, dna.offsets, T.codon_table())
    ntl = np.diff(dna.offsets.astype(np.int64))
    dbm, _, _ = orc.tantan_mask(fc, fo, oeng_b62())
    qm, _, _ = orc.tantan_mask(qs.codes, qs.offsets, oeng_b62())
    want = oeng.search_batch(fc, fo, qs.codes, qs.offsets, P, tn.se.matrix, 11, 1, gapped_protein("BLOSUM62", 11, 1),
                             tn.se.scan_params, dbm.view(np.uint8), qm.view(np.uint8),
                             stats_size=(int(ntl.sum()) // 3, ntl.size))
    total = 0
    for qi in range(len(qs)):
        exp = []
        for h in want[qi]:
            w = dict(h)
            s, f = h["subject"] // 6, h["subject"] % 6
            w["s_start"], w["s_end"], lab = oeng.frame_nt_range(f, h["s_start"], h["s_end"], int(ntl[s]))
            w["subject"] = s
            exp.append(w)
            assert lab == T.frame_label(f)
        _compare_results(got[qi], exp)
        total += len(exp)
    assert total > 0
    assert tn.se.stats.db_length == int(ntl.sum()) // 3 and tn.se.stats.db_num_seqs == ntl.size


def oeng_b62():
    from saber_gb300.scoring import matrix
    return matrix("BLOSUM62")
