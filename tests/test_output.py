"""Output formats (output.rs): the reference's writer tests
(output.rs:283-376) and Rust float formatting, on CPU; on the GPU, every
format rendered from a real search agrees with the hit records (m8 equals
the engine's m8 rows, the aligned strings rescore to the hit)."""
import json

import numpy as np
import pytest

from saber_gb300 import output as O
from saber_gb300.search import Hit


def _sample():
    h = Hit(subject=0, score=100, evalue=1e-10, bitscore=50.0, q_start=1, q_end=100, s_start=1, s_end=100,
            columns=100, matches=95, mismatches=5, positives=97, gap_opens=0, gap_columns=0, q_len=100, s_len=100,
            ops=[("M", 100)], exact=False)
    a = O.alignment_result(h, "q1", "s1")
    a["identity"] = 95.5
    a["query_seq"], a["subject_seq"], a["match_string"] = "ACGT", "ACGT", "||||"
    return a


def test_m8_has_12_tab_columns():
    assert len(O.write_results([_sample()], "m8").rstrip("\n").split("\t")) == 12


def test_sam_nm_counts_mismatches_and_indels():
    a = _sample()
    a["mismatches"], a["gaps"], a["cigar"] = 4, 3, "50M2I47M1D1M"
    assert "\tNM:i:7\t" in O.write_results([a], "sam")


def test_format_evalue():
    assert "e" in O.format_evalue(1e-50) and O.format_evalue(0.5) == "0.500"


def test_json_writer_emits_array():
    s = O.write_results([_sample(), _sample()], "json")
    assert s.startswith("[") and s.rstrip().endswith("]") and '"query_id":"q1"' in s
    rows = json.loads(s)
    assert len(rows) == 2 and rows[0]["query_range"] == [1, 100] and rows[0]["evalue"] == 1e-10


def test_rust_float_is_ryu_shortest():
    cases = {50.0: "50.0", 95.5: "95.5", 0.5: "0.5", 1e-10: "1e-10", 1.234e-5: "0.00001234", 1e-5: "0.00001",
             9.9e-6: "9.9e-6", 1e16: "1e16", 1.5e300: "1.5e300", 123456789.0: "123456789.0",
             1234567890123456.0: "1234567890123456.0", 0.1: "0.1", 100.0: "100.0", 3.0e-7: "3e-7",
             2.5e-308: "2.5e-308", 0.0: "0.0", -1.5: "-1.5"}
    for x, want in cases.items():
        assert O.rust_float(x) == want, (x, O.rust_float(x), want)


def test_other_writers_layout():
    a = _sample()
    assert O.write_results([a], "m9").startswith("# SABER 1.4.0\n# Fields: query id, subject id, % identity")
    csv = O.write_results([a], "csv").splitlines()
    assert csv[0].startswith("query_id,subject_id") and csv[1].split(",")[0] == "q1"
    m0 = O.write_results([a], "m0")
    assert ">s1\n Score = 50.0 bits (100), Expect = 1.00e-10\n" in m0
    assert "Query       1  ACGT  4\n               ||||\nSbjct       1  ACGT  4\n" in m0
    b = dict(a, query_id='a,"b"')
    assert O.write_results([b], "csv").splitlines()[1].startswith('"a,""b""",s1,')
    with pytest.raises(ValueError):
        O.write_results([a], "xml")


@pytest.mark.gpu
def test_formats_from_a_search(dev):
    from saber_gb300 import synth
    from saber_gb300.scoring import matrix
    from saber_gb300.search import Searcher, SearchParams, m8_row
    from oracle import oracle as orc
    qs, ss, _ = synth.protein_db(31, 8, 300)
    se = Searcher(dev, ss.codes, ss.offsets, SearchParams("default"))
    hits = se.search(qs.codes, qs.offsets)
    b62 = matrix("BLOSUM62")
    res, m8 = [], []
    for qi, hq in enumerate(hits):
        for h in hq:
            res.append(O.alignment_result(h, "q%d" % qi, "s%d" % h["subject"], qs.seq(qi), ss.seq(h["subject"]), b62))
            m8.append(m8_row("q%d" % qi, "s%d" % h["subject"], h) + "\n")
    assert len(res) > 0
    assert O.write_results(res, "m8") == "".join(m8)
    for a, h, in zip(res, [h for hq in hits for h in hq]):
        q = a["query_seq"].replace("-", "")
        s = a["subject_seq"].replace("-", "")
        assert len(q) == a["query_end"] - a["query_start"] + 1 and len(s) == a["subject_end"] - a["subject_start"] + 1
        assert sum(c not in " +" for c in a["match_string"]) == a["matches"]
        assert sum(c != " " for c in a["match_string"]) == a["positives"]
    js = json.loads(O.write_results(res, "json"))
    assert [r["score"] for r in js] == [a["score"] for a in res]
    for fmt in O.FORMATS:
        assert O.write_results(res, fmt)
