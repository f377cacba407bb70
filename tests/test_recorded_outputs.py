"""Known answers recorded by the reference binary itself (v1.2.0,
bench/results/v1.2.0/defects.json on bench/defects/*.fa; fixture made by
tests/golden/make_golden.py): score, CIGAR, coordinates and bit score of the
single hit of each defect case.  The oracle (CPU) and the full GPU search
pipeline must both reproduce them."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from saber_gb300.bias import composition_bias
from saber_gb300.scoring import encode_protein, matrix
from saber_gb300.stats import SearchStatistics, gapped_protein

HERE = os.path.dirname(os.path.abspath(__file__))
B62 = matrix("BLOSUM62")


def _cases():
    with open(os.path.join(HERE, "golden", "defects.json")) as f:
        for c in json.load(f)["cases"]:
            for run, want in c["recorded"].items():
                yield c, run, want


def _cigar(ops):
    return "".join("%d%s" % (l, o) for o, l in ops)


@pytest.mark.parametrize("case,run,want", list(_cases()), ids=lambda x: x if isinstance(x, str) else None)
def test_oracle_reproduces_recorded_alignment(case, run, want):
    q = encode_protein(case["query"][0][1])
    s = encode_protein(case["db"][0][1])
    bias = None if "--comp-bias off" in run else composition_bias(q, B62)
    if bias is not None and not np.any(bias != 0):
        bias = None
    al = orc.banded_align(q, s, bias, B62, 11, 1, -len(q), len(s))
    assert al["score"] == want["score"]
    assert _cigar(al["ops"]) == want["cigar"]
    assert [al["q_start"] + 1, al["q_end"]] == want["query_range"]
    assert [al["s_start"] + 1, al["s_end"]] == want["subject_range"]
    st = SearchStatistics(gapped_protein("BLOSUM62", 11, 1), len(s), 1).for_query(len(q))
    assert "%.1f" % st.bitscore(al["score"]) == "%.1f" % want["bitscore"]


@pytest.mark.gpu
@pytest.mark.parametrize("case,run,want", list(_cases()), ids=lambda x: x if isinstance(x, str) else None)
def test_gpu_search_reproduces_recorded_hit(dev, case, run, want):
    from saber_gb300.search import Searcher, SearchParams
    q = encode_protein(case["query"][0][1])
    s = encode_protein(case["db"][0][1])
    # sat (4000 W): every Murphy-10 seed of the run has the same code, which
    # the 1.4 frequent-seed cap drops (v1.2.0 seeded differently); the
    # exhaustive preset scores the pair without seeding
    preset = "exhaustive" if case["name"] == "sat" else "default"
    # the runs without --masking none used the reference's default tantan
    # masking of the query and the database
    P = SearchParams(preset, comp_bias="--comp-bias off" not in run,
                     masking="none" if "--masking none" in run else "tantan")
    se = Searcher(dev, s, np.array([0, len(s)], np.uint64), P)
    hits = se.search(q, np.array([0, len(q)], np.uint64))[0]
    assert len(hits) == 1
    h = hits[0]
    assert h["score"] == want["score"]
    assert h.cigar() == want["cigar"]
    assert [h["q_start"], h["q_end"]] == want["query_range"]
    assert [h["s_start"], h["s_end"]] == want["subject_range"]
    assert "%.1f" % h["bitscore"] == "%.1f" % want["bitscore"]
