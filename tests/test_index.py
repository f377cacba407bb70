"""SABERIDX v4 database files (index.rs, crc32.rs): the CRC-32 known answer,
write/read round trips of every section read, the open-time checks the
reference makes (magic, version, header and metadata checksums, size,
section bounds), and on the GPU a search over a loaded index (mask runs
expanded on the device) equal to the oracle engine with the same mask."""
import numpy as np
import pytest

from saber_gb300 import index as IX
from saber_gb300 import synth


def _db(tmp_path, translated=False):
    qs, ss, _ = synth.protein_db(51, 6, 400)
    runs = np.array([[3, 10], [100, 130], [5000, 5004]], np.uint64)
    ids = ["sub%d|x" % i for i in range(len(ss))]
    kw = {}
    if translated:
        kw = dict(translated=True, nt_lengths=np.arange(len(ss) // 6) + 30, genetic_code="Standard")
    p = str(tmp_path / "db.sdx")
    IX.write_index(p, ss.codes, ss.offsets, ids=ids, mask_runs=runs, **kw)
    return p, qs, ss, runs, ids


def test_crc32_known_vector():
    """crc32.rs:52-61."""
    assert IX.crc32(b"123456789") == 0xCBF43926


def test_round_trip(tmp_path):
    p, qs, ss, runs, ids = _db(tmp_path)
    idx = IX.SeedIndex(p, verify_sections=True)
    assert np.array_equal(idx.residues, ss.codes) and np.array_equal(idx.subject_offsets, ss.offsets)
    assert idx.num_subjects == len(ss) and idx.subject_id(7) == ids[7]
    assert np.array_equal(idx.mask_runs, runs)
    assert idx.stats_size() == (int(ss.codes.size), len(ss)) and not idx.is_translated
    with open(p, "rb") as f:
        head = f.read(16)
    assert head[:8] == b"SABERIDX" and int.from_bytes(head[8:12], "little") == 4


def test_translated_stats(tmp_path):
    p, qs, ss, runs, ids = _db(tmp_path, translated=True)
    idx = IX.SeedIndex(p)
    nl = idx.nt_lengths
    assert idx.is_translated and idx.stats_size() == (int(nl.sum()) // 3, nl.size)


@pytest.mark.parametrize("damage,msg", [
    (lambda b: b.__setitem__(slice(0, 8), b"NOTANIDX"), "not a SABER index"),
    (lambda b: b.__setitem__(slice(8, 12), (3).to_bytes(4, "little")), "format v3"),
    (lambda b: b.__setitem__(100, b[100] ^ 1), "header checksum"),
    (lambda b: b.extend(b"\0" * 8), "header says"),
])
def test_open_checks(tmp_path, damage, msg):
    p, *_ = _db(tmp_path)
    b = bytearray(open(p, "rb").read())
    damage(b)
    open(p, "wb").write(bytes(b))
    with pytest.raises(IX.IndexError_, match=msg):
        IX.SeedIndex(p)


def test_section_checksum(tmp_path):
    p, *_ = _db(tmp_path)
    idx = IX.SeedIndex(p)
    o = idx._sec["enc"][0]
    idx.close()
    b = bytearray(open(p, "rb").read())
    b[o + 5] ^= 1
    open(p, "wb").write(bytes(b))
    IX.SeedIndex(p)  # sections are checked on request, as verify_checksums
    with pytest.raises(IX.IndexError_, match="section 'enc' checksum"):
        IX.SeedIndex(p, verify_sections=True)


@pytest.mark.gpu
def test_search_over_index(dev, tmp_path):
    from oracle import engine as oeng
    from oracle import oracle as orc
    from saber_gb300.masking import mask_runs
    from saber_gb300.scoring import matrix
    from saber_gb300.search import Searcher, SearchParams
    from saber_gb300.stats import gapped_protein
    from tests.test_search_gpu import _compare
    qs, ss, _ = synth.protein_db(52, 10, 800)
    b62 = matrix("BLOSUM62")
    dbm, _, _ = orc.tantan_mask(ss.codes, ss.offsets, b62)
    runs = mask_runs(dbm, ss.offsets)
    p = str(tmp_path / "db.sdx")
    IX.write_index(p, ss.codes, ss.offsets, mask_runs=runs)
    idx = IX.SeedIndex(p, verify_sections=True)
    P = SearchParams("default")
    se = Searcher.from_index(dev, idx, P)
    got = se.search(qs.codes, qs.offsets)
    qm, _, _ = orc.tantan_mask(qs.codes, qs.offsets, b62)
    want = oeng.search_batch(ss.codes, ss.offsets, qs.codes, qs.offsets, P, se.matrix, 11, 1,
                             gapped_protein("BLOSUM62", 11, 1), se.scan_params, dbm.view(np.uint8), qm.view(np.uint8))
    assert sum(len(h) for h in want) > 0
    _compare(got, want)


def test_empty_database(tmp_path):
    p = str(tmp_path / "empty.sdx")
    IX.write_index(p, np.zeros(0, np.uint8), np.zeros(1, np.uint64), ids=[])
    idx = IX.SeedIndex(p, verify_sections=True)
    assert idx.num_subjects == 0 and idx.residues.size == 0 and idx.mask_runs is None
