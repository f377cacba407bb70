"""SABERIDX v4 database files (index.rs:55-75, 240-330, 948-1004, 1680-1710):
read the residues, subject offsets, identifiers, tantan mask runs and (for a
translated database) the nucleotide lengths straight from a memory map, and
load them into a device handle; write the same layout for a scan-only
database (no seed postings: the scan schedule needs only these sections).

File layout, little-endian: a 256-byte header (magic "SABERIDX", format
version 4, endian mark 0x01020304, file size, metadata offset / length /
CRC-32, header CRC-32 over bytes 0..252 at byte 252), the sections at
8-byte-aligned offsets, then the metadata as JSON (IndexMeta, whose
`sections` list names, offsets, lengths and CRC-32s).  Sections read here:
`enc` (residue codes), `enc_off` (u64, subjects + 1), `ids` / `id_off`
(identifier bytes and u64 offsets), `maskruns` (u64 pairs, half-open runs
of database residues) and `nt_len` (u64 per nucleotide sequence of a
translated database).
"""
import json
import mmap
import os
import zlib

import numpy as np

MAGIC = b"SABERIDX"
FORMAT_VERSION = 4
HEADER_BYTES = 256
ENDIAN_MARK = 0x01020304


class IndexError_(Exception):
    """A file that is not a readable SABERIDX v4 database."""


def crc32(data):
    """IEEE 802.3 CRC-32 (reflected 0xEDB88320, as crc32.rs)."""
    return zlib.crc32(data) & 0xFFFFFFFF


class SeedIndex:
    """A SABERIDX v4 file opened read-only through a memory map."""

    def __init__(self, path, verify_sections=False):
        self.path = path
        f = open(path, "rb")
        try:
            size = os.fstat(f.fileno()).st_size
            if size < 16:
                raise IndexError_("%s: not a SABER index file" % path)
            self._mm = mmap.mmap(f.fileno(), 0, access=mmap.ACCESS_READ)
        finally:
            f.close()
        mm = self._mm
        if mm[0:8] != MAGIC:
            raise IndexError_("%s: not a SABER index file" % path)
        rd32 = lambda o: int.from_bytes(mm[o:o + 4], "little")  # noqa: E731
        rd64 = lambda o: int.from_bytes(mm[o:o + 8], "little")  # noqa: E731
        version = rd32(8)
        if version != FORMAT_VERSION:
            raise IndexError_("%s: SABER index format v%d, this reader reads v%d" % (path, version, FORMAT_VERSION))
        if size < HEADER_BYTES:
            raise IndexError_("%s: truncated index (header incomplete)" % path)
        if rd32(12) != ENDIAN_MARK:
            raise IndexError_("%s: index byte order differs from this machine" % path)
        if crc32(mm[0:252]) != rd32(252):
            raise IndexError_("%s: index header checksum mismatch (corrupt file)" % path)
        if rd64(16) != size:
            raise IndexError_("%s: index is %d bytes but its header says %d" % (path, size, rd64(16)))
        moff, mlen, mcrc = rd64(24), rd64(32), rd32(40)
        if moff + mlen > size:
            raise IndexError_("%s: index metadata out of bounds" % path)
        mbytes = mm[moff:moff + mlen]
        if crc32(mbytes) != mcrc:
            raise IndexError_("%s: index metadata checksum mismatch" % path)
        self.meta = json.loads(mbytes)
        self._sec = {}
        for s in self.meta["sections"]:
            o, l = int(s["offset"]), int(s["len"])
            if o % 8 or o < HEADER_BYTES or o + l > moff:
                raise IndexError_("%s: index section '%s' out of bounds or misaligned" % (path, s["name"]))
            self._sec[s["name"]] = (o, l, int(s["crc32"]))
        for name in ("enc", "enc_off", "ids", "id_off"):
            if name not in self._sec:
                raise IndexError_("%s: index is missing section '%s'" % (path, name))
        if verify_sections:
            self.verify_checksums()
        n = self.num_subjects
        off = self.subject_offsets
        if (off.size != n + 1 or off[0] != 0 or int(off[-1]) != self._sec["enc"][1]
                or int(off[-1]) != int(self.meta["total_residues"])):
            raise IndexError_("%s: subject offsets do not match the residue section" % path)
        if self.meta.get("translated") and "nt_len" not in self._sec:
            raise IndexError_("%s: translated index is missing its nucleotide-length section" % path)

    def _u8(self, name):
        o, l, _ = self._sec[name]
        return np.frombuffer(self._mm, np.uint8, l, o)

    def _u64(self, name):
        o, l, _ = self._sec[name]
        return np.frombuffer(self._mm, np.uint64, l // 8, o)

    def verify_checksums(self):
        """CRC-32 of every section against the metadata (verify_checksums)."""
        for name, (o, l, c) in self._sec.items():
            if crc32(self._mm[o:o + l]) != c:
                raise IndexError_("%s: section '%s' checksum mismatch" % (self.path, name))

    @property
    def num_subjects(self):
        return int(self.meta["num_subjects"])

    @property
    def is_translated(self):
        return bool(self.meta.get("translated", False))

    @property
    def residues(self):
        """Residue codes of all subjects (a view of the map)."""
        return self._u8("enc")

    @property
    def subject_offsets(self):
        return self._u64("enc_off")

    def subject_id(self, i):
        off = self._u64("id_off")
        return bytes(self._u8("ids")[int(off[i]):int(off[i + 1])]).decode("utf-8", "replace")

    @property
    def mask_runs(self):
        """Tantan mask runs as an (n, 2) array of half-open residue ranges, or None."""
        if "maskruns" not in self._sec:
            return None
        return self._u64("maskruns").reshape(-1, 2)

    @property
    def nt_lengths(self):
        return self._u64("nt_len") if "nt_len" in self._sec else None

    def stats_size(self):
        """db_stats_size (driver.rs:575-583): (length, sequences) of the statistics."""
        m = self.meta
        if self.is_translated:
            return max(int(m["nt_residues"]) // 3, 1), max(int(m["nt_sequences"]), 1)
        return int(m["total_residues"]), self.num_subjects

    def load(self, dev):
        """Upload the residues and offsets into the handle and install the
        index's seed mask runs (expanded on the device); returns self."""
        dev.load_db(self.residues, self.subject_offsets)
        runs = self.mask_runs
        if runs is not None:
            dev.load_db_mask_runs(runs)
        return self

    def close(self):
        self._mm.close()


def write_index(path, codes, offsets, ids=None, mask_runs=None, kind="Protein", translated=False,
                nt_lengths=None, genetic_code="", masking="tantan", source="", saber_version="1.4.0"):
    """Write a scan-only SABERIDX v4 file (no seed postings: `postings` false)
    with the layout of IndexBuilder::finish_to_file (index.rs:1680-1710)."""
    codes = np.ascontiguousarray(codes, np.uint8)
    offsets = np.ascontiguousarray(offsets, np.uint64)
    n = offsets.size - 1
    ids = ids if ids is not None else ["s%d" % i for i in range(n)]
    idb = [s.encode() for s in ids]
    id_off = np.zeros(n + 1, np.uint64)
    id_off[1:] = np.cumsum([len(b) for b in idb])
    sections = [("enc", codes.tobytes()), ("enc_off", offsets.tobytes()), ("ids", b"".join(idb)),
                ("id_off", id_off.tobytes())]
    if mask_runs is not None:
        sections.append(("maskruns", np.ascontiguousarray(mask_runs, np.uint64).reshape(-1).tobytes()))
    if translated:
        sections.append(("nt_len", np.ascontiguousarray(nt_lengths, np.uint64).tobytes()))
    body, metas, pos = [], [], HEADER_BYTES
    for name, data in sections:
        pad = (-pos) % 8
        body.append(b"\0" * pad)
        pos += pad
        metas.append({"name": name, "offset": pos, "len": len(data), "crc32": crc32(data)})
        body.append(data)
        pos += len(data)
    pad = (-pos) % 8
    body.append(b"\0" * pad)
    pos += pad
    lens = np.diff(offsets.astype(np.int64))
    parts = []
    for first in range(0, max(n, 1), 65535):
        cnt = min(65535, n - first)
        if cnt <= 0:
            break
        pl = lens[first:first + cnt]
        parts.append({"first_subject": first, "num_subjects": cnt, "residues": int(pl.sum()),
                      "max_len": int(pl.max()) if cnt else 0, "compact": True, "postings": [], "sparse": []})
    meta = {
        "format_version": FORMAT_VERSION, "saber_version": saber_version, "kind": kind,
        "alphabet_name": "murphy10" if kind == "Protein" else "acgt", "alphabet_size": 10 if kind == "Protein" else 4,
        "alphabet_map": [], "shapes": [], "minimizer_window": 1, "masking": masking, "masking_matrix": "BLOSUM62",
        "num_subjects": n, "total_residues": int(codes.size), "max_subject_len": int(lens.max()) if n else 0,
        "partitions": parts, "sections": metas, "source": source, "total_postings": [],
        "translated": bool(translated), "genetic_code": genetic_code,
        "nt_sequences": int(len(nt_lengths)) if translated else 0,
        "nt_residues": int(np.sum(nt_lengths)) if translated else 0, "postings": False, "scan_totals": [],
        "scan_freq_min": 128,
    }
    js = json.dumps(meta, separators=(",", ":")).encode()
    hdr = bytearray(HEADER_BYTES)
    hdr[0:8] = MAGIC
    hdr[8:12] = FORMAT_VERSION.to_bytes(4, "little")
    hdr[12:16] = ENDIAN_MARK.to_bytes(4, "little")
    hdr[16:24] = (pos + len(js)).to_bytes(8, "little")
    hdr[24:32] = pos.to_bytes(8, "little")
    hdr[32:40] = len(js).to_bytes(8, "little")
    hdr[40:44] = crc32(js).to_bytes(4, "little")
    hdr[252:256] = crc32(bytes(hdr[0:252])).to_bytes(4, "little")
    with open(path, "wb") as f:
        f.write(bytes(hdr))
        for b in body:
            f.write(b)
        f.write(js)
    return path
