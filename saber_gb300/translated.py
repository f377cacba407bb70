"""Translated searches (driver.rs:387-503): nx (blastx) and pn (tblastn).

nx: each nucleotide query record is searched as its six translated frames
(one engine query per frame, record-major), and the frames' hits are merged
per record: best score first, at most max_hsps per subject and
max_target_seqs subjects (finish_record, driver.rs:473-503).

pn: the nucleotide database is stored as six translated frames per sequence
(subject 6 * s + f, index.rs:1351-1368) and the statistics use the
nucleotides / 3 and the sequence count (db_stats_size, driver.rs:575-583).

Both report nucleotide coordinates on the original strand (start > end on
the minus strand) and the frame as +1..+3 / -1..-3 (to_result,
driver.rs:405-471).  The frames are translated on the GPU.
"""
import numpy as np

from .search import Hit, Searcher, format_evalue
from .translation import codon_table, frame_label, protein_to_nt


def merge_record(all_hits, max_target_seqs, max_hsps):
    """finish_record's merge of one nx record (driver.rs:481-501): (frame, hit)
    pairs sorted by score desc, subject, frame (stable), then the per-subject
    and per-record limits."""
    order = sorted(all_hits, key=lambda fh: (-fh[1]["score"], fh[1]["subject"], fh[0]))
    per, kept, subjects = {}, [], 0
    for f, h in order:
        c = per.get(h["subject"], 0)
        if c >= max_hsps:
            continue
        if c == 0:
            if subjects >= max_target_seqs:
                continue
            subjects += 1
        per[h["subject"]] = c + 1
        kept.append((f, h))
    return kept


def to_result(h, q_frame=None, q_nt_len=None, s_frame=None, s_seq=None, s_nt_len=None):
    """to_result (driver.rs:405-471): the engine hit with nucleotide
    coordinates and frames; q_frame / s_frame 0..5 or None."""
    r = Hit(h)
    r["query_frame"], r["subject_frame"] = 0, 0
    # identity and coverages come from the engine hit (frame coordinates and
    # lengths), as to_result computes them before mapping
    r["query_cover_engine"], r["subject_cover_engine"] = h.query_cover(), h.subject_cover()
    r["q_start_engine"], r["s_start_engine"] = h["q_start"], h["s_start"]
    if q_frame is not None:
        r["q_start"], r["q_end"] = protein_to_nt(q_frame, h["q_start"], h["q_end"], q_nt_len)
        r["query_frame"] = frame_label(q_frame)
        r["q_len"] = q_nt_len
    if s_frame is not None:
        r["s_start"], r["s_end"] = protein_to_nt(s_frame, h["s_start"], h["s_end"], s_nt_len)
        r["subject_frame"] = frame_label(s_frame)
        r["subject"] = s_seq
        r["s_len"] = s_nt_len
    return r


def m8_row(query_id, subject_id, r):
    """write_m8_row (output.rs:20-36) of a translated result: the IDs carry
    the "|frame+N" suffix (driver.rs:444-451)."""
    qid = "%s|frame%+d" % (query_id, r["query_frame"]) if r["query_frame"] else query_id
    sid = "%s|frame%+d" % (subject_id, r["subject_frame"]) if r["subject_frame"] else subject_id
    return "%s\t%s\t%.2f\t%d\t%d\t%d\t%d\t%d\t%d\t%d\t%s\t%.1f" % (
        qid, sid, r.identity(), r["columns"], r["mismatches"], r["gap_opens"], r["q_start"], r["q_end"],
        r["s_start"], r["s_end"], format_evalue(r["evalue"]), r["bitscore"])


class BlastxSearcher:
    """nx: nucleotide query records (codes 0..3, 4 = N) against a protein database."""

    def __init__(self, dev, db_codes, db_offsets, params=None, genetic_code="standard", **kw):
        self.se = Searcher(dev, db_codes, db_offsets, params, **kw)
        self.codon = codon_table(genetic_code)

    @property
    def counters(self):
        return self.se.counters

    def search(self, nt_codes, nt_offsets):
        """Results per record (lists of Hit with nucleotide query coordinates)."""
        nt_offsets = np.ascontiguousarray(nt_offsets, np.uint64)
        nrec = nt_offsets.size - 1
        frames, foffs = self.se.dev.translate6(nt_codes, nt_offsets, self.codon)
        hits = self.se.search(frames, foffs) if nrec else []
        P = self.se.p
        out = []
        for r in range(nrec):
            nl = int(nt_offsets[r + 1] - nt_offsets[r])
            all_hits = [(f, h) for f in range(6) for h in hits[6 * r + f]]
            kept = merge_record(all_hits, P.max_target_seqs, P.max_hsps)
            out.append([to_result(h, q_frame=f, q_nt_len=nl) for f, h in kept])
        return out


class TblastnSearcher:
    """pn: protein queries against a nucleotide database (codes 0..3, 4 = N)
    stored as its six translated frames."""

    def __init__(self, dev, nt_codes, nt_offsets, params=None, genetic_code="standard", **kw):
        self.codon = codon_table(genetic_code)
        nt_offsets = np.ascontiguousarray(nt_offsets, np.uint64)
        self.nt_len = np.diff(nt_offsets.astype(np.int64))
        nseq = self.nt_len.size
        frames, foffs = dev.translate6(nt_codes, nt_offsets, self.codon)
        total = int(self.nt_len.sum())
        self.se = Searcher(dev, frames, foffs, params, stats_size=(max(total // 3, 1), max(nseq, 1)), **kw)

    @property
    def counters(self):
        return self.se.counters

    def search(self, q_codes, q_offsets):
        """Results per query (lists of Hit with nucleotide subject coordinates;
        `subject` is the nucleotide sequence index)."""
        hits = self.se.search(q_codes, q_offsets)
        return [[to_result(h, s_frame=h["subject"] % 6, s_seq=h["subject"] // 6,
                           s_nt_len=int(self.nt_len[h["subject"] // 6])) for h in hq] for hq in hits]
