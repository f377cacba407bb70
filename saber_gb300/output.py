"""Output formats from the same hit records (output.rs): m8, m9, m0, SAM,
BAM-as-text, JSON and CSV, byte-identical to the reference's writers.

`alignment_result` builds the reference's AlignmentResult (driver.rs:405-471)
from a hit, with the aligned strings and midline of make_hit
(engine.rs:1447-1530); `write_results` renders a stream of them with the
format's header and footer.  Floats follow Rust's formatting: `{:.N}` is
round-half-even on the exact binary value (as Python's %-formatting), and
the JSON numbers are serde_json's shortest representation (`ryu`).
"""
import json

from .search import format_evalue
_PROTEIN_ALPHABET = "ARNDCQEGHILKMFPSTWYVBZX*"  # alphabet.rs:22

OUTPUT_VERSION = "1.4.0"  # the reference release whose writers these reproduce (Cargo.toml)
_NT_ALPHABET = "ACGTN"


def aligned_strings(q_codes, s_codes, q_start, s_start, ops, matrix, is_protein=True):
    """make_hit's aligned query, subject and midline (engine.rs:1459-1512):
    q_start / s_start 0-based in q_codes / s_codes; the midline holds the
    letter where identical (standard residues only), '+' where the matrix
    score is positive, ' ' otherwise and under gaps."""
    def dec(c):
        c = int(c)
        if is_protein:
            return _PROTEIN_ALPHABET[c] if c < 24 else "X"
        return _NT_ALPHABET[min(c, 4)]

    qa, sa, mid = [], [], []
    i, j = q_start, s_start
    for op, l in ops:
        if op == "M":
            for _ in range(l):
                a, b = int(q_codes[i]), int(s_codes[j])
                identical = a == b and ((is_protein and a < 20) or (not is_protein and a < 4))
                ai, bi = (a if a < 24 else 22), (b if b < 24 else 22)
                positive = identical or int(matrix[ai][bi]) > 0
                qa.append(dec(a))
                sa.append(dec(b))
                mid.append(dec(a) if identical else ("+" if positive else " "))
                i += 1
                j += 1
        elif op == "I":
            for k in range(l):
                qa.append(dec(q_codes[i + k]))
                sa.append("-")
                mid.append(" ")
            i += l
        else:
            for k in range(l):
                qa.append("-")
                sa.append(dec(s_codes[j + k]))
                mid.append(" ")
            j += l
    return "".join(qa), "".join(sa), "".join(mid)


def alignment_result(h, query_id, subject_id, q_codes=None, s_codes=None, matrix=None, is_protein=True,
                     calibrated=True):
    """AlignmentResult of a hit (to_result, driver.rs:405-471).  A translated
    result (saber_gb300.translated) already carries nucleotide coordinates,
    frames and the engine-level coverages.  q_codes / s_codes: the query and
    the subject (engine coordinates; the frame for translated sides) for the
    aligned strings, or None to leave them empty."""
    qf, sf = h.get("query_frame", 0), h.get("subject_frame", 0)
    r = {
        "query_id": "%s|frame%+d" % (query_id, qf) if qf else str(query_id),
        "subject_id": "%s|frame%+d" % (subject_id, sf) if sf else str(subject_id),
        "score": int(h["score"]), "evalue": float(h["evalue"]), "bitscore": float(h["bitscore"]),
        "identity": h.identity(),
        "query_coverage": h["query_cover_engine"] if "query_cover_engine" in h else h.query_cover(),
        "subject_coverage": h["subject_cover_engine"] if "subject_cover_engine" in h else h.subject_cover(),
        "query_start": int(h["q_start"]), "query_end": int(h["q_end"]),
        "subject_start": int(h["s_start"]), "subject_end": int(h["s_end"]),
        "align_length": int(h["columns"]), "matches": int(h["matches"]), "mismatches": int(h["mismatches"]),
        "gaps": int(h["gap_columns"]), "cigar": h.cigar(), "gap_opens": int(h["gap_opens"]),
        "positives": int(h["positives"]), "query_length": int(h["q_len"]), "subject_length": int(h["s_len"]),
        "query_frame": int(qf), "subject_frame": int(sf), "evalue_calibrated": bool(calibrated),
        "exact": bool(h.get("exact", False)), "query_seq": "", "subject_seq": "", "match_string": "",
    }
    if q_codes is not None and s_codes is not None and matrix is not None:
        qs0 = int(h.get("q_start_engine", h["q_start"])) - 1
        ss0 = int(h.get("s_start_engine", h["s_start"])) - 1
        r["query_seq"], r["subject_seq"], r["match_string"] = aligned_strings(
            q_codes, s_codes, qs0, ss0, h["ops"], matrix, is_protein)
    return r


def rust_float(x):
    """serde_json's f64 text (the ryu crate's shortest round-trip digits,
    decimal for 1e-5 <= |x| < 1e16, else d.ddde±X without padding)."""
    x = float(x)
    if x != x or x in (float("inf"), float("-inf")):
        return "null"
    if x == 0.0:
        return "-0.0" if str(x).startswith("-") else "0.0"
    r = repr(x)
    mant, _, exp = r.partition("e")
    digits = mant.replace("-", "").replace(".", "").lstrip("0") or "0"
    neg = r.startswith("-")
    # decimal exponent: value = 0.digits * 10^kk
    if exp:
        e = int(exp)
        ip = mant.replace("-", "").split(".")[0]
        kk = e + len(ip.lstrip("0") or "0")
    else:
        ip, _, fp = mant.replace("-", "").partition(".")
        ip_s = ip.lstrip("0")
        kk = len(ip_s) if ip_s else -(len(fp) - len(fp.lstrip("0")))
    digits = digits.rstrip("0") or "0"
    n = len(digits)
    sign = "-" if neg else ""
    if 0 <= kk - n and kk <= 16:
        return sign + digits + "0" * (kk - n) + ".0"
    if 0 < kk <= 16:
        return sign + digits[:kk] + "." + digits[kk:]
    if -5 < kk <= 0:
        return sign + "0." + "0" * (-kk) + digits
    if n == 1:
        return "%s%se%d" % (sign, digits, kk - 1)
    return "%s%s.%se%d" % (sign, digits[0], digits[1:], kk - 1)


def _m8(a):
    return "%s\t%s\t%.2f\t%d\t%d\t%d\t%d\t%d\t%d\t%d\t%s\t%.1f\n" % (
        a["query_id"], a["subject_id"], a["identity"], a["align_length"], a["mismatches"], a["gap_opens"],
        a["query_start"], a["query_end"], a["subject_start"], a["subject_end"], format_evalue(a["evalue"]),
        a["bitscore"])


def _m0(a):
    L = max(a["align_length"], 1)
    pct_gaps = 100.0 * a["gaps"] / a["align_length"] if a["align_length"] > 0 else 0.0
    pct_pos = 100.0 * a["positives"] / a["align_length"] if a["align_length"] > 0 else 0.0
    out = [">%s\n" % a["subject_id"],
           " Score = %.1f bits (%d), Expect = %s\n" % (a["bitscore"], a["score"], format_evalue(a["evalue"])),
           " Identities = %d/%d (%.0f%%), Positives = %d/%d (%.0f%%), Gaps = %d/%d (%.0f%%)\n" % (
               a["matches"], L, a["identity"], a["positives"], L, pct_pos, a["gaps"], L, pct_gaps)]
    if not a["evalue_calibrated"]:
        out.append(" WARNING: E-value computed with UNCALIBRATED statistical parameters\n")
    out.append("\n")
    qb, sb, mb = a["query_seq"], a["subject_seq"], a["match_string"]
    q, s, i = a["query_start"], a["subject_start"], 0
    while i < len(qb):
        j = min(i + 60, len(qb))
        qs_, ss_, ms_ = qb[i:j], sb[i:j], mb[i:j]
        qc = sum(1 for c in qs_ if c != "-")
        sc = sum(1 for c in ss_ if c != "-")
        out.append("Query  %6d  %s  %d\n" % (q, qs_, q + max(qc - 1, 0)))
        out.append("               %s\n" % ms_)
        out.append("Sbjct  %6d  %s  %d\n" % (s, ss_, s + max(sc - 1, 0)))
        out.append("\n")
        q += qc
        s += sc
        i = j
    return "".join(out)


def _sam(a):
    mapq = 60 if (a["evalue"] == a["evalue"] and abs(a["evalue"]) != float("inf") and a["evalue"] < 0.001) else 30
    cigar = a["cigar"] or "*"
    seq = a["query_seq"].replace("-", "") if a["query_seq"] else "*"
    return "%s\t0\t%s\t%d\t%d\t%s\t*\t0\t0\t%s\t*\tAS:i:%d\tNM:i:%d\tEV:f:%s\n" % (
        a["query_id"], a["subject_id"], a["subject_start"], mapq, cigar, seq, a["score"],
        a["mismatches"] + a["gaps"], format_evalue(a["evalue"]))


_JSON_FIELDS = ("query_id", "subject_id", "score", "evalue", "bitscore", "identity", "align_length", "matches",
                "mismatches", "gaps", "query_range", "subject_range", "cigar", "gap_opens", "positives",
                "query_length", "subject_length", "query_cover", "subject_cover", "query_frame", "subject_frame",
                "evalue_calibrated", "exact")


def _json(a):
    v = dict(a)
    v["query_range"] = (a["query_start"], a["query_end"])
    v["subject_range"] = (a["subject_start"], a["subject_end"])
    v["query_cover"], v["subject_cover"] = a["query_coverage"], a["subject_coverage"]
    parts = []
    for k in _JSON_FIELDS:
        x = v[k]
        if isinstance(x, bool):
            t = "true" if x else "false"
        elif isinstance(x, float):
            t = rust_float(x)
        elif isinstance(x, tuple):
            t = "[%d,%d]" % x
        elif isinstance(x, str):
            t = json.dumps(x, ensure_ascii=False)
        else:
            t = str(int(x))
        parts.append('"%s":%s' % (k, t))
    return "{" + ",".join(parts) + "}"


def _csv_escape(s):
    if "," in s or '"' in s or "\n" in s:
        return '"%s"' % s.replace('"', '""')
    return s


def _csv(a):
    return "%s,%s,%.2f,%d,%d,%d,%d,%d,%d,%d,%s,%.1f\n" % (
        _csv_escape(a["query_id"]), _csv_escape(a["subject_id"]), a["identity"], a["align_length"],
        a["mismatches"], a["gaps"], a["query_start"], a["query_end"], a["subject_start"], a["subject_end"],
        format_evalue(a["evalue"]), a["bitscore"])


FORMATS = ("m8", "m9", "m0", "sam", "bam", "json", "csv")
NEEDS_STRINGS = ("m0", "sam", "bam")


def write_results(results, fmt="m8"):
    """The text a Writer produces for a stream of AlignmentResults: header,
    one record per result, footer (output.rs:12-282)."""
    if fmt not in FORMATS:
        raise ValueError("unknown output format '%s'" % fmt)
    out = []
    if fmt == "m9":
        out.append("# SABER %s\n" % OUTPUT_VERSION)
    elif fmt == "m0":
        out.append("SABER %s  https://github.com/raw937/saber\n\n" % OUTPUT_VERSION)
    elif fmt in ("sam", "bam"):
        out.append("@HD\tVN:1.6\tSO:unsorted\n@PG\tID:saber\tPN:SABER\tVN:%s\n" % OUTPUT_VERSION)
    elif fmt == "json":
        out.append("[\n")
    elif fmt == "csv":
        out.append("query_id,subject_id,identity,align_length,mismatches,gaps,q_start,q_end,s_start,s_end,evalue,"
                   "bitscore\n")
    first = True
    for a in results:
        if fmt == "m8":
            out.append(_m8(a))
        elif fmt == "m9":
            if first:
                out.append("# Fields: query id, subject id, % identity, alignment length, mismatches, gap opens, "
                           "q. start, q. end, s. start, s. end, evalue, bit score\n")
            out.append(_m8(a))
        elif fmt == "m0":
            out.append(_m0(a))
        elif fmt in ("sam", "bam"):
            out.append(_sam(a))
        elif fmt == "json":
            out.append(("" if first else ",\n") + "  " + _json(a))
        else:
            out.append(_csv(a))
        first = False
    if fmt == "json":
        out.append("\n]\n")
    return "".join(out)
