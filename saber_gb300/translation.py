"""Six-frame translation for the translated modes (translation.rs).

nx (blastx): nucleotide queries, each searched as its six translated frames
against a protein database, the frames' hits merged per record.  pn
(tblastn): protein queries against a nucleotide database stored as six
translated frames per sequence (subject = 6 * sequence + frame).  The frames
are translated on the GPU (`saber_gpu_translate6`); this module holds the
genetic codes, the codon table and the coordinate mapping back to
nucleotides (translation.rs:277-337).
"""
import numpy as np

from .scoring import encode_protein

# The standard genetic code (NCBI table 1), codons in TCAG order.
_STANDARD_TCAG = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG"

# Each code as its differences from the standard one, as the reference
# defines them (translation.rs:158-247).
_CODES = {
    "standard": {},
    "vertebrate": {"AGA": "*", "AGG": "*", "ATA": "M", "TGA": "W"},
    "yeast": {"CTT": "T", "CTC": "T", "CTA": "T", "CTG": "T", "ATA": "M", "TGA": "W"},
    "mold": {"TGA": "W"},
    "invertebrate": {"AGA": "S", "AGG": "S", "ATA": "M", "TGA": "W"},
    "ciliate": {"TAA": "Q", "TAG": "Q"},
    "echinoderm": {"AAA": "N", "AGA": "S", "AGG": "S", "TGA": "W"},
    "bacterial": {},
    "alt-yeast": {"CTG": "S"},
    "archaeal": {},  # NCBI 11, as bacterial
    "blepharisma": {"TAG": "Q"},
}
_ALIASES = {"1": "standard", "2": "vertebrate", "3": "yeast", "4": "mold", "5": "invertebrate", "6": "ciliate",
            "9": "echinoderm", "11": "bacterial", "12": "alt-yeast", "altyeast": "alt-yeast", "15": "blepharisma"}


def parse_genetic_code(s):
    """TranslationTable::from_str (translation.rs:35-53): a name or an NCBI number."""
    v = str(s).lower()
    v = _ALIASES.get(v, v)
    if v not in _CODES:
        raise ValueError("Unknown genetic code: %s" % s)
    return v


def _standard():
    bases = "TCAG"
    out = {}
    for i, aa in enumerate(_STANDARD_TCAG):
        out[bases[i // 16] + bases[(i // 4) % 4] + bases[i % 4]] = aa
    return out


def codon_table(code="standard"):
    """CodonTable::new (translation.rs:254-268): protein codes (alignment
    encoding) of the 64 codons, index a*16 + b*4 + c with A=0, C=1, G=2, T=3."""
    name = parse_genetic_code(code)
    m = _standard()
    m.update(_CODES[name])
    nts = "ACGT"
    letters = "".join(m[nts[a] + nts[b] + nts[c]] for a in range(4) for b in range(4) for c in range(4))
    return encode_protein(letters).astype(np.uint8)


_NT = np.full(256, 4, np.uint8)
for _c, _v in (("A", 0), ("C", 1), ("G", 2), ("T", 3), ("U", 3)):
    _NT[ord(_c)] = _v
    _NT[ord(_c.lower())] = _v


def encode_nucleotide(ascii_seq):
    """encode_nucleotide (alphabet.rs:249): ACGTU (any case) -> 0..3, anything else -> 4 (N)."""
    b = np.frombuffer(ascii_seq.encode() if isinstance(ascii_seq, str) else bytes(ascii_seq), np.uint8)
    return _NT[b]


def frame_lengths(n):
    """Residues of frames 0..5 of a sequence of n nucleotides (translate_codes, translation.rs:277-299)."""
    return [max(n - (f % 3), 0) // 3 for f in range(6)]


def frame_label(frame):
    """+1..+3 forward, -1..-3 reverse (translation.rs:316-318)."""
    return frame + 1 if frame < 3 else -((frame - 3) + 1)


def protein_to_nt(frame, p_start, p_end, nt_len):
    """1-based inclusive protein coordinates of a frame -> 1-based nucleotide
    coordinates on the original strand, start > end on the minus strand
    (translation.rs:323-337)."""
    if frame < 3:
        return frame + 3 * (p_start - 1) + 1, frame + 3 * p_end
    off = frame - 3
    rs = off + 3 * (p_start - 1) + 1
    re_ = off + 3 * p_end
    return nt_len - rs + 1, nt_len - re_ + 1
