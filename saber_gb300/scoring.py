"""Residue alphabet and substitution tables.

ALPHABET is the 24-letter NCBI matrix order of src/alphabet.rs:22 (unknown
letters encode as X = 22, alphabet.rs:48-60).  The protein tables are the
public NCBI BLOSUM/PAM matrices in that order (src/scoring/matrices.rs:145+),
stored as data in data/matrices.json; ``nucleotide`` is
ScoreMatrix::nucleotide (matrices.rs:85-91).
"""
import json
import os

import numpy as np

ALPHABET = b"ARNDCQEGHILKMFPSTWYVBZX*"
_ENC = np.full(256, 22, dtype=np.uint8)
for _i, _c in enumerate(ALPHABET):
    _ENC[_c] = _i
    if 65 <= _c <= 90:
        _ENC[_c + 32] = _i

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "matrices.json")
_MATS = None


def encode_protein(ascii_seq):
    """ASCII protein -> codes 0..23 (unknown -> X = 22)."""
    if isinstance(ascii_seq, str):
        ascii_seq = ascii_seq.encode()
    return _ENC[np.frombuffer(ascii_seq, dtype=np.uint8)]


def matrix(name="BLOSUM62"):
    """24x24 int32 substitution matrix by name (BLOSUM45/50/62/80/90, PAM30/70/250)."""
    global _MATS
    if _MATS is None:
        with open(_DATA) as f:
            _MATS = json.load(f)
    return np.asarray(_MATS[name.upper()], dtype=np.int32)


def nucleotide(match=2, mismatch=-3):
    m = np.full((24, 24), mismatch, dtype=np.int32)
    for i in range(4):
        m[i, i] = match
    return m
