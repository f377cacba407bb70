"""Seed alphabets, spaced-seed shapes and search presets.

The values restate the reference's configuration tables so the GPU path
accepts the same presets: the Murphy et al. (2000) 10-letter alphabet
(src/alphabet.rs:325-328), DIAMOND's 16 weight-7 spaced seeds (DS16) and
the 8 weight-6 seeds W6X8 (src/search/presets.rs:47-92), and the preset
table (presets.rs:98-197).
"""
from .scoring import ALPHABET

MURPHY10_GROUPS = "A KR EDNQ C G H ILVM FYW P ST"

DS16 = ["11110111", "11100100111", "110010101011", "11010001001011", "10101100001101", "110100100100011",
        "1010010100010011", "1100101000001011", "11100000100010101", "11000100010010011", "11010000001000111",
        "110001001000010011", "1010001000100001011", "1100010100000010011", "1100100000101000011",
        "1101000010000001011"]
W6X8 = ["100111011", "1011100011", "1010011011", "11110101", "1101000111", "1111100001", "10101111", "1010010111"]


def alphabet_map(groups=MURPHY10_GROUPS):
    """(map[24] reduced letter per code or 255, size) from a group string (alphabet.rs:299-322)."""
    amap = [255] * 24
    n = 0
    for g in groups.split():
        for ch in g.encode():
            code = ALPHABET.index(ch)
            if code >= 20 or amap[code] != 255:
                raise ValueError("bad group letter %r" % chr(ch))
            amap[code] = n
        n += 1
    return amap, n


def full_alphabet():
    return [i if i < 20 else 255 for i in range(24)], 20


# name -> (alphabet, shapes, hit_filter_ids, exact_weight, hsp_threshold,
#          max_candidates, hsp_floor_fraction, score_band, prefilter_band, exhaustive)
PRESETS = {
    "very-fast": ("murphy10", DS16[:4], 28, 2, 40, 5000, 0.7, 48, 0, False),
    "fast": ("murphy10", DS16[:8], 27, 2, 40, 5000, 0.7, 48, 0, False),
    "default": ("murphy10", DS16, 27, 2, 40, 5000, 0.65, 48, 16, False),
    "sensitive": ("murphy10", W6X8, 27, 2, 40, 5000, 0.65, 48, 16, False),
    "more-sensitive": ("murphy10", DS16 + W6X8, 27, 2, 40, 8000, 0.65, 48, 16, False),
    "legacy": ("full", ["1111"], 0, 0, 40, 5000, 0.0, 0, 0, False),
    "exhaustive": ("full", ["1111"], 0, 0, 0, 2 ** 32 - 1, 0.0, 0, 0, True),
}
