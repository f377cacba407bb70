"""Learned triage of candidate regions (host side).

The network and its kernels live in the library (saber_gb300/csrc/triage.cu):
a 3-layer MLP over 24 per-region features (seed hits, HSPs, best ungapped
X-drop score and its E-value, diagonal spread, query / subject lengths and
composition entropy, low-complexity fractions, rank of the region), bf16
weights with fp32 accumulation, trained on the GPU with the library's own
forward / backward / Adam kernels.  This module builds training sets from
plain searches (labels: the region produced a reported hit), initialises and
trains the model, picks a conservative logit threshold and measures what it
keeps.  The plain path stays the arbiter: with a model installed every kept
region is still scored exactly, and the lost-hit rate is measured against
the plain search of the same batch.
"""
import numpy as np

from .gpu import TRIAGE_MODEL_FLOATS, TRIAGE_ROW_FLOATS

IN, FEAT, HID = 32, 24, 256
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
OFF_MU = OFF_B3 + 1
OFF_ISD = OFF_MU + IN
assert OFF_ISD + IN == TRIAGE_MODEL_FLOATS

FEATURES = ("best", "log2_best", "best_over_region_threshold", "bitscore", "neg_log10_evalue_estimate",
            "log2_hsps", "log2_seed_hits", "mean_hsp_score", "log2_hsp_score_sum", "log2_diagonal_spread",
            "spread_over_query", "log2_query_len", "log2_subject_len", "log2_length_ratio", "diagonal_overlap",
            "log2_rank_in_query", "best_over_query_top", "log2_regions_of_query", "query_entropy",
            "query_low_complexity", "query_max_residue_freq", "subject_entropy", "subject_low_complexity",
            "subject_max_residue_freq")
assert len(FEATURES) == FEAT


def init_model(seed=0, rows=None):
    """He-initialised weights (seeded); the input normalisation from `rows`
    (feature means and inverse standard deviations) when given."""
    rng = np.random.default_rng(seed)
    m = np.zeros(TRIAGE_MODEL_FLOATS, np.float32)
    w1 = np.zeros((IN, HID), np.float32)
    w1[:FEAT] = rng.normal(0.0, np.sqrt(2.0 / FEAT), size=(FEAT, HID))
    m[OFF_W1:OFF_B1] = w1.ravel()
    m[OFF_W2:OFF_B2] = rng.normal(0.0, np.sqrt(2.0 / HID), size=HID * HID)
    m[OFF_W3:OFF_B3] = rng.normal(0.0, np.sqrt(1.0 / HID), size=HID)
    mu = np.zeros(IN, np.float32)
    isd = np.ones(IN, np.float32)
    if rows is not None and len(rows):
        x = np.asarray(rows, np.float64)[:, :FEAT]
        mu[:FEAT] = x.mean(axis=0)
        sd = x.std(axis=0)
        isd[:FEAT] = 1.0 / np.where(sd > 1e-6, sd, 1.0)
    m[OFF_MU:OFF_ISD] = mu
    m[OFF_ISD:] = isd
    return m


def collect(searcher, q_codes, q_offsets):
    """One plain search with feature collection: (rows, labels, hits)."""
    dev = searcher.dev
    dev.set_triage(None)
    dev.collect_regions(True)
    try:
        hits = searcher.search(q_codes, q_offsets)
        rows, y, _ = dev.collected_regions()
    finally:
        dev.collect_regions(False)
    return rows, y, hits


def train(dev, rows, labels, seed=0, epochs=12, batch=2048, lr=2e-3, pos_weight=None):
    """Train a model on (rows, labels); positives up-weighted to balance the classes."""
    y = np.asarray(labels, np.uint8)
    npos = max(int(y.sum()), 1)
    if pos_weight is None:
        pos_weight = float(min(max((y.size - npos) / npos, 1.0), 200.0))
    model = init_model(seed, rows)
    model, st = dev.triage_train(model, rows, y, epochs=epochs, batch=batch, lr=lr, pos_weight=pos_weight, seed=seed)
    st["pos_weight"] = pos_weight
    return model, st


def threshold_for_recall(logits, labels, recall=0.999, margin=1.0):
    """The logit threshold that keeps `recall` of the positives of a
    calibration set, lowered by `margin` (a conservative cut)."""
    z = np.asarray(logits, np.float64)[np.asarray(labels) > 0]
    if z.size == 0:
        return -np.inf
    z = np.sort(z)
    k = int(np.floor((1.0 - recall) * z.size))
    return float(z[min(k, z.size - 1)] - margin)


def hit_key(h):
    return (h["subject"], h["score"], h["q_start"], h["q_end"], h["s_start"], h["s_end"], h["evalue"])


def compare_hits(plain, triaged):
    """(kept, total, identical): plain hits found by the triaged search with
    identical scores, coordinates and E-values."""
    kept = total = 0
    identical = True
    for a, b in zip(plain, triaged):
        kb = {hit_key(h) for h in b}
        for h in a:
            total += 1
            kept += hit_key(h) in kb
        ka = {hit_key(h) for h in a}
        for h in b:
            if hit_key(h) not in ka:
                identical = False
    return kept, total, identical
