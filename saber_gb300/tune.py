"""Autotuner of the banded scoring launch shape.

The packed int16 kernel's launch has three shape knobs that change speed,
never results:

* the band tile, rows per strip (`Device.strip_rows`, 8 or 16): 16-row strips
  halve the boundary traffic per cell, 8-row strips waste fewer cells at the
  band's left triangle and at query ends;
* lanes per region (`Device.pair_steps`): a job whose 16-row sweep is longer
  than the threshold gets a whole lane as paired 32-row strips (half the
  critical path) instead of half a lane; the threshold is the bin edge
  between the two classes;
* the long-job bin edge (`Device.long_steps`): a job whose one-lane sweep is
  longer than this goes to the warp-per-job int32 kernel's pipelined strips
  (a whole warp on one job) instead of a lane of the int16 kernel; the
  default picks it per call from the batch's in-band cells per lane (the
  power of two at or above four times a lane's even share of the sweep
  steps, at least 2048).

`autotune_scoring` times settings on the caller's own batch (the
device-resident entry point, same stream) by coordinate descent: starting
from the first candidate of each knob, it times every candidate of one knob
with the others held, keeps the fastest, and goes round the knobs until a
full round changes nothing (or after `rounds` rounds).  Every timed setting
must give scores identical to the first one's.  The fastest setting is left
on the device and the table of timed settings is returned.  The reference
has no counterpart (its AVX2 kernels have fixed vector widths and one job
per vector lane).
"""
import time

PAIR_NEVER = 0xFFFFFFFF
LONG_AUTO = 0xFFFFFFFE

# candidates per knob; the first of each is the starting point
KNOBS = (
    ("strip_rows", (16, 8)),
    ("pair_steps", (2048, 1024, 4096, 8192, PAIR_NEVER)),
    ("long_steps", (LONG_AUTO, 4096, 8192, 16384, 65536)),
)


def autotune_scoring(dev, d_jobs, d_scores, knobs=KNOBS, reps=3, rounds=2):
    """Pick the fastest (strip_rows, pair_steps, long_steps) for scoring `d_jobs`.

    d_jobs: CUDA uint8 tensor holding saber_band_job records; d_scores: CUDA
    int32 tensor of one score per job (overwritten).  Returns a dict with the
    chosen setting and every timed setting's best time (ms)."""
    import torch

    njobs = d_scores.numel()
    ref = [None]
    timed = {}

    def run(setting):
        key = tuple(setting[name] for name, _ in knobs)
        if key in timed:
            return timed[key]
        for name, _ in knobs:
            setattr(dev, name, setting[name])
        dev.score_band_jobs_dev(d_jobs.data_ptr(), njobs, d_scores.data_ptr())  # warm: scratch sizes
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            dev.score_band_jobs_dev(d_jobs.data_ptr(), njobs, d_scores.data_ptr())
            best = min(best, time.perf_counter() - t0)
        if ref[0] is None:
            ref[0] = d_scores.clone()
        elif not torch.equal(ref[0], d_scores):
            raise RuntimeError("scores differ between kernel shapes %s" % (setting,))
        timed[key] = best
        return best

    cur = {name: cands[0] for name, cands in knobs}
    cur_t = run(cur)
    for _ in range(rounds):
        changed = False
        for name, cands in knobs:
            for v in cands:
                trial = dict(cur, **{name: v})
                t = run(trial)
                if t < cur_t:
                    cur, cur_t, changed = trial, t, True
        if not changed:
            break
    for name, _ in knobs:
        setattr(dev, name, cur[name])
    table = [dict(zip([n for n, _ in knobs], k), ms=round(t * 1e3, 3)) for k, t in timed.items()]
    return dict(cur, candidates=table)
