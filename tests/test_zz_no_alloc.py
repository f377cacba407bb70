"""GPU test of the allocation-free scoring entry point
(saber_gpu_score_band_jobs_noalloc).

That entry point serves callers that cannot allocate GPU memory while they
score (device memory owned by another allocator or reserved in a fixed
budget, a path that cannot afford cudaMalloc's implicit device
synchronisation): its only scratch is a fixed array compiled into the
library.  This test calls it through the C ABI on two calls in a row (the
second with fewer jobs than the first) and checks every score against the
regular (allocating) entry point — exact equality, as for all integer scores
here — then the errors: a width limit beyond the maximum, a job wider than
the limit and a job outside the loaded queries (each naming the job), a good
call after a failed one, and a call with no jobs.  The file sorts last so a
run that stops at the first failure has run every other test first; it also
passes on its own.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_no_alloc_entry_point_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from saber_gb300 import Device, synth
    from saber_gb300.gpu import SaberGpuError
    from saber_gb300.scoring import matrix

    qs, ss, planted = synth.protein_db(77, 24, 1500)
    bias = synth.query_bias(78, qs)
    dev = Device(0)

    def run(jobs, max_w):
        d_jobs = torch.from_numpy(jobs.view(np.uint8).copy()).cuda()
        d_out = torch.full((max(jobs.size, 1),), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        dev.score_band_jobs_noalloc(d_jobs.data_ptr(), jobs.size, max_w, d_out.data_ptr())
        return d_out.cpu().numpy()[:jobs.size]

    try:
        dev.set_scheme(matrix("BLOSUM62"), 11, 1)
        dev.load_db(ss.codes, ss.offsets)
        dev.load_queries(qs.codes, qs.offsets, bias)
        for call, nj in enumerate((3500, 3000)):
            jobs = synth.band_jobs(90 + call, qs, ss, planted, nj, half_min=1, half_max=128)
            want, _ = dev.score_band_jobs(jobs)
            got = run(jobs, 257)
            assert np.array_equal(got, want), "call %d: %d scores differ" % (call, int(np.sum(got != want)))
        # sizes beyond the stated maximum are rejected with a clear error
        with pytest.raises(SaberGpuError, match="max_band_width"):
            run(jobs, 5000)
        with pytest.raises(SaberGpuError, match=r"wider than max_band_width \(job \d+\)"):
            run(jobs, 16)
        bad = jobs[:200].copy()
        bad["query"][123] = len(qs)
        with pytest.raises(SaberGpuError, match=r"outside the loaded data \(job 123\)"):
            run(bad, 257)
        # the next call starts from a cleared status word
        assert np.array_equal(run(jobs[:200], 257), want[:200])
        assert run(jobs[:0], 257).size == 0
    finally:
        dev.close()
