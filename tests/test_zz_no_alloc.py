"""GPU test of the allocation-free scoring entry point
(saber_gpu_score_band_jobs_noalloc).

That entry point serves callers that cannot allocate GPU memory while they
score (a CUDA graph being captured, memory owned by another allocator or a
fixed budget, a path that cannot afford cudaMalloc's implicit device
synchronisation): it uses a fixed scratch array compiled into the library.
This test calls it through the C ABI twice in a row and checks every score
against the regular (allocating) entry point — exact equality, as for all
integer scores here.  The file sorts last so a run that stops at the first
failure has run every other test first; it also passes on its own.
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
    try:
        dev.set_scheme(matrix("BLOSUM62"), 11, 1)
        dev.load_db(ss.codes, ss.offsets)
        dev.load_queries(qs.codes, qs.offsets, bias)
        for call in range(2):
            jobs = synth.band_jobs(90 + call, qs, ss, planted, 3000 + 500 * call, half_min=1, half_max=128)
            want, _ = dev.score_band_jobs(jobs)
            d_jobs = torch.from_numpy(jobs.view(np.uint8).copy()).cuda()
            d_out = torch.full((jobs.size,), -7, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            dev.score_band_jobs_noalloc(d_jobs.data_ptr(), jobs.size, 257, d_out.data_ptr())
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            assert np.array_equal(got, want), "call %d: %d scores differ" % (call, int(np.sum(got != want)))
        # sizes beyond the stated maximum are rejected with a clear error
        with pytest.raises(SaberGpuError, match="max_band_width"):
            dev.score_band_jobs_noalloc(d_jobs.data_ptr(), jobs.size, 5000, d_out.data_ptr())
        with pytest.raises(SaberGpuError, match="wider than max_band_width"):
            dev.score_band_jobs_noalloc(d_jobs.data_ptr(), jobs.size, 16, d_out.data_ptr())
    finally:
        dev.close()
