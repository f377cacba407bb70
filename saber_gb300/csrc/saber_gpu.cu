// C-ABI runtime of libsaber_gb300.so: handle, device-resident database and
// query sets, and the banded scoring pipeline
//   classify -> radix sort by (strips, width, query) -> packed int16 kernel
//   (64 consecutive jobs per warp task) -> int32 kernel (narrow bands and
//   int16 overflows)
// all on the handle's stream.  See include/saber_gpu.h for the contract.
#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "band_common.cuh"
#include "saber_gpu.h"

#include "runtime.cuh"

namespace saber {

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------
// Database seed mask from half-open runs [runs[2r], runs[2r+1]): one warp per
// run, lanes over its bytes (the index's mask runs, index.rs:613-617).
__global__ void k_fill_runs(const uint64_t* __restrict__ runs, uint64_t nruns, uint8_t* __restrict__ mask) {
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    for (uint64_t r = warp; r < nruns; r += nwarps)
        for (uint64_t i = runs[2 * r] + lane; i < runs[2 * r + 1]; i += 32) mask[i] = 1;
}

__global__ void k_canon(uint8_t* __restrict__ r, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint8_t c = r[i];
        if (c >= 24) r[i] = 22;  // alphabet.rs:39-41
    }
}

// Query profile P[c][i] = S(q_i, c) + bias_i + go for c < 24 and i < m, the
// sentinel score + go elsewhere (row 24 and rows past the query end).  The
// gap-open cost is folded in for the packed kernel, which adds the profile
// to H - go; the int32 kernels and the traceback subtract it again.  When
// every real entry lies in [-127, 127], an int8 copy with sentinel -128 is
// written too (prof8, else null): the packed kernel then reads half the
// bytes.  The reference builds the same per-query table (without go) for its
// ungapped extension (engine.rs:387-388) and a per-subject one in its int16
// kernel (banded_simd.rs:425-469).
__global__ void k_profile(const uint8_t* __restrict__ codes, const uint64_t* __restrict__ qoffs,
                          const int8_t* __restrict__ bias, const int32_t* __restrict__ matrix,
                          const uint64_t* __restrict__ prof_off, const uint32_t* __restrict__ prof_mpad,
                          int go, int16_t* __restrict__ prof, int8_t* __restrict__ prof8) {
    const uint32_t q = blockIdx.x;
    const uint64_t q0 = qoffs[q];
    const int m = (int)(qoffs[q + 1] - q0);
    const int mpad = (int)prof_mpad[q];
    int16_t* P = prof + prof_off[q];
    for (int t = threadIdx.x; t < kProfRows * mpad; t += blockDim.x) {
        int c = t / mpad, i = t - c * mpad;
        int v = kSent16;
        const bool real = c < 24 && i < m;
        if (real) {
            int qc = codes[q0 + i];
            if (qc >= 24) qc = 22;
            v = matrix[qc * 24 + c] + (bias ? (int)bias[q0 + i] : 0);
        }
        P[t] = (int16_t)(v + go);
        if (prof8) prof8[prof_off[q] + t] = real ? (int8_t)(v + go) : (int8_t)-128;
    }
}

// Widest clipped band (out[0]) and in-band cell total (out[1]) of the jobs
// that reference a loaded query.
__global__ void k_job_wmax(const saber_band_job* __restrict__ jobs, uint64_t njobs,
                           const uint64_t* __restrict__ qoffs, uint32_t nq, unsigned long long* __restrict__ out) {
    unsigned long long wm = 0, cells = 0;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < njobs; t += (uint64_t)gridDim.x * blockDim.x) {
        const saber_band_job j = jobs[t];
        if (j.query >= nq) continue;
        const int64_t m = (int64_t)(qoffs[j.query + 1] - qoffs[j.query]);
        int64_t lo = j.band_lo, hi = j.band_hi;
        const int64_t w = clip_band(m, j.win_len, lo, hi);
        wm = max(wm, (unsigned long long)w);
        if (w > 0) cells += band_cells(m, j.win_len, lo, hi);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        wm = max(wm, __shfl_xor_sync(0xffffffffu, wm, o));
        cells += __shfl_xor_sync(0xffffffffu, cells, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (wm) atomicMax(out, wm);
        if (cells) atomicAdd(out + 1, cells);
    }
}

// stats layout (uint64): 0 cells, 1 wmax of the R-row class, 2 wmax of the
//   int32 class, 3 bad job count, 4 cells of the packed classes, 5 wmax of
//   the 8-row class
// counts layout (uint32): 0 jobs in the R-row class (paired ones included),
//   1 int32 class, 4 empty, 5 int32 list length (class + rescued), 6 task
//   counter of the R-row launch, 7 jobs in the 8-row class, 8 task counter of
//   the 8-row launch, 9 paired jobs of the R-row class
//
// Classes (the top two key bits, so the sort makes them contiguous):
//   0: width >= R (R = the handle's strip rows), packed int16 kernel with R rows
//   1: 8 <= width < R when R = 16, packed int16 kernel with 8 rows
//   2: narrower bands, out-of-range sizes and sweeps longer than long_steps
//      column steps in one lane: the warp-per-job int32 kernel, largest first
//   3: empty jobs (score 0, written here)
// Packed-class keys order jobs by (strips, width, query) so that the 64
// consecutive jobs of a warp task share their loop counts and widths; within
// class 0 the paired jobs (bit 61; their strips counted in 2R rows) sort last.
__global__ void k_classify(const saber_band_job* __restrict__ jobs, uint64_t njobs, const uint32_t* __restrict__ n_real,
                           int R, uint32_t pair_steps, uint32_t long_steps, const uint64_t* __restrict__ qoffs,
                           uint32_t nq, uint64_t n_res,
                           uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                           int32_t* __restrict__ scores, uint32_t* __restrict__ counts,
                           unsigned long long* __restrict__ stats) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t cells = 0, fcells = 0;
    uint32_t c0 = 0, c1 = 0, c2 = 0, c3 = 0, cp = 0, bad = 0;
    unsigned long long w0 = 0, w1 = 0, w2 = 0;
    // padded launches (captured graphs): entries past the real job count sort
    // last as empty jobs and are neither scored nor counted
    const uint64_t nreal = n_real ? *n_real : njobs;
    for (; t < njobs; t += (uint64_t)gridDim.x * blockDim.x) {
        vals[t] = (uint32_t)t;
        if (t >= nreal) {
            keys[t] = (3ull << 62) | t;
            continue;
        }
        saber_band_job j = jobs[t];
        bool ok = j.query < nq && j.win_begin + (uint64_t)j.win_len <= n_res;
        int64_t m = ok ? (int64_t)(qoffs[j.query + 1] - qoffs[j.query]) : 0;
        int64_t lo = j.band_lo, hi = j.band_hi;
        int64_t w = ok ? clip_band(m, j.win_len, lo, hi) : 0;
        if (!ok) bad++;
        if (w == 0) {
            scores[t] = 0;
            keys[t] = 3ull << 62;
            c3++;
            continue;
        }
        const uint64_t jc = band_cells(m, j.win_len, lo, hi);
        cells += jc;
        // strips of `rows` rows holding the job's in-window rows
        const int64_t first = hi < 0 ? -hi : 0;
        int64_t last = (int64_t)j.win_len - 1 - lo;
        if (last > m - 1) last = m - 1;
        int cls = 2;
        int rows = R;
        if (w >= R) cls = 0;
        else if (R > kStripRowsMin && w >= kStripRowsMin) {
            cls = 1;
            rows = kStripRowsMin;
        }
        int64_t ns = last / rows - first / rows + 1;
        // long R-row sweeps go to paired strips (one job per lane, 2R rows)
        uint64_t pair = 0;
        if (cls == 0 && R == kStripRows && w >= 2 * R + 1 && (uint64_t)ns * (uint64_t)(w + R - 1) > pair_steps) {
            pair = 1;
            ns = last / (2 * R) - first / (2 * R) + 1;
        }
        if (cls != 2 && (w >= (1 << 16) || ns >= (1 << 13))) cls = 2;
        // a sweep longer than long_steps column steps in one lane goes to the
        // warp-per-job int32 kernel
        if (cls != 2) {
            // the sweep's steps per strip: the band's, or the window's when
            // the band is wider (the kernels sweep window columns only)
            const int64_t srw = pair ? 2 * R : rows;
            const int64_t span = w + srw - 1 < (int64_t)j.win_len + srw ? w + srw - 1 : (int64_t)j.win_len + srw;
            if ((uint64_t)ns * (uint64_t)span > long_steps) cls = 2;
        }
        if (cls == 2) {
            // largest first, so that the warps' static share ends together
            const uint64_t sz = jc >> 4 < 0x7FFFFFFFull ? jc >> 4 : 0x7FFFFFFFull;
            keys[t] = (2ull << 62) | ((0x7FFFFFFFull - sz) << 31) | t;
            c2++;
            w2 = max(w2, (unsigned long long)w);
        } else {
            // within (strips, width): jobs ordered by the first strip's
            // window geometry (steps before column -1, steps to the last
            // column), so that a warp's jobs share the step range it sweeps
            const int64_t srows = pair ? 2 * R : rows;
            const int64_t col0 = lo + (first / srows) * srows;
            const int64_t left = col0 < -1 ? -col0 - 1 : 0;
            const int64_t right = (int64_t)j.win_len - (pair ? 0 : 1) - col0;
            const uint64_t low = ((uint64_t)(left < 65535 ? left : 65535) << 16) |
                                 (uint64_t)(right < 0 ? 0 : (right < 65535 ? right : 65535));
            keys[t] = ((uint64_t)cls << 62) | (pair << 61) | ((uint64_t)ns << 48) | ((uint64_t)w << 32) | low;
            cp += (uint32_t)pair;
            fcells += jc;
            if (cls == 0) {
                c0++;
                w0 = max(w0, (unsigned long long)w);
            } else {
                c1++;
                w1 = max(w1, (unsigned long long)w);
            }
        }
    }
    // block totals in shared memory, then one global atomic per counter and block
    __shared__ unsigned long long b_sum[4];  // cells, bad, fast cells, unused
    __shared__ unsigned long long b_max[3];  // w0, w2, w1
    __shared__ uint32_t b_cnt[5];            // c0, c1, c2, c3, paired
    if (threadIdx.x < 5) b_cnt[threadIdx.x] = 0;
    if (threadIdx.x < 4) {
        b_sum[threadIdx.x] = 0;
        if (threadIdx.x < 3) b_max[threadIdx.x] = 0;
    }
    __syncthreads();
    c0 = __reduce_add_sync(0xffffffffu, c0);
    c1 = __reduce_add_sync(0xffffffffu, c1);
    c2 = __reduce_add_sync(0xffffffffu, c2);
    c3 = __reduce_add_sync(0xffffffffu, c3);
    cp = __reduce_add_sync(0xffffffffu, cp);
    bad = __reduce_add_sync(0xffffffffu, bad);
    for (int o = 16; o > 0; o >>= 1) {
        cells += __shfl_xor_sync(0xffffffffu, cells, o);
        fcells += __shfl_xor_sync(0xffffffffu, fcells, o);
        w0 = max(w0, __shfl_xor_sync(0xffffffffu, w0, o));
        w1 = max(w1, __shfl_xor_sync(0xffffffffu, w1, o));
        w2 = max(w2, __shfl_xor_sync(0xffffffffu, w2, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&b_cnt[0], c0);
        atomicAdd(&b_cnt[1], c1);
        atomicAdd(&b_cnt[2], c2);
        atomicAdd(&b_cnt[3], c3);
        atomicAdd(&b_cnt[4], cp);
        atomicAdd(&b_sum[0], (unsigned long long)cells);
        atomicAdd(&b_sum[1], (unsigned long long)bad);
        atomicAdd(&b_sum[2], (unsigned long long)fcells);
        atomicMax(&b_max[0], w0);
        atomicMax(&b_max[1], w2);
        atomicMax(&b_max[2], w1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(&counts[0], b_cnt[0]);
        atomicAdd(&counts[7], b_cnt[1]);
        atomicAdd(&counts[1], b_cnt[2]);
        atomicAdd(&counts[4], b_cnt[3]);
        atomicAdd(&counts[9], b_cnt[4]);
        atomicAdd(&stats[0], b_sum[0]);
        atomicMax(&stats[1], b_max[0]);
        atomicMax(&stats[2], b_max[1]);
        atomicAdd(&stats[3], b_sum[1]);
        atomicAdd(&stats[4], b_sum[2]);
        atomicMax(&stats[5], b_max[2]);
    }
}


// ---------------------------------------------------------------------------
// the scoring pipeline (device-resident jobs and scores)
// ---------------------------------------------------------------------------
// The long-job threshold of a call.  In the automatic mode a one-lane sweep
// goes to the warp-pipelined int32 kernel when it is longer than about four
// times the sweep steps each int16 lane gets if the batch's cells were
// spread evenly (a lane sweeps 32 cells per step), as a power of two, at
// least kLongStepsSmall: such a job would otherwise set the launch's length
// while most lanes are done.  Measured on one GB300 (threshold -> result):
// the blastn batch (26.8 k kilobase regions, about 6.9 k steps per lane)
// 2048 / 16384 / 32768 / none -> scoring 80 / 61 / 56 / 82 ms; the 1 M-job
// microbench (about 11.6 k) 16384 / 65536 / none -> 8.66 / 8.71 / 8.67 ms;
// the 11,000-query protein search (about 60 k) 32768 / none -> 64.1 /
// 64.1 ms of device scoring.
static uint32_t long_steps_for(const saber_gpu* h, uint64_t cells) {
    if (h->long_steps != kLongStepsAuto) return h->long_steps;
    const uint64_t lanes = (uint64_t)h->sm_count * band_fast_blocks_per_sm(h->strip_rows, false) * 256;
    const uint64_t load = cells / 32 / (lanes ? lanes : 1);
    uint64_t t = kLongStepsSmall;
    while (t < 4 * load && t < (1ull << 30)) t <<= 1;
    return (uint32_t)t;
}

// In-band cells of the device jobs (for the automatic long-job threshold):
// one reduction and an 8-byte read-back, only in the automatic mode.
static int jobs_cells(saber_gpu* h, const QuerySet& qs, const saber_band_job* d_jobs, uint64_t njobs,
                      uint64_t* cells) {
    *cells = 0;
    if (h->long_steps != kLongStepsAuto || !qs.has || njobs == 0) return SABER_OK;
    CUALLOC(h, h->g_wmax, 16);
    CU(h, cudaMemsetAsync(h->g_wmax.p, 0, 16, h->stream));
    k_job_wmax<<<nblocks(njobs, 256, h->sm_count * 8), 256, 0, h->stream>>>(
        d_jobs, njobs, qs.offsets.as<uint64_t>(), qs.nq, h->g_wmax.as<unsigned long long>());
    CU(h, cudaGetLastError());
    unsigned long long r[2] = {0, 0};
    CU(h, cudaMemcpyAsync(r, h->g_wmax.p, 16, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    *cells = r[1];
    return SABER_OK;
}

static int score_pipeline(saber_gpu* h, const Scheme& sch, const Dataset& ds, const saber_band_job* d_jobs,
                          uint64_t njobs, int32_t* d_scores, saber_score_stats* st) {
    if (!sch.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    if (!ds.has_db) return fail(h, SABER_ERR_STATE, "no database loaded");
    if (!ds.qs.has) return fail(h, SABER_ERR_STATE, "no query set loaded");
    if (njobs >= (1ull << 31))
        return fail(h, SABER_ERR_ARG, "too many jobs in one call (%llu)", (unsigned long long)njobs);
    saber_score_stats local{};
    if (njobs == 0) {
        if (st) *st = local;
        return SABER_OK;
    }
    cudaStream_t s = h->stream;
    const uint32_t n = (uint32_t)njobs;
    CUALLOC(h, h->keys_in, njobs * 8);
    CUALLOC(h, h->keys_out, njobs * 8);
    CUALLOC(h, h->vals_in, njobs * 4);
    CUALLOC(h, h->vals_out, njobs * 4);
    CUALLOC(h, h->counts, 16 * 4);
    CUALLOC(h, h->stats, 8 * 8);
    CUALLOC(h, h->list, njobs * 4);
    uint32_t* counts = h->counts.as<uint32_t>();
    unsigned long long* stats = h->stats.as<unsigned long long>();
    CU(h, cudaMemsetAsync(counts, 0, 16 * 4, s));
    CU(h, cudaMemsetAsync(stats, 0, 8 * 8, s));

    const QuerySet& qs = ds.qs;
    uint64_t job_cells = 0;
    int rc0 = jobs_cells(h, qs, d_jobs, njobs, &job_cells);
    if (rc0 != SABER_OK) return rc0;
    const uint32_t long_steps = long_steps_for(h, job_cells);
    cudaEvent_t ev[4];
    for (int i = 0; i < 4; i++) CU(h, cudaEventCreate(&ev[i]));
    struct EvGuard {
        cudaEvent_t* e;
        ~EvGuard() {
            for (int i = 0; i < 4; i++) cudaEventDestroy(e[i]);
        }
    } evg{ev};
    CU(h, cudaEventRecord(ev[0], s));
    k_classify<<<nblocks(njobs, 256, h->sm_count * 8), 256, 0, s>>>(
        d_jobs, njobs, nullptr, h->strip_rows, h->pair_steps, long_steps, qs.offsets.as<uint64_t>(), qs.nq,
        ds.n_res,
        h->keys_in.as<uint64_t>(),
        h->vals_in.as<uint32_t>(), d_scores, counts, stats);
    CU(h, cudaGetLastError());
    local.kernel_launches++;

    // CUB temp storage of the radix sort
    size_t t_sort = 0;
    CU(h, cub::DeviceRadixSort::SortPairs(nullptr, t_sort, h->keys_in.as<uint64_t>(),
                                          h->keys_out.as<uint64_t>(), h->vals_in.as<uint32_t>(),
                                          h->vals_out.as<uint32_t>(), (int)n, 0, 64, s));
    CUALLOC(h, h->cub_tmp, t_sort);
    size_t tb = h->cub_tmp.cap;
    CU(h, cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, tb, h->keys_in.as<uint64_t>(),
                                          h->keys_out.as<uint64_t>(), h->vals_in.as<uint32_t>(),
                                          h->vals_out.as<uint32_t>(), (int)n, 0, 64, s));
    local.library_launches += 9;  // onesweep radix sort: histogram + 8 digit passes

    // one small read-back: class counts and widths size the scratch
    uint32_t hc[10];
    unsigned long long hs[6];
    CU(h, cudaMemcpyAsync(hc, counts, 10 * 4, cudaMemcpyDeviceToHost, s));
    CU(h, cudaMemcpyAsync(hs, stats, 6 * 8, cudaMemcpyDeviceToHost, s));
    CU(h, cudaStreamSynchronize(s));
    if (hs[3] != 0)
        return fail(h, SABER_ERR_ARG, "%llu job(s) reference a query or window outside the loaded data", hs[3]);
    const uint32_t n_fast = hc[0], n_gen = hc[1], n_fast8 = hc[7];
    local.jobs = njobs;
    local.banded_cells = hs[0];
    local.fast_cells = hs[4];
    local.fast_jobs = n_fast + n_fast8;
    local.generic_jobs = n_gen;
    local.empty_jobs = hc[4];
    const uint64_t wmax_fast = std::max<uint64_t>(hs[1], hs[5]);
    const uint64_t wmax_all = std::max<uint64_t>(wmax_fast, hs[2]);

    const uint32_t* order = h->vals_out.as<uint32_t>();
    // generic list: class-1 jobs, then int16 overflows appended by the fast kernel
    if (n_gen)
        CU(h, cudaMemcpyAsync(h->list.as<uint32_t>(), order + n_fast + n_fast8, (size_t)n_gen * 4,
                              cudaMemcpyDeviceToDevice, s));
    CU(h, cudaMemcpyAsync(counts + 5, &n_gen, 4, cudaMemcpyHostToDevice, s));

    CU(h, cudaEventRecord(ev[1], s));
    // packed int16 launches: the R-row class, then the 8-row class; persistent
    // warps, one boundary buffer of (wmax + 1) x 32 lanes per warp, shared by
    // the two launches (same stream)
    for (int pass = 0; pass < 2; pass++) {
        const uint32_t nj = pass == 0 ? n_fast : n_fast8;
        if (nj == 0) continue;
        const int rows = pass == 0 ? h->strip_rows : kStripRowsMin;
        const int bps = band_fast_blocks_per_sm(rows, qs.p8);
        const unsigned grid = (unsigned)(h->sm_count * bps);
        const uint64_t warps = (uint64_t)grid * 256 / 32;
        const uint32_t stride = (uint32_t)(wmax_fast + 1);
        CUALLOC(h, h->bufs, warps * stride * 32 * sizeof(uint2));
        FastArgs a;
        a.res = ds.res.as<uint8_t>();
        a.prof = qs.prof.as<int16_t>();
        a.prof8 = qs.p8 ? qs.prof8.as<int8_t>() : nullptr;
        a.prof_off = qs.prof_off.as<uint64_t>();
        a.prof_mpad = qs.prof_mpad.as<uint32_t>();
        a.qoffs = qs.offsets.as<uint64_t>();
        a.jobs = d_jobs;
        a.order = order + (pass == 0 ? 0 : n_fast);
        a.n_ptr = counts + (pass == 0 ? 0 : 7);
        a.np_ptr = pass == 0 ? counts + 9 : nullptr;
        a.order_skip = nullptr;
        a.wt_counter = counts + (pass == 0 ? 6 : 8);
        a.bufs = h->bufs.as<uint2>();
        a.buf_stride = stride;
        a.go = sch.go;
        a.ge = sch.ge;
        a.scores = d_scores;
        a.rescue = h->list.as<uint32_t>();
        a.rescue_count = counts + 5;
        a.strip_rows = rows;
        CU(h, launch_band_fast(grid, s, a));
        local.kernel_launches++;
    }
    CU(h, cudaEventRecord(ev[2], s));
    {
        // int32 kernel over narrow bands and rescued jobs (count read on the device)
        const unsigned T = 128;
        const unsigned grid = (unsigned)(h->sm_count * 4);
        const uint64_t warps = (uint64_t)grid * T / 32;
        const uint32_t stride = (uint32_t)(wmax_all + 1);
        CUALLOC(h, h->slabs, warps * stride * 4 * sizeof(int32_t));
        GenericArgs a;
        a.res = ds.res.as<uint8_t>();
        a.prof = qs.prof.as<int16_t>();
        a.prof_off = qs.prof_off.as<uint64_t>();
        a.prof_mpad = qs.prof_mpad.as<uint32_t>();
        a.qoffs = qs.offsets.as<uint64_t>();
        a.jobs = d_jobs;
        a.list = h->list.as<uint32_t>();
        a.list_count = counts + 5;
        a.slabs = h->slabs.as<int32_t>();
        a.slab_stride = stride;
        a.go = sch.go;
        a.ge = sch.ge;
        a.scores = d_scores;
        CU(h, launch_band_generic(grid, T, s, a));
        CU(h, cudaEventRecord(ev[3], s));
        local.kernel_launches++;
    }
    uint32_t glist = 0;
    CU(h, cudaMemcpyAsync(&glist, counts + 5, 4, cudaMemcpyDeviceToHost, s));
    CU(h, cudaStreamSynchronize(s));
    local.i16_rescored = glist - n_gen;
    float t01 = 0, t12 = 0, t23 = 0;
    CU(h, cudaEventElapsedTime(&t01, ev[0], ev[1]));
    CU(h, cudaEventElapsedTime(&t12, ev[1], ev[2]));
    CU(h, cudaEventElapsedTime(&t23, ev[2], ev[3]));
    local.t_prep_ms = t01;
    local.t_fast_ms = t12;
    local.t_generic_ms = t23;
    local.prof8 = qs.p8 ? 1 : 0;
    if (st) *st = local;
    return SABER_OK;
}

// Generic list for a captured scoring graph: the int32 class's jobs (after
// the R-row and 8-row classes in the sorted order), counts read on the device.
__global__ void k_copy_generic(const uint32_t* __restrict__ order, uint32_t* __restrict__ counts,
                               uint32_t* __restrict__ list) {
    const uint32_t n_fast = counts[0], n_fast8 = counts[7], n_gen = counts[1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_gen; i += gridDim.x * blockDim.x)
        list[i] = order[n_fast + n_fast8 + i];
    if (blockIdx.x == 0 && threadIdx.x == 0) counts[5] = n_gen;
}

static uint64_t pow2_at_least(uint64_t v, uint64_t lo) {
    uint64_t p = lo;
    while (p < v) p <<= 1;
    return p;
}

// The scoring pipeline as a CUDA graph: the same kernels as score_pipeline
// with every count kept on the device (the real job count in a device word,
// padded entries sorted last as empty jobs), scratch sized for a power-of-two
// job count and band width, captured once per (size bucket, buffers,
// settings) and replayed.  Jobs and scores live in the handle's buffers.
static int score_pipeline_graph(saber_gpu* h, const Scheme& sch, const Dataset& ds, uint64_t njobs, uint64_t wmax,
                                uint64_t job_cells, saber_score_stats* st) {
    if (!sch.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    if (!ds.has_db) return fail(h, SABER_ERR_STATE, "no database loaded");
    if (!ds.qs.has) return fail(h, SABER_ERR_STATE, "no query set loaded");
    const uint64_t npad = pow2_at_least(njobs, 1 << 12);
    const uint64_t wcap = pow2_at_least(wmax + 1, 64);
    if (npad >= (1ull << 31)) return fail(h, SABER_ERR_ARG, "too many jobs in one call");
    cudaStream_t s = h->stream;
    const QuerySet& qs = ds.qs;
    CUALLOC(h, h->keys_in, npad * 8);
    CUALLOC(h, h->keys_out, npad * 8);
    CUALLOC(h, h->vals_in, npad * 4);
    CUALLOC(h, h->vals_out, npad * 4);
    CUALLOC(h, h->counts, 16 * 4);
    CUALLOC(h, h->stats, 8 * 8);
    CUALLOC(h, h->list, npad * 4);
    CUALLOC(h, h->g_nreal, 16);
    const int rows0 = h->strip_rows;
    const unsigned grid0 = (unsigned)(h->sm_count * band_fast_blocks_per_sm(rows0, qs.p8));
    const unsigned grid8 = (unsigned)(h->sm_count * band_fast_blocks_per_sm(kStripRowsMin, qs.p8));
    const uint64_t warps = (uint64_t)std::max(grid0, grid8) * 256 / 32;
    CUALLOC(h, h->bufs, warps * wcap * 32 * sizeof(uint2));
    const unsigned gT = 128, gGrid = (unsigned)(h->sm_count * 4);
    CUALLOC(h, h->slabs, (uint64_t)gGrid * (gT / 32) * wcap * 4 * sizeof(int32_t));
    size_t t_sort = 0;
    CU(h, cub::DeviceRadixSort::SortPairs(nullptr, t_sort, h->keys_in.as<uint64_t>(), h->keys_out.as<uint64_t>(),
                                          h->vals_in.as<uint32_t>(), h->vals_out.as<uint32_t>(), (int)npad, 0, 64, s));
    CUALLOC(h, h->cub_tmp, t_sort);
    GraphKey key;
    std::memset(&key, 0, sizeof(key));
    key.npad = npad;
    key.wcap = wcap;
    key.rows = rows0;
    key.go = sch.go;
    key.ge = sch.ge;
    key.pair_steps = h->pair_steps;
    const uint32_t long_steps = long_steps_for(h, job_cells);
    key.long_steps = long_steps;
    key.n_res = ds.n_res;  // scalar kernel parameters baked into the graph
    key.nq = qs.nq;
    key.prof8 = qs.p8 ? qs.prof8.p : nullptr;  // which packed kernel the graph launches
    const void* ptrs[16] = {h->jobs_dev.p, h->scores_dev.p, h->keys_in.p, h->keys_out.p, h->vals_in.p,
                            h->vals_out.p, h->counts.p, h->stats.p, h->list.p, h->bufs.p, h->slabs.p,
                            h->cub_tmp.p, ds.res.p, qs.prof.p, qs.offsets.p, qs.prof_off.p};
    std::memcpy(key.ptrs, ptrs, sizeof(ptrs));
    const void* extra = qs.prof_mpad.p;  // (pointer identity of the last profile table)
    cudaGraphExec_t exec = nullptr;
    for (auto& e : h->graphs)
        if (e.first == key && e.second.extra == extra) exec = e.second.exec;
    if (!exec) {
        uint32_t* counts = h->counts.as<uint32_t>();
        unsigned long long* stats = h->stats.as<unsigned long long>();
        const saber_band_job* d_jobs = h->jobs_dev.as<saber_band_job>();
        int32_t* d_scores = h->scores_dev.as<int32_t>();
        CU(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        bool ok = true;
        auto chk = [&](cudaError_t e) {
            if (e != cudaSuccess) ok = false;
        };
        chk(cudaMemsetAsync(counts, 0, 16 * 4, s));
        chk(cudaMemsetAsync(stats, 0, 8 * 8, s));
        k_classify<<<nblocks(npad, 256, h->sm_count * 8), 256, 0, s>>>(
            d_jobs, npad, h->g_nreal.as<uint32_t>(), rows0, h->pair_steps, long_steps,
            qs.offsets.as<uint64_t>(), qs.nq,
            ds.n_res, h->keys_in.as<uint64_t>(), h->vals_in.as<uint32_t>(), d_scores, counts, stats);
        chk(cudaGetLastError());
        size_t tb = h->cub_tmp.cap;
        chk(cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, tb, h->keys_in.as<uint64_t>(), h->keys_out.as<uint64_t>(),
                                            h->vals_in.as<uint32_t>(), h->vals_out.as<uint32_t>(), (int)npad, 0, 64,
                                            s));
        const uint32_t* order = h->vals_out.as<uint32_t>();
        k_copy_generic<<<h->sm_count * 4, 256, 0, s>>>(order, counts, h->list.as<uint32_t>());
        chk(cudaGetLastError());
        for (int pass = 0; pass < 2; pass++) {
            FastArgs a;
            a.res = ds.res.as<uint8_t>();
            a.prof = qs.prof.as<int16_t>();
            a.prof8 = qs.p8 ? qs.prof8.as<int8_t>() : nullptr;
            a.prof_off = qs.prof_off.as<uint64_t>();
            a.prof_mpad = qs.prof_mpad.as<uint32_t>();
            a.qoffs = qs.offsets.as<uint64_t>();
            a.jobs = d_jobs;
            a.order = order;
            a.n_ptr = counts + (pass == 0 ? 0 : 7);
            a.np_ptr = pass == 0 ? counts + 9 : nullptr;
            a.order_skip = pass == 0 ? nullptr : counts + 0;
            a.wt_counter = counts + (pass == 0 ? 6 : 8);
            a.bufs = h->bufs.as<uint2>();
            a.buf_stride = (uint32_t)wcap;
            a.go = sch.go;
            a.ge = sch.ge;
            a.scores = d_scores;
            a.rescue = h->list.as<uint32_t>();
            a.rescue_count = counts + 5;
            a.strip_rows = pass == 0 ? rows0 : kStripRowsMin;
            chk(launch_band_fast(pass == 0 ? grid0 : grid8, s, a));
        }
        GenericArgs g;
        g.res = ds.res.as<uint8_t>();
        g.prof = qs.prof.as<int16_t>();
        g.prof_off = qs.prof_off.as<uint64_t>();
        g.prof_mpad = qs.prof_mpad.as<uint32_t>();
        g.qoffs = qs.offsets.as<uint64_t>();
        g.jobs = d_jobs;
        g.list = h->list.as<uint32_t>();
        g.list_count = counts + 5;
        g.slabs = h->slabs.as<int32_t>();
        g.slab_stride = (uint32_t)wcap;
        g.go = sch.go;
        g.ge = sch.ge;
        g.scores = d_scores;
        chk(launch_band_generic(gGrid, gT, s, g));
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (e != cudaSuccess || !ok || !graph) {
            if (graph) cudaGraphDestroy(graph);
            return fail(h, SABER_ERR_CUDA, "capture of the scoring graph failed: %s", cudaGetErrorString(e));
        }
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(h, SABER_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
        if (h->graphs.size() >= 8) {
            cudaGraphExecDestroy(h->graphs.front().second.exec);
            h->graphs.erase(h->graphs.begin());
        }
        GraphEntry ge_{exec, extra};
        h->graphs.push_back({key, ge_});
        h->graph_captures++;
    }
    const uint32_t nreal = (uint32_t)njobs;
    CU(h, cudaMemcpyAsync(h->g_nreal.p, &nreal, 4, cudaMemcpyHostToDevice, s));
    cudaEvent_t e0, e1;
    CU(h, cudaEventCreate(&e0));
    CU(h, cudaEventCreate(&e1));
    CU(h, cudaEventRecord(e0, s));
    CU(h, cudaGraphLaunch(exec, s));
    CU(h, cudaEventRecord(e1, s));
    uint32_t hc[10];
    unsigned long long hs[6];
    CU(h, cudaMemcpyAsync(hc, h->counts.p, 10 * 4, cudaMemcpyDeviceToHost, s));
    CU(h, cudaMemcpyAsync(hs, h->stats.p, 6 * 8, cudaMemcpyDeviceToHost, s));
    CU(h, cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (hs[3] != 0)
        return fail(h, SABER_ERR_ARG, "%llu job(s) reference a query or window outside the loaded data", hs[3]);
    if (std::max<uint64_t>(std::max<uint64_t>(hs[1], hs[5]), hs[2]) + 1 > wcap)
        return fail(h, SABER_ERR_STATE, "band width above the graph's capacity");
    if (st) {
        saber_score_stats local{};
        local.jobs = njobs;
        local.banded_cells = hs[0];
        local.fast_cells = hs[4];
        local.fast_jobs = hc[0] + hc[7];
        local.generic_jobs = hc[1];
        local.empty_jobs = hc[4];
        local.i16_rescored = hc[5] - hc[1];
        local.kernel_launches = 5;
        local.library_launches = 9;
        local.t_fast_ms = ms;
        local.prof8 = qs.p8 ? 1 : 0;
        *st = local;
    }
    return SABER_OK;
}

static int build_profiles(saber_gpu* h, const Scheme& sch, QuerySet& q) {
    q.p8 = false;
    if (!q.has || !sch.has || q.nq == 0) return SABER_OK;
    // int8 copy when every real entry S + bias + go lies in [-127, 127]
    // (bounded over the whole matrix and the set's bias range)
    int smin = sch.matrix[0], smax = sch.matrix[0];
    for (int i = 1; i < 576; i++) {
        smin = std::min(smin, (int)sch.matrix[i]);
        smax = std::max(smax, (int)sch.matrix[i]);
    }
    const bool fits8 = smin + q.bias_min + sch.go >= -127 && smax + q.bias_max + sch.go <= 127;
    if (fits8) CUALLOC(h, q.prof8, q.prof_elems + 64);
    k_profile<<<q.nq, 256, 0, h->stream>>>(q.codes.as<uint8_t>(), q.offsets.as<uint64_t>(),
                                           q.has_bias ? q.bias.as<int8_t>() : nullptr, sch.d_matrix.as<int32_t>(),
                                           q.prof_off.as<uint64_t>(), q.prof_mpad.as<uint32_t>(), sch.go,
                                           q.prof.as<int16_t>(), fits8 ? q.prof8.as<int8_t>() : nullptr);
    CU(h, cudaGetLastError());
    CU(h, cudaStreamSynchronize(h->stream));
    q.p8 = fits8;
    return SABER_OK;
}

static int load_queries(saber_gpu* h, const Scheme& sch, QuerySet& q, const uint8_t* codes, const uint64_t* offsets,
                        const int8_t* bias, uint32_t nq) {
    if (!offsets) return fail(h, SABER_ERR_ARG, "null query offsets");
    if (offsets[0] != 0) return fail(h, SABER_ERR_ARG, "query offsets must start at 0");
    for (uint32_t i = 0; i < nq; i++)
        if (offsets[i + 1] < offsets[i]) return fail(h, SABER_ERR_ARG, "query offsets must be non-decreasing");
    const uint64_t total = offsets[nq];
    if (total && !codes) return fail(h, SABER_ERR_ARG, "null query codes");
    q.has = false;
    q.nq = nq;
    q.offs.assign(offsets, offsets + nq + 1);
    q.poff.clear();
    q.pmpad.clear();
    std::vector<uint64_t> poff(nq ? nq : 1, 0);
    std::vector<uint32_t> pm(nq ? nq : 1, kStripRows);
    uint64_t acc = 0;
    for (uint32_t i = 0; i < nq; i++) {
        uint64_t m = offsets[i + 1] - offsets[i];
        uint64_t mpad = (m + kProfPad - 1) / kProfPad * kProfPad;
        if (mpad == 0) mpad = kProfPad;
        if (mpad > (1ull << 30)) return fail(h, SABER_ERR_ARG, "query %u too long", i);
        poff[i] = acc;
        pm[i] = (uint32_t)mpad;
        acc += (uint64_t)kProfRows * mpad;
    }
    CUALLOC(h, q.codes, total + 16);
    CUALLOC(h, q.offsets, (uint64_t)(nq + 1) * 8);
    CUALLOC(h, q.prof_off, poff.size() * 8);
    CUALLOC(h, q.prof_mpad, pm.size() * 4);
    CUALLOC(h, q.prof, acc * 2 + 16);
    cudaStream_t s = h->stream;
    if (total) CU(h, cudaMemcpyAsync(q.codes.p, codes, total, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemcpyAsync(q.offsets.p, offsets, (uint64_t)(nq + 1) * 8, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemcpyAsync(q.prof_off.p, poff.data(), poff.size() * 8, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemcpyAsync(q.prof_mpad.p, pm.data(), pm.size() * 4, cudaMemcpyHostToDevice, s));
    q.has_bias = bias != nullptr && total > 0;
    q.bias_min = 0;
    q.bias_max = 0;
    if (q.has_bias) {
        CUALLOC(h, q.bias, total + 16);
        CU(h, cudaMemcpyAsync(q.bias.p, bias, total, cudaMemcpyHostToDevice, s));
        int bmin = bias[0], bmax = bias[0];
        for (uint64_t i = 1; i < total; i++) {
            bmin = std::min(bmin, (int)bias[i]);
            bmax = std::max(bmax, (int)bias[i]);
        }
        q.bias_min = bmin;
        q.bias_max = bmax;
    }
    q.prof_elems = acc;
    CU(h, cudaStreamSynchronize(s));
    q.poff.assign(poff.begin(), poff.begin() + nq);
    q.pmpad.assign(pm.begin(), pm.begin() + nq);
    q.has = true;
    return build_profiles(h, sch, q);
}

static int load_db(saber_gpu* h, Dataset& ds, const uint8_t* residues, uint64_t n_res, const uint64_t* offsets,
                   uint64_t nsub) {
    if ((!residues && n_res) || !offsets) return fail(h, SABER_ERR_ARG, "null database arrays");
    if (offsets[0] != 0 || offsets[nsub] != n_res)
        return fail(h, SABER_ERR_ARG, "subject offsets must run from 0 to n_residues");
    uint64_t max_len = 0;
    for (uint64_t i = 0; i < nsub; i++) {
        if (offsets[i + 1] < offsets[i]) return fail(h, SABER_ERR_ARG, "subject offsets must be non-decreasing");
        max_len = std::max<uint64_t>(max_len, offsets[i + 1] - offsets[i]);
    }
    ds.has_db = false;
    CUALLOC(h, ds.res, n_res + 64);
    CUALLOC(h, ds.soff, (nsub + 1) * 8);
    cudaStream_t s = h->stream;
    if (n_res) CU(h, cudaMemcpyAsync(ds.res.p, residues, n_res, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemsetAsync(ds.res.as<uint8_t>() + n_res, 22, 64, s));
    CU(h, cudaMemcpyAsync(ds.soff.p, offsets, (nsub + 1) * 8, cudaMemcpyHostToDevice, s));
    if (n_res) {
        k_canon<<<nblocks(n_res, 256, h->sm_count * 16), 256, 0, s>>>(ds.res.as<uint8_t>(), n_res);
        CU(h, cudaGetLastError());
    }
    CU(h, cudaStreamSynchronize(s));
    ds.n_res = n_res;
    ds.nsub = nsub;
    ds.max_len = max_len;
    ds.has_db = true;
    if (&ds == &h->main) {
        h->sc_key = 0;
        h->has_db_mask = false;
    }
    return SABER_OK;
}

static int set_scheme(saber_gpu* h, Scheme& sch, const int32_t* matrix, int32_t go, int32_t ge) {
    if (!matrix) return fail(h, SABER_ERR_ARG, "null matrix");
    if (ge < 0 || go < ge || go > 1000) return fail(h, SABER_ERR_ARG, "gap costs need 0 <= extend <= open <= 1000");
    for (int i = 0; i < 576; i++)
        if (matrix[i] < -512 || matrix[i] > 512)
            return fail(h, SABER_ERR_ARG, "substitution scores must lie in [-512, 512]");
    memcpy(sch.matrix, matrix, sizeof(sch.matrix));
    sch.go = go;
    sch.ge = ge;
    sch.has = false;
    CUALLOC(h, sch.d_matrix, 576 * 4);
    CU(h, cudaMemcpyAsync(sch.d_matrix.p, sch.matrix, 576 * 4, cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    sch.has = true;
    return SABER_OK;
}

// One query against many windows on the per-call dataset (score_banded_many
// and ScoreBackend::score_windows): the windows become the per-call database.
static int one_query_jobs(saber_gpu* h, const Scheme& sch, const uint8_t* query, uint32_t m, const int8_t* bias,
                          const uint8_t* subjects, const uint64_t* offs, const int64_t* blo, const int64_t* bhi,
                          uint64_t njobs, bool full, int32_t* scores) {
    if (njobs == 0) return SABER_OK;
    if (!offs || (!query && m)) return fail(h, SABER_ERR_ARG, "null argument");
    Dataset& ds = h->eph;
    int rc = load_db(h, ds, subjects, offs[njobs], offs, njobs);
    if (rc != SABER_OK) return rc;
    uint64_t qoff[2] = {0, m};
    rc = load_queries(h, sch, ds.qs, query, qoff, bias, 1);
    if (rc != SABER_OK) return rc;
    std::vector<saber_band_job> jobs(njobs);
    for (uint64_t t = 0; t < njobs; t++) {
        saber_band_job& j = jobs[t];
        uint64_t n = offs[t + 1] - offs[t];
        if (n > 0x7FFFFFFFull) return fail(h, SABER_ERR_ARG, "window %llu too long", (unsigned long long)t);
        j.query = 0;
        j.subject = (uint32_t)t;
        j.win_begin = offs[t];
        j.win_len = (uint32_t)n;
        int64_t lo = full ? -(int64_t)m : blo[t];
        int64_t hi = full ? (int64_t)n : bhi[t];
        // clip in 64 bits first (Band::clip never widens) so any band fits int32
        if (lo < -(int64_t)m) lo = -(int64_t)m;
        if (hi > (int64_t)n) hi = (int64_t)n;
        if (hi < lo) {
            lo = 1;
            hi = 0;
        }
        j.band_lo = (int32_t)lo;
        j.band_hi = (int32_t)hi;
        j.flags = 0;
    }
    CUALLOC(h, h->jobs_dev, njobs * sizeof(saber_band_job));
    CUALLOC(h, h->scores_dev, njobs * 4);
    CU(h, cudaMemcpyAsync(h->jobs_dev.p, jobs.data(), njobs * sizeof(saber_band_job), cudaMemcpyHostToDevice,
                          h->stream));
    rc = score_pipeline(h, sch, ds, h->jobs_dev.as<saber_band_job>(), njobs, h->scores_dev.as<int32_t>(), nullptr);
    if (rc != SABER_OK) return rc;
    CU(h, cudaMemcpyAsync(scores, h->scores_dev.p, njobs * 4, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    return SABER_OK;
}

// ---------------------------------------------------------------------------
// banded traceback: batched banded_align_until and the widening driver
// ---------------------------------------------------------------------------
struct AlignReq {
    const uint8_t* win;
    const int16_t* prof;
    uint64_t dir_off;
    uint64_t ops_off;
    int32_t m, n, lo, w;
    int32_t mpad;
    int32_t stop_at;
    int32_t want_dir;
    int32_t pad_;
};
struct AlignOut {
    int32_t status;
    int32_t score;
    uint32_t q_start, q_end, s_start, s_end;
    uint32_t n_ops;
    uint32_t pad_;
    uint64_t cells;
};
cudaError_t launch_band_align(unsigned grid, cudaStream_t s, const AlignReq* reqs, uint32_t nreq, uint8_t* dir_pool,
                              uint8_t* opbytes, uint32_t* runs, int32_t* slabs, uint32_t slab_stride, int go, int ge,
                              AlignOut* outs);

__global__ void k_pack_runs(const uint32_t* __restrict__ runs, const uint64_t* __restrict__ src_off,
                            const uint64_t* __restrict__ dst_off, const uint32_t* __restrict__ counts, uint32_t n,
                            uint32_t* __restrict__ packed) {
    for (uint32_t t = blockIdx.x; t < n; t += gridDim.x)
        for (uint32_t k = threadIdx.x; k < counts[t]; k += blockDim.x) packed[dst_off[t] + k] = runs[src_off[t] + k];
}

struct AlignHostReq {
    uint32_t query;
    uint64_t win_begin;
    uint32_t win_len;
    int64_t lo, hi;  // band (unclipped)
    int32_t stop_at;
    bool want_dir;
};
struct AlignResult {
    int status = 0;  // 1 alignment, 0 none, SABER_ERR_CAP over the direction-byte cap
    int32_t score = 0;
    uint32_t q_start = 0, q_end = 0, s_start = 0, s_end = 0;
    uint64_t cells = 0;
    // op runs ((len << 8) | op): n_runs from run_off of pools[pool], the
    // packed runs of the launch that produced the result
    uint32_t pool = 0, n_runs = 0;
    uint64_t run_off = 0;
};
using RunPools = std::vector<std::vector<uint32_t>>;

// Budget of the direction-byte pool per launch (larger batches are split).
// A launch ends with its longest job, so few launches per round matter: the
// blastn batch's first round (14.6 k alignments of kilobase windows, about
// 6.6 GB of direction bytes) fits one launch.
constexpr uint64_t kDirPoolBudget = 8ull << 30;
constexpr uint64_t kAlignSlabBudget = 512ull << 20;

static int align_batch(saber_gpu* h, const Scheme& sch, const Dataset& ds, const std::vector<AlignHostReq>& in,
                       uint64_t max_dir_bytes, std::vector<AlignResult>& out, RunPools& pools) {
    if (!sch.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    if (!ds.has_db || !ds.qs.has) return fail(h, SABER_ERR_STATE, "no database or query set loaded");
    const QuerySet& qs = ds.qs;
    out.assign(in.size(), AlignResult());
    std::vector<size_t> todo;
    todo.reserve(in.size());
    for (size_t t = 0; t < in.size(); t++) {
        const AlignHostReq& r = in[t];
        if (r.query >= qs.nq || r.win_begin + r.win_len > ds.n_res)
            return fail(h, SABER_ERR_ARG, "traceback job %zu references data outside the loaded set", t);
        int64_t m = (int64_t)(qs.offs[r.query + 1] - qs.offs[r.query]);
        int64_t lo = r.lo, hi = r.hi;
        int64_t w = clip_band(m, r.win_len, lo, hi);
        if (w == 0) continue;  // Ok(None)
        if (r.want_dir && (uint64_t)m * (uint64_t)w > max_dir_bytes) {
            out[t].status = SABER_ERR_CAP;
            continue;
        }
        todo.push_back(t);
    }
    // largest size class first (classes of log2 of the band cells, input
    // order within a class, one counting pass): warp w takes jobs w, w +
    // warps, ..., so the longest ones start together and the short ones fill
    // in behind them; within a class jobs of one query stay together.  Each
    // job is independent and results go back by index.
    {
        std::vector<uint8_t> cls(todo.size());
        size_t count[65] = {0};
        for (size_t k = 0; k < todo.size(); k++) {
            const AlignHostReq& r = in[todo[k]];
            int64_t lo = r.lo, hi = r.hi;
            const int64_t m = (int64_t)(qs.offs[r.query + 1] - qs.offs[r.query]);
            const uint64_t cells = (uint64_t)m * (uint64_t)clip_band(m, r.win_len, lo, hi);
            cls[k] = (uint8_t)(cells ? 64 - __builtin_clzll(cells) : 0);  // 1 + floor(log2), 0 for none
            count[cls[k]]++;
        }
        size_t start[65];
        size_t acc = 0;
        for (int c = 64; c >= 0; c--) {
            start[c] = acc;
            acc += count[c];
        }
        std::vector<size_t> sorted(todo.size());
        for (size_t k = 0; k < todo.size(); k++) sorted[start[cls[k]]++] = todo[k];
        todo.swap(sorted);
    }
    cudaStream_t s = h->stream;
    size_t pos = 0;
    while (pos < todo.size()) {
        // one launch: as many jobs as fit the pool budget
        std::vector<AlignReq> reqs;
        std::vector<size_t> idx;
        uint64_t dir_tot = 0, ops_tot = 0;
        int64_t wmax = 1;
        while (pos < todo.size()) {
            const AlignHostReq& r = in[todo[pos]];
            int64_t m = (int64_t)(qs.offs[r.query + 1] - qs.offs[r.query]);
            int64_t lo = r.lo, hi = r.hi;
            int64_t w = clip_band(m, r.win_len, lo, hi);
            uint64_t dbytes = r.want_dir ? (uint64_t)m * (uint64_t)w : 0;
            if (!reqs.empty() && dir_tot + dbytes > kDirPoolBudget) break;
            AlignReq q;
            q.win = ds.res.as<uint8_t>() + r.win_begin;
            q.prof = qs.prof.as<int16_t>() + qs.poff[r.query];
            q.dir_off = dir_tot;
            q.ops_off = ops_tot;
            q.m = (int32_t)m;
            q.n = (int32_t)r.win_len;
            q.lo = (int32_t)lo;
            q.w = (int32_t)w;
            q.mpad = (int32_t)qs.pmpad[r.query];
            q.stop_at = r.stop_at;
            q.want_dir = r.want_dir ? 1 : 0;
            q.pad_ = 0;
            dir_tot += (dbytes + 15) / 16 * 16;
            if (r.want_dir) ops_tot += (uint64_t)m + r.win_len + 2;
            wmax = std::max(wmax, w);
            reqs.push_back(q);
            idx.push_back(todo[pos]);
            pos++;
        }
        const uint32_t nreq = (uint32_t)reqs.size();
        const uint32_t stride = (uint32_t)(wmax + 1);
        // warp-per-job kernel: one row-buffer set per warp, one job per warp
        uint64_t warps = kAlignSlabBudget / ((uint64_t)stride * 16);
        if (warps < 4) warps = 4;
        warps = std::min<uint64_t>(std::min<uint64_t>(warps, ((uint64_t)nreq + 3) / 4 * 4),
                                   (uint64_t)h->sm_count * 6 * 4);
        const uint64_t thr = std::max<uint64_t>(warps / 4 * 4, 4) * 32;
        const unsigned grid = (unsigned)(thr / 128);
        CUALLOC(h, h->al_reqs, nreq * sizeof(AlignReq));
        CUALLOC(h, h->al_outs, nreq * sizeof(AlignOut));
        CUALLOC(h, h->al_dir, dir_tot + 16);
        CUALLOC(h, h->al_opbytes, ops_tot + 16);
        CUALLOC(h, h->al_runs, (ops_tot + 16) * 4);
        CUALLOC(h, h->al_slabs, (thr / 32) * stride * 16);
        CU(h, cudaMemcpyAsync(h->al_reqs.p, reqs.data(), nreq * sizeof(AlignReq), cudaMemcpyHostToDevice, s));
        CU(h, launch_band_align(grid, s, h->al_reqs.as<AlignReq>(), nreq, h->al_dir.as<uint8_t>(),
                                h->al_opbytes.as<uint8_t>(), h->al_runs.as<uint32_t>(), h->al_slabs.as<int32_t>(),
                                stride, sch.go, sch.ge, h->al_outs.as<AlignOut>()));
        std::vector<AlignOut> outs(nreq);
        CU(h, cudaMemcpyAsync(outs.data(), h->al_outs.p, nreq * sizeof(AlignOut), cudaMemcpyDeviceToHost, s));
        CU(h, cudaStreamSynchronize(s));
        // gather the op runs of the alignments into one packed copy
        std::vector<uint64_t> src(nreq), dst(nreq);
        std::vector<uint32_t> cnt(nreq);
        uint64_t packed = 0;
        for (uint32_t t = 0; t < nreq; t++) {
            src[t] = reqs[t].ops_off;
            dst[t] = packed;
            cnt[t] = outs[t].n_ops;
            packed += outs[t].n_ops;
        }
        std::vector<uint32_t> hostruns(packed);
        if (packed) {
            CUALLOC(h, h->al_pack_off, (uint64_t)nreq * 20 + 64);
            uint64_t* d_src = h->al_pack_off.as<uint64_t>();
            uint64_t* d_dst = d_src + nreq;
            uint32_t* d_cnt = reinterpret_cast<uint32_t*>(d_dst + nreq);
            CUALLOC(h, h->al_packed, packed * 4);
            CU(h, cudaMemcpyAsync(d_src, src.data(), nreq * 8, cudaMemcpyHostToDevice, s));
            CU(h, cudaMemcpyAsync(d_dst, dst.data(), nreq * 8, cudaMemcpyHostToDevice, s));
            CU(h, cudaMemcpyAsync(d_cnt, cnt.data(), nreq * 4, cudaMemcpyHostToDevice, s));
            k_pack_runs<<<std::min<uint32_t>(nreq, 4096), 32, 0, s>>>(h->al_runs.as<uint32_t>(), d_src, d_dst, d_cnt,
                                                                      nreq, h->al_packed.as<uint32_t>());
            CU(h, cudaGetLastError());
            CU(h, cudaMemcpyAsync(hostruns.data(), h->al_packed.p, packed * 4, cudaMemcpyDeviceToHost, s));
            CU(h, cudaStreamSynchronize(s));
        }
        const uint32_t pid = (uint32_t)pools.size();
        pools.push_back(std::move(hostruns));
        for (uint32_t t = 0; t < nreq; t++) {
            AlignResult& r = out[idx[t]];
            const AlignOut& o = outs[t];
            r.status = o.status;
            r.score = o.score;
            r.q_start = o.q_start;
            r.q_end = o.q_end;
            r.s_start = o.s_start;
            r.s_end = o.s_end;
            r.cells = o.cells;
            r.pool = pid;
            r.run_off = dst[t];
            r.n_runs = cnt[t];
        }
    }
    return SABER_OK;
}

static void put_alignment(const AlignResult& r, const RunPools& pools, int status, saber_alignment* o, uint32_t* ops,
                          uint64_t ops_cap, uint64_t& ops_used, bool& overflow) {
    o->status = status;
    o->score = r.score;
    o->q_start = r.q_start;
    o->q_end = r.q_end;
    o->s_start = r.s_start;
    o->s_end = r.s_end;
    o->cells = r.cells;
    o->n_ops = r.n_runs;
    o->ops_offset = (uint32_t)ops_used;
    if (ops_used + r.n_runs > ops_cap) {
        overflow = true;
    } else if (r.n_runs) {
        memcpy(ops + ops_used, pools[r.pool].data() + r.run_off, (size_t)r.n_runs * 4);
    }
    ops_used += r.n_runs;
}

// Engine::traceback (src/search/engine.rs:1328-1393) and traceback_from_end
// (engine.rs:1403-1445) for a batch of regions: each widening round of every
// unresolved region is one align_batch launch.
struct TbState {
    int phase = 0;        // 0 region band, 1 end-anchored, 2 done
    int64_t pad = 16;
    bool has_best = false;
    AlignResult best;
    int64_t d_end = 0, target = 0;
    int64_t slo = 0, shi = 0;  // scope of the end-anchored search
    int status = 0;       // final: 1 exact, 2 inexact, 0 none
};

static int traceback_driver(saber_gpu* h, const saber_traceback_job* jobs, uint64_t n, int32_t band_pad,
                            uint64_t max_dir_bytes, saber_alignment* out, uint32_t* ops, uint64_t ops_cap,
                            saber_traceback_stats* st) {
    const Dataset& ds = h->main;
    const QuerySet& qs = ds.qs;
    if (!ds.qs.has || !ds.has_db) return fail(h, SABER_ERR_STATE, "no database or query set loaded");
    saber_traceback_stats local{};
    std::vector<TbState> S(n);
    const int64_t pad0 = band_pad > 4 ? band_pad : 4;
    for (uint64_t t = 0; t < n; t++) {
        if (jobs[t].query >= qs.nq) return fail(h, SABER_ERR_ARG, "traceback job %llu: bad query", (unsigned long long)t);
        S[t].pad = pad0;
    }
    auto mlen = [&](uint64_t t) { return (int64_t)(qs.offs[jobs[t].query + 1] - qs.offs[jobs[t].query]); };
    std::vector<AlignResult> res;
    RunPools pools;
    for (int round = 0; round < 64; round++) {
        std::vector<AlignHostReq> reqs;
        std::vector<uint64_t> who;
        std::vector<int> kind;  // 0 region band, 1 end-anchored band, 2 end-finding score pass
        std::vector<char> covers;
        for (uint64_t t = 0; t < n; t++) {
            TbState& x = S[t];
            if (x.phase == 2) continue;
            const saber_traceback_job& j = jobs[t];
            const int64_t m = mlen(t), nn = j.win_len;
            AlignHostReq r;
            r.query = j.query;
            r.win_begin = j.win_begin;
            r.win_len = j.win_len;
            r.want_dir = true;
            if (x.phase == 0) {
                // engine.rs:1342-1356
                const bool full = (j.flags & 1u) != 0;
                int64_t lo = full ? -m : (int64_t)j.d_min - x.pad;
                int64_t hi = full ? nn : (int64_t)j.d_max + x.pad;
                bool cov = lo <= -(m - 1) && hi >= nn - 1;
                if (j.flags & 2u) {
                    lo = std::max<int64_t>(lo, j.limit_lo);
                    hi = std::min<int64_t>(hi, j.limit_hi);
                    cov = cov || (lo <= j.limit_lo && hi >= j.limit_hi);
                }
                r.lo = lo;
                r.hi = hi;
                r.stop_at = j.want;
                reqs.push_back(r);
                who.push_back(t);
                kind.push_back(0);
                covers.push_back(cov);
            } else if (x.phase == 3) {
                // engine.rs:1412-1414: score pass over the scope for the end cell
                r.lo = x.slo;
                r.hi = x.shi;
                r.stop_at = INT32_MAX;
                r.want_dir = false;
                reqs.push_back(r);
                who.push_back(t);
                kind.push_back(2);
                covers.push_back(1);
            } else {
                // engine.rs:1422-1427
                int64_t lo = std::max<int64_t>(x.d_end - x.pad, x.slo);
                int64_t hi = std::min<int64_t>(x.d_end + x.pad, x.shi);
                reqs.push_back(AlignHostReq{j.query, j.win_begin, j.win_len, lo, hi, (int32_t)x.target, true});
                who.push_back(t);
                kind.push_back(1);
                covers.push_back(lo <= x.slo && hi >= x.shi);
            }
        }
        if (reqs.empty()) break;
        int rc = align_batch(h, h->scheme, ds, reqs, max_dir_bytes, res, pools);
        if (rc != SABER_OK) return rc;
        local.launches++;
        for (size_t k = 0; k < reqs.size(); k++) {
            const uint64_t t = who[k];
            TbState& x = S[t];
            const saber_traceback_job& j = jobs[t];
            AlignResult& r = res[k];
            const bool cov = covers[k] != 0;
            if (kind[k] != 2) local.tracebacks++;
            // the reference adds the cells of an alignment pass only when it
            // returns an alignment, and those of the score pass always
            if (kind[k] == 2 || r.status == 1) local.banded_cells += r.cells;
            if (kind[k] == 0) {
                if (r.status == 1) {
                    bool done = r.score >= j.want || cov;
                    x.best = r;
                    x.has_best = true;
                    if (done) {
                        x.status = r.score >= j.want ? 1 : 2;
                        x.phase = 2;
                        continue;
                    }
                } else if (r.status == 0) {
                    if (cov) {
                        x.status = 0;
                        x.phase = 2;
                        continue;
                    }
                } else {  // over the cap: traceback_from_end
                    const int64_t m = mlen(t);
                    if (j.flags & 2u) {
                        x.slo = j.limit_lo;
                        x.shi = j.limit_hi;
                    } else {
                        x.slo = -m;
                        x.shi = j.win_len;
                    }
                    x.phase = 3;
                    continue;
                }
                local.band_widenings++;
                x.pad *= 2;
            } else if (kind[k] == 2) {
                if (r.status != 1 || r.score <= 0) {
                    // no end cell: report the best so far, flagged (engine.rs:1384-1387)
                    local.band_capped++;
                    x.status = x.has_best ? 2 : 0;
                    x.phase = 2;
                    continue;
                }
                local.end_anchored++;
                x.target = std::max<int64_t>(r.score, j.want);
                x.d_end = (int64_t)r.s_end - (int64_t)r.q_end;
                x.pad = pad0;
                x.phase = 1;
            } else {
                if (r.status == 1) {
                    if (r.score >= x.target || cov) {
                        x.best = r;
                        x.has_best = true;
                        x.status = r.score >= j.want ? 1 : 2;
                        x.phase = 2;
                        continue;
                    }
                } else if (r.status == 0) {
                    if (cov) {
                        local.band_capped++;
                        x.status = x.has_best ? 2 : 0;
                        x.phase = 2;
                        continue;
                    }
                } else {
                    local.band_capped++;
                    x.status = x.has_best ? 2 : 0;
                    x.phase = 2;
                    continue;
                }
                local.band_widenings++;
                x.pad *= 2;
            }
        }
    }
    uint64_t used = 0;
    bool overflow = false;
    for (uint64_t t = 0; t < n; t++) {
        const TbState& x = S[t];
        if (x.phase != 2) return fail(h, SABER_ERR_DEVICE, "traceback of job %llu did not converge",
                                      (unsigned long long)t);
        if (x.status == 0 || !x.has_best) {
            memset(&out[t], 0, sizeof(out[t]));
            out[t].ops_offset = (uint32_t)used;
            continue;
        }
        put_alignment(x.best, pools, x.status, &out[t], ops, ops_cap, used, overflow);
    }
    if (st) *st = local;
    if (overflow) return fail(h, SABER_ERR_ARG, "ops buffer too small: %llu runs needed", (unsigned long long)used);
    return SABER_OK;
}

}  // namespace saber

using namespace saber;

extern "C" int saber_probe_int_peak_impl(int device, cudaStream_t s, double* dpx, double* i32);
extern "C" int saber_probe_pipe_rates_impl(int device, cudaStream_t s, double* rates);

// ---------------------------------------------------------------------------
// exported C ABI
// ---------------------------------------------------------------------------
#define ENTER(h)                          \
    if (!(h)) return SABER_ERR_ARG;       \
    std::lock_guard<std::mutex> g_((h)->mu); \
    cudaSetDevice((h)->device);           \
    (h)->err.clear()

namespace saber {
double tantan_implied_lambda(const int32_t* m);
int tantan_mask_host(saber_gpu* h, const saber_tantan_params* p, const int32_t* matrix576, const uint8_t* codes,
                     const uint64_t* offsets, uint64_t nseq, uint8_t* mask, float* probs, uint64_t* n_masked,
                     double* lambda_out);
int tantan_mask_db(saber_gpu* h, const saber_tantan_params* p, const int32_t* matrix576, uint64_t* n_masked,
                   double* lambda_out);
int translate6_host(saber_gpu* h, const uint8_t* nt, const uint64_t* nt_offsets, uint64_t nseq,
                    const uint8_t* codon64, uint8_t* out, uint64_t out_cap, uint64_t* out_offsets);
// Pinned host staging for the host engine (engine.cpp).
void* pinned_scratch(saber_gpu* h, int slot, size_t bytes) {
    if (!h || slot < 0 || slot >= 4) return nullptr;
    cudaSetDevice(h->device);
    return h->pin_scratch[slot].reserve(std::max<size_t>(bytes, 64)) == cudaSuccess ? h->pin_scratch[slot].p : nullptr;
}

// The batch's candidate regions for the host engine (engine.cpp): capped per
// query and triaged on the device, kept ones in pinned memory (sink).
int scan_search_regions(saber_gpu* h, const saber_scan_params* p, const uint8_t* q_mask, const int32_t* region_thr,
                        RegionSink& sink, saber_scan_stats* st) {
    ENTER(h);
    uint64_t n = 0;
    return scan_regions(h, p, q_mask, region_thr, nullptr, 0, &n, st, &sink);
}

int triage_grads(saber_gpu* h, const float* model, const float* X, const uint8_t* y, uint32_t n, float pos_weight,
                 float* grads, double* loss);
int triage_train(saber_gpu* h, float* model, const float* X, const uint8_t* y, uint64_t n,
                 const saber_triage_train_cfg* cfg, saber_triage_train_stats* st);
int triage_predict_host(saber_gpu* h, const float* model, const float* X, uint64_t n, float* logits);
int triage_predict(saber_gpu* h, DevBuf& model, DevBuf& wb, const float* d_X, uint64_t n, float* d_logit);
int triage_upload_model(saber_gpu* h, DevBuf& model, DevBuf& wb, const float* host_model);

// Labels of the collected regions (1 = produced a reported hit).
void triage_set_labels(saber_gpu* h, const std::vector<uint64_t>& hit_regions) {
    std::lock_guard<std::mutex> g_(h->mu);
    if (!h->tr_collect) return;
    for (uint64_t i : hit_regions)
        if (i < h->tr_labels.size()) h->tr_labels[i] = 1;
}

// The handle's scoring matrix, for the host engine (engine.cpp).
int scheme_matrix(saber_gpu* h, int32_t* out576) {
    ENTER(h);
    if (!h->scheme.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    std::memcpy(out576, h->scheme.matrix, sizeof(int32_t) * 576);
    return SABER_OK;
}
}  // namespace saber

extern "C" {

int saber_gpu_open(int device, saber_gpu** out) {
    if (!out) return SABER_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return SABER_ERR_CUDA;
    if (device < 0 || device >= ndev) return SABER_ERR_ARG;
    saber_gpu* h = new saber_gpu();
    h->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        delete h;
        return SABER_ERR_CUDA;
    }
    *out = h;
    return SABER_OK;
}

int saber_gpu_close(saber_gpu* h) {
    if (!h) return SABER_ERR_ARG;
    cudaSetDevice(h->device);
    if (h->stream) {
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->stream);
    }
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.second.exec);
    h->graphs.clear();
    delete h;
    return SABER_OK;
}

const char* saber_gpu_last_error(const saber_gpu* h) { return h ? h->err.c_str() : "null handle"; }

void* saber_gpu_stream(saber_gpu* h) { return h ? (void*)h->stream : nullptr; }

int saber_gpu_set_scheme(saber_gpu* h, const int32_t* matrix576, int32_t go, int32_t ge) {
    ENTER(h);
    int rc = set_scheme(h, h->scheme, matrix576, go, ge);
    if (rc == SABER_OK) rc = build_profiles(h, h->scheme, h->main.qs);
    return rc;
}

int saber_gpu_load_db(saber_gpu* h, const uint8_t* residues, uint64_t n_res, const uint64_t* offsets,
                      uint64_t nsub) {
    ENTER(h);
    return load_db(h, h->main, residues, n_res, offsets, nsub);
}

int saber_gpu_load_queries(saber_gpu* h, const uint8_t* codes, const uint64_t* offsets, const int8_t* bias,
                           uint32_t nq) {
    ENTER(h);
    return load_queries(h, h->scheme, h->main.qs, codes, offsets, bias, nq);
}

int saber_gpu_score_band_jobs_dev(saber_gpu* h, const saber_band_job* d_jobs, uint64_t njobs, int32_t* d_scores,
                                  saber_score_stats* stats) {
    ENTER(h);
    if (njobs && (!d_jobs || !d_scores)) return fail(h, SABER_ERR_ARG, "null job or score buffer");
    return score_pipeline(h, h->scheme, h->main, d_jobs, njobs, d_scores, stats);
}

int saber_gpu_score_band_jobs(saber_gpu* h, const saber_band_job* jobs, uint64_t njobs, int32_t* scores,
                              saber_score_stats* stats) {
    ENTER(h);
    if (njobs && (!jobs || !scores)) return fail(h, SABER_ERR_ARG, "null job or score buffer");
    if (njobs == 0) {
        if (stats) *stats = saber_score_stats{};
        return SABER_OK;
    }
    int rc;
    if (h->use_graphs) {
        // the widest clipped band sizes the graph's scratch and the cell total
        // sets the automatic long-job threshold: one reduction on the device
        // after the copy, 16 bytes read back
        const QuerySet& qs = h->main.qs;
        const uint64_t npad = pow2_at_least(njobs, 1 << 12);
        CUALLOC(h, h->jobs_dev, npad * sizeof(saber_band_job));
        CUALLOC(h, h->scores_dev, npad * 4);
        CUALLOC(h, h->g_wmax, 16);
        CU(h, cudaMemcpyAsync(h->jobs_dev.p, jobs, njobs * sizeof(saber_band_job), cudaMemcpyHostToDevice, h->stream));
        CU(h, cudaMemsetAsync(h->g_wmax.p, 0, 16, h->stream));
        if (qs.has)
            k_job_wmax<<<nblocks(njobs, 256, h->sm_count * 8), 256, 0, h->stream>>>(
                h->jobs_dev.as<saber_band_job>(), njobs, qs.offsets.as<uint64_t>(), qs.nq,
                h->g_wmax.as<unsigned long long>());
        CU(h, cudaGetLastError());
        unsigned long long r[2] = {0, 0};
        CU(h, cudaMemcpyAsync(r, h->g_wmax.p, 16, cudaMemcpyDeviceToHost, h->stream));
        CU(h, cudaStreamSynchronize(h->stream));
        rc = score_pipeline_graph(h, h->scheme, h->main, njobs, r[0], r[1], stats);
    } else {
        CUALLOC(h, h->jobs_dev, njobs * sizeof(saber_band_job));
        CUALLOC(h, h->scores_dev, njobs * 4);
        CU(h, cudaMemcpyAsync(h->jobs_dev.p, jobs, njobs * sizeof(saber_band_job), cudaMemcpyHostToDevice,
                              h->stream));
        rc = score_pipeline(h, h->scheme, h->main, h->jobs_dev.as<saber_band_job>(), njobs,
                            h->scores_dev.as<int32_t>(), stats);
    }
    if (rc != SABER_OK) return rc;
    CU(h, cudaMemcpyAsync(scores, h->scores_dev.p, njobs * 4, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    return SABER_OK;
}

int saber_gpu_score_banded_many(saber_gpu* h, const uint8_t* query, uint32_t m, const int8_t* bias,
                                const uint8_t* subjects, const uint64_t* sub_offsets, const int64_t* band_lo,
                                const int64_t* band_hi, uint64_t njobs, int32_t* scores) {
    ENTER(h);
    if (!h->scheme.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    if (njobs && (!band_lo || !band_hi || !scores)) return fail(h, SABER_ERR_ARG, "null argument");
    return one_query_jobs(h, h->scheme, query, m, bias, subjects, sub_offsets, band_lo, band_hi, njobs, false,
                          scores);
}

int saber_gpu_score_windows(saber_gpu* h, const uint8_t* query, uint32_t m, const int8_t* bias,
                            const uint8_t* windows, const uint64_t* win_offsets, uint32_t nwin,
                            const int32_t* matrix576, int32_t go, int32_t ge, int32_t* scores) {
    ENTER(h);
    if (nwin && !scores) return fail(h, SABER_ERR_ARG, "null argument");
    int rc = set_scheme(h, h->eph_scheme, matrix576, go, ge);
    if (rc != SABER_OK) return rc;
    return one_query_jobs(h, h->eph_scheme, query, m, bias, windows, win_offsets, nullptr, nullptr, nwin, true,
                          scores);
}

int saber_gpu_probe_int_peak(saber_gpu* h, double* dpx, double* i32) {
    ENTER(h);
    int rc = saber_probe_int_peak_impl(h->device, h->stream, dpx, i32);
    if (rc != SABER_OK) return fail(h, rc, "integer peak probe failed");
    return SABER_OK;
}

int saber_gpu_probe_pipe_rates(saber_gpu* h, double rates[5]) {
    ENTER(h);
    if (!rates) return fail(h, SABER_ERR_ARG, "null argument");
    int rc = saber_probe_pipe_rates_impl(h->device, h->stream, rates);
    if (rc != SABER_OK) return fail(h, rc, "pipe rate probe failed");
    return SABER_OK;
}

int saber_gpu_score_band_jobs_noalloc(saber_gpu* h, const saber_band_job* d_jobs, uint64_t njobs,
                                      int32_t max_band_width, int32_t* d_scores) {
    ENTER(h);
    if (!h->scheme.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    if (!h->main.has_db) return fail(h, SABER_ERR_STATE, "no database loaded");
    if (!h->main.qs.has) return fail(h, SABER_ERR_STATE, "no query set loaded");
    if (njobs && (!d_jobs || !d_scores)) return fail(h, SABER_ERR_ARG, "null job or score buffer");
    const QuerySet& qs = h->main.qs;
    NoAllocArgs a;
    a.res = h->main.res.as<uint8_t>();
    a.prof = qs.prof.as<int16_t>();
    a.prof_off = qs.prof_off.as<uint64_t>();
    a.prof_mpad = qs.prof_mpad.as<uint32_t>();
    a.qoffs = qs.offsets.as<uint64_t>();
    a.nq = qs.nq;
    a.n_res = h->main.n_res;
    a.jobs = d_jobs;
    a.njobs = njobs;
    a.max_band_width = max_band_width;
    a.go = h->scheme.go;
    a.ge = h->scheme.ge;
    a.scores = d_scores;
    const char* msg = "";
    uint32_t bad_job = UINT32_MAX;
    int rc = noalloc_score_band_jobs(h->device, h->stream, a, &msg, &bad_job);
    if (rc != SABER_OK) {
        if (bad_job != UINT32_MAX) return fail(h, rc, "%s (job %u)", msg, bad_job);
        return fail(h, rc, "%s", msg);
    }
    return SABER_OK;
}

int saber_gpu_set_strip_rows(saber_gpu* h, int32_t strip_rows) {
    ENTER(h);
    if (strip_rows != 8 && strip_rows != 16) return fail(h, SABER_ERR_ARG, "strip_rows must be 8 or 16");
    h->strip_rows = strip_rows;
    return SABER_OK;
}

int32_t saber_gpu_get_strip_rows(saber_gpu* h) { return h ? h->strip_rows : 0; }

int saber_gpu_triage_grads(saber_gpu* h, const float* model, const float* rows, const uint8_t* labels, uint32_t n,
                           float pos_weight, float* grads, double* loss) {
    ENTER(h);
    if (!model || !grads || (n && (!rows || !labels))) return fail(h, SABER_ERR_ARG, "null argument");
    return triage_grads(h, model, rows, labels, n, pos_weight, grads, loss);
}

int saber_gpu_triage_train(saber_gpu* h, float* model, const float* rows, const uint8_t* labels, uint64_t n,
                           const saber_triage_train_cfg* cfg, saber_triage_train_stats* stats) {
    ENTER(h);
    if (!model || !cfg || (n && (!rows || !labels))) return fail(h, SABER_ERR_ARG, "null argument");
    return triage_train(h, model, rows, labels, n, cfg, stats);
}

int saber_gpu_triage_predict(saber_gpu* h, const float* model, const float* rows, uint64_t n, float* logits) {
    ENTER(h);
    if (!model || (n && (!rows || !logits))) return fail(h, SABER_ERR_ARG, "null argument");
    return triage_predict_host(h, model, rows, n, logits);
}

int saber_gpu_set_triage(saber_gpu* h, const float* model, float threshold) {
    ENTER(h);
    if (!model) {
        h->tr_on = false;
        return SABER_OK;
    }
    int rc = triage_upload_model(h, h->tr_model, h->tr_wb, model);
    if (rc != SABER_OK) return rc;
    CU(h, cudaStreamSynchronize(h->stream));
    h->tr_threshold = threshold;
    h->tr_on = true;
    return SABER_OK;
}

int saber_gpu_collect_regions(saber_gpu* h, int32_t collect) {
    ENTER(h);
    h->tr_collect = collect != 0;
    h->tr_rows.clear();
    h->tr_labels.clear();
    h->tr_logits.clear();
    return SABER_OK;
}

int saber_gpu_collected_regions(saber_gpu* h, float* rows, uint8_t* labels, float* logits, uint64_t cap,
                                uint64_t* n) {
    ENTER(h);
    const uint64_t m = h->tr_labels.size();
    if (n) *n = m;
    if (m > cap) return fail(h, SABER_ERR_CAP, "%llu collected regions", (unsigned long long)m);
    if (rows) std::memcpy(rows, h->tr_rows.data(), m * SABER_TRIAGE_ROW_FLOATS * 4);
    if (labels) std::memcpy(labels, h->tr_labels.data(), m);
    if (logits) std::memcpy(logits, h->tr_logits.data(), m * 4);
    return SABER_OK;
}

int saber_gpu_set_graphs(saber_gpu* h, int32_t on) {
    ENTER(h);
    h->use_graphs = on != 0;
    return SABER_OK;
}

int32_t saber_gpu_get_graphs(saber_gpu* h) { return h ? (h->use_graphs ? 1 : 0) : 0; }

uint64_t saber_gpu_graph_captures(saber_gpu* h) { return h ? h->graph_captures : 0; }

int saber_gpu_set_pair_steps(saber_gpu* h, uint32_t steps) {
    ENTER(h);
    h->pair_steps = steps;
    return SABER_OK;
}

uint32_t saber_gpu_get_pair_steps(saber_gpu* h) { return h ? h->pair_steps : 0u; }

int saber_gpu_set_long_steps(saber_gpu* h, uint32_t steps) {
    ENTER(h);
    h->long_steps = steps;
    return SABER_OK;
}

uint32_t saber_gpu_get_long_steps(saber_gpu* h) { return h ? h->long_steps : 0u; }

int saber_gpu_set_scan_table_bytes(saber_gpu* h, uint64_t bytes) {
    ENTER(h);
    h->scan_table_bytes = bytes;
    return SABER_OK;
}

uint64_t saber_gpu_get_scan_table_bytes(saber_gpu* h) { return h ? h->scan_table_bytes : 0u; }

int saber_gpu_banded_align(saber_gpu* h, const saber_align_job* jobs, uint64_t njobs, uint64_t max_dir_bytes,
                           saber_alignment* out, uint32_t* ops, uint64_t ops_cap) {
    ENTER(h);
    if (njobs && (!jobs || !out)) return fail(h, SABER_ERR_ARG, "null argument");
    std::vector<AlignHostReq> reqs(njobs);
    for (uint64_t t = 0; t < njobs; t++)
        reqs[t] = AlignHostReq{jobs[t].query, jobs[t].win_begin, jobs[t].win_len, jobs[t].band_lo, jobs[t].band_hi,
                               jobs[t].stop_at, true};
    std::vector<AlignResult> res;
    RunPools pools;
    int rc = align_batch(h, h->scheme, h->main, reqs, max_dir_bytes, res, pools);
    if (rc != SABER_OK) return rc;
    uint64_t used = 0;
    bool overflow = false;
    for (uint64_t t = 0; t < njobs; t++)
        put_alignment(res[t], pools, res[t].status, &out[t], ops, ops_cap, used, overflow);
    if (overflow) return fail(h, SABER_ERR_ARG, "ops buffer too small: %llu runs needed", (unsigned long long)used);
    return SABER_OK;
}

int saber_gpu_banded_align_one(saber_gpu* h, const uint8_t* query, uint32_t m, const int8_t* bias,
                               const uint8_t* subject, uint32_t n, int64_t band_lo, int64_t band_hi,
                               uint64_t max_dir_bytes, int32_t stop_at, saber_alignment* out, uint32_t* ops,
                               uint64_t ops_cap) {
    ENTER(h);
    if (!out) return fail(h, SABER_ERR_ARG, "null argument");
    if (!h->scheme.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    memset(out, 0, sizeof(*out));
    if (m == 0 || n == 0 || band_hi < band_lo) return SABER_OK;
    Dataset& ds = h->eph;
    uint64_t offs[2] = {0, n};
    int rc = load_db(h, ds, subject, n, offs, 1);
    if (rc != SABER_OK) return rc;
    uint64_t qoff[2] = {0, m};
    rc = load_queries(h, h->scheme, ds.qs, query, qoff, bias, 1);
    if (rc != SABER_OK) return rc;
    int64_t lo = std::max<int64_t>(band_lo, -(int64_t)m - 1), hi = std::min<int64_t>(band_hi, (int64_t)n + 1);
    if (hi < lo) return SABER_OK;
    std::vector<AlignHostReq> reqs(1, AlignHostReq{0, 0, n, lo, hi, stop_at, true});
    std::vector<AlignResult> res;
    RunPools pools;
    rc = align_batch(h, h->scheme, ds, reqs, max_dir_bytes, res, pools);
    if (rc != SABER_OK) return rc;
    uint64_t used = 0;
    bool overflow = false;
    put_alignment(res[0], pools, res[0].status, out, ops, ops_cap, used, overflow);
    if (overflow) return fail(h, SABER_ERR_ARG, "ops buffer too small: %llu runs needed", (unsigned long long)used);
    return SABER_OK;
}

int saber_gpu_traceback(saber_gpu* h, const saber_traceback_job* jobs, uint64_t njobs, int32_t band_pad,
                        uint64_t max_dir_bytes, saber_alignment* out, uint32_t* ops, uint64_t ops_cap,
                        saber_traceback_stats* stats) {
    ENTER(h);
    if (njobs && (!jobs || !out)) return fail(h, SABER_ERR_ARG, "null argument");
    if (!h->scheme.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    return traceback_driver(h, jobs, njobs, band_pad, max_dir_bytes, out, ops, ops_cap, stats);
}

int saber_gpu_load_db_mask(saber_gpu* h, const uint8_t* mask, uint64_t n_residues) {
    ENTER(h);
    h->sc_key = 0;  // the scan's database state depends on the mask
    if (!mask) {
        h->has_db_mask = false;
        return SABER_OK;
    }
    if (!h->main.has_db || n_residues != h->main.n_res)
        return fail(h, SABER_ERR_ARG, "mask length must equal the loaded database's residues");
    CUALLOC(h, h->db_mask, n_residues + 64);
    if (n_residues) CU(h, cudaMemcpyAsync(h->db_mask.p, mask, n_residues, cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    h->has_db_mask = true;
    return SABER_OK;
}

double saber_tantan_implied_lambda(const int32_t* matrix576) {
    return matrix576 ? saber::tantan_implied_lambda(matrix576) : NAN;
}

int saber_gpu_tantan_mask(saber_gpu* h, const saber_tantan_params* params, const int32_t* matrix576,
                          const uint8_t* codes, const uint64_t* offsets, uint64_t nseq, uint8_t* mask, float* probs,
                          uint64_t* n_masked, double* lambda_out) {
    ENTER(h);
    return saber::tantan_mask_host(h, params, matrix576, codes, offsets, nseq, mask, probs, n_masked, lambda_out);
}

int saber_gpu_tantan_mask_db(saber_gpu* h, const saber_tantan_params* params, const int32_t* matrix576,
                             uint64_t* n_masked, double* lambda_out) {
    ENTER(h);
    return saber::tantan_mask_db(h, params, matrix576, n_masked, lambda_out);
}

int saber_gpu_translate6(saber_gpu* h, const uint8_t* nt, const uint64_t* nt_offsets, uint64_t nseq,
                         const uint8_t* codon64, uint8_t* out, uint64_t out_cap, uint64_t* out_offsets) {
    ENTER(h);
    return saber::translate6_host(h, nt, nt_offsets, nseq, codon64, out, out_cap, out_offsets);
}

int saber_gpu_load_db_mask_runs(saber_gpu* h, const uint64_t* runs, uint64_t nruns) {
    ENTER(h);
    h->sc_key = 0;  // the scan's database state depends on the mask
    if (!h->main.has_db) return fail(h, SABER_ERR_STATE, "no database loaded");
    if (nruns && !runs) return fail(h, SABER_ERR_ARG, "null runs");
    const uint64_t n = h->main.n_res;
    for (uint64_t r = 0; r < nruns; r++)
        if (runs[2 * r] > runs[2 * r + 1] || runs[2 * r + 1] > n)
            return fail(h, SABER_ERR_ARG, "mask run %llu out of the database", (unsigned long long)r);
    CUALLOC(h, h->db_mask, n + 64);
    CU(h, cudaMemsetAsync(h->db_mask.p, 0, n + 64, h->stream));
    if (nruns) {
        CUALLOC(h, h->mask_runs, nruns * 2 * sizeof(uint64_t));
        CU(h, cudaMemcpyAsync(h->mask_runs.p, runs, nruns * 2 * sizeof(uint64_t), cudaMemcpyHostToDevice,
                              h->stream));
        k_fill_runs<<<nblocks(nruns * 32, 256, h->sm_count * 16), 256, 0, h->stream>>>(
            (const uint64_t*)h->mask_runs.p, nruns, h->db_mask.as<uint8_t>());
        CU(h, cudaGetLastError());
    }
    CU(h, cudaStreamSynchronize(h->stream));
    h->has_db_mask = true;
    return SABER_OK;
}

int saber_gpu_scan(saber_gpu* h, const saber_scan_params* params, const uint8_t* q_mask, const int32_t* region_thr,
                   saber_region* out, uint64_t out_cap, uint64_t* n_out, saber_scan_stats* stats) {
    // (the batch engine, engine.cpp, takes every region through scan_regions_all)
    ENTER(h);
    if (!params || (out_cap && !out)) return fail(h, SABER_ERR_ARG, "null argument");
    return scan_regions(h, params, q_mask, region_thr, out, out_cap, n_out, stats);
}

uint64_t saber_band_cells(uint64_t m, uint64_t n, int64_t band_lo, int64_t band_hi) {
    int64_t lo = band_lo, hi = band_hi;
    if (clip_band((int64_t)m, (int64_t)n, lo, hi) == 0) return 0;
    return band_cells((int64_t)m, (int64_t)n, lo, hi);
}

}  // extern "C"
