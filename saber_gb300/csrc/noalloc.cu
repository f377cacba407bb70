// Allocation-free banded scoring (saber_gpu_score_band_jobs_noalloc).
//
// Who needs it: callers that must not allocate GPU memory while they score —
// a host process whose device memory is owned by another allocator or
// reserved up front in a fixed budget, or a latency-bound service path where
// a cudaMalloc (an implicit device synchronisation) is not acceptable.  The
// regular entry points grow their work buffers with cudaMalloc on demand;
// this one uses only the fixed scratch array below, the caller's input and
// output buffers, and the database and query set already resident in the
// handle.
//
// The call runs on the handle's stream and returns when the scores are
// written: it reads the control block back to the host and waits for the
// stream.  The handle's stream is not ordered after the caller's streams, so
// the caller finishes writing the jobs before the call.
//
// The scratch is a file-scope __device__ array, so every GPU that loads this
// library holds kNoAllocScratchBytes for the life of the process.  Its
// device address is looked up once per device (cudaGetSymbolAddress with that
// device current) on the first call on that device; make that first call
// before any stream capture.  All calls share the array and it keeps the
// previous call's contents: the control block is cleared at the start of
// every call, and calls that overlap on the GPU (several streams or handles
// at once) race on it.
//
// Threads per call: each thread keeps four int32 rows of max_band_width + 1
// entries (interleaved across threads, so a warp's row accesses coalesce), so
// (16 MiB - 256 B) / (16 (max_band_width + 1)) threads fit: about 4,000 at a
// width of 257, 255 at 4096.  Pick the smallest max_band_width that covers
// the jobs.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "band_common.cuh"
#include "saber_gpu.h"

namespace saber {

// 16 MiB: a 256-byte control block (error word, offending job) followed by
// per-thread int32 H/F rows of the banded recurrence.
constexpr size_t kNoAllocScratchBytes = 16u << 20;
constexpr size_t kNoAllocControlBytes = 256;
constexpr unsigned kNoAllocBlock = 32;  // one warp per block: the few threads a wide band allows spread over SMs
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host-side device addresses of g_noalloc_scratch, one per device ordinal.
constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kMaxDevices];

// Scalar banded recurrence of banded.rs:134-224 in int32, one job per thread,
// rows in the static scratch: row r entry k of thread t at
// rows[(r * (max_w + 1) + k) * nthreads + t].  ctl[0] = error flags, ctl[1] =
// index of an offending job.
__global__ void __launch_bounds__(kNoAllocBlock) k_band_noalloc(
    const uint8_t* __restrict__ res, const int16_t* __restrict__ prof, const uint64_t* __restrict__ prof_off,
    const uint32_t* __restrict__ prof_mpad, const uint64_t* __restrict__ qoffs, uint32_t nq, uint64_t n_res,
    const saber_band_job* __restrict__ jobs, uint32_t njobs, int32_t max_w, unsigned char* __restrict__ scratch,
    int go, int ge, int32_t* __restrict__ scores) {
    const int NEG = INT32_MIN / 4;
    unsigned int* ctl = reinterpret_cast<unsigned int*>(scratch);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nth = (size_t)gridDim.x * blockDim.x;
    const size_t stride = (size_t)max_w + 1;
    int32_t* rows = reinterpret_cast<int32_t*>(scratch + kNoAllocControlBytes) + tid;
    int32_t* hp = rows;
    int32_t* fp = rows + stride * nth;
    int32_t* hc = rows + 2 * stride * nth;
    int32_t* fc = rows + 3 * stride * nth;
#define AT(row, k) (row)[(size_t)(k) * nth]
    for (uint32_t t = tid; t < njobs; t += (uint32_t)nth) {
        const saber_band_job jj = jobs[t];
        if (jj.query >= nq || jj.win_begin + (uint64_t)jj.win_len > n_res) {
            atomicOr(&ctl[0], 2u);
            atomicExch(&ctl[1], t);
            continue;
        }
        const uint32_t q = jj.query;
        const int64_t m = (int64_t)(qoffs[q + 1] - qoffs[q]);
        const int64_t nn = jj.win_len;
        int64_t lo = jj.band_lo, hi = jj.band_hi;
        const int64_t w = clip_band(m, nn, lo, hi);
        if (w == 0) {
            scores[t] = 0;
            continue;
        }
        if (w > max_w) {
            atomicOr(&ctl[0], 1u);
            atomicExch(&ctl[1], t);
            continue;
        }
        const int16_t* qprof = prof + prof_off[q];
        const int64_t mpad = prof_mpad[q];
        const uint8_t* s = res + jj.win_begin;
        int32_t* a_hp = hp;
        int32_t* a_fp = fp;
        int32_t* a_hc = hc;
        int32_t* a_fc = fc;
        for (int64_t k = 0; k <= w; k++) {
            AT(a_hp, k) = NEG;
            AT(a_fp, k) = NEG;
            AT(a_hc, k) = NEG;
            AT(a_fc, k) = NEG;
        }
        int32_t best = 0;
        for (int64_t i = 0; i < m; i++) {
            int64_t kmin = -(i + lo);
            if (kmin < 0) kmin = 0;
            int64_t kmax = nn - 1 - i - lo;
            if (kmax > w - 1) kmax = w - 1;
            if (kmin > kmax) {
                for (int64_t k = 0; k < w; k++) {
                    AT(a_hc, k) = NEG;
                    AT(a_fc, k) = NEG;
                }
            } else {
                int32_t e = NEG, h_left = NEG;
                const int64_t base = i + lo;
                for (int64_t k = kmin; k <= kmax; k++) {
                    const int64_t j = base + k;
                    int32_t ecand = max(h_left - go, e - ge);
                    e = k > kmin ? ecand : NEG;
                    int32_t f = i >= 1 ? max(AT(a_hp, k + 1) - go, AT(a_fp, k + 1) - ge) : NEG;
                    int32_t hd = (i >= 1 && j >= 1) ? AT(a_hp, k) : 0;
                    int32_t h = max(max(max(hd + ((int32_t)qprof[(size_t)s[j] * mpad + i] - go), e), f), 0);
                    AT(a_hc, k) = h;
                    AT(a_fc, k) = f;
                    h_left = h;
                    best = max(best, h);
                }
                for (int64_t k = 0; k < kmin; k++) {
                    AT(a_hc, k) = NEG;
                    AT(a_fc, k) = NEG;
                }
                for (int64_t k = kmax + 1; k < w; k++) {
                    AT(a_hc, k) = NEG;
                    AT(a_fc, k) = NEG;
                }
            }
            int32_t* tmp = a_hp;
            a_hp = a_hc;
            a_hc = tmp;
            tmp = a_fp;
            a_fp = a_fc;
            a_fc = tmp;
        }
        scores[t] = best;
    }
#undef AT
}

// Set-up (once per device, that device current) and launch.  Returns a
// SABER_* status; *msg receives a static description on error and *bad_job
// the index of an offending job (or UINT32_MAX).
int noalloc_score_band_jobs(int device, cudaStream_t s, const NoAllocArgs& a, const char** msg, uint32_t* bad_job) {
    *msg = "";
    *bad_job = UINT32_MAX;
    if (device < 0 || device >= kMaxDevices) {
        *msg = "device ordinal out of range for the allocation-free entry point";
        return SABER_ERR_ARG;
    }
    if (a.max_band_width < 1 || a.max_band_width > kNoAllocMaxBandWidth) {
        *msg = "max_band_width must lie in [1, 4096] for the allocation-free entry point";
        return SABER_ERR_ARG;
    }
    if (a.njobs >= (1ull << 31)) {
        *msg = "too many jobs in one call";
        return SABER_ERR_ARG;
    }
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> g(g_noalloc_mu);
        if (!g_noalloc_ptr[device]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                *msg = "cudaGetSymbolAddress of the static scratch array failed";
                return SABER_ERR_CUDA;
            }
            g_noalloc_ptr[device] = p;
        }
        base = g_noalloc_ptr[device];
    }
    if (a.njobs == 0) return SABER_OK;
    // threads whose rows fit in the scratch after the control block
    const size_t per_thread = 4 * ((size_t)a.max_band_width + 1) * sizeof(int32_t);
    size_t threads = (kNoAllocScratchBytes - kNoAllocControlBytes) / per_thread;
    const size_t want = ((size_t)a.njobs + kNoAllocBlock - 1) / kNoAllocBlock * kNoAllocBlock;
    if (threads > want) threads = want;
    if (threads > 65536) threads = 65536;
    const unsigned grid = (unsigned)(threads / kNoAllocBlock);
    if (grid == 0) {
        *msg = "static scratch too small for one block";
        return SABER_ERR_ARG;
    }
    if (cudaMemsetAsync(base, 0, kNoAllocControlBytes, s) != cudaSuccess) {
        *msg = "clearing the control block failed";
        return SABER_ERR_CUDA;
    }
    k_band_noalloc<<<grid, kNoAllocBlock, 0, s>>>(a.res, a.prof, a.prof_off, a.prof_mpad, a.qoffs, a.nq, a.n_res,
                                                  a.jobs, (uint32_t)a.njobs, a.max_band_width,
                                                  static_cast<unsigned char*>(base), a.go, a.ge, a.scores);
    if (cudaGetLastError() != cudaSuccess) {
        *msg = "kernel launch failed";
        return SABER_ERR_CUDA;
    }
    unsigned int ctl[2] = {0, 0};
    if (cudaMemcpyAsync(ctl, base, sizeof(ctl), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "reading the control block failed";
        return SABER_ERR_CUDA;
    }
    if (ctl[0] & 2u) {
        *msg = "a job references a query or window outside the loaded data";
        *bad_job = ctl[1];
        return SABER_ERR_ARG;
    }
    if (ctl[0] & 1u) {
        *msg = "a job's clipped band is wider than max_band_width";
        *bad_job = ctl[1];
        return SABER_ERR_ARG;
    }
    return SABER_OK;
}

}  // namespace saber
