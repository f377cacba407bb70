// Shared definitions of the banded scoring kernels (device + host helpers).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "saber_gpu.h"

namespace saber {

// Rows per strip of the packed int16 kernel (one strip = R query rows swept
// along the subject window; see band_kernels.cu): 8 or 16, chosen per handle
// (tuning); query profiles are padded to the largest.
constexpr int kStripRows = 16;
constexpr int kStripRowsMin = 8;
// Query profiles are padded to a multiple of the paired kernel's super-strip
// (2 x 16 rows).
constexpr int kProfPad = 32;
// Default pairing threshold: a job whose R-row sweep takes more than this
// many column steps (strips x (width + R - 1)) is swept as paired strips.
constexpr uint32_t kPairStepsDefault = 2048;
constexpr uint32_t kLongStepsNever = 0xFFFFFFFFu;
constexpr uint32_t kLongStepsAuto = 0xFFFFFFFEu;  // from the batch's cells per lane, at least kLongStepsSmall
constexpr uint32_t kLongStepsSmall = 2048;
constexpr uint32_t kLongStepsDefault = kLongStepsAuto;
// Residue code used for positions outside a window or a query: its profile
// entries are kSent, so such cells never beat a real cell (banded.rs:123-131
// excludes them; the kernels compute them harmlessly instead of branching).
constexpr int kSentCode = 24;
constexpr int kProfRows = 25;  // 24 codes + sentinel
// int16 domain of the packed kernel.
constexpr int kNeg16 = -16000;   // unreachable (banded_simd.rs:336 uses -31000 with saturation)
constexpr int kSent16 = -16000;  // substitution score of sentinel cells
// A job whose int16 best reaches this value is rescored in int32: below it,
// no in-band H + S + bias can have left the int16 range (|S + bias| <= 767).
constexpr int kLimit16 = 32000;

// Clip a band to an m x n rectangle (banded.rs:45-47) and return its width
// (banded.rs:41-43); 0 means an empty job (score 0).
__host__ __device__ inline int64_t clip_band(int64_t m, int64_t n, int64_t& lo, int64_t& hi) {
    if (m <= 0 || n <= 0 || hi < lo) return 0;
    if (lo < -(m - 1)) lo = -(m - 1);
    if (hi > n - 1) hi = n - 1;
    int64_t w = hi - lo + 1;
    return w > 0 ? w : 0;
}

// Number of in-band cells of a clipped band, counted as the reference counts
// them (sum over rows of the row_range span, banded.rs:123-131,208):
// sum over diagonals d in [lo, hi] of |{i : 0 <= i < m, 0 <= i + d < n}|.
__host__ __device__ inline uint64_t band_cells(int64_t m, int64_t n, int64_t lo, int64_t hi) {
    if (hi < lo) return 0;
    // term(d) = min(m, n - d) - max(0, -d), positive on the clipped range.
    auto sum_range = [](int64_t a, int64_t b) -> int64_t {  // sum of integers a..b
        return b < a ? 0 : (a + b) * (b - a + 1) / 2;
    };
    int64_t total = 0;
    // sum of min(m, n - d): equals m for d <= n - m, n - d above.
    int64_t split = n - m;
    int64_t a1 = lo, b1 = hi < split ? hi : split;
    if (b1 >= a1) total += m * (b1 - a1 + 1);
    int64_t a2 = lo > split + 1 ? lo : split + 1, b2 = hi;
    if (b2 >= a2) total += n * (b2 - a2 + 1) - sum_range(a2, b2);
    // minus sum of max(0, -d) for d < 0: sum of -d over d in [lo, min(hi, -1)].
    int64_t b3 = hi < -1 ? hi : -1;
    if (b3 >= lo) total -= -sum_range(lo, b3);
    return (uint64_t)total;
}

// Arguments of the scoring kernels (launch wrappers in band_kernels.cu).
struct FastArgs {
    const uint8_t* res;
    const int16_t* prof;
    const int8_t* prof8;    // int8 copy of the profile (every entry fits), or null: the int16 kernel
    const uint64_t* prof_off;
    const uint32_t* prof_mpad;
    const uint64_t* qoffs;
    const saber_band_job* jobs;
    const uint32_t* order;  // sorted job indices of this launch's class
    const uint32_t* n_ptr;  // device count of those jobs
    const uint32_t* np_ptr; // device count of the paired jobs among them (at the end), or null
    const uint32_t* order_skip;  // device count of leading entries of order to skip, or null
    uint32_t* wt_counter;
    uint2* bufs;
    uint32_t buf_stride;
    int go, ge;
    int32_t* scores;
    uint32_t* rescue;
    uint32_t* rescue_count;
    int strip_rows;  // 8 or 16
};
struct GenericArgs {
    const uint8_t* res;
    const int16_t* prof;
    const uint64_t* prof_off;
    const uint32_t* prof_mpad;
    const uint64_t* qoffs;
    const saber_band_job* jobs;
    const uint32_t* list;
    const uint32_t* list_count;
    int32_t* slabs;
    uint32_t slab_stride;
    int go, ge;
    int32_t* scores;
};
// Allocation-free entry point (noalloc.cu).
constexpr int32_t kNoAllocMaxBandWidth = 4096;
struct NoAllocArgs {
    const uint8_t* res;
    const int16_t* prof;
    const uint64_t* prof_off;
    const uint32_t* prof_mpad;
    const uint64_t* qoffs;
    uint32_t nq;
    uint64_t n_res;
    const saber_band_job* jobs;
    uint64_t njobs;
    int32_t max_band_width;
    int go, ge;
    int32_t* scores;
};
int noalloc_score_band_jobs(int device, cudaStream_t s, const NoAllocArgs& a, const char** msg, uint32_t* bad_job);

int band_fast_blocks_per_sm(int strip_rows, bool prof8);
cudaError_t launch_band_fast(unsigned grid, cudaStream_t s, const FastArgs& a);
cudaError_t launch_band_generic(unsigned grid, unsigned block, cudaStream_t s, const GenericArgs& a);

}  // namespace saber
