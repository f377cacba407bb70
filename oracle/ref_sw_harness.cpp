// Host harness that compiles the reference's CUDA SW kernel source
// (src/gpu/kernels/sw.cu) as plain C++ and exposes it through a C function,
// so the oracle can be checked against the reference's own compiled code.
// Test infrastructure only.  The CUDA built-ins the kernel uses are given
// host definitions here; the kernel runs one thread per block, so its
// cooperative shared-memory fill completes before use.
#include <cstdint>
#include <vector>

namespace refsw {
struct dim3_t { unsigned x, y, z; };
static dim3_t threadIdx, blockIdx, blockDim;
static inline void __syncthreads() {}
#define __global__
#define __shared__ static
#define __restrict__ __restrict
#include REF_SW_CU
#undef __global__
#undef __shared__
#undef __restrict__
}  // namespace refsw

extern "C" int ref_sw_score_windows(const uint8_t* query, int32_t qlen, const int8_t* bias,
                                    const uint8_t* subjects, const uint32_t* offsets,
                                    int32_t nsub, const int32_t* matrix, int32_t go,
                                    int32_t ge, int32_t* scores) {
    std::vector<int8_t> zeros;
    if (!bias) { zeros.assign(qlen > 0 ? qlen : 1, 0); bias = zeros.data(); }
    std::vector<int32_t> H((size_t)(qlen > 0 ? qlen : 1) * (nsub > 0 ? nsub : 1));
    std::vector<int32_t> E(H.size());
    const uint8_t one_x = 22;
    const uint8_t* subj = subjects ? subjects : &one_x;
    refsw::blockDim = {1, 1, 1};
    for (int b = 0; b < nsub; b++) {
        refsw::blockIdx = {(unsigned)b, 0, 0};
        refsw::threadIdx = {0, 0, 0};
        refsw::saber_sw_score_i32(query, qlen, bias, subj, offsets, nsub, matrix, go, ge,
                                  H.data(), E.data(), scores);
    }
    return 0;
}
