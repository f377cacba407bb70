// Integer-pipe throughput probe (roofline denominator of the scoring kernels):
// independent chains of the DPX packed-int16 instructions the banded kernel
// uses, and of plain int32 max, timed with CUDA events at full occupancy.
#include <cuda_runtime.h>

#include <cstdint>

#include "saber_gpu.h"

namespace saber {

constexpr int kChains = 8;
constexpr int kProbeIters = 4096;

// Each iteration issues kChains x 2 DPX instructions (viaddmax + vimax3).
__global__ void __launch_bounds__(256) k_probe_dpx(uint32_t seed, uint32_t* out) {
    uint32_t a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = seed * (threadIdx.x + 3 * c + 1);
    const uint32_t b = seed ^ 0x00050003u, d = seed ^ 0x7f007f00u;
    for (int it = 0; it < kProbeIters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            a[c] = __viaddmax_s16x2(a[c], b, d);
            a[c] = __vimax3_s16x2(a[c], b + c, d ^ it);
        }
    }
    uint32_t x = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) x ^= a[c];
    if (x == 0x12345678u) out[0] = x;
}

// Each iteration issues kChains x 2 int32 max instructions.
__global__ void __launch_bounds__(256) k_probe_i32(int32_t seed, int32_t* out) {
    int32_t a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = seed * (int32_t)(threadIdx.x + 3 * c + 1);
    const int32_t b = seed ^ 0x5003, d = seed ^ 0x7f00;
    for (int it = 0; it < kProbeIters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            a[c] = max(a[c], b ^ it);
            a[c] = max(a[c] + c, d);
        }
    }
    int32_t x = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) x ^= a[c];
    if (x == 0x12345678) out[0] = x;
}

// Per-instruction throughput of the packed cell's instructions: kChains
// independent chains of two dependent instructions per iteration.  OP 0:
// __viaddmax_s16x2, 1: __vimax3_s16x2_relu, 2: __vadd2, 3: byte permute
// (prmt), 4: a viaddmax chain and a vadd2 chain side by side (instructions
// of two pipes).
template <int OP>
__global__ void __launch_bounds__(256) k_probe_op(uint32_t seed, uint32_t* out) {
    uint32_t a[kChains], x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        a[c] = seed * (threadIdx.x + 3 * c + 1);
        x[c] = seed ^ (threadIdx.x * 7 + c);
    }
    const uint32_t b = seed ^ 0x00050003u, d = seed ^ 0x7f007f00u;
    for (int it = 0; it < kProbeIters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            if constexpr (OP == 0) {
                a[c] = __viaddmax_s16x2(a[c], b, d);
                a[c] = __viaddmax_s16x2(a[c], d, b);
            } else if constexpr (OP == 1) {
                a[c] = __vimax3_s16x2_relu(a[c], b, d);
                a[c] = __vimax3_s16x2_relu(a[c], d, b);
            } else if constexpr (OP == 2) {
                a[c] = __vadd2(a[c], b);
                a[c] = __vadd2(a[c], d);
            } else if constexpr (OP == 3) {
                a[c] = __byte_perm(a[c], b, 0x5410);
                a[c] = __byte_perm(a[c], d, 0x7632);
            } else {
                a[c] = __viaddmax_s16x2(a[c], b, d);
                x[c] = __vadd2(x[c], b);
            }
        }
    }
    uint32_t r = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) r ^= a[c] ^ x[c];
    if (r == 0x12345678u) out[0] = r;
}

}  // namespace saber

extern "C" int saber_probe_int_peak_impl(int device, cudaStream_t s, double* dpx, double* i32) {
    using namespace saber;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return SABER_ERR_CUDA;
    int bps = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_probe_dpx, 256, 0);
    if (bps < 1) bps = 1;
    const unsigned grid = (unsigned)(sms * bps * 4);
    uint32_t* out = nullptr;
    if (cudaMalloc(&out, 64) != cudaSuccess) return SABER_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best_dpx = 0, best_i32 = 0;
    const double instr = (double)grid * 256 * kProbeIters * kChains * 2;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0, s);
        k_probe_dpx<<<grid, 256, 0, s>>>(0x00010002u + rep, out);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0) best_dpx = instr / (ms * 1e-3) > best_dpx ? instr / (ms * 1e-3) : best_dpx;
        cudaEventRecord(e0, s);
        k_probe_i32<<<grid, 256, 0, s>>>(17 + rep, reinterpret_cast<int32_t*>(out));
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0) best_i32 = instr / (ms * 1e-3) > best_i32 ? instr / (ms * 1e-3) : best_i32;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return SABER_ERR_CUDA;
    if (dpx) *dpx = best_dpx;
    if (i32) *i32 = best_i32;
    return SABER_OK;
}

// Lane-instructions per second of each k_probe_op kind (rates[0..4], best of
// three timed launches after one warm-up).
extern "C" int saber_probe_pipe_rates_impl(int device, cudaStream_t s, double* rates) {
    using namespace saber;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return SABER_ERR_CUDA;
    uint32_t* out = nullptr;
    if (cudaMalloc(&out, 64) != cudaSuccess) return SABER_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    void (*kernels[5])(uint32_t, uint32_t*) = {k_probe_op<0>, k_probe_op<1>, k_probe_op<2>, k_probe_op<3>,
                                               k_probe_op<4>};
    for (int k = 0; k < 5; k++) {
        int bps = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernels[k], 256, 0);
        if (bps < 1) bps = 1;
        const unsigned grid = (unsigned)(sms * bps * 4);
        const double instr = (double)grid * 256 * kProbeIters * kChains * 2;
        double best = 0;
        for (int rep = 0; rep < 4; rep++) {
            cudaEventRecord(e0, s);
            kernels[k]<<<grid, 256, 0, s>>>(0x00010002u + rep, out);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms > 0 && instr / (ms * 1e-3) > best) best = instr / (ms * 1e-3);
        }
        rates[k] = best;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return err == cudaSuccess ? SABER_OK : SABER_ERR_CUDA;
}
