// Learned triage of candidate regions: a 3-layer MLP (24 features -> 256 ->
// 256 -> 1 logit, ReLU) with bf16 weights and fp32 accumulation, trained on
// the GPU by the kernels below (forward, backward, Adam) on labels that the
// plain search produces (the region yields a reported hit at the E-value
// cut), and used by the batch engine to drop candidate regions before the
// banded scoring.  Every surviving region is still scored exactly; the plain
// path (no model installed) is unchanged.  No reference counterpart: the
// reference scores every candidate region.
//
// Model layout (floats, host and ABI): W1[32][256] (input-major, rows 24..31
// unused), b1[256], W2[256][256], b2[256], W3[256], b3, mu[32], isd[32]
// (the input normalisation x' = (x - mu) * isd).  The forward pass rounds the
// weights to bf16; training keeps fp32 master weights.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <type_traits>
#include <vector>

#include "runtime.cuh"

namespace saber {

static_assert(SABER_TRIAGE_ROW_FLOATS == 32, "feature row width");
constexpr int kTIn = 32, kTFeat = 24, kTHid = 256;
constexpr size_t kOffW1 = 0, kOffB1 = kOffW1 + kTIn * kTHid, kOffW2 = kOffB1 + kTHid,
                 kOffB2 = kOffW2 + kTHid * kTHid, kOffW3 = kOffB2 + kTHid, kOffB3 = kOffW3 + kTHid,
                 kOffMu = kOffB3 + 1, kOffIsd = kOffMu + kTIn, kModelFloats = kOffIsd + kTIn;
static_assert(kModelFloats == SABER_TRIAGE_MODEL_FLOATS, "model layout");

// ---- per-sequence composition features --------------------------------------
// One warp per sequence: Shannon entropy of the 20 standard residues (bits),
// the fraction of positions starting a 12-residue window with at most 4
// distinct residues (low complexity), the largest residue frequency, and the
// fraction of non-standard codes.
__global__ void k_seq_feats(const uint8_t* __restrict__ codes, const uint64_t* __restrict__ offs, uint64_t n,
                            float4* __restrict__ out) {
    __shared__ uint32_t hist[8][24];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint64_t s = (uint64_t)blockIdx.x * 8 + w; s < n; s += (uint64_t)gridDim.x * 8) {
        if (lane < 24) hist[w][lane] = 0;
        __syncwarp();
        const uint64_t b = offs[s], e = offs[s + 1];
        const uint64_t len = e - b;
        uint32_t lc = 0;
        for (uint64_t i = b + lane; i < e; i += 32) {
            const uint32_t c = codes[i];
            atomicAdd(&hist[w][c < 24 ? c : 23], 1u);
            if (i + 12 <= e) {
                uint32_t seen = 0;
                for (int k = 0; k < 12; k++) seen |= 1u << min((uint32_t)codes[i + k], 23u);
                lc += __popc(seen) <= 4;
            }
        }
        lc = __reduce_add_sync(0xffffffffu, lc);
        __syncwarp();
        if (lane == 0) {
            float ent = 0.f, mx = 0.f;
            uint32_t std20 = 0;
            for (int c = 0; c < 20; c++) std20 += hist[w][c];
            for (int c = 0; c < 20; c++) {
                if (!hist[w][c]) continue;
                const float p = (float)hist[w][c] / (float)std20;
                ent -= p * log2f(p);
                mx = fmaxf(mx, p);
            }
            const float nl = len ? (float)len : 1.f;
            const float win = len >= 12 ? (float)(len - 11) : 1.f;
            out[s] = make_float4(ent, (float)lc / win, mx, (float)(len - std20) / nl);
        }
        __syncwarp();
    }
}

// ---- per-region features ------------------------------------------------------
struct RegionFeatArgs {
    const saber_region* reg;
    const uint4* rstat;       // HSPs, score sum, seed hits
    const uint32_t* rquery;   // query of each region (batch index)
    const uint32_t* rrank;    // rank of the region within its query (region order)
    const float4* qinfo;      // per query: length, region threshold, top best, regions
    const float4* qfeat;      // per query sequence features
    const float4* sfeat;      // per subject sequence features
    const uint64_t* soffs;    // subject offsets
    float lambda, logk;
    uint64_t n;
    float* X;                 // n x 32
};

__global__ void k_region_feats(RegionFeatArgs a) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x) {
        const saber_region r = a.reg[i];
        const uint4 st = a.rstat[i];
        const uint32_t q = a.rquery[i];
        const float4 qi = a.qinfo[q];
        const float qlen = fmaxf(qi.x, 1.f), thr = fmaxf(qi.y, 1.f), top = fmaxf(qi.z, 1.f), nreg = qi.w;
        const float slen = fmaxf((float)(a.soffs[r.subject + 1] - a.soffs[r.subject]), 1.f);
        const float best = (float)r.best, spread = (float)(r.d_max - r.d_min);
        const float nh = (float)st.x, ssum = (float)st.y, hits = (float)st.z;
        const float dmid = 0.5f * (float)(r.d_min + r.d_max);
        const float ov = fmaxf(fminf(qlen, slen - dmid) - fmaxf(0.f, -dmid), 0.f);
        const float4 qf = a.qfeat[q], sf = a.sfeat[r.subject];
        float f[kTIn];
        f[0] = best / 100.f;
        f[1] = log2f(1.f + fmaxf(best, 0.f));
        f[2] = best / thr;
        f[3] = (a.lambda * best - a.logk) / 0.69314718f / 100.f;
        f[4] = (a.lambda * best - a.logk - logf(qlen) - logf(slen)) / 2.30258509f / 10.f;
        f[5] = log2f(1.f + nh);
        f[6] = log2f(1.f + hits);
        f[7] = nh > 0.f ? ssum / (100.f * nh) : 0.f;
        f[8] = log2f(1.f + ssum);
        f[9] = log2f(1.f + fmaxf(spread, 0.f));
        f[10] = spread / qlen;
        f[11] = log2f(qlen);
        f[12] = log2f(slen);
        f[13] = log2f(qlen) - log2f(slen);
        f[14] = ov / fminf(qlen, slen);
        f[15] = log2f(1.f + (float)a.rrank[i]);
        f[16] = best / top;
        f[17] = log2f(1.f + nreg);
        f[18] = qf.x;
        f[19] = qf.y;
        f[20] = qf.z;
        f[21] = sf.x;
        f[22] = sf.y;
        f[23] = sf.z;
        for (int k = kTFeat; k < kTIn; k++) f[k] = 0.f;
        float4* o = reinterpret_cast<float4*>(a.X + i * kTIn);
        for (int k = 0; k < kTIn / 4; k++) o[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
    }
}

// ---- generic tiled GEMM: C[m][n] (=|+=) act(sum_k A[m][k] B[k][n] + bias[n]) ----------
// A[m][k] at A[m * sam + k * sak], B[k][n] at B[k * sbk + n * sbn]; fp32
// accumulation; ACT 0 none, 1 ReLU; ACC: add into C; MASK: multiply the
// result by (M[m][n] > 0) (ReLU derivative of a stored activation).
template <class TA, class TB>
__device__ __forceinline__ float ld_as_f(const TA* p) {
    if constexpr (std::is_same<TA, __nv_bfloat16>::value) return __bfloat162float(*p);
    else return (float)*p;
}

template <class TA, class TB, int ACT, bool ACC, bool MASK>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const TA* __restrict__ A, long sam, long sak,
                                              const TB* __restrict__ B, long sbk, long sbn, const float* __restrict__ bias,
                                              const float* __restrict__ Mk, float* __restrict__ C, long ldc) {
    __shared__ float As[16][64 + 1];
    __shared__ float Bs[16][64 + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int t = threadIdx.x; t < 16 * 64; t += 256) {
            const int kk = t / 64, mm = t % 64;
            const int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < K) ? ld_as_f<TA, TA>(A + (long)gm * sam + (long)gk * sak) : 0.f;
            const int gn = n0 + mm;
            Bs[kk][mm] = (gn < N && gk < K) ? ld_as_f<TB, TB>(B + (long)gk * sbk + (long)gn * sbn) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= N) continue;
            float v = acc[i][j] + (bias ? bias[gn] : 0.f);
            if (ACT == 1) v = fmaxf(v, 0.f);
            if (MASK) v = Mk[(long)gm * ldc + gn] > 0.f ? v : 0.f;
            float* c = C + (long)gm * ldc + gn;
            *c = ACC ? *c + v : v;
        }
    }
}

template <class TA, class TB, int ACT, bool ACC, bool MASK>
static void gemm(cudaStream_t s, int M, int N, int K, const TA* A, long sam, long sak, const TB* B, long sbk, long sbn,
                 const float* bias, const float* Mk, float* C, long ldc) {
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    k_gemm<TA, TB, ACT, ACC, MASK><<<grid, 256, 0, s>>>(M, N, K, A, sam, sak, B, sbk, sbn, bias, Mk, C, ldc);
}

// normalised inputs: Xn = (X - mu) * isd
__global__ void k_normalize(const float* __restrict__ X, uint64_t n, const float* __restrict__ model,
                            float* __restrict__ Xn) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * kTIn; t += (uint64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t % kTIn);
        Xn[t] = k < kTFeat ? (X[t] - model[kOffMu + k]) * model[kOffIsd + k] : 0.f;
    }
}

__global__ void k_to_bf16(const float* __restrict__ src, uint64_t n, __nv_bfloat16* __restrict__ dst) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x)
        dst[t] = __float2bfloat16_rn(src[t]);
}

// binary cross-entropy on logits, positives weighted by pos_weight, mean over
// the batch: dz = w (sigmoid(z) - y) / n; loss accumulated in double
__global__ void k_bce(const float* __restrict__ z, const uint8_t* __restrict__ y, int n, float pos_weight,
                      float* __restrict__ dz, double* __restrict__ loss) {
    double l = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float zi = z[i];
        const float yi = y[i] ? 1.f : 0.f;
        const float w = y[i] ? pos_weight : 1.f;
        const float p = 1.f / (1.f + expf(-zi));
        dz[i] = w * (p - yi) / (float)n;
        // log(1 + exp(-|z|)) + max(z, 0) - y z
        const float li = log1pf(expf(-fabsf(zi))) + fmaxf(zi, 0.f) - yi * zi;
        l += (double)(w * li) / n;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// column sums: out[j] (=|+=) sum_i G[i][j]
__global__ void k_colsum(const float* __restrict__ G, int rows, int cols, float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.f;
    for (int i = 0; i < rows; i++) s += G[(long)i * cols + j];
    out[j] = s;
}

// dH2[i][j] = dz[i] * W3[j] * (H2[i][j] > 0)
__global__ void k_outer_mask(const float* __restrict__ dz, int n, const __nv_bfloat16* __restrict__ w3,
                             const float* __restrict__ H2, float* __restrict__ dH2) {
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < (long)n * kTHid; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t / kTHid), j = (int)(t % kTHid);
        dH2[t] = H2[t] > 0.f ? dz[i] * __bfloat162float(w3[j]) : 0.f;
    }
}

// Adam (bias-corrected), fp32 masters, weights only (the normalisation
// entries mu / isd are not trained)
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       uint64_t n, float lr, float b1, float b2, float eps, float c1, float c2, float wd) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        if (t >= kOffMu) continue;
        const float gt = g[t] + wd * w[t];
        const float mt = b1 * m[t] + (1.f - b1) * gt;
        const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
        m[t] = mt;
        v[t] = vt;
        w[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
    }
}

// ---- fused inference on the tensor cores -------------------------------------
// One warp per 16 regions, mma.sync m16n8k16 (bf16 operands, fp32
// accumulation).  The weights are bf16 already; the activations (the
// normalised inputs and the layer-1 outputs) are fp32 and enter as a
// bf16 pair hi + lo (lo = the rounding residual), two products per tile, so
// the result matches the fp32-activation forward pass of training to about
// 2^-16 relative.  Layer 1 runs in chunks of 16 hidden units whose
// accumulator tiles are, register for register, the A operand of layer 2;
// layer 3 (256 -> 1) is a quad reduction of the layer-2 accumulators.
constexpr size_t kPackOff = ((kModelFloats * 2 + 255) / 256) * 256;        // bytes into the bf16 buffer
constexpr size_t kPackBytes = (size_t)(2 + 16) * 32 * 32 * sizeof(uint2);  // W1 and W2 fragments

// B fragments of a row-major [K][256] bf16 weight, K = 16 kt: for tile (kt,
// nt) and lane l, {W[k][n], W[k + 1][n]} and {W[k + 8][n], W[k + 9][n]} with
// k = 16 kt + 2 (l % 4), n = 8 nt + l / 4.
__global__ void k_pack_b(const __nv_bfloat16* __restrict__ W, int kt_n, uint2* __restrict__ out) {
    const int total = kt_n * 32 * 32;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const int lane = t & 31, nt = (t >> 5) & 31, kt = t >> 10;
        const int k = kt * 16 + 2 * (lane & 3), n = nt * 8 + (lane >> 2);
        auto u = [&](int kk) { return (uint32_t)__bfloat16_as_ushort(W[(size_t)kk * kTHid + n]); };
        out[t] = make_uint2(u(k) | (u(k + 1) << 16), u(k + 8) | (u(k + 9) << 16));
    }
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint2 b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b.x), "r"(b.y));
}

// (x, y) -> packed bf16 pairs hi and lo with x ~ hi.x + lo.x, y ~ hi.y + lo.y
__device__ __forceinline__ void split2(float x, float y, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
    const __nv_bfloat162 l = __floats2bfloat162_rn(x - __bfloat162float(h.x), y - __bfloat162float(h.y));
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

__global__ void __launch_bounds__(128) k_mlp_infer(const float* __restrict__ X, uint64_t n,
                                                   const float* __restrict__ model, const uint2* __restrict__ pk,
                                                   const __nv_bfloat16* __restrict__ wb, float* __restrict__ logit) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t r0 = warp * 16;
    if (r0 >= n) return;
    const int qr = lane >> 2, qc = 2 * (lane & 3);
    const uint64_t ra = r0 + qr, rb = r0 + qr + 8;
    // layer-1 A operand: normalised inputs, 2 k-steps of 16, hi and lo
    uint32_t xa[2][4], xl[2][4];
#pragma unroll
    for (int ks = 0; ks < 2; ks++) {
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {  // k and k + 8
            const int k = ks * 16 + hf * 8 + qc;
            float v[2][2];
#pragma unroll
            for (int rr = 0; rr < 2; rr++) {
                const uint64_t r = rr ? rb : ra;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int kk = k + e;
                    v[rr][e] = (r < n && kk < kTFeat) ? (X[r * kTIn + kk] - model[kOffMu + kk]) * model[kOffIsd + kk]
                                                      : 0.f;
                }
            }
            split2(v[0][0], v[0][1], xa[ks][hf * 2 + 0], xl[ks][hf * 2 + 0]);
            split2(v[1][0], v[1][1], xa[ks][hf * 2 + 1], xl[ks][hf * 2 + 1]);
        }
    }
    const uint2* P1 = pk;
    const uint2* P2 = pk + 2 * 32 * 32;
    float acc[32][4];
#pragma unroll
    for (int nt = 0; nt < 32; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll 1
    for (int ch = 0; ch < 16; ch++) {
        // layer 1, hidden units 16 ch .. 16 ch + 15 (n-tiles 2 ch, 2 ch + 1)
        float h[2][4];
#pragma unroll
        for (int j = 0; j < 2; j++) {
            h[j][0] = h[j][1] = h[j][2] = h[j][3] = 0.f;
            const int nt = 2 * ch + j;
#pragma unroll
            for (int ks = 0; ks < 2; ks++) {
                const uint2 b = P1[(ks * 32 + nt) * 32 + lane];
                mma_bf16(h[j], xa[ks][0], xa[ks][1], xa[ks][2], xa[ks][3], b);
                mma_bf16(h[j], xl[ks][0], xl[ks][1], xl[ks][2], xl[ks][3], b);
            }
            const float b0 = model[kOffB1 + nt * 8 + qc], b1 = model[kOffB1 + nt * 8 + qc + 1];
            h[j][0] = fmaxf(h[j][0] + b0, 0.f);
            h[j][1] = fmaxf(h[j][1] + b1, 0.f);
            h[j][2] = fmaxf(h[j][2] + b0, 0.f);
            h[j][3] = fmaxf(h[j][3] + b1, 0.f);
        }
        // the two accumulator tiles are the layer-2 A operand of k-step ch
        uint32_t ah[4], al[4];
        split2(h[0][0], h[0][1], ah[0], al[0]);
        split2(h[0][2], h[0][3], ah[1], al[1]);
        split2(h[1][0], h[1][1], ah[2], al[2]);
        split2(h[1][2], h[1][3], ah[3], al[3]);
#pragma unroll
        for (int nt = 0; nt < 32; nt++) {
            const uint2 b = P2[(ch * 32 + nt) * 32 + lane];
            mma_bf16(acc[nt], ah[0], ah[1], ah[2], ah[3], b);
            mma_bf16(acc[nt], al[0], al[1], al[2], al[3], b);
        }
    }
    // layer 3
    const __nv_bfloat16* W3 = wb + kOffW3;
    float sa = 0.f, sb = 0.f;
#pragma unroll
    for (int nt = 0; nt < 32; nt++) {
        const int c = nt * 8 + qc;
        const float b0 = model[kOffB2 + c], b1 = model[kOffB2 + c + 1];
        const float w0 = __bfloat162float(W3[c]), w1 = __bfloat162float(W3[c + 1]);
        sa = fmaf(fmaxf(acc[nt][0] + b0, 0.f), w0, sa);
        sa = fmaf(fmaxf(acc[nt][1] + b1, 0.f), w1, sa);
        sb = fmaf(fmaxf(acc[nt][2] + b0, 0.f), w0, sb);
        sb = fmaf(fmaxf(acc[nt][3] + b1, 0.f), w1, sb);
    }
    sa += __shfl_xor_sync(0xffffffffu, sa, 1);
    sa += __shfl_xor_sync(0xffffffffu, sa, 2);
    sb += __shfl_xor_sync(0xffffffffu, sb, 1);
    sb += __shfl_xor_sync(0xffffffffu, sb, 2);
    if ((lane & 3) == 0) {
        if (ra < n) logit[ra] = sa + model[kOffB3];
        if (rb < n) logit[rb] = sb + model[kOffB3];
    }
}

__global__ void k_gather_rows(const float* __restrict__ Xn, const uint8_t* __restrict__ y,
                              const uint32_t* __restrict__ idx, int nb, float* __restrict__ Xb, uint8_t* __restrict__ yb) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nb * kTIn; t += gridDim.x * blockDim.x) {
        const int i = t / kTIn, k = t % kTIn;
        Xb[t] = Xn[(size_t)idx[i] * kTIn + k];
        if (k == 0) yb[i] = y[idx[i]];
    }
}

// ---- host side -------------------------------------------------------------------
struct TriageDev {
    DevBuf model, wb, X, Xn, y, H1, H2, z, dz, dH2, dH1, grad, m, v, loss;
};

int triage_upload_model(saber_gpu* h, DevBuf& model, DevBuf& wb, const float* host_model);
static int upload_model(saber_gpu* h, DevBuf& model, DevBuf& wb, const float* host_model) {
    return triage_upload_model(h, model, wb, host_model);
}

int triage_upload_model(saber_gpu* h, DevBuf& model, DevBuf& wb, const float* host_model) {
    CUALLOC(h, model, kModelFloats * 4);
    CUALLOC(h, wb, kPackOff + kPackBytes);
    CU(h, cudaMemcpyAsync(model.p, host_model, kModelFloats * 4, cudaMemcpyHostToDevice, h->stream));
    k_to_bf16<<<nblocks(kModelFloats, 256), 256, 0, h->stream>>>(model.as<float>(), kModelFloats,
                                                                 wb.as<__nv_bfloat16>());
    // tensor-core fragments of W1 (2 x 32 tiles) and W2 (16 x 32 tiles)
    const __nv_bfloat16* w = wb.as<__nv_bfloat16>();
    uint2* pk = reinterpret_cast<uint2*>(wb.as<uint8_t>() + kPackOff);
    k_pack_b<<<nblocks(2 * 32 * 32, 256), 256, 0, h->stream>>>(w + kOffW1, 2, pk);
    k_pack_b<<<nblocks(16 * 32 * 32, 256), 256, 0, h->stream>>>(w + kOffW2, 16, pk + 2 * 32 * 32);
    CU(h, cudaGetLastError());
    return SABER_OK;
}

// forward + backward of one batch (inputs already normalised in Xn, labels
// in y): gradients written to grad (model layout), loss added to *loss
static int fwd_bwd(saber_gpu* h, TriageDev& d, int n, float pos_weight) {
    cudaStream_t s = h->stream;
    const float* mdl = d.model.as<float>();
    const __nv_bfloat16* wb = d.wb.as<__nv_bfloat16>();
    float* H1 = d.H1.as<float>();
    float* H2 = d.H2.as<float>();
    float* z = d.z.as<float>();
    float* g = d.grad.as<float>();
    // forward
    gemm<float, __nv_bfloat16, 1, false, false>(s, n, kTHid, kTIn, d.Xn.as<float>(), kTIn, 1, wb + kOffW1, kTHid, 1,
                                                mdl + kOffB1, nullptr, H1, kTHid);
    gemm<float, __nv_bfloat16, 1, false, false>(s, n, kTHid, kTHid, H1, kTHid, 1, wb + kOffW2, kTHid, 1, mdl + kOffB2,
                                                nullptr, H2, kTHid);
    gemm<float, __nv_bfloat16, 0, false, false>(s, n, 1, kTHid, H2, kTHid, 1, wb + kOffW3, 1, 1, mdl + kOffB3, nullptr,
                                                z, 1);
    // loss and dz
    k_bce<<<nblocks(n, 256, 1024), 256, 0, s>>>(z, d.y.as<uint8_t>(), n, pos_weight, d.dz.as<float>(),
                                                 d.loss.as<double>());
    // output layer: dW3 = H2^T dz, db3 = sum dz
    gemm<float, float, 0, false, false>(s, kTHid, 1, n, H2, 1, kTHid, d.dz.as<float>(), 1, 1, nullptr, nullptr,
                                        g + kOffW3, 1);
    k_colsum<<<1, 32, 0, s>>>(d.dz.as<float>(), n, 1, g + kOffB3);
    // dH2 = dz W3^T * relu'(H2)
    k_outer_mask<<<nblocks((uint64_t)n * kTHid, 256), 256, 0, s>>>(d.dz.as<float>(), n, wb + kOffW3, H2,
                                                                      d.dH2.as<float>());
    // dW2 = H1^T dH2, db2
    gemm<float, float, 0, false, false>(s, kTHid, kTHid, n, H1, 1, kTHid, d.dH2.as<float>(), kTHid, 1, nullptr, nullptr,
                                        g + kOffW2, kTHid);
    k_colsum<<<(kTHid + 127) / 128, 128, 0, s>>>(d.dH2.as<float>(), n, kTHid, g + kOffB2);
    // dH1 = dH2 W2^T * relu'(H1)
    gemm<float, __nv_bfloat16, 0, false, true>(s, n, kTHid, kTHid, d.dH2.as<float>(), kTHid, 1, wb + kOffW2, 1, kTHid,
                                               nullptr, H1, d.dH1.as<float>(), kTHid);
    // dW1 = Xn^T dH1, db1
    gemm<float, float, 0, false, false>(s, kTIn, kTHid, n, d.Xn.as<float>(), 1, kTIn, d.dH1.as<float>(), kTHid, 1,
                                        nullptr, nullptr, g + kOffW1, kTHid);
    k_colsum<<<(kTHid + 127) / 128, 128, 0, s>>>(d.dH1.as<float>(), n, kTHid, g + kOffB1);
    CU(h, cudaMemsetAsync(g + kOffMu, 0, 2 * kTIn * 4, s));
    CU(h, cudaGetLastError());
    return SABER_OK;
}

static int reserve_batch(saber_gpu* h, TriageDev& d, uint64_t n) {
    CUALLOC(h, d.Xn, n * kTIn * 4);
    CUALLOC(h, d.y, n + 16);
    CUALLOC(h, d.H1, n * kTHid * 4);
    CUALLOC(h, d.H2, n * kTHid * 4);
    CUALLOC(h, d.z, n * 4 + 16);
    CUALLOC(h, d.dz, n * 4 + 16);
    CUALLOC(h, d.dH2, n * kTHid * 4);
    CUALLOC(h, d.dH1, n * kTHid * 4);
    CUALLOC(h, d.grad, kModelFloats * 4);
    CUALLOC(h, d.loss, 16);
    return SABER_OK;
}

int triage_grads(saber_gpu* h, const float* model, const float* X, const uint8_t* y, uint32_t n, float pos_weight,
                 float* grads, double* loss) {
    TriageDev d;
    int rc = upload_model(h, d.model, d.wb, model);
    if (rc != SABER_OK) return rc;
    rc = reserve_batch(h, d, std::max<uint32_t>(n, 1));
    if (rc != SABER_OK) return rc;
    cudaStream_t s = h->stream;
    CUALLOC(h, d.X, (uint64_t)std::max<uint32_t>(n, 1) * kTIn * 4);
    CU(h, cudaMemcpyAsync(d.X.p, X, (uint64_t)n * kTIn * 4, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemcpyAsync(d.y.p, y, n, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemsetAsync(d.loss.p, 0, 8, s));
    k_normalize<<<nblocks((uint64_t)n * kTIn, 256), 256, 0, s>>>(d.X.as<float>(), n, d.model.as<float>(),
                                                                  d.Xn.as<float>());
    rc = fwd_bwd(h, d, (int)n, pos_weight);
    if (rc != SABER_OK) return rc;
    CU(h, cudaMemcpyAsync(grads, d.grad.p, kModelFloats * 4, cudaMemcpyDeviceToHost, s));
    double l = 0;
    CU(h, cudaMemcpyAsync(&l, d.loss.p, 8, cudaMemcpyDeviceToHost, s));
    CU(h, cudaStreamSynchronize(s));
    if (loss) *loss = l;
    return SABER_OK;
}

int triage_train(saber_gpu* h, float* model, const float* X, const uint8_t* y, uint64_t n,
                 const saber_triage_train_cfg* cfg, saber_triage_train_stats* st) {
    if (n == 0) return fail(h, SABER_ERR_ARG, "no training samples");
    cudaStream_t s = h->stream;
    const int B = (int)std::max<uint32_t>(32, cfg->batch);
    TriageDev d;
    int rc = upload_model(h, d.model, d.wb, model);
    if (rc != SABER_OK) return rc;
    rc = reserve_batch(h, d, (uint64_t)B);
    if (rc != SABER_OK) return rc;
    DevBuf Xall, yall;
    CUALLOC(h, Xall, n * kTIn * 4);
    CUALLOC(h, yall, n + 16);
    CUALLOC(h, d.m, kModelFloats * 4);
    CUALLOC(h, d.v, kModelFloats * 4);
    CU(h, cudaMemcpyAsync(Xall.p, X, n * kTIn * 4, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemcpyAsync(yall.p, y, n, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemsetAsync(d.m.p, 0, kModelFloats * 4, s));
    CU(h, cudaMemsetAsync(d.v.p, 0, kModelFloats * 4, s));
    // normalised copy of every sample; each epoch's batches gather rows
    // through a shuffled order (seeded)
    DevBuf Xnall, didx;
    CUALLOC(h, Xnall, n * kTIn * 4);
    CUALLOC(h, didx, n * 4);
    k_normalize<<<nblocks(n * kTIn, 256), 256, 0, s>>>(Xall.as<float>(), n, d.model.as<float>(), Xnall.as<float>());
    std::vector<uint32_t> order(n);
    for (uint64_t i = 0; i < n; i++) order[i] = (uint32_t)i;
    std::mt19937_64 rng(cfg->seed);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    uint64_t step = 0;
    double last_loss = 0;
    for (uint32_t ep = 0; ep < cfg->epochs; ep++) {
        std::shuffle(order.begin(), order.end(), rng);
        CU(h, cudaMemcpyAsync(didx.p, order.data(), n * 4, cudaMemcpyHostToDevice, s));
        CU(h, cudaMemsetAsync(d.loss.p, 0, 8, s));
        uint32_t nb = 0;
        for (uint64_t b0 = 0; b0 < n; b0 += B) {
            const int nbat = (int)std::min<uint64_t>(B, n - b0);
            k_gather_rows<<<nblocks((uint64_t)nbat * kTIn, 256), 256, 0, s>>>(
                Xnall.as<float>(), yall.as<uint8_t>(), didx.as<uint32_t>() + b0, nbat, d.Xn.as<float>(),
                d.y.as<uint8_t>());
            rc = fwd_bwd(h, d, nbat, cfg->pos_weight);
            if (rc != SABER_OK) return rc;
            step++;
            const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
            k_adam<<<nblocks(kModelFloats, 256), 256, 0, s>>>(d.model.as<float>(), d.grad.as<float>(), d.m.as<float>(),
                                                              d.v.as<float>(), kModelFloats, cfg->lr, b1, b2, eps, c1, c2,
                                                              cfg->weight_decay);
            k_to_bf16<<<nblocks(kModelFloats, 256), 256, 0, s>>>(d.model.as<float>(), kModelFloats,
                                                                 d.wb.as<__nv_bfloat16>());
            CU(h, cudaGetLastError());
            nb++;
        }
        double l = 0;
        CU(h, cudaMemcpyAsync(&l, d.loss.p, 8, cudaMemcpyDeviceToHost, s));
        CU(h, cudaStreamSynchronize(s));
        last_loss = nb ? l / nb : 0.0;
    }
    CU(h, cudaMemcpyAsync(model, d.model.p, kModelFloats * 4, cudaMemcpyDeviceToHost, s));
    CU(h, cudaStreamSynchronize(s));
    if (st) {
        st->steps = step;
        st->final_loss = last_loss;
    }
    return SABER_OK;
}

// logits of n feature rows with the installed model or the given one
int triage_predict(saber_gpu* h, DevBuf& model, DevBuf& wb, const float* d_X, uint64_t n, float* d_logit) {
    if (n == 0) return SABER_OK;
    const uint64_t warps = (n + 15) / 16;
    k_mlp_infer<<<(unsigned)((warps + 3) / 4), 128, 0, h->stream>>>(
        d_X, n, model.as<float>(), reinterpret_cast<const uint2*>(wb.as<uint8_t>() + kPackOff),
        wb.as<__nv_bfloat16>(), d_logit);
    CU(h, cudaGetLastError());
    return SABER_OK;
}

int triage_predict_host(saber_gpu* h, const float* model, const float* X, uint64_t n, float* logits) {
    DevBuf m, wb, dX, dz;
    int rc = upload_model(h, m, wb, model);
    if (rc != SABER_OK) return rc;
    CUALLOC(h, dX, std::max<uint64_t>(n, 1) * kTIn * 4);
    CUALLOC(h, dz, std::max<uint64_t>(n, 1) * 4);
    CU(h, cudaMemcpyAsync(dX.p, X, n * kTIn * 4, cudaMemcpyHostToDevice, h->stream));
    rc = triage_predict(h, m, wb, dX.as<float>(), n, dz.as<float>());
    if (rc != SABER_OK) return rc;
    CU(h, cudaMemcpyAsync(logits, dz.p, n * 4, cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    return SABER_OK;
}

// Region features for the engine: uploads the batch's regions and computes
// the feature rows on the device (kept in h->tr_X); sequence features of the
// database are computed once per loaded database.
int triage_region_features(saber_gpu* h, const saber_region* d_reg, const uint4* d_rstat, const uint32_t* d_rq,
                           const uint32_t* d_rrank, const float4* d_qinfo, uint64_t n, float lambda, float logk) {
    const Dataset& ds = h->main;
    const QuerySet& qs = ds.qs;
    cudaStream_t s = h->stream;
    if (!h->tr_sfeat_ok || h->tr_sfeat_key != (uint64_t)(uintptr_t)ds.res.p + ds.n_res) {
        CUALLOC(h, h->tr_sfeat, std::max<uint64_t>(ds.nsub, 1) * sizeof(float4));
        if (ds.nsub)
            k_seq_feats<<<(unsigned)std::min<uint64_t>((ds.nsub + 7) / 8, 65535u * 8), 256, 0, s>>>(
                ds.res.as<uint8_t>(), ds.soff.as<uint64_t>(), ds.nsub, h->tr_sfeat.as<float4>());
        CU(h, cudaGetLastError());
        h->tr_sfeat_ok = true;
        h->tr_sfeat_key = (uint64_t)(uintptr_t)ds.res.p + ds.n_res;
    }
    CUALLOC(h, h->tr_qfeat, std::max<uint64_t>(qs.nq, 1) * sizeof(float4));
    if (qs.nq)
        k_seq_feats<<<(unsigned)std::min<uint64_t>((qs.nq + 7) / 8, 65535u * 8), 256, 0, s>>>(
            qs.codes.as<uint8_t>(), qs.offsets.as<uint64_t>(), qs.nq, h->tr_qfeat.as<float4>());
    const uint64_t nn = std::max<uint64_t>(n, 1);
    CUALLOC(h, h->tr_X, nn * kTIn * 4);
    CUALLOC(h, h->tr_logit, nn * 4);
    RegionFeatArgs a;
    a.reg = d_reg;
    a.rstat = d_rstat;
    a.rquery = d_rq;
    a.rrank = d_rrank;
    a.qinfo = d_qinfo;
    a.qfeat = h->tr_qfeat.as<float4>();
    a.sfeat = h->tr_sfeat.as<float4>();
    a.soffs = ds.soff.as<uint64_t>();
    a.lambda = lambda;
    a.logk = logk;
    a.n = n;
    a.X = h->tr_X.as<float>();
    if (n) k_region_feats<<<nblocks(n, 256), 256, 0, s>>>(a);
    CU(h, cudaGetLastError());
    return SABER_OK;
}

}  // namespace saber
