// Tantan seed masking on the GPU: the posterior probability that each
// residue lies in a tandem repeat, from the scaled forward-backward pass of
// tantan's HMM (one background state B, repeat states F_1..F_W), and the
// seed mask posterior >= min_prob.  The query side is masked per batch, the
// database side once per load (masking.rs:1-31; the reference applies it in
// Engine::prepare, engine.rs:758-786, and when building the scan database,
// scan.rs:1078-1123).
//
// Bit-exact with the reference's f32 arithmetic: every operation is an
// explicitly rounded __fadd_rn / __fmul_rn / __fdiv_rn (never contracted to a
// fused multiply-add), and the state sums keep the reference's summation
// order — eight accumulators over the states in chunks of eight, the fixed
// combination tree ((a0+a1)+(a2+a3))+((a4+a5)+(a6+a7)), then the remaining
// states one by one (sum8 / dot8, masking.rs:121-152).
//
// Layout: one warp per sequence, lane l holding repeat states l and l+32
// (W <= 64), so each state sum is five chunk shuffles, a three-level xor
// tree and the remainder.  The forward pass stores each position's
// normalised F row (64 floats, two coalesced 128-byte stores) and its B value
// and scale (one float2 per position, staged in lanes and written 32 at a
// time) in a scratch region; the backward pass reads them in reverse order.
// Sequences run longest first and in launches whose scratch stays under a
// fixed budget.
//
// The model tables (lambda implied by the matrix, the emission ratios
// exp(lambda S(a,b)) and the B->F_i entry probabilities) are computed on the
// host in f64 exactly as Tantan::with_params computes them (masking.rs:
// 162-179, 531-612); this file's host code is built without floating-point
// contraction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "runtime.cuh"

namespace saber {

constexpr int kTtMaxW = 64;
constexpr unsigned kTtWarps = 8;  // warps (sequences) per block
constexpr uint32_t kFull = 0xffffffffu;

struct TantanModel {
    float lr[24 * 32];     // exp(lambda * S(a, b)) as f32; columns 24..31 are 0 (no partner residue)
    float b2f[kTtMaxW];    // B -> F_i, zero beyond w
    float b2b, f2f, f2b;   // 1 - r, 1 - e, e
    int w;                 // repeat states
    double min_prob;       // mask threshold
};

// ---- host: the model tables (masking.rs:162-179, 531-612) ----------------------

// Rust's f64::powi: binary exponentiation by the running square.
static double powi_bin(double a, int b) {
    const bool recip = b < 0;
    if (recip) b = -b;
    double r = 1.0;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return recip ? 1.0 / r : r;
}

// Gauss-Jordan inverse of a 20x20 matrix with partial pivoting (invert20,
// masking.rs:586-612); false when a pivot magnitude is below 1e-300.
static bool invert20(double (*a)[20], double (*inv)[20]) {
    for (int i = 0; i < 20; i++)
        for (int j = 0; j < 20; j++) inv[i][j] = i == j ? 1.0 : 0.0;
    for (int col = 0; col < 20; col++) {
        int piv = col;
        for (int r = col + 1; r < 20; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (std::fabs(a[piv][col]) < 1e-300) return false;
        if (piv != col)
            for (int j = 0; j < 20; j++) {
                std::swap(a[col][j], a[piv][j]);
                std::swap(inv[col][j], inv[piv][j]);
            }
        const double d = a[col][col];
        for (int j = 0; j < 20; j++) {
            a[col][j] /= d;
            inv[col][j] /= d;
        }
        for (int r = 0; r < 20; r++) {
            if (r == col) continue;
            const double f = a[r][col];
            if (f == 0.0) continue;
            for (int j = 0; j < 20; j++) {
                a[r][j] -= f * a[col][j];
                inv[r][j] -= f * inv[col][j];
            }
        }
    }
    return true;
}

// sum of the entries of (e^{l S})^-1 minus 1, and whether every implied
// letter frequency (row and column sum) is positive.
static bool lambda_gap(const int32_t* m, double l, double& v, bool& positive) {
    double a[20][20], inv[20][20];
    for (int i = 0; i < 20; i++)
        for (int j = 0; j < 20; j++) a[i][j] = std::exp(l * (double)m[i * 24 + j]);
    if (!invert20(a, inv)) return false;
    double total = 0.0;
    positive = true;
    for (int i = 0; i < 20; i++) {
        double rs = 0.0, cs = 0.0;
        for (int k = 0; k < 20; k++) rs += inv[i][k];
        for (int k = 0; k < 20; k++) cs += inv[k][i];
        if (rs <= 0.0 || cs <= 0.0) positive = false;
        total += rs;
    }
    v = total - 1.0;
    return true;
}

// The matrix's implied lambda: the first sign change of lambda_gap on the
// grid 0.02, 0.03, ... < 3, bisected 80 times, whose implied frequencies are
// positive.  NaN when there is none.
double tantan_implied_lambda(const int32_t* m) {
    bool have = false;
    double pl = 0.0, pv = 0.0;
    for (double l = 0.02; l < 3.0; l += 0.01) {
        double v;
        bool pos;
        if (!lambda_gap(m, l, v, pos)) continue;
        if (have && ((pv > 0.0) != (v > 0.0))) {
            double lo = pl, hi = l, vlo = pv;
            for (int it = 0; it < 80; it++) {
                const double mid = 0.5 * (lo + hi);
                double vm;
                bool pm;
                if (!lambda_gap(m, mid, vm, pm)) return NAN;
                if ((vm > 0.0) == (vlo > 0.0)) {
                    lo = mid;
                    vlo = vm;
                } else {
                    hi = mid;
                }
            }
            const double root = 0.5 * (lo + hi);
            double vr;
            bool pr;
            if (lambda_gap(m, root, vr, pr) && pr) return root;
        }
        have = true;
        pl = l;
        pv = v;
    }
    return NAN;
}

static int tantan_model(saber_gpu* h, const int32_t* m, const saber_tantan_params* p, TantanModel& M,
                        double& lambda) {
    if (!m || !p) return fail(h, SABER_ERR_ARG, "null tantan argument");
    const uint32_t w = p->max_period ? p->max_period : 1;
    if (w > (uint32_t)kTtMaxW) return fail(h, SABER_ERR_ARG, "tantan max_period %u above %d", w, kTtMaxW);
    lambda = p->lambda;
    if (!(lambda > 0.0)) {
        // implied by the matrix; cached per handle (a grid scan and 80
        // bisection steps, each a 20x20 inversion)
        if (h->tt_lambda_matrix.size() == 576 && std::equal(m, m + 576, h->tt_lambda_matrix.begin())) {
            lambda = h->tt_lambda;
        } else {
            lambda = tantan_implied_lambda(m);
            if (std::isnan(lambda)) lambda = 0.3176;  // masking.rs:163
            h->tt_lambda_matrix.assign(m, m + 576);
            h->tt_lambda = lambda;
        }
    }
    std::memset(&M, 0, sizeof(M));
    for (int a = 0; a < 24; a++)
        for (int b = 0; b < 24; b++) M.lr[a * 32 + b] = (float)std::exp(lambda * (double)m[a * 24 + b]);
    const double first = std::fabs(p->decay - 1.0) < 1e-12 ? 1.0 / (double)w
                                                          : (1.0 - p->decay) / (1.0 - powi_bin(p->decay, (int)w));
    for (uint32_t i = 0; i < w; i++) M.b2f[i] = (float)(p->repeat_start * first * powi_bin(p->decay, (int)i));
    M.b2b = (float)(1.0 - p->repeat_start);
    M.f2f = (float)(1.0 - p->repeat_end);
    M.f2b = (float)p->repeat_end;
    M.w = (int)w;
    M.min_prob = p->min_prob;
    return SABER_OK;
}

// ---- device ---------------------------------------------------------------------

// The reference's sum8 over the states 0..w-1 held as v0 = state lane,
// v1 = state lane + 32: lanes 0..7 accumulate the full chunks of eight
// states in order, the xor tree combines them as
// ((a0+a1)+(a2+a3))+((a4+a5)+(a6+a7)) in lane 0 (IEEE addition commutes, so
// the partner order within each pair does not matter), then the remaining
// w mod 8 states are added one at a time.  Every lane returns the sum.
template <int WC>
__device__ __forceinline__ float tt_sum8(float v0, float v1, int wrt) {
    const int w = WC ? WC : wrt;
    const int chunks = w >> 3;
    float acc = 0.f;
    if (chunks > 0) {
        float c[kTtMaxW / 8];
#pragma unroll
        for (int j = 1; j < kTtMaxW / 8; j++)
            c[j] = j < chunks ? __shfl_down_sync(kFull, (j >> 2) ? v1 : v0, 8 * (j & 3)) : 0.f;
        acc = __fadd_rn(0.f, v0);
#pragma unroll
        for (int j = 1; j < kTtMaxW / 8; j++)
            if (j < chunks) acc = __fadd_rn(acc, c[j]);
    }
    acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 1));
    acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 2));
    acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 4));
    float t = __shfl_sync(kFull, acc, 0);
    const int rem0 = chunks * 8;
#pragma unroll
    for (int r = 0; r < 7; r++) {
        const int s = rem0 + r;
        if (s < w) t = __fadd_rn(t, __shfl_sync(kFull, s < 32 ? v0 : v1, s & 31));
    }
    return t;
}

// One warp per sequence (ord[k] for k in [k0, k1)); base[k] is the sequence's
// first scratch row.  Writes mask[offs[sid] + p] (and probs when non-null) and
// adds the masked positions to *n_masked.
template <int WC>  // repeat states when fixed at compile time (0: M.w)
__global__ void __launch_bounds__(kTtWarps * 32, 4) k_tantan(const __grid_constant__ TantanModel M,
                                                          const uint8_t* __restrict__ codes,
                                                          const uint64_t* __restrict__ offs,
                                                          const uint32_t* __restrict__ ord,
                                                          const uint64_t* __restrict__ base, uint64_t k0, uint64_t k1,
                                                          float* __restrict__ fwdF, float2* __restrict__ fwdBS,
                                                          uint8_t* __restrict__ mask, float* __restrict__ probs,
                                                          unsigned long long* __restrict__ n_masked) {
    __shared__ float lr[24 * 32];
    for (int i = threadIdx.x; i < 24 * 32; i += blockDim.x) lr[i] = M.lr[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint64_t k = k0 + (uint64_t)blockIdx.x * kTtWarps + (threadIdx.x >> 5);
    if (k >= k1) return;
    const uint32_t sid = ord[k];
    const uint64_t st = offs[sid];
    const int64_t n = (int64_t)(offs[sid + 1] - st);
    if (n <= 0) return;
    const uint8_t* x = codes + st;
    float* F = fwdF + base[k] * (uint64_t)kTtMaxW;
    float2* BS = fwdBS + base[k];
    const int w = WC ? WC : M.w;
    const float b2f0 = M.b2f[lane], b2f1 = M.b2f[lane + 32];
    const float b2b = M.b2b, f2f = M.f2f, f2b = M.f2b;

    // ---- forward (masking.rs:476-497) ----
    float pb = 1.f, pf0 = 0.f, pf1 = 0.f;
    int h0 = 24, h1 = 24;  // codes x[p-1-lane], x[p-33-lane]; 24 = no partner (ratio 0)
    int cw = 0;
    float mb = 0.f, ms = 0.f;
    for (int64_t p = 0; p < n; p++) {
        const int j = (int)(p & 31);
        if (j == 0) {
            const int64_t q = p + lane;
            cw = q < n ? min((int)x[q], 23) : 0;
        }
        const int xp = __shfl_sync(kFull, cw, j);
        const float e0 = lr[xp * 32 + h0], e1 = lr[xp * 32 + h1];
        const float sum_f = tt_sum8<WC>(pf0, pf1, w);
        const float c0 = __fmul_rn(__fadd_rn(__fmul_rn(pb, b2f0), __fmul_rn(pf0, f2f)), e0);
        const float c1 = __fmul_rn(__fadd_rn(__fmul_rn(pb, b2f1), __fmul_rn(pf1, f2f)), e1);
        const float cb = __fadd_rn(__fmul_rn(pb, b2b), __fmul_rn(sum_f, f2b));
        const float tot = __fadd_rn(cb, tt_sum8<WC>(c0, c1, w));
        const float s = tot > 0.f ? __fdiv_rn(1.f, tot) : 1.f;
        pb = __fmul_rn(cb, s);
        pf0 = __fmul_rn(c0, s);
        pf1 = __fmul_rn(c1, s);
        F[p * kTtMaxW + lane] = pf0;
        F[p * kTtMaxW + 32 + lane] = pf1;
        if (lane == j) {
            mb = pb;
            ms = s;
        }
        if (j == 31 || p == n - 1) {
            const int64_t q = (p & ~(int64_t)31) + lane;
            if (q < n) BS[q] = make_float2(mb, ms);
        }
        const int t31 = __shfl_sync(kFull, h0, 31);
        h0 = __shfl_up_sync(kFull, h0, 1);
        h1 = __shfl_up_sync(kFull, h1, 1);
        if (lane == 0) {
            h0 = xp;
            h1 = t31;
        }
    }
    __syncwarp();

    // ---- backward with the same scales (masking.rs:499-528) ----
    // The F row of position p and the partner codes x[p-1-lane], x[p-33-lane]
    // are loaded one position ahead.
    float nb = 1.f, nf0 = f2b, nf1 = f2b;
    float2 bs = make_float2(0.f, 0.f);
    float keep = 0.f;
    unsigned masked = 0;
    float r0 = F[(n - 1) * kTtMaxW + lane], r1 = F[(n - 1) * kTtMaxW + 32 + lane];
    int g0 = n - 2 - lane >= 0 ? min((int)x[n - 2 - lane], 23) : 24;
    int g1 = n - 34 - lane >= 0 ? min((int)x[n - 34 - lane], 23) : 24;
    for (int64_t p = n - 1; p >= 0; p--) {
        const int j = (int)(p & 31);
        if (j == 31 || p == n - 1) {
            const int64_t q = (p & ~(int64_t)31) + lane;
            bs = q < n ? BS[q] : make_float2(0.f, 0.f);
            cw = q < n ? min((int)x[q], 23) : 0;
        }
        float r0n = 0.f, r1n = 0.f;
        int g0n = 24, g1n = 24;
        if (p > 0) {
            r0n = F[(p - 1) * kTtMaxW + lane];
            r1n = F[(p - 1) * kTtMaxW + 32 + lane];
            const int64_t q0 = p - 2 - lane, q1 = p - 34 - lane;
            if (q0 >= 0) g0n = min((int)x[q0], 23);
            if (q1 >= 0) g1n = min((int)x[q1], 23);
        }
        const float rb = __shfl_sync(kFull, bs.x, j), s = __shfl_sync(kFull, bs.y, j);
        const int xp = __shfl_sync(kFull, cw, j);
        const float onb = nb, onf0 = nf0, onf1 = nf1;
        if (p > 0) {
            const float be0 = __fmul_rn(lr[xp * 32 + g0], onf0), be1 = __fmul_rn(lr[xp * 32 + g1], onf1);
            const float to_fg = tt_sum8<WC>(__fmul_rn(b2f0, be0), __fmul_rn(b2f1, be1), w);
            const float fb = __fmul_rn(f2b, onb);
            nf0 = __fmul_rn(__fadd_rn(__fmul_rn(f2f, be0), fb), s);
            nf1 = __fmul_rn(__fadd_rn(__fmul_rn(f2f, be1), fb), s);
            nb = __fmul_rn(__fadd_rn(__fmul_rn(b2b, onb), to_fg), s);
        }
        const float pbv = __fmul_rn(rb, onb);
        const float pfv = tt_sum8<WC>(__fmul_rn(r0, onf0), __fmul_rn(r1, onf1), w);
        const float z = __fadd_rn(pbv, pfv);
        const float post = z > 0.f ? __fdiv_rn(pfv, z) : 0.f;
        if (lane == j) keep = post;
        if (j == 0) {
            const int64_t q = p + lane;
            const bool ok = q < n;
            const bool m = ok && (double)keep >= M.min_prob;
            if (ok) {
                mask[st + q] = m ? 1 : 0;
                if (probs) probs[st + q] = keep;
            }
            masked += __popc(__ballot_sync(kFull, m));
        }
        r0 = r0n;
        r1 = r1n;
        g0 = g0n;
        g1 = g1n;
    }
    if (lane == 0 && masked) atomicAdd(n_masked, (unsigned long long)masked);
}

// ---- eight lanes per sequence ------------------------------------------------------
//
// The default model (W = 50) runs four sequences per warp, eight lanes each:
// lane k of a group holds states k + 8j (j = 0..7, registers v[j]), so each
// of the reference's eight accumulators is one lane's in-register chain over
// the full chunks, the combination tree is three xor shuffles inside the group
// (every lane ends with the same sum: each level adds a pair in both orders,
// and IEEE addition commutes), and the remaining states W mod 8 sit in
// register W/8 of lanes 0.. and are added by broadcast, in order.
//
// Partner codes come from a per-group ring of 128 codes in shared memory,
// stored twice (slots q & 127 and 128 + (q & 127)) so that the code of
// position p-1-k-8j is at the fixed offset ((p-1-k) & 127) + 128 - 8j; ring
// slots of positions before the sequence hold 24 (no partner, ratio 0).
// The scratch row of a position keeps lane k's eight states contiguous
// (index 8k + j: two 16-byte stores per lane).
constexpr int kTg = 8;          // lanes per sequence
constexpr int kTgSeqs = 4;      // sequences per warp
constexpr int kRingPitch = 264; // bytes per group ring (256 + 8: the two words a group reads never share a
                                // bank with the neighbouring groups')

template <int W>
__device__ __forceinline__ float tg_sum(const float (&v)[8]) {
    constexpr int C = W / 8, R = W % 8;
    float acc = 0.f;
    if (C > 0) {
        acc = __fadd_rn(0.f, v[0]);
#pragma unroll
        for (int j = 1; j < C; j++) acc = __fadd_rn(acc, v[j]);
    }
    acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 1, kTg));
    acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 2, kTg));
    acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 4, kTg));
#pragma unroll
    for (int r = 0; r < R; r++) acc = __fadd_rn(acc, __shfl_sync(kFull, v[C < 8 ? C : 7], r, kTg));
    return acc;
}

// Ring chunk c (positions 32c .. 32c+31) of one group: lane k loads the
// codes of positions 32c + 4k .. 32c + 4k + 3 (24 before the sequence) as
// one word and stores it into both copies of the ring.
__device__ __forceinline__ uint32_t tg_load(const uint8_t* __restrict__ x, int64_t n, int64_t c, int k) {
    const int64_t q0 = 32 * c + 4 * k;
    uint32_t word = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const int64_t q = q0 + t;
        const uint32_t code = q < 0 ? 24u : (q < n ? (uint32_t)min((int)x[q], 23) : 0u);
        word |= code << (8 * t);
    }
    return word;
}
__device__ __forceinline__ void tg_store(uint8_t* ring, int64_t c, int k, uint32_t word) {
    const int slot = (int)((32 * c + 4 * k) & 127);
    *reinterpret_cast<uint32_t*>(ring + slot) = word;
    *reinterpret_cast<uint32_t*>(ring + 128 + slot) = word;
}

template <int W>
__global__ void __launch_bounds__(kTtWarps * 32, 4) k_tantan8(const __grid_constant__ TantanModel M,
                                                              const uint8_t* __restrict__ codes,
                                                              const uint64_t* __restrict__ offs,
                                                              const uint32_t* __restrict__ ord,
                                                              const uint64_t* __restrict__ base, uint64_t k0,
                                                              uint64_t k1, float* __restrict__ fwdF,
                                                              float2* __restrict__ fwdBS, uint8_t* __restrict__ mask,
                                                              float* __restrict__ probs,
                                                              unsigned long long* __restrict__ n_masked) {
    static_assert(W >= 1 && W <= kTtMaxW, "repeat states");
    constexpr int J = (W + 7) / 8;  // registers holding states
    __shared__ float lr[24 * 33];
    __shared__ __align__(16) uint8_t rings[kTtWarps * kTgSeqs * kRingPitch];
    for (int i = threadIdx.x; i < 24 * 33; i += blockDim.x) {
        const int r = i / 33, c = i % 33;
        lr[i] = c < 32 ? M.lr[r * 32 + c] : 0.f;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 3, k = lane & 7;
    const int wib = threadIdx.x >> 5;
    uint8_t* ring = rings + (wib * kTgSeqs + g) * kRingPitch;
    const uint64_t kk = k0 + ((uint64_t)blockIdx.x * (blockDim.x >> 5) + wib) * kTgSeqs + g;
    int64_t n = 0;
    uint64_t st = 0;
    float* F = fwdF;
    float2* BS = fwdBS;
    if (kk < k1) {
        const uint32_t sid = ord[kk];
        st = offs[sid];
        n = (int64_t)(offs[sid + 1] - st);
        F = fwdF + base[kk] * (uint64_t)kTtMaxW + 8 * k;
        BS = fwdBS + base[kk];
    }
    const int64_t nmax = (int64_t)__reduce_max_sync(kFull, (unsigned)n);
    if (nmax == 0) return;
    const uint8_t* x = codes + st;
    float b2f[8];
#pragma unroll
    for (int j = 0; j < 8; j++) b2f[j] = j < J ? M.b2f[k + 8 * j] : 0.f;
    const float b2b = M.b2b, f2f = M.f2f, f2b = M.f2b;
    // ring: 24 everywhere (positions before the sequence), then chunks 0 and 1
#pragma unroll
    for (int t = 0; t < 8; t++) *reinterpret_cast<uint32_t*>(ring + 32 * t + 4 * k) = 0x18181818u;
    __syncwarp();

    // ---- forward (masking.rs:476-497) ----
    float pb = 1.f, pf[8];
#pragma unroll
    for (int j = 0; j < 8; j++) pf[j] = 0.f;
    float mb = 0.f, ms = 0.f;
    uint32_t wnext = tg_load(x, n, 0, k);  // codes one chunk ahead
    for (int64_t p = 0; p < nmax; p++) {
        if ((p & 31) == 0) {
            __syncwarp();
            tg_store(ring, p >> 5, k, wnext);
            __syncwarp();
            wnext = tg_load(x, n, (p >> 5) + 1, k);
        }
        const int xrow = 33 * (int)ring[p & 127];
        const uint8_t* rp = ring + ((p - 1 - k) & 127) + 128;
        float e[8];
#pragma unroll
        for (int j = 0; j < 8; j++) e[j] = j < J ? lr[xrow + rp[-8 * j]] : 0.f;
        const float sum_f = tg_sum<W>(pf);
        float c[8];
#pragma unroll
        for (int j = 0; j < 8; j++) c[j] = __fmul_rn(__fadd_rn(__fmul_rn(pb, b2f[j]), __fmul_rn(pf[j], f2f)), e[j]);
        const float cb = __fadd_rn(__fmul_rn(pb, b2b), __fmul_rn(sum_f, f2b));
        const float tot = __fadd_rn(cb, tg_sum<W>(c));
        const float s = tot > 0.f ? __fdiv_rn(1.f, tot) : 1.f;
        pb = __fmul_rn(cb, s);
#pragma unroll
        for (int j = 0; j < 8; j++) pf[j] = __fmul_rn(c[j], s);
        if (p < n) {
            float4* row = reinterpret_cast<float4*>(F + p * kTtMaxW);
            row[0] = make_float4(pf[0], pf[1], pf[2], pf[3]);
            row[1] = make_float4(pf[4], pf[5], pf[6], pf[7]);
        }
        const int j8 = (int)(p & 7);
        if (k == j8) {
            mb = pb;
            ms = s;
        }
        if (j8 == 7 || p == nmax - 1) {
            const int64_t q = (p & ~(int64_t)7) + k;
            if (q < n && q <= p) BS[q] = make_float2(mb, ms);
        }
    }

    // ---- backward with the same scales (masking.rs:499-528) ----
    float nb = 1.f, nf[8];
#pragma unroll
    for (int j = 0; j < 8; j++) nf[j] = f2b;
    // B values and scales one block of eight positions ahead, codes one
    // chunk ahead, the F row one position ahead
    auto bs_load = [&](int64_t blk) {
        const int64_t q = 8 * blk + k;
        return blk >= 0 && q < n ? BS[q] : make_float2(0.f, 0.f);
    };
    float2 bs = bs_load((nmax - 1) >> 3), bsn = bs_load(((nmax - 1) >> 3) - 1);
    float keep = 0.f;
    unsigned masked = 0;
    float4 ra = make_float4(0.f, 0.f, 0.f, 0.f), rb4 = ra;
    {
        const int64_t p = nmax - 1;
        if (p < n) {
            const float4* row = reinterpret_cast<const float4*>(F + p * kTtMaxW);
            ra = row[0];
            rb4 = row[1];
        }
        const uint32_t w0 = tg_load(x, n, p >> 5, k), w1 = tg_load(x, n, (p >> 5) - 1, k),
                       w2 = tg_load(x, n, (p >> 5) - 2, k);
        __syncwarp();
        tg_store(ring, p >> 5, k, w0);
        tg_store(ring, (p >> 5) - 1, k, w1);
        tg_store(ring, (p >> 5) - 2, k, w2);
        __syncwarp();
        wnext = tg_load(x, n, (p >> 5) - 3, k);
    }
    for (int64_t p = nmax - 1; p >= 0; p--) {
        if ((p & 31) == 31 && p != nmax - 1) {
            __syncwarp();
            tg_store(ring, (p >> 5) - 2, k, wnext);
            __syncwarp();
            wnext = tg_load(x, n, (p >> 5) - 3, k);
        }
        const int j8 = (int)(p & 7);
        if (j8 == 7 && p != nmax - 1) {
            bs = bsn;
            bsn = bs_load((p >> 3) - 1);
        }
        float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb4 = na;
        if (p > 0 && p - 1 < n) {
            const float4* row = reinterpret_cast<const float4*>(F + (p - 1) * kTtMaxW);
            na = row[0];
            nb4 = row[1];
        }
        const float rbv = __shfl_sync(kFull, bs.x, j8, kTg), s = __shfl_sync(kFull, bs.y, j8, kTg);
        const float r[8] = {ra.x, ra.y, ra.z, ra.w, rb4.x, rb4.y, rb4.z, rb4.w};
        const bool active = p < n;
        const float onb = nb;
        float onf[8];
#pragma unroll
        for (int j = 0; j < 8; j++) onf[j] = nf[j];
        {
            const int xrow = 33 * (int)ring[p & 127];
            const uint8_t* rp = ring + ((p - 1 - k) & 127) + 128;
            float be[8], t[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                be[j] = j < J ? __fmul_rn(lr[xrow + rp[-8 * j]], onf[j]) : 0.f;
                t[j] = __fmul_rn(b2f[j], be[j]);
            }
            const float to_fg = tg_sum<W>(t);
            if (active && p > 0) {
                const float fb = __fmul_rn(f2b, onb);
#pragma unroll
                for (int j = 0; j < 8; j++) nf[j] = __fmul_rn(__fadd_rn(__fmul_rn(f2f, be[j]), fb), s);
                nb = __fmul_rn(__fadd_rn(__fmul_rn(b2b, onb), to_fg), s);
            }
        }
        float pr[8];
#pragma unroll
        for (int j = 0; j < 8; j++) pr[j] = __fmul_rn(r[j], onf[j]);
        const float pbv = __fmul_rn(rbv, onb);
        const float pfv = tg_sum<W>(pr);
        const float z = __fadd_rn(pbv, pfv);
        const float post = z > 0.f ? __fdiv_rn(pfv, z) : 0.f;
        if (k == j8) keep = post;
        if (j8 == 0) {
            const int64_t q = p + k;
            const bool ok = q < n;
            const bool m = ok && (double)keep >= M.min_prob;
            if (ok) {
                mask[st + q] = m ? 1 : 0;
                if (probs) probs[st + q] = keep;
            }
            masked += __popc(__ballot_sync(kFull, m));
        }
        ra = na;
        rb4 = nb4;
    }
    if (lane == 0 && masked) atomicAdd(n_masked, (unsigned long long)masked);
}

// ---- host driver ------------------------------------------------------------------

// Scratch rows (positions) per launch: 64 F floats + one float2 each.
constexpr uint64_t kTtRowsPerLaunch = 8ull << 20;

// Masks the sequences [offs[i], offs[i+1]) of the device residues d_codes
// (offsets on the host: h_offs; on the device: d_offs) into d_mask (one byte
// per residue) and, when d_probs is non-null, their posteriors.  Returns the
// masked count in *n_masked.
int tantan_run(saber_gpu* h, const TantanModel& M, const uint8_t* d_codes, const uint64_t* h_offs,
               const uint64_t* d_offs, uint64_t nseq, uint8_t* d_mask, float* d_probs, uint64_t* n_masked) {
    *n_masked = 0;
    if (nseq == 0) return SABER_OK;
    if (nseq > 0xffffffffull) return fail(h, SABER_ERR_ARG, "too many sequences for tantan");
    for (uint64_t i = 0; i < nseq; i++)
        if (h_offs[i + 1] - h_offs[i] >= (1ull << 31)) return fail(h, SABER_ERR_ARG, "sequence too long for tantan");
    // longest first (a counting sort on the length, lengths above 2^22 in one
    // bucket; ties by index), then launches bounded by the scratch budget
    uint64_t maxn = 0;
    for (uint64_t i = 0; i < nseq; i++) maxn = std::max(maxn, h_offs[i + 1] - h_offs[i]);
    const uint64_t nb = std::min<uint64_t>(maxn, 1ull << 22) + 1;
    std::vector<uint32_t> bucket(nb + 1, 0);
    for (uint64_t i = 0; i < nseq; i++) bucket[nb - 1 - std::min<uint64_t>(h_offs[i + 1] - h_offs[i], nb - 1)]++;
    for (uint64_t b = 0, acc = 0; b <= nb; b++) {
        const uint32_t c = bucket[b];
        bucket[b] = (uint32_t)acc;
        acc += c;
    }
    const uint64_t cap = std::max<uint64_t>(kTtRowsPerLaunch, maxn);
    std::vector<uint32_t> ord(nseq);
    std::vector<uint64_t> base(nseq);
    for (uint64_t i = 0; i < nseq; i++)
        ord[bucket[nb - 1 - std::min<uint64_t>(h_offs[i + 1] - h_offs[i], nb - 1)]++] = (uint32_t)i;
    std::vector<uint64_t> cuts{0};
    uint64_t rows = 0;
    for (uint64_t k = 0; k < nseq; k++) {
        const uint64_t n = h_offs[ord[k] + 1] - h_offs[ord[k]];
        if (rows + n > cap) {
            cuts.push_back(k);
            rows = 0;
        }
        base[k] = rows;
        rows += n;
    }
    cuts.push_back(nseq);
    uint64_t rows_max = 0;
    for (size_t c = 0; c + 1 < cuts.size(); c++) {
        const uint64_t k = cuts[c + 1] - 1;
        rows_max = std::max(rows_max, base[k] + (h_offs[ord[k] + 1] - h_offs[ord[k]]));
    }
    CUALLOC(h, h->tt_ord, nseq * sizeof(uint32_t));
    CUALLOC(h, h->tt_base, nseq * sizeof(uint64_t));
    CUALLOC(h, h->tt_F, std::max<uint64_t>(rows_max, 1) * kTtMaxW * sizeof(float));
    CUALLOC(h, h->tt_BS, std::max<uint64_t>(rows_max, 1) * sizeof(float2));
    CUALLOC(h, h->tt_count, sizeof(unsigned long long));
    CU(h, cudaMemcpyAsync(h->tt_ord.p, ord.data(), nseq * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemcpyAsync(h->tt_base.p, base.data(), nseq * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemsetAsync(h->tt_count.p, 0, sizeof(unsigned long long), h->stream));
    for (size_t c = 0; c + 1 < cuts.size(); c++) {
        const uint64_t k0 = cuts[c], k1 = cuts[c + 1];
        if (M.w == 50) {  // tantan's protein default: eight lanes per sequence
            // a batch too small to fill every SM with full blocks (a query
            // batch) runs two warps per block: more SMs, less contention
            // on each sequence's serial chain
            const unsigned warps = (k1 - k0) < (uint64_t)h->sm_count * kTtWarps * kTgSeqs ? 2u : kTtWarps;
            const uint64_t per_block = (uint64_t)warps * kTgSeqs;
            const unsigned blocks = (unsigned)((k1 - k0 + per_block - 1) / per_block);
            k_tantan8<50><<<blocks, warps * 32, 0, h->stream>>>(
                M, d_codes, d_offs, (const uint32_t*)h->tt_ord.p, (const uint64_t*)h->tt_base.p, k0, k1,
                (float*)h->tt_F.p, (float2*)h->tt_BS.p, d_mask, d_probs, (unsigned long long*)h->tt_count.p);
            CU(h, cudaGetLastError());
            continue;
        }
        const unsigned blocks = (unsigned)((k1 - k0 + kTtWarps - 1) / kTtWarps);
        k_tantan<0><<<blocks, kTtWarps * 32, 0, h->stream>>>(
            M, d_codes, d_offs, (const uint32_t*)h->tt_ord.p, (const uint64_t*)h->tt_base.p, k0, k1,
            (float*)h->tt_F.p, (float2*)h->tt_BS.p, d_mask, d_probs, (unsigned long long*)h->tt_count.p);
        CU(h, cudaGetLastError());
    }
    unsigned long long total = 0;
    CU(h, cudaMemcpyAsync(&total, h->tt_count.p, sizeof(total), cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    *n_masked = total;
    return SABER_OK;
}

int tantan_mask_host(saber_gpu* h, const saber_tantan_params* p, const int32_t* matrix576, const uint8_t* codes,
                     const uint64_t* offsets, uint64_t nseq, uint8_t* mask, float* probs, uint64_t* n_masked,
                     double* lambda_out) {
    if (!offsets || (nseq && !codes) || !mask || !n_masked) return fail(h, SABER_ERR_ARG, "null argument");
    TantanModel M;
    double lambda;
    int rc = tantan_model(h, matrix576, p, M, lambda);
    if (rc) return rc;
    if (lambda_out) *lambda_out = lambda;
    const uint64_t n0 = nseq ? offsets[0] : 0;
    const uint64_t total = nseq ? offsets[nseq] - n0 : 0;
    for (uint64_t i = 0; i < nseq; i++)
        if (offsets[i + 1] < offsets[i]) return fail(h, SABER_ERR_ARG, "offsets must be non-decreasing");
    *n_masked = 0;
    if (total == 0) return SABER_OK;
    std::vector<uint64_t> rel(nseq + 1);
    for (uint64_t i = 0; i <= nseq; i++) rel[i] = offsets[i] - n0;
    CUALLOC(h, h->tt_codes, total);
    CUALLOC(h, h->tt_offs, (nseq + 1) * sizeof(uint64_t));
    CUALLOC(h, h->tt_mask, total);
    if (probs) CUALLOC(h, h->tt_probs, total * sizeof(float));
    CU(h, cudaMemcpyAsync(h->tt_codes.p, codes + n0, total, cudaMemcpyHostToDevice, h->stream));
    CU(h, cudaMemcpyAsync(h->tt_offs.p, rel.data(), (nseq + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                          h->stream));
    rc = tantan_run(h, M, (const uint8_t*)h->tt_codes.p, rel.data(), (const uint64_t*)h->tt_offs.p, nseq,
                    (uint8_t*)h->tt_mask.p, probs ? (float*)h->tt_probs.p : nullptr, n_masked);
    if (rc) return rc;
    CU(h, cudaMemcpyAsync(mask + n0, h->tt_mask.p, total, cudaMemcpyDeviceToHost, h->stream));
    if (probs)
        CU(h, cudaMemcpyAsync(probs + n0, h->tt_probs.p, total * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    return SABER_OK;
}

int tantan_mask_db(saber_gpu* h, const saber_tantan_params* p, const int32_t* matrix576, uint64_t* n_masked,
                   double* lambda_out) {
    if (!n_masked) return fail(h, SABER_ERR_ARG, "null argument");
    if (!h->main.has_db) return fail(h, SABER_ERR_ARG, "no database loaded");
    TantanModel M;
    double lambda;
    int rc = tantan_model(h, matrix576, p, M, lambda);
    if (rc) return rc;
    if (lambda_out) *lambda_out = lambda;
    const uint64_t nsub = h->main.nsub, nres = h->main.n_res;
    std::vector<uint64_t> offs(nsub + 1);
    CU(h, cudaMemcpyAsync(offs.data(), h->main.soff.p, (nsub + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                          h->stream));
    CU(h, cudaStreamSynchronize(h->stream));
    CUALLOC(h, h->db_mask, nres + 64);
    CU(h, cudaMemsetAsync(h->db_mask.p, 0, nres + 64, h->stream));
    rc = tantan_run(h, M, (const uint8_t*)h->main.res.p, offs.data(), (const uint64_t*)h->main.soff.p, nsub,
                    (uint8_t*)h->db_mask.p, nullptr, n_masked);
    if (rc) return rc;
    h->sc_key = 0;  // the scan's database state depends on the mask
    h->has_db_mask = true;
    return SABER_OK;
}

}  // namespace saber
