// Banded affine-gap Smith-Waterman score kernels for sm_103a.
//
// Semantics: the reference's banded_score (src/algorithm/banded.rs:134-224,
// dispatched at banded.rs:408-449): the optimal local alignment restricted to
// lo <= j - i <= hi, with SABER's recurrences
//   E(i,j) = max(H(i,j-1) - go, E(i,j-1) - ge)
//   F(i,j) = max(H(i-1,j) - go, F(i-1,j) - ge)
//   H(i,j) = max(0, H(i-1,j-1) + S(q_i,s_j) + bias_i, E(i,j), F(i,j))
//
// Fast kernel (k_band_fast): one warp takes 32 pairs of jobs of one query,
// each lane two jobs held in the two int16 halves of every register (DPX
// s16x2 max/add instructions), and sweeps the band as strips of R query rows
// along the subject window.  Per strip the lane keeps H(i, j-1) and E(i, j-1)
// of its R rows in registers; the H/F values of the row above the strip come
// from a per-lane boundary buffer (indexed by band offset k = j - i - lo) in
// global memory, laid out [k][lane] so a warp reads and writes 256 contiguous
// bytes per step.  All lanes of a warp run the same column schedule, so the
// rows entering the band at the left edge are handled by compile-time
// unrolling and only the ragged right edge (different band widths) is masked.
// Substitution scores come from a per-query profile P[c][i] = S(q_i, c) +
// bias_i (int16, built at query upload) — one 16-byte load per 8 rows.
//
// Cells outside the window (j < 0 or j >= n) and rows past the query end use
// a sentinel code whose profile value is kSent16; such cells only ever hold
// values below the band optimum and never feed an in-window cell (except the
// j = -1 column, which holds exactly H = 0 as the reference's "hd = 0 when
// j == 0" rule requires), so they need no masks.
//
// A job whose int16 best reaches kLimit16 is re-run by the int32 kernel
// (k_band_generic), as the reference re-runs its int16 kernel in int32
// (banded_simd.rs:581-583 -> banded.rs:435-439).
#include "band_common.cuh"

#include <cuda_runtime.h>

namespace saber {

__device__ __forceinline__ uint32_t pk2(int v) { return (uint32_t)(uint16_t)(int16_t)v * 0x10001u; }
__device__ __forceinline__ uint32_t pk2(int lo, int hi) {
    return (uint32_t)(uint16_t)(int16_t)lo | ((uint32_t)(uint16_t)(int16_t)hi << 16);
}
__device__ __forceinline__ int lo16(uint32_t v) { return (int)(int16_t)(v & 0xFFFFu); }
__device__ __forceinline__ int hi16(uint32_t v) { return (int)(int16_t)(v >> 16); }

struct PackedConsts {
    uint32_t ngo2, nge2, neg2;
};

// One cell pair of one row: updates E (row state), computes F and H.
__device__ __forceinline__ void cell(uint32_t& E, uint32_t Hleft, uint32_t Hup, uint32_t Fup,
                                     uint32_t diag, uint32_t sub, const PackedConsts& c,
                                     uint32_t& H, uint32_t& F) {
    uint32_t ee = __viaddmax_s16x2(E, c.nge2, c.neg2);      // max(E - ge, NEG)
    E = __viaddmax_s16x2(Hleft, c.ngo2, ee);                // max(H(i,j-1) - go, ...)
    uint32_t fe = __viaddmax_s16x2(Fup, c.nge2, c.neg2);
    F = __viaddmax_s16x2(Hup, c.ngo2, fe);                  // max(H(i-1,j) - go, ...)
    uint32_t ef = __vimax_s16x2_relu(E, F);                 // max(E, F, 0)
    H = __viaddmax_s16x2_relu(diag, sub, ef);               // max(diag + S, E, F, 0)
}

template <int R>
struct StripState {
    uint32_t Hd[R];  // H(row r, previous column)
    uint32_t E[R];   // E(row r, previous column)
};

struct LaneJob {
    const uint8_t* win;  // window start (may be null when n == 0)
    int n;               // window length
    int lo;              // clipped band lo
    int w;               // clipped band width
};

__device__ __forceinline__ int load_code(const LaneJob& j, int col) {
    return ((unsigned)col < (unsigned)j.n) ? (int)__ldg(j.win + col) : kSentCode;
}

// Loads the packed substitution scores of R rows (starting at the strip's
// first row) for the two halves' residue codes.
template <int R>
__device__ __forceinline__ void load_sub(const int16_t* __restrict__ prof, int mpad, int i0, int ca,
                                         int cb, uint32_t (&sub)[R]) {
    const uint4* pa = reinterpret_cast<const uint4*>(prof + (size_t)ca * mpad + i0);
    const uint4* pb = reinterpret_cast<const uint4*>(prof + (size_t)cb * mpad + i0);
#pragma unroll
    for (int g = 0; g < R / 8; g++) {
        uint4 a = __ldg(pa + g);
        uint4 b = __ldg(pb + g);
        sub[8 * g + 0] = __byte_perm(a.x, b.x, 0x5410);
        sub[8 * g + 1] = __byte_perm(a.x, b.x, 0x7632);
        sub[8 * g + 2] = __byte_perm(a.y, b.y, 0x5410);
        sub[8 * g + 3] = __byte_perm(a.y, b.y, 0x7632);
        sub[8 * g + 4] = __byte_perm(a.z, b.z, 0x5410);
        sub[8 * g + 5] = __byte_perm(a.z, b.z, 0x7632);
        sub[8 * g + 6] = __byte_perm(a.w, b.w, 0x5410);
        sub[8 * g + 7] = __byte_perm(a.w, b.w, 0x7632);
    }
}

// Mask of the halves whose row r is still inside its band at this step
// (row r is in band while r >= thr_half, thr = u - w + 1).
__device__ __forceinline__ uint32_t ragged_mask(int r, int thr_a, int thr_b) {
    uint32_t ma = (r >= thr_a) ? 0x0000FFFFu : 0u;
    uint32_t mb = (r >= thr_b) ? 0xFFFF0000u : 0u;
    return ma | mb;
}

// One column step of a strip.  MODE 0: left triangle, rows 0..U computed
// (compile-time U); MODE 1: all rows, no masks; MODE 2: all rows, ragged
// right-edge masks.
template <int R, int MODE, int U>
__device__ __forceinline__ void strip_step(StripState<R>& st, uint32_t& diag0, uint2* __restrict__ buf,
                                           int u, int wmax, const uint32_t (&sub)[R],
                                           const PackedConsts& c, uint32_t& best, int thr_a,
                                           int thr_b) {
    int kin = u + 1 <= wmax ? u + 1 : wmax;
    uint2 top = buf[(size_t)kin * 32];
    uint32_t Hup = top.x, Fup = top.y;
    uint32_t diag = diag0;
    diag0 = top.x;
#pragma unroll
    for (int r = 0; r < R; r++) {
        if (MODE == 0 && r > U) break;
        uint32_t H, F;
        uint32_t hold = st.Hd[r];
        cell(st.E[r], hold, Hup, Fup, diag, sub[r], c, H, F);
        if (MODE == 2) {
            uint32_t mk = ragged_mask(r, thr_a, thr_b);
            H = (H & mk) | (c.neg2 & ~mk);
            F = (F & mk) | (c.neg2 & ~mk);
        }
        diag = hold;
        st.Hd[r] = H;
        Hup = H;
        Fup = F;
        best = __vimax_s16x2_relu(best, H);
    }
    if (MODE != 0 || U == R - 1) {
        int kout = u - R + 1;
        buf[(size_t)kout * 32] = make_uint2(Hup, Fup);
    }
}

template <int R, int U>
struct LeftTriangle {
    __device__ __forceinline__ static void run(StripState<R>& st, uint32_t& diag0, uint2* buf, int wmax,
                                               const int16_t* prof, int mpad, int i0,
                                               const LaneJob& ja, const LaneJob& jb,
                                               const PackedConsts& c, uint32_t& best) {
        LeftTriangle<R, U - 1>::run(st, diag0, buf, wmax, prof, mpad, i0, ja, jb, c, best);
        uint32_t sub[R];
        int ca = load_code(ja, ja.lo + i0 + U);
        int cb = load_code(jb, jb.lo + i0 + U);
        load_sub<R>(prof, mpad, i0, ca, cb, sub);
        strip_step<R, 0, U>(st, diag0, buf, U, wmax, sub, c, best, 0, 0);
    }
};
template <int R>
struct LeftTriangle<R, -1> {
    __device__ __forceinline__ static void run(StripState<R>&, uint32_t&, uint2*, int, const int16_t*, int,
                                               int, const LaneJob&, const LaneJob&, const PackedConsts&,
                                               uint32_t&) {}
};

struct FastTask {
    uint32_t pair_begin;  // index of the first pair in the pair list
};

// Persistent warps over warp tasks (32 pairs of one query each).
// pairs[p] = (sorted position of the first job, 1 or 2 jobs).
template <int R>
__global__ void __launch_bounds__(256) k_band_fast(
    const uint8_t* __restrict__ res, const int16_t* __restrict__ prof,
    const uint64_t* __restrict__ prof_off, const uint32_t* __restrict__ prof_mpad,
    const uint64_t* __restrict__ qoffs, const saber_band_job* __restrict__ jobs,
    const uint32_t* __restrict__ order, const uint2* __restrict__ pairs,
    const uint32_t* __restrict__ wtask_pair, const uint32_t* __restrict__ counts,
    uint32_t* __restrict__ wt_counter, uint2* __restrict__ bufs, uint32_t buf_stride, int go, int ge,
    int32_t* __restrict__ scores, uint32_t* __restrict__ rescue, uint32_t* __restrict__ rescue_count,
    uint32_t rescue_base) {
    const int lane = threadIdx.x & 31;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint2* mybuf = bufs + (size_t)gwarp * buf_stride * 32 + lane;
    const uint32_t n_wtasks = counts[3];
    const uint32_t n_pairs = counts[2];
    PackedConsts c;
    c.ngo2 = pk2(-go);
    c.nge2 = pk2(-ge);
    c.neg2 = pk2(kNeg16);

    for (;;) {
        uint32_t wt = 0;
        if (lane == 0) wt = atomicAdd(wt_counter, 1u);
        wt = __shfl_sync(0xffffffffu, wt, 0);
        if (wt >= n_wtasks) break;
        const uint32_t p0 = wtask_pair[wt];
        if (p0 >= n_pairs) continue;  // defensive: never index past the pair list
        const uint32_t qid = jobs[order[pairs[p0].x]].query;
        const uint32_t p = p0 + lane;
        bool has_pair = p < n_pairs;
        uint2 pr = has_pair ? pairs[p] : make_uint2(0, 0);
        uint32_t ja_idx = 0, jb_idx = 0;
        bool has_a = false, has_b = false;
        if (has_pair) {
            ja_idx = order[pr.x];
            has_a = jobs[ja_idx].query == qid;
            if (has_a && pr.y == 2) {
                jb_idx = order[pr.x + 1];
                has_b = true;
            }
        }
        const uint64_t q0 = qoffs[qid];
        const int m = (int)(qoffs[qid + 1] - q0);
        const int16_t* qprof = prof + prof_off[qid];
        const int mpad = (int)prof_mpad[qid];

        LaneJob ja{nullptr, 0, 0, 0}, jb{nullptr, 0, 0, 0};
        int first_a = 1 << 30, last_a = -1, first_b = 1 << 30, last_b = -1;
        if (has_a) {
            saber_band_job jj = jobs[ja_idx];
            int64_t lo = jj.band_lo, hi = jj.band_hi;
            int64_t w = clip_band(m, jj.win_len, lo, hi);
            ja.win = res + jj.win_begin;
            ja.n = (int)jj.win_len;
            ja.lo = (int)lo;
            ja.w = (int)w;
            first_a = (int)(hi < 0 ? -hi : 0);
            int64_t la = (int64_t)jj.win_len - 1 - lo;
            last_a = (int)(la < m - 1 ? la : m - 1);
        }
        if (has_b) {
            saber_band_job jj = jobs[jb_idx];
            int64_t lo = jj.band_lo, hi = jj.band_hi;
            int64_t w = clip_band(m, jj.win_len, lo, hi);
            jb.win = res + jj.win_begin;
            jb.n = (int)jj.win_len;
            jb.lo = (int)lo;
            jb.w = (int)w;
            first_b = (int)(hi < 0 ? -hi : 0);
            int64_t lb = (int64_t)jj.win_len - 1 - lo;
            last_b = (int)(lb < m - 1 ? lb : m - 1);
        }
        const int big = 1 << 30;
        int wmin_l = min(has_a ? ja.w : big, has_b ? jb.w : big);
        int wmax_l = max(has_a ? ja.w : 0, has_b ? jb.w : 0);
        const int wmin = __reduce_min_sync(0xffffffffu, wmin_l);
        const int wmax = __reduce_max_sync(0xffffffffu, wmax_l);
        if (!has_a) ja.w = wmin;
        if (!has_b) jb.w = wmin;
        const int s_first = __reduce_min_sync(0xffffffffu, min(first_a, first_b)) / R;
        const int s_last = __reduce_max_sync(0xffffffffu, max(last_a, last_b)) / R;

        // Boundary of the row above the first strip: H = 0 (the reference's
        // hd = 0 on row 0), F unreachable; position wmax is outside every band.
        for (int k = 0; k < wmax; k++) mybuf[(size_t)k * 32] = make_uint2(0u, c.neg2);
        mybuf[(size_t)wmax * 32] = make_uint2(c.neg2, c.neg2);

        uint32_t best = 0;
        for (int s = s_first; s <= s_last; s++) {
            const int i0 = s * R;
            StripState<R> st;
#pragma unroll
            for (int r = 0; r < R; r++) {
                st.Hd[r] = c.neg2;
                st.E[r] = c.neg2;
            }
            uint32_t diag0 = mybuf[0].x;
            LeftTriangle<R, R - 1>::run(st, diag0, mybuf, wmax, qprof, mpad, i0, ja, jb, c, best);
            int u = R;
            for (; u < wmin; u++) {
                uint32_t sub[R];
                int ca = load_code(ja, ja.lo + i0 + u);
                int cb = load_code(jb, jb.lo + i0 + u);
                load_sub<R>(qprof, mpad, i0, ca, cb, sub);
                strip_step<R, 1, 0>(st, diag0, mybuf, u, wmax, sub, c, best, 0, 0);
            }
            const int uend = wmax + R - 1;
            for (; u < uend; u++) {
                uint32_t sub[R];
                int ca = load_code(ja, ja.lo + i0 + u);
                int cb = load_code(jb, jb.lo + i0 + u);
                load_sub<R>(qprof, mpad, i0, ca, cb, sub);
                strip_step<R, 2, 0>(st, diag0, mybuf, u, wmax, sub, c, best, u - ja.w + 1,
                                    u - jb.w + 1);
            }
        }
        int sa = lo16(best), sb = hi16(best);
        if (has_a) {
            if (sa >= kLimit16) {
                uint32_t slot = atomicAdd(rescue_count, 1u);
                rescue[rescue_base + slot] = ja_idx;
            } else {
                scores[ja_idx] = sa;
            }
        }
        if (has_b) {
            if (sb >= kLimit16) {
                uint32_t slot = atomicAdd(rescue_count, 1u);
                rescue[rescue_base + slot] = jb_idx;
            } else {
                scores[jb_idx] = sb;
            }
        }
    }
}

// int32 kernel, one job per thread: the scalar recurrence of
// banded.rs:134-224 with H/F rows in a per-thread global slab.  Used for
// bands narrower than a strip and to rescore int16 results at the limit.
__global__ void __launch_bounds__(128) k_band_generic(
    const uint8_t* __restrict__ res, const int16_t* __restrict__ prof,
    const uint64_t* __restrict__ prof_off, const uint32_t* __restrict__ prof_mpad,
    const uint64_t* __restrict__ qoffs, const saber_band_job* __restrict__ jobs,
    const uint32_t* __restrict__ list, const uint32_t* __restrict__ list_count, int32_t* __restrict__ slabs,
    uint32_t slab_stride, int go, int ge, int32_t* __restrict__ scores) {
    const int NEG = INT32_MIN / 4;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t n = *list_count;
    int32_t* hp = slabs + (size_t)tid * slab_stride * 4;
    int32_t* fp = hp + slab_stride;
    int32_t* hc = fp + slab_stride;
    int32_t* fc = hc + slab_stride;
    for (uint32_t t = tid; t < n; t += nthreads) {
        const uint32_t jid = list[t];
        const saber_band_job jj = jobs[jid];
        const uint32_t q = jj.query;
        const int64_t m = (int64_t)(qoffs[q + 1] - qoffs[q]);
        const int64_t nn = jj.win_len;
        int64_t lo = jj.band_lo, hi = jj.band_hi;
        const int64_t w = clip_band(m, nn, lo, hi);
        if (w == 0) {
            scores[jid] = 0;
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
            a_hp[k] = NEG;
            a_fp[k] = NEG;
            a_hc[k] = NEG;
            a_fc[k] = NEG;
        }
        int32_t best = 0;
        for (int64_t i = 0; i < m; i++) {
            int64_t kmin = -(i + lo);
            if (kmin < 0) kmin = 0;
            int64_t kmax = nn - 1 - i - lo;
            if (kmax > w - 1) kmax = w - 1;
            if (kmin > kmax) {
                for (int64_t k = 0; k < w; k++) {
                    a_hc[k] = NEG;
                    a_fc[k] = NEG;
                }
            } else {
                int32_t e = NEG, h_left = NEG;
                const int64_t base = i + lo;
                for (int64_t k = kmin; k <= kmax; k++) {
                    const int64_t j = base + k;
                    int32_t ecand = max(h_left - go, e - ge);
                    e = k > kmin ? ecand : NEG;
                    int32_t f = i >= 1 ? max(a_hp[k + 1] - go, a_fp[k + 1] - ge) : NEG;
                    int32_t hd = (i >= 1 && j >= 1) ? a_hp[k] : 0;
                    int32_t sub = (int32_t)qprof[(size_t)s[j] * mpad + i];
                    int32_t diag = hd + sub;
                    int32_t h = max(max(max(diag, e), f), 0);
                    a_hc[k] = h;
                    a_fc[k] = f;
                    h_left = h;
                    best = max(best, h);
                }
                for (int64_t k = 0; k < kmin; k++) {
                    a_hc[k] = NEG;
                    a_fc[k] = NEG;
                }
                for (int64_t k = kmax + 1; k < w; k++) {
                    a_hc[k] = NEG;
                    a_fc[k] = NEG;
                }
            }
            int32_t* tmp = a_hp;
            a_hp = a_hc;
            a_hc = tmp;
            tmp = a_fp;
            a_fp = a_fc;
            a_fc = tmp;
        }
        scores[jid] = best;
    }
}

// ---- host-side launch wrappers (the runtime TU calls these) ----
int band_fast_blocks_per_sm() {
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_band_fast<kStripRows>, 256, 0) != cudaSuccess)
        return 1;
    return bps < 1 ? 1 : bps;
}

cudaError_t launch_band_fast(unsigned grid, cudaStream_t s, const FastArgs& a) {
    k_band_fast<kStripRows><<<grid, 256, 0, s>>>(a.res, a.prof, a.prof_off, a.prof_mpad, a.qoffs, a.jobs,
                                                 a.order, a.pairs, a.wtask_pair, a.counts, a.wt_counter,
                                                 a.bufs, a.buf_stride, a.go, a.ge, a.scores, a.rescue,
                                                 a.rescue_count, 0u);
    return cudaGetLastError();
}

cudaError_t launch_band_generic(unsigned grid, unsigned block, cudaStream_t s, const GenericArgs& a) {
    k_band_generic<<<grid, block, 0, s>>>(a.res, a.prof, a.prof_off, a.prof_mpad, a.qoffs, a.jobs, a.list,
                                          a.list_count, a.slabs, a.slab_stride, a.go, a.ge, a.scores);
    return cudaGetLastError();
}

}  // namespace saber
