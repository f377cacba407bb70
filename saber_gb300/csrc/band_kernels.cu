// Banded affine-gap Smith-Waterman score kernels for sm_103a.
//
// Semantics: the reference's banded_score (src/algorithm/banded.rs:134-224,
// dispatched at banded.rs:408-449): the optimal local alignment restricted to
// lo <= j - i <= hi, with SABER's recurrences
//   E(i,j) = max(H(i,j-1) - go, E(i,j-1) - ge)
//   F(i,j) = max(H(i-1,j) - go, F(i-1,j) - ge)
//   H(i,j) = max(0, H(i-1,j-1) + S(q_i,s_j) + bias_i, E(i,j), F(i,j))
//
// Fast kernel (k_band_fast<R>): a warp takes 64 jobs (consecutive in the
// (strips, width, query) order the runtime sorts them in); each lane holds
// two independent jobs in the two int16 halves of every register and
// updates both with one DPX s16x2 instruction per operation.  A job is swept
// as strips of R query rows along its subject window: per strip the lane
// keeps G(i, j-1) = H(i, j-1) - go and E(i, j-1) of its R rows in registers,
// and the G/F values of the row above the strip come from a per-lane boundary buffer
// indexed by band offset k = j - i - lo, laid out [k][lane] so the warp
// reads and writes 256 contiguous bytes per step.  All lanes run the same
// column schedule: the rows entering the band at its left edge are handled
// by compile-time unrolling, the middle steps need no masks, and only the
// right edge (band widths differ within a warp) is masked per half.  The
// boundary value, residue codes and substitution scores of a step are
// fetched one to two steps ahead.  Substitution scores come from per-query
// profiles P[c][i] = S(q_i, c) + bias_i + go built at query upload (the
// packed cell adds them to G = H - go): an int8 copy (sentinel -128) when
// every entry of the query set lies in [-127, 127], one 16-byte load per 16
// rows and step, else the int16 profile, one 32-byte load.  The L1 data pipe
// bounds the kernel, so the int8 copy's half-size loads are what set its
// speed; one byte permute with sign replication widens them.
//
// Cells outside the window (j < 0 or j >= n), rows past the query end and
// the strips of a half that has finished use a sentinel code / sentinel
// profile whose value is kSent16 (+ go in the query profiles): such cells
// only ever hold values below the
// band optimum and never feed an in-window cell (except the j = -1 column,
// which holds exactly H = 0 as the reference's "hd = 0 when j == 0" rule
// requires), so they need no masks.
//
// A job whose int16 best reaches kLimit16 is re-run by the int32 kernel
// (k_band_generic), as the reference re-runs its int16 kernel in int32
// (banded_simd.rs:581-583 -> banded.rs:435-439).
#include "band_common.cuh"

#include <cuda_runtime.h>

namespace saber {

// Boundary-row stores: plain write-back stores, so that the lane's later
// loads of the same entries (cached in L1) see them.
template <class T>
__device__ __forceinline__ void stbuf(T* p, T v) { *p = v; }

__device__ __forceinline__ uint32_t pk2(int v) { return (uint32_t)(uint16_t)(int16_t)v * 0x10001u; }
__device__ __forceinline__ int lo16(uint32_t v) { return (int)(int16_t)(v & 0xFFFFu); }
__device__ __forceinline__ int hi16(uint32_t v) { return (int)(int16_t)(v >> 16); }

// R int16 sentinel profile entries: the profile of a half whose job has no
// strip left (32-byte aligned for the vector loads).
__device__ __align__(32) int16_t g_sent_profile[64] = {
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16,
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16,
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16,
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16,
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16,
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16,
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16,
    kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16, kSent16};

// The same for the int8 profiles: -128 is their sentinel score (S + bias +
// go of every real entry lies in [-127, 127]).
__device__ __align__(32) int8_t g_sent_profile8[64] = {
    -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128,
    -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128,
    -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128,
    -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128, -128,
};

template <class T>
__device__ __forceinline__ const T* sent_profile();
template <>
__device__ __forceinline__ const int16_t* sent_profile<int16_t>() { return g_sent_profile; }
template <>
__device__ __forceinline__ const int8_t* sent_profile<int8_t>() { return g_sent_profile8; }

struct PackedConsts {
    uint32_t ngo2, nge2, neg2, go2;
};

// One cell pair of one row.  The kernel keeps G = H - go instead of H (the
// value both gap recurrences open from) and E, F unshifted, and the profile
// holds S + bias + go:
//   E(i,j) = max(E(i,j-1) - ge, G(i,j-1))
//   F(i,j) = max(F(i-1,j) - ge, G(i-1,j))
//   H(i,j) = max(E, F, G(i-1,j-1) + (S + go), 0),   G(i,j) = H(i,j) - go
// so that a cell is three DPX instructions on the ALU pipe (two fused
// add-max, one three-input max with relu) and two packed adds on the FMA
// pipe (the diagonal sum and G), which issue beside them.  In-band values
// stay inside int16 without clamping: G >= kNeg16 (the unreachable value of
// cells outside the band) and the profile >= kSent16, so the diagonal sum is
// >= -32000; below kLimit16 it is < 32767 (|S + bias| <= 767, go <= 1000).
// E and F start at kNeg16 and never fall below it (E >= G), and where the
// reference holds E or F at its NEG sentinel these hold values <= 0, which
// no H can tell apart (H is clamped at 0).
__device__ __forceinline__ void cell(uint32_t& E, uint32_t Gleft, uint32_t Gup, uint32_t Fup,
                                     uint32_t gdiag, uint32_t sub, const PackedConsts& c,
                                     uint32_t& G, uint32_t& F) {
    E = __viaddmax_s16x2(E, c.nge2, Gleft);
    F = __viaddmax_s16x2(Fup, c.nge2, Gup);
    const uint32_t ds = __vadd2(gdiag, sub);
    const uint32_t H = __vimax3_s16x2_relu(E, F, ds);
    G = __vadd2(H, c.ngo2);
}

template <int R>
struct StripState {
    uint32_t Gd[R];  // G = H - go of (row r, previous column)
    uint32_t E[R];   // E(row r, previous column)
};

// One job of a half: its window, clipped band and rows.  T is the profile's
// element type: int16 S + bias + go, or int8 where every entry fits.
template <class T>
struct HalfJob {
    const T* prof;        // query profile (rows c = 0..24, stride mpad)
    const uint8_t* win;   // window start (unused when n == 0)
    int mpad;
    int n;                // window length (0: every column is a sentinel)
    int lo;               // clipped band lo
    int w;                // clipped band width
    int s0;               // first strip
    int ns;               // number of strips
};

// Per-strip view of a half: profile row base for this strip's rows.
template <class T>
struct HalfStrip {
    const T* rows;        // prof + i0 (sentinel block when the half is done)
    const uint8_t* win;
    int mpad;
    int n;
    int col0;             // window column of step 0 (= lo + i0)
};

template <class T>
__device__ __forceinline__ HalfStrip<T> half_strip(const HalfJob<T>& h, int t, int R) {
    HalfStrip<T> v;
    if (t < h.ns) {
        int i0 = (h.s0 + t) * R;
        v.rows = h.prof + i0;
        v.win = h.win;
        v.mpad = h.mpad;
        v.n = h.n;
        v.col0 = h.lo + i0;
    } else {
        v.rows = sent_profile<T>();
        v.win = nullptr;
        v.mpad = 0;
        v.n = 0;
        v.col0 = 0;
    }
    return v;
}

// Residue codes of steps u .. u + 3 of a strip (window columns col0 + u ..),
// one byte each, the sentinel code outside the window.  Interior groups take
// one or two aligned 32-bit loads; the residue buffer is padded past its end,
// so the second word never leaves the allocation.
template <class T>
__device__ __forceinline__ uint32_t code_word(const HalfStrip<T>& h, int u) {
    const int c = h.col0 + u;
    if (c >= 0 && c + 4 <= h.n) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(h.win + c);
        const uint32_t* p = reinterpret_cast<const uint32_t*>(a & ~(uintptr_t)3);
        const uint32_t sh = (uint32_t)(a & 3u) * 8u;
        const uint32_t w0 = __ldg(p);
        const uint32_t w1 = sh ? __ldg(p + 1) : 0u;
        return __funnelshift_r(w0, w1, sh);
    }
    if (c + 4 <= 0 || c >= h.n) return 0x01010101u * kSentCode;
    uint32_t r = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int col = c + i;
        const uint32_t b = ((unsigned)col < (unsigned)h.n) ? (uint32_t)__ldg(h.win + col) : (uint32_t)kSentCode;
        r |= b << (8 * i);
    }
    return r;
}

// Raw profile words of one step for both halves (R rows of T each: 32, 16
// or 8 bytes).
template <int R, class T>
struct StepLoads {
    static constexpr int kW = R * (int)sizeof(T) / 4;
    uint32_t a[kW];
    uint32_t b[kW];
    uint2 top;  // (G, F) of the row above at band offset u + 1
};

// Read-only load of one half's profile words for a step: one request per
// lane (32-byte loads exist on sm_100 and later).
template <int W>
__device__ __forceinline__ void ld_prof(uint32_t (&d)[W], const void* p) {
    if constexpr (W == 8) {
        asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
            : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]), "=r"(d[6]), "=r"(d[7])
            : "l"(p));
    } else if constexpr (W == 4) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
        d[3] = v.w;
    } else {
        static_assert(W == 2, "8, 16 or 32 bytes of profile per half and step");
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
        d[0] = v.x;
        d[1] = v.y;
    }
}

template <int R, class T>
__device__ __forceinline__ void fetch_step(StepLoads<R, T>& L, const HalfStrip<T>& ha, const HalfStrip<T>& hb,
                                           int ca, int cb, const uint2* __restrict__ buf, int kin) {
    static_assert(R == 8 || R == 16, "strip rows are 8 or 16");
    ld_prof(L.a, ha.rows + (size_t)ca * ha.mpad);
    ld_prof(L.b, hb.rows + (size_t)cb * hb.mpad);
    L.top = __ldca(buf + (size_t)kin * 32);  // boundary rows: the lane's own writes, cached in L1
}

// Byte permute with the selector's sign-replicate bit (PTX prmt, default
// mode): a selector nibble 8 | b writes the sign of source byte b.
__device__ __forceinline__ uint32_t prmt(uint32_t x, uint32_t y, uint32_t sel) {
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(x), "r"(y), "r"(sel));
    return d;
}

// Packed substitution scores (half a low, half b high) of row r of a step:
// one byte permute per row, from int16 pairs or, with sign extension, from
// int8 quads.
template <int R, class T>
__device__ __forceinline__ uint32_t sub_of(const StepLoads<R, T>& L, int r) {
    if constexpr (sizeof(T) == 2) {
        const uint32_t x = L.a[r / 2], y = L.b[r / 2];
        return (r & 1) ? __byte_perm(x, y, 0x7632) : __byte_perm(x, y, 0x5410);
    } else {
        const uint32_t x = L.a[r / 4], y = L.b[r / 4];
        const uint32_t k = (uint32_t)(r & 3);
        return prmt(x, y, k | ((8u | k) << 4) | ((4u + k) << 8) | ((12u + k) << 12));
    }
}

// Right-edge masks: a half's row r is in band while r >= thr (thr = u - w +
// 1).  ragged_nthr packs -thr of both halves, thr clamped to [0, rows] so
// that r - thr fits int16 (once per step); ragged_out gives 0xFFFF in the
// halves whose row r is out of band: one packed add (FMA pipe) and one
// permute that replicates each half's sign.
__device__ __forceinline__ uint32_t ragged_nthr(int thr_a, int thr_b, int rows) {
    thr_a = min(max(thr_a, 0), rows);
    thr_b = min(max(thr_b, 0), rows);
    return (uint32_t)(uint16_t)(-thr_a) | ((uint32_t)(uint16_t)(-thr_b) << 16);
}
__device__ __forceinline__ uint32_t ragged_out(int r, uint32_t nthr2) {
    return prmt(__vadd2((uint32_t)r * 0x10001u, nthr2), 0u, 0xBB99u);
}

// One column step of a strip.  MODE 0: left triangle, rows 0..U computed
// (compile-time U); MODE 1: all rows, no masks; MODE 2: all rows, ragged
// right-edge masks.  `best` is the running maximum of G (H - go) over the
// lane's in-band cells.
template <int R, class T, int MODE, int U>
__device__ __forceinline__ void strip_step(StripState<R>& st, uint32_t& diag0, uint2* __restrict__ buf, int u,
                                           const StepLoads<R, T>& L, const PackedConsts& c, uint32_t& best,
                                           int thr_a, int thr_b) {
    uint32_t Gup = L.top.x, Fup = L.top.y;
    uint32_t diag = diag0;
    diag0 = L.top.x;
    uint32_t gprev = 0;
    const uint32_t nthr2 = MODE == 2 ? ragged_nthr(thr_a, thr_b, R) : 0u;
#pragma unroll
    for (int r = 0; r < R; r++) {
        if (MODE == 0 && r > U) break;
        uint32_t G, F;
        uint32_t gold = st.Gd[r];
        cell(st.E[r], gold, Gup, Fup, diag, sub_of<R, T>(L, r), c, G, F);
        if (MODE == 2) {
            const uint32_t out = ragged_out(r, nthr2);
            G = (G & ~out) | (c.neg2 & out);
            F = (F & ~out) | (c.neg2 & out);
        }
        diag = gold;
        st.Gd[r] = G;
        Gup = G;
        Fup = F;
        // running best over row pairs: one three-input max per two rows
        if (r & 1) best = __vimax3_s16x2(best, gprev, G);
        else if (r == R - 1 || (MODE == 0 && r == U)) best = __vmaxs2(best, G);
        else gprev = G;
    }
    if (MODE != 0 || U == R - 1) stbuf(buf + (size_t)(u - R + 1) * 32, make_uint2(Gup, Fup));
}

// The pipelined column loop state of one strip: the loads of step u + 1 are
// in flight while step u computes; the residue codes come four steps to a
// word, the word of the next group loaded a group ahead.
template <int R, class T>
struct Pipe {
    StepLoads<R, T> cur, nxt;
    uint32_t wa, wb;    // codes of the group of step u + 1 (byte i: step 4g + i)
    uint32_t wa2, wb2;  // codes of the group after it
};

// Called before computing step u: cur <- nxt (step u), issue step u + 1.
// K = (u + 1) & 3 when known at compile time, else -1.
template <int R, class T, int K>
__device__ __forceinline__ void pipe_advance(Pipe<R, T>& p, const HalfStrip<T>& ha, const HalfStrip<T>& hb,
                                             const uint2* buf, int u, int wmax) {
    p.cur = p.nxt;
    const int v = u + 1;
    const int k = K >= 0 ? K : (v & 3);
    if (k == 0) {
        p.wa = p.wa2;
        p.wb = p.wb2;
        p.wa2 = code_word(ha, v + 4);
        p.wb2 = code_word(hb, v + 4);
    }
    const uint32_t sel = 0x4440u | (uint32_t)k;
    const int ca = (int)__byte_perm(p.wa, 0u, sel), cb = (int)__byte_perm(p.wb, 0u, sel);
    const int k1 = u + 2 <= wmax ? u + 2 : wmax;
    fetch_step<R, T>(p.nxt, ha, hb, ca, cb, buf, k1);
}

template <int R, class T, int U>
struct LeftTriangle {
    __device__ __forceinline__ static void run(StripState<R>& st, uint32_t& diag0, uint2* buf, int wmax,
                                               Pipe<R, T>& p, const HalfStrip<T>& ha, const HalfStrip<T>& hb,
                                               const PackedConsts& c, uint32_t& best) {
        LeftTriangle<R, T, U - 1>::run(st, diag0, buf, wmax, p, ha, hb, c, best);
        pipe_advance<R, T, (U + 1) & 3>(p, ha, hb, buf, U, wmax);
        strip_step<R, T, 0, U>(st, diag0, buf, U, p.cur, c, best, 0, 0);
    }
};
template <int R, class T>
struct LeftTriangle<R, T, -1> {
    __device__ __forceinline__ static void run(StripState<R>&, uint32_t&, uint2*, int, Pipe<R, T>&,
                                               const HalfStrip<T>&, const HalfStrip<T>&, const PackedConsts&,
                                               uint32_t&) {}
};

// ---- paired strips (one job per lane) --------------------------------------
// A job whose sweep as R-row strips would be long takes a whole lane: the
// lane sweeps super-strips of 2R rows, rows 0 .. R-1 in the low halves and
// rows R .. 2R-1 in the high halves one column behind, so the high half's row
// above (the low half's last row) comes from the previous step's registers
// and its residue code is the low half's code of the previous step.  The
// boundary buffer then carries one job per lane: 32-bit words G | F << 16
// of the super-strip's last row.  A warp task is 32 such jobs; the job's
// critical path is about half of its R-row sweep.
template <int R, class T>
struct PairPipe {
    StepLoads<R, T> cur, nxt;  // top.x: boundary word of the low half's row above
    uint32_t w, w2;         // code words of the low half: group of step g + 1, next group
    int cprev;              // low half's code at step g (the high half's at step g + 1)
    // int8 profiles: rows R .. 2R-1 of the low half's last 32-byte block, the
    // high half's rows at the next step (one load serves both halves)
    uint32_t hi[sizeof(T) == 1 ? StepLoads<R, T>::kW : 1];
};

// One aligned 2R-row block of an int8 profile at code c: rows 0 .. R-1 to lo,
// rows R .. 2R-1 to hi.
template <int R, class T>
__device__ __forceinline__ void ld_block(uint32_t (&lo)[StepLoads<R, T>::kW], uint32_t (&hi)[StepLoads<R, T>::kW],
                                         const T* p) {
    static_assert(sizeof(T) == 1 && R == 16, "one 32-byte load covers 32 int8 rows");
    uint32_t d[8];
    ld_prof(d, p);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        lo[i] = d[i];
        hi[i] = d[4 + i];
    }
}

// Called before computing step g: cur <- nxt (step g), issue step g + 1.
template <int R, class T, int K>
__device__ __forceinline__ void pair_advance(PairPipe<R, T>& p, const HalfStrip<T>& ha, const T* hb_rows,
                                             const uint32_t* pbuf, int g, int wmax) {
    p.cur = p.nxt;
    const int v = g + 1;
    const int k = K >= 0 ? K : (v & 3);
    if (k == 0) {
        p.w = p.w2;
        p.w2 = code_word(ha, v + 4);
    }
    const int ca = (int)__byte_perm(p.w, 0u, 0x4440u | (uint32_t)k);
    const int cb = p.cprev;
    p.cprev = ca;
    const int kin = g + 2 <= wmax ? g + 2 : wmax;
    if constexpr (sizeof(T) == 1) {
        // the high half's rows at code cb came with the low half's block last step
#pragma unroll
        for (int i = 0; i < StepLoads<R, T>::kW; i++) p.nxt.b[i] = p.hi[i];
        ld_block<R, T>(p.nxt.a, p.hi, ha.rows + (size_t)ca * ha.mpad);
    } else {
        ld_prof(p.nxt.a, ha.rows + (size_t)ca * ha.mpad);
        ld_prof(p.nxt.b, hb_rows + (size_t)cb * ha.mpad);
    }
    p.nxt.top.x = __ldca(pbuf + (size_t)kin * 32);
}

// One step g of a super-strip.  PH 0: compile-time step G <= 2R (low rows
// r > G not yet in band, high rows r > G - R - 1 not yet in band); PH 1: every
// row of both halves in band; PH 2: right-edge masks from the thresholds.
// Values are G = H - go and F, as in strip_step.
template <int R, class T, int PH, int G>
__device__ __forceinline__ void pair_step(StripState<R>& st, uint32_t& diag0, uint32_t& lastG, uint32_t& lastF,
                                          uint32_t* __restrict__ pbuf, int g, const StepLoads<R, T>& L,
                                          const PackedConsts& c, uint32_t& best, int thr_a, int thr_b) {
    const uint32_t top = L.top.x;
    uint32_t Gup = __byte_perm(top, lastG, 0x5410);
    uint32_t Fup = __byte_perm(top, lastF, 0x5432);
    uint32_t diag = diag0;
    diag0 = Gup;
    uint32_t gprev = 0;
    const uint32_t nthr2 = PH == 2 ? ragged_nthr(thr_a, thr_b, R) : 0u;
#pragma unroll
    for (int r = 0; r < R; r++) {
        if (PH == 0 && r > G) break;
        uint32_t Gv, F;
        uint32_t gold = st.Gd[r];
        cell(st.E[r], gold, Gup, Fup, diag, sub_of<R, T>(L, r), c, Gv, F);
        if (PH == 0 && r > G - R - 1) {
            Gv = (Gv & 0x0000FFFFu) | (c.neg2 & 0xFFFF0000u);
            F = (F & 0x0000FFFFu) | (c.neg2 & 0xFFFF0000u);
        }
        if (PH == 2) {
            const uint32_t out = ragged_out(r, nthr2);
            Gv = (Gv & ~out) | (c.neg2 & out);
            F = (F & ~out) | (c.neg2 & out);
        }
        diag = gold;
        st.Gd[r] = Gv;
        Gup = Gv;
        Fup = F;
        if (r & 1) best = __vimax3_s16x2(best, gprev, Gv);
        else if (r == R - 1 || (PH == 0 && r == G)) best = __vmaxs2(best, Gv);
        else gprev = Gv;
    }
    lastG = Gup;
    lastF = Fup;
    if (g >= 2 * R) stbuf(pbuf + (size_t)(g - 2 * R) * 32, __byte_perm(Gup, Fup, 0x7632));
}

template <int R, class T, int G>
struct PairTriangle {
    __device__ __forceinline__ static void run(PairPipe<R, T>& p, StripState<R>& st, uint32_t& diag0,
                                               uint32_t& lastG, uint32_t& lastF, uint32_t* pbuf, int wmax,
                                               const HalfStrip<T>& ha, const T* hb_rows, const PackedConsts& c,
                                               uint32_t& best) {
        PairTriangle<R, T, G - 1>::run(p, st, diag0, lastG, lastF, pbuf, wmax, ha, hb_rows, c, best);
        pair_advance<R, T, (G + 1) & 3>(p, ha, hb_rows, pbuf, G, wmax);
        pair_step<R, T, 0, G>(st, diag0, lastG, lastF, pbuf, G, p.cur, c, best, 0, 0);
    }
};
template <int R, class T>
struct PairTriangle<R, T, -1> {
    __device__ __forceinline__ static void run(PairPipe<R, T>&, StripState<R>&, uint32_t&, uint32_t&, uint32_t&,
                                               uint32_t*, int, const HalfStrip<T>&, const T*, const PackedConsts&,
                                               uint32_t&) {}
};

template <class T>
__device__ __forceinline__ void load_half(HalfJob<T>& h, const saber_band_job& j, const T* prof,
                                          const uint64_t* prof_off, const uint32_t* prof_mpad,
                                          const uint64_t* qoffs, const uint8_t* res, int R) {
    const uint32_t q = j.query;
    const int64_t m = (int64_t)(qoffs[q + 1] - qoffs[q]);
    int64_t lo = j.band_lo, hi = j.band_hi;
    int64_t w = clip_band(m, j.win_len, lo, hi);
    h.prof = prof + prof_off[q];
    h.mpad = (int)prof_mpad[q];
    h.win = res + j.win_begin;
    h.n = (int)j.win_len;
    h.lo = (int)lo;
    h.w = (int)w;
    int64_t first = hi < 0 ? -hi : 0;
    int64_t last = (int64_t)j.win_len - 1 - lo;
    if (last > m - 1) last = m - 1;
    h.s0 = (int)(first / R);
    h.ns = (int)(last / R - first / R + 1);
}

// One paired task: sorted positions [32t, 32t + 32) of the paired range,
// lane l takes position 32t + l.
template <int R, class T>
__device__ __noinline__ void pair_task(const uint8_t* __restrict__ res, const T* __restrict__ prof,
                                       const uint64_t* __restrict__ prof_off, const uint32_t* __restrict__ prof_mpad,
                                       const uint64_t* __restrict__ qoffs, const saber_band_job* __restrict__ jobs,
                                       const uint32_t* __restrict__ porder, uint32_t n_pair, uint32_t task, int lane,
                                       uint32_t* __restrict__ pbuf, const PackedConsts& c,
                                       int32_t* __restrict__ scores, uint32_t* __restrict__ rescue,
                                       uint32_t* __restrict__ rescue_count) {
    const uint32_t pos = task * 32 + lane;
    const bool has = pos < n_pair;
    const uint32_t jidx = has ? porder[pos] : 0u;
    HalfJob<T> J{sent_profile<T>(), nullptr, 0, 0, 0, 0, 0, 0};
    if (has) load_half(J, jobs[jidx], prof, prof_off, prof_mpad, qoffs, res, 2 * R);
    const int big = 1 << 30;
    const int wmin = __reduce_min_sync(0xffffffffu, has ? J.w : big);
    const int wmax = __reduce_max_sync(0xffffffffu, has ? J.w : 0);
    const int nsmax = __reduce_max_sync(0xffffffffu, J.ns);
    if (!has) J.w = wmin;
    const uint32_t top0 = (c.neg2 & 0xFFFF0000u) | (c.ngo2 & 0x0000FFFFu);  // G = -go (H = 0), F unreachable
    for (int k = 0; k < wmax; k++) stbuf(pbuf + (size_t)k * 32, top0);
    stbuf(pbuf + (size_t)wmax * 32, c.neg2);

    uint32_t best = c.ngo2;  // G of H = 0
    const int gfull = wmax + 2 * R;
    for (int t = 0; t < nsmax; t++) {
        const HalfStrip<T> ha = half_strip(J, t, 2 * R);
        const T* hb_rows = ha.rows + R;
        // Step g reads window column col0 + g in the low half and col0 + g - 1
        // in the high half.  As in the two-job lanes, the warp sweeps only the
        // steps that reach a window column of one of its jobs, a late start
        // being = 1 (mod 4) past the triangle, from rows of H = 0, with the
        // boundary entries of the skipped steps set as those steps would set
        // them.
        int s_lo = 1 << 30, s_hi = -1;
        if (ha.n > 0) {
            const int a0 = max(0, -ha.col0 - 1), a1 = min(gfull - 1, ha.n - ha.col0);
            if (a0 <= a1) {
                s_lo = a0;
                s_hi = a1;
            }
        }
        const int w_lo = __reduce_min_sync(0xffffffffu, s_lo), w_hi = __reduce_max_sync(0xffffffffu, s_hi);
        int g0 = 0, gend = gfull;
        if (w_hi >= 0 && w_lo <= w_hi) {
            g0 = ((w_lo - 1) & ~3) + 1;  // largest value = 1 (mod 4) not above w_lo
            if (g0 < 2 * R + 1) g0 = 0;
            gend = w_hi + 1 < gfull ? w_hi + 1 : gfull;
        }
        StripState<R> st;
        uint32_t diag0, lastG, lastF;
        PairPipe<R, T> p;
        int g;
        if (g0 == 0) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                st.Gd[r] = c.neg2;
                st.E[r] = c.neg2;
            }
            diag0 = __byte_perm(__ldca(pbuf), c.neg2, 0x5410);
            lastG = c.neg2;
            lastF = c.neg2;
            p.w = code_word(ha, 0);
            p.w2 = code_word(ha, 4);
            const int ca0 = (int)(p.w & 0xFFu);
            if constexpr (sizeof(T) == 1) ld_block<R, T>(p.nxt.a, p.hi, ha.rows + (size_t)ca0 * ha.mpad);
            else ld_prof(p.nxt.a, ha.rows + (size_t)ca0 * ha.mpad);
            ld_prof(p.nxt.b, hb_rows + (size_t)kSentCode * ha.mpad);
            p.nxt.top.x = __ldca(pbuf + 32);
            p.cprev = ca0;
            PairTriangle<R, T, 2 * R>::run(p, st, diag0, lastG, lastF, pbuf, wmax, ha, hb_rows, c, best);
            g = 2 * R + 1;
        } else {
#pragma unroll
            for (int r = 0; r < R; r++) {
                st.Gd[r] = c.ngo2;
                st.E[r] = c.neg2;
            }
            const int kskip = min(g0 - 2 * R, wmax);
            for (int k = 0; k < kskip; k++) stbuf(pbuf + (size_t)k * 32, top0);
            diag0 = c.ngo2;
            lastG = c.ngo2;
            lastF = c.neg2;
            // code words of the groups holding steps g0 - 1 .. g0 + 2 and the next
            p.w = code_word(ha, g0 - 1);
            p.w2 = code_word(ha, g0 + 3);
            const int ca0 = (int)((p.w >> 8) & 0xFFu);  // step g0 (= 1 mod 4)
            const int cb0 = (int)(p.w & 0xFFu);         // the high half's: the low half's at g0 - 1
            if constexpr (sizeof(T) == 1) ld_block<R, T>(p.nxt.a, p.hi, ha.rows + (size_t)ca0 * ha.mpad);
            else ld_prof(p.nxt.a, ha.rows + (size_t)ca0 * ha.mpad);
            ld_prof(p.nxt.b, hb_rows + (size_t)cb0 * ha.mpad);
            p.nxt.top.x = __ldca(pbuf + (size_t)(g0 + 1 <= wmax ? g0 + 1 : wmax) * 32);
            p.cprev = ca0;
            g = g0;
        }
        const int gmid = wmin < gend ? wmin : gend;
        // middle steps, one per iteration (the code byte's selector is a
        // register; a short loop body keeps the hot code in the instruction cache)
        for (; g < gmid; g++) {
            pair_advance<R, T, -1>(p, ha, hb_rows, pbuf, g, wmax);
            pair_step<R, T, 1, 0>(st, diag0, lastG, lastF, pbuf, g, p.cur, c, best, 0, 0);
        }
        for (; g < gend; g++) {
            pair_advance<R, T, -1>(p, ha, hb_rows, pbuf, g, wmax);
            pair_step<R, T, 2, 0>(st, diag0, lastG, lastF, pbuf, g, p.cur, c, best, g - J.w + 1, g - R - J.w);
        }
    }
    const int sc = max(lo16(best), hi16(best)) + lo16(c.go2);
    if (has) {
        if (sc >= kLimit16) rescue[atomicAdd(rescue_count, 1u)] = jidx;
        else scores[jidx] = sc;
    }
}

// Persistent warps over warp tasks: task t = sorted positions [64t, 64t + 64)
// of the fast class, taken largest first; lane l takes positions 64t + 2l
// (low half) and 64t + 2l + 1 (high half).
template <int R, class T>
__global__ void __launch_bounds__(256, 2) k_band_fast(
    const uint8_t* __restrict__ res, const T* __restrict__ prof,
    const uint64_t* __restrict__ prof_off, const uint32_t* __restrict__ prof_mpad,
    const uint64_t* __restrict__ qoffs, const saber_band_job* __restrict__ jobs,
    const uint32_t* __restrict__ order, const uint32_t* __restrict__ n_ptr, const uint32_t* __restrict__ np_ptr,
    const uint32_t* __restrict__ order_skip, uint32_t* __restrict__ wt_counter, uint2* __restrict__ bufs,
    uint32_t buf_stride, int go, int ge, int32_t* __restrict__ scores, uint32_t* __restrict__ rescue,
    uint32_t* __restrict__ rescue_count) {
    if (order_skip) order += *order_skip;
    const int lane = threadIdx.x & 31;
    const uint32_t gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint2* mybuf = bufs + (size_t)gwarp * buf_stride * 32 + lane;
    // sorted positions [0, n_fast - n_pair): R-row strips, two jobs per lane;
    // [n_fast - n_pair, n_fast): paired strips, one job per lane
    const uint32_t n_all = *n_ptr;
    const uint32_t n_pair = (R == 16 && np_ptr) ? *np_ptr : 0u;
    const uint32_t n_fast = n_all - n_pair;
    const uint32_t n_ptasks = (n_pair + 31) / 32;
    const uint32_t n_wtasks = (n_fast + 63) / 64;
    PackedConsts c;
    c.ngo2 = pk2(-go);
    c.nge2 = pk2(-ge);
    c.neg2 = pk2(kNeg16);
    c.go2 = pk2(go);

    for (;;) {
        uint32_t wt = 0;
        if (lane == 0) wt = atomicAdd(wt_counter, 1u);
        wt = __shfl_sync(0xffffffffu, wt, 0);
        if (wt >= n_ptasks + n_wtasks) break;
        // largest tasks first: paired tasks, then R-row tasks; each sorted
        // range is ascending in strips and width
        bool paired = false;
        if constexpr (R == 16) paired = wt < n_ptasks;
        if (paired) {
            if constexpr (R == 16)
                pair_task<R, T>(res, prof, prof_off, prof_mpad, qoffs, jobs, order + n_fast, n_pair, n_ptasks - 1 - wt,
                             lane, reinterpret_cast<uint32_t*>(bufs + (size_t)gwarp * buf_stride * 32) + lane, c,
                             scores, rescue, rescue_count);
            continue;
        }
        const uint32_t task = n_wtasks - 1 - (wt - n_ptasks);
        const uint32_t pa = task * 64 + 2 * lane, pb = pa + 1;
        const bool has_a = pa < n_fast, has_b = pb < n_fast;
        const uint32_t ja_idx = has_a ? order[pa] : 0u;
        const uint32_t jb_idx = has_b ? order[pb] : 0u;
        HalfJob<T> A{sent_profile<T>(), nullptr, 0, 0, 0, 0, 0, 0}, B{sent_profile<T>(), nullptr, 0, 0, 0, 0, 0, 0};
        if (has_a) load_half(A, jobs[ja_idx], prof, prof_off, prof_mpad, qoffs, res, R);
        if (has_b) load_half(B, jobs[jb_idx], prof, prof_off, prof_mpad, qoffs, res, R);
        const int big = 1 << 30;
        const int wmin = __reduce_min_sync(0xffffffffu, min(has_a ? A.w : big, has_b ? B.w : big));
        const int wmax = __reduce_max_sync(0xffffffffu, max(has_a ? A.w : 0, has_b ? B.w : 0));
        const int nsmax = __reduce_max_sync(0xffffffffu, max(A.ns, B.ns));
        if (!has_a) A.w = wmin;
        if (!has_b) B.w = wmin;

        // Boundary of the row above each job's first strip: H = 0 (the
        // reference's hd = 0 on row 0, stored as G = -go), F unreachable;
        // position wmax lies outside every band.
        for (int k = 0; k < wmax; k++) stbuf(mybuf + (size_t)k * 32, make_uint2(c.ngo2, c.neg2));
        stbuf(mybuf + (size_t)wmax * 32, make_uint2(c.neg2, c.neg2));

        uint32_t best = c.ngo2;  // G of H = 0
        const int ufull = wmax + R - 1;
        for (int t = 0; t < nsmax; t++) {
            const HalfStrip<T> ha = half_strip(A, t, R), hb = half_strip(B, t, R);
            // Step u reads window column col0 + u in every row of a half.  The
            // warp sweeps only the steps that reach a window column of one of
            // its halves: steps left of column -1 hold sentinel cells only (H =
            // 0, E and F below zero, whatever came before), steps right of the
            // last column feed nothing that a later strip reads (its own
            // columns end R steps earlier).  A sweep that starts late starts
            // at a multiple of 4 past the left triangle, from H = 0 rows.
            int s_lo = 1 << 30, s_hi = -1;
            if (ha.n > 0) {
                const int a0 = max(0, -ha.col0 - 1), a1 = min(ufull - 1, ha.n - 1 - ha.col0);
                if (a0 <= a1) {
                    s_lo = a0;
                    s_hi = a1;
                }
            }
            if (hb.n > 0) {
                const int b0 = max(0, -hb.col0 - 1), b1 = min(ufull - 1, hb.n - 1 - hb.col0);
                if (b0 <= b1) {
                    s_lo = min(s_lo, b0);
                    s_hi = max(s_hi, b1);
                }
            }
            const int w_lo = __reduce_min_sync(0xffffffffu, s_lo), w_hi = __reduce_max_sync(0xffffffffu, s_hi);
            int u0 = 0, uend = ufull;
            if (w_hi >= 0 && w_lo <= w_hi) {
                u0 = (w_lo >> 2) << 2;
                if (u0 < R) u0 = 0;
                uend = w_hi + 1;
            }
            StripState<R> st;
            uint32_t diag0;
            Pipe<R, T> p;
            int u;
            if (u0 == 0) {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    st.Gd[r] = c.neg2;
                    st.E[r] = c.neg2;
                }
                diag0 = __ldca(mybuf).x;
                p.wa = code_word(ha, 0);
                p.wb = code_word(hb, 0);
                p.wa2 = code_word(ha, 4);
                p.wb2 = code_word(hb, 4);
                fetch_step<R, T>(p.nxt, ha, hb, (int)(p.wa & 0xFFu), (int)(p.wb & 0xFFu), mybuf, 1);
                LeftTriangle<R, T, R - 1>::run(st, diag0, mybuf, wmax, p, ha, hb, c, best);
                u = R;
            } else {
                // the skipped columns are sentinel columns: H = 0 (G = -go) to
                // the left and on the diagonal, E below zero; the boundary entries the
                // skipped steps would have written get those values too (a
                // later strip that sweeps from step 0 reads them)
#pragma unroll
                for (int r = 0; r < R; r++) {
                    st.Gd[r] = c.ngo2;
                    st.E[r] = c.neg2;
                }
                const int kskip = min(u0 - R + 1, wmax);
                for (int k = 0; k < kskip; k++) stbuf(mybuf + (size_t)k * 32, make_uint2(c.ngo2, c.neg2));
                diag0 = c.ngo2;
                p.wa = code_word(ha, u0);
                p.wb = code_word(hb, u0);
                p.wa2 = code_word(ha, u0 + 4);
                p.wb2 = code_word(hb, u0 + 4);
                fetch_step<R, T>(p.nxt, ha, hb, (int)(p.wa & 0xFFu), (int)(p.wb & 0xFFu), mybuf,
                              u0 + 1 <= wmax ? u0 + 1 : wmax);
                u = u0;
            }
            // middle steps (every row in band for every half), one step per
            // iteration: the code byte's selector is a register, and the
            // short loop body keeps the hot code in the instruction cache
            const int umid = wmin < uend ? wmin : uend;
            for (; u < umid; u++) {
                pipe_advance<R, T, -1>(p, ha, hb, mybuf, u, wmax);
                strip_step<R, T, 1, 0>(st, diag0, mybuf, u, p.cur, c, best, 0, 0);
            }
            // the rest, with the right-edge masks (all ones while u < wmin)
            for (; u < uend; u++) {
                pipe_advance<R, T, -1>(p, ha, hb, mybuf, u, wmax);
                strip_step<R, T, 2, 0>(st, diag0, mybuf, u, p.cur, c, best, u - A.w + 1, u - B.w + 1);
            }
        }
        const int sa = lo16(best) + go, sb = hi16(best) + go;
        if (has_a) {
            if (sa >= kLimit16) rescue[atomicAdd(rescue_count, 1u)] = ja_idx;
            else scores[ja_idx] = sa;
        }
        if (has_b) {
            if (sb >= kLimit16) rescue[atomicAdd(rescue_count, 1u)] = jb_idx;
            else scores[jb_idx] = sb;
        }
    }
}

// One long job on a warp, int32 (banded_score_i32, banded.rs:134-224): the
// lanes sweep consecutive strips of kPipeRows rows in a pipeline, lane l on
// strips first + l, first + l + 32, ..., each kPipeLag steps behind the lane
// before it.  A strip reads the row above from one boundary row per warp
// (band index k holds (H, F) of the last row of the latest strip that passed
// it) and writes its own last row there; kPipeLag > kPipeRows steps of lag
// put every read after the write it needs, and a round period of at least
// 31 kPipeLag + kPipeRows + 1 steps does the same for lane 0's next strip.
// Step u of a strip is window column col0 + u in every row (row r at band
// index u - r); a strip sweeps only the steps of window columns.  Cells
// outside the band, the window or the query are NEG (the reference's
// kmin / kmax), the diagonal of column 0 is 0 and row 0 has no F.
constexpr int kPipeRows = 8;
constexpr int kPipeLag = kPipeRows + 1;

__device__ __forceinline__ void band_pipe_job(const int16_t* __restrict__ qprof, int64_t mpad,
                                              const uint8_t* __restrict__ s, int m, int nn, int lo, int w,
                                              int first, int last, int go, int ge, int2* __restrict__ buf,
                                              int lane, int32_t& best_out) {
    const int NEG = INT32_MIN / 4;
    constexpr int RR = kPipeRows;
    const int s0 = first / RR, ns = last / RR - s0 + 1;
    for (int k = lane; k <= w; k += 32) buf[k] = make_int2(NEG, NEG);
    // each strip's steps: window columns [0, nn) only
    auto ustart = [&](int st) { const int c0 = lo + st * RR; return c0 < 0 ? -c0 : 0; };
    auto uend = [&](int st) {  // exclusive
        const int c0 = lo + st * RR;
        const int e = nn - c0;
        return e < w + RR - 1 ? e : w + RR - 1;
    };
    int lmax = 1;
    for (int st = s0 + lane; st < s0 + ns; st += 32) lmax = max(lmax, uend(st) - ustart(st));
    lmax = __reduce_max_sync(0xffffffffu, lmax);
    const int P = max(lmax, 31 * kPipeLag + RR + 1);
    const int rounds = (ns + 31) / 32;
    const long long T = (long long)(rounds - 1) * P + 31 * kPipeLag + lmax;
    __syncwarp();
    int Hl[RR], El[RR];
    int best = 0;
    int u = 0, ue = 0, i0 = 0, col0 = 0;
    int diag0 = NEG;
    int c = -lane * kPipeLag, st = s0 + lane;  // this lane's count within its round, and its strip
    for (long long tg = 0; tg < T; tg++) {
        if (c == 0 && st < s0 + ns) {
            i0 = st * RR;
            col0 = lo + i0;
            u = ustart(st);
            ue = uend(st);
#pragma unroll
            for (int r = 0; r < RR; r++) {
                Hl[r] = NEG;
                El[r] = NEG;
            }
            diag0 = buf[u < w ? u : w].x;
        }
        const bool act = c >= 0 && st < s0 + ns && u < ue;
        if (act) {
            const int j = col0 + u;
            const bool colok = j >= 0 && j < nn;
            const int code = colok ? s[j] : 0;
            int sub[RR];
            {
                const uint4 pv = *reinterpret_cast<const uint4*>(qprof + (size_t)code * mpad + i0);
                const uint32_t wv[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
                for (int r = 0; r < RR; r++) sub[r] = (int)(int16_t)((wv[r >> 1] >> (16 * (r & 1))) & 0xFFFFu) - go;
            }
            const int2 top = buf[u + 1 < w ? u + 1 : w];  // entry w stays NEG
            int Hup = top.x, Fup = top.y;
            int diag = diag0;
            diag0 = top.x;  // the next step's diagonal of row 0: this step's row above
#pragma unroll
            for (int r = 0; r < RR; r++) {
                const int k = u - r, i = i0 + r;
                const bool valid = colok && k >= 0 && k < w && i < m;
                const int F = i >= 1 ? max(Hup - go, Fup - ge) : NEG;
                const int d = (i >= 1 && j >= 1) ? diag : 0;
                const int E = max(Hl[r] - go, El[r] - ge);
                int H = max(max(d + sub[r], E), max(F, 0));
                const int hold = Hl[r];
                Hl[r] = valid ? H : NEG;
                El[r] = valid ? E : NEG;
                Hup = Hl[r];
                Fup = valid ? F : NEG;
                diag = hold;
                if (valid) best = max(best, H);
            }
            const int kl = u - RR + 1;
            if (kl >= 0 && kl < w) buf[kl] = make_int2(Hup, Fup);
            u++;
        }
        __syncwarp();
        if (++c == P) {  // next round: strip + 32
            c = 0;
            st += 32;
        }
    }
    best_out = __reduce_max_sync(0xffffffffu, best);
}

// int32 banded scoring, one warp per job (banded_score_i32, banded.rs:134-224,
// the recurrence of the reference's scalar kernel): narrow bands, the jobs
// whose strip sweep in one lane would be long, and int16 results at the
// overflow limit.  The warp sweeps the band row by row, 32 band cells per
// lane step.  Per row i and band cell k (j = i + lo + k): F and the diagonal
// come from the previous row's H and F (k + 1 and k); H0 = max(diag, F, 0).
// E along the row is an exclusive max-scan of H0[k'] + k' ge over the row's
// cells k' < k, minus go + (k - 1) ge: with ge <= go, reopening after a gap
// run never beats extending it, so E of H0 equals E of H.  H = max(H0, E).
// The profile column of row i is staged in shared memory.  Row buffers (H and
// F, previous and current, w + 1 entries with entry w kept at NEG) are per
// warp in global scratch.
__global__ void __launch_bounds__(128) k_band_generic(
    const uint8_t* __restrict__ res, const int16_t* __restrict__ prof,
    const uint64_t* __restrict__ prof_off, const uint32_t* __restrict__ prof_mpad,
    const uint64_t* __restrict__ qoffs, const saber_band_job* __restrict__ jobs,
    const uint32_t* __restrict__ list, const uint32_t* __restrict__ list_count, int32_t* __restrict__ slabs,
    uint32_t slab_stride, int go, int ge, int32_t* __restrict__ scores) {
    const int NEG = INT32_MIN / 4;
    const int VNEG = INT32_MIN / 2;  // below every scanned value
    __shared__ int32_t col[4][24];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t n = *list_count;
    int32_t* const base_hp = slabs + (size_t)warp * slab_stride * 4;
    for (uint32_t t = warp; t < n; t += nwarps) {
        const uint32_t jid = list[t];
        const saber_band_job jj = jobs[jid];
        const uint32_t q = jj.query;
        const int64_t m = (int64_t)(qoffs[q + 1] - qoffs[q]);
        const int64_t nn = jj.win_len;
        int64_t lo = jj.band_lo, hi = jj.band_hi;
        const int w = (int)clip_band(m, nn, lo, hi);
        if (w == 0) {
            if (lane == 0) scores[jid] = 0;
            continue;
        }
        const int16_t* qprof = prof + prof_off[q];
        const int64_t mpad = prof_mpad[q];
        const uint8_t* s = res + jj.win_begin;
        {
            // long jobs: strips pipelined over the lanes
            const int64_t first = hi < 0 ? -hi : 0;
            int64_t last = nn - 1 - lo;
            if (last > m - 1) last = m - 1;
            if (w >= 32 && last / kPipeRows - first / kPipeRows + 1 >= 8) {
                int32_t b;
                band_pipe_job(qprof, mpad, s, (int)m, (int)nn, (int)lo, w, (int)first, (int)last, go, ge,
                              reinterpret_cast<int2*>(base_hp), lane, b);
                if (lane == 0) scores[jid] = b;
                __syncwarp();
                continue;
            }
        }
        int32_t* hp = base_hp;
        int32_t* fp = hp + slab_stride;
        int32_t* hc = fp + slab_stride;
        int32_t* fc = hc + slab_stride;
        for (int k = lane; k <= w; k += 32) {
            hp[k] = NEG;
            fp[k] = NEG;
            hc[k] = NEG;
            fc[k] = NEG;
        }
        int32_t best = 0;
        for (int64_t i = 0; i < m; i++) {
            __syncwarp();
            if (lane < 24) col[wib][lane] = qprof[(size_t)lane * mpad + i] - go;
            __syncwarp();
            int64_t kmin64 = -(i + lo);
            if (kmin64 < 0) kmin64 = 0;
            int64_t kmax64 = nn - 1 - i - lo;
            if (kmax64 > w - 1) kmax64 = w - 1;
            const int kmin = (int)(kmin64 > w ? w : kmin64), kmax = (int)(kmax64 < -1 ? -1 : kmax64);
            const int64_t jb = i + lo;
            int carry = VNEG;
            for (int c0 = 0; c0 < w; c0 += 32) {
                const int k = c0 + lane;
                const bool valid = k >= kmin && k <= kmax;
                int h0 = NEG, f = NEG;
                if (valid) {
                    const int64_t j = jb + k;
                    f = i >= 1 ? max(hp[k + 1] - go, fp[k + 1] - ge) : NEG;
                    const int hd = (i >= 1 && j >= 1) ? hp[k] : 0;
                    h0 = max(max(hd + (int)col[wib][s[j]], f), 0);
                }
                const int v = valid ? h0 + k * ge : VNEG;
                int incl = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl = max(incl, u);
                }
                int excl = __shfl_up_sync(0xffffffffu, incl, 1);
                if (lane == 0) excl = VNEG;
                excl = max(excl, carry);
                carry = max(carry, __shfl_sync(0xffffffffu, incl, 31));
                const int e = excl - go - (k - 1) * ge;
                const int h = valid ? max(h0, e) : NEG;
                if (k < w) {
                    hc[k] = h;
                    fc[k] = valid ? f : NEG;
                }
                best = max(best, h);
            }
            __syncwarp();
            int32_t* tmp = hp;
            hp = hc;
            hc = tmp;
            tmp = fp;
            fp = fc;
            fc = tmp;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
        if (lane == 0) scores[jid] = best;
        __syncwarp();
    }
}

// ---- host-side launch wrappers (the runtime TU calls these) ----
template <int R, class T>
static int fast_blocks_per_sm() {
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_band_fast<R, T>, 256, 0) != cudaSuccess) return 1;
    return bps < 1 ? 1 : bps;
}

int band_fast_blocks_per_sm(int strip_rows, bool prof8) {
    if (prof8) return strip_rows == 8 ? fast_blocks_per_sm<8, int8_t>() : fast_blocks_per_sm<16, int8_t>();
    return strip_rows == 8 ? fast_blocks_per_sm<8, int16_t>() : fast_blocks_per_sm<16, int16_t>();
}

template <int R, class T>
static void launch_fast(unsigned grid, cudaStream_t s, const FastArgs& a, const T* prof) {
    k_band_fast<R, T><<<grid, 256, 0, s>>>(a.res, prof, a.prof_off, a.prof_mpad, a.qoffs, a.jobs, a.order, a.n_ptr,
                                           a.np_ptr, a.order_skip, a.wt_counter, a.bufs, a.buf_stride, a.go, a.ge,
                                           a.scores, a.rescue, a.rescue_count);
}

// The int8 profile when the query set has one (every entry fits), else the
// int16 profile.
cudaError_t launch_band_fast(unsigned grid, cudaStream_t s, const FastArgs& a) {
    if (a.prof8) {
        if (a.strip_rows == 8) launch_fast<8>(grid, s, a, a.prof8);
        else launch_fast<16>(grid, s, a, a.prof8);
    } else {
        if (a.strip_rows == 8) launch_fast<8>(grid, s, a, a.prof);
        else launch_fast<16>(grid, s, a, a.prof);
    }
    return cudaGetLastError();
}

cudaError_t launch_band_generic(unsigned grid, unsigned block, cudaStream_t s, const GenericArgs& a) {
    k_band_generic<<<grid, block, 0, s>>>(a.res, a.prof, a.prof_off, a.prof_mpad, a.qoffs, a.jobs, a.list,
                                          a.list_count, a.slabs, a.slab_stride, a.go, a.ge, a.scores);
    return cudaGetLastError();
}

}  // namespace saber
