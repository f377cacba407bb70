/*
 * SIMD-class CPU restatement of the reference's banded scoring — TEST AND
 * CPU-BASELINE INFRASTRUCTURE ONLY.  bench.py times it as the CPU baseline and
 * as the reference arm; tests/test_simd_baseline.py holds it to the scalar
 * oracle (orc_banded_score).  The product library never links it.
 *
 * What it restates (paths relative to the reference crate root):
 *
 *   score_banded_many   src/algorithm/band_simd8.rs:78-185
 *       per query: bands of width hi - lo <= 126 are sorted by (width,
 *       subject length, input order) and scored 32 at a time by batch_u8;
 *       lanes whose maximum may have saturated, and wider bands, go to
 *       banded_score.  The substitution offset `off` and the 8-bit limit
 *       255 - pmax are the reference's.
 *   batch_u8            src/algorithm/band_simd8.rs:236-388
 *       Rognes' inter-sequence layout: lane l holds job l in lane
 *       coordinates c = j - lo_l, unsigned saturating 8-bit H/E/F, cells
 *       outside a lane's band or subject forced to 0.
 *   banded_score        src/algorithm/banded.rs:408-449
 *       the 16-bit row kernel banded_avx2_16 (src/algorithm/banded_simd.rs:
 *       393-599: saturating i16, E along the row by a max-plus prefix scan
 *       with a chunk carry, the limit 32767 - 16 ge - 192), re-run in 32 bits
 *       when a row's best passes the limit (here by the scalar oracle, which
 *       the reference proves equal to its 32-bit vector kernel).
 *
 * Vector width.  The reference's kernels are AVX2 (256-bit).  The machine
 * that times this baseline is aarch64, so they are restated for 128-bit
 * NEON: batch_u8 keeps its 32 lanes as two registers, and the 16-bit row
 * kernel works on chunks of 8 band cells (one register) instead of 16.
 * Scores do not depend on the chunk width.  On other hosts the same kernels
 * run on a portable emulation of the dozen NEON operations they use (GCC
 * vector extensions), so the tests here exercise the same code.
 */
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#if defined(__aarch64__)
#include <arm_neon.h>
#endif

namespace {

/* ------------------------------------------------------------------------
 * The vector operations the kernels use: NEON on aarch64, GCC vector
 * extensions elsewhere.
 * ---------------------------------------------------------------------- */
#if defined(__aarch64__)
typedef uint8x16_t vu8;
typedef int16x8_t vs16;
typedef uint16x8_t vm16;
struct Tbl32 { uint8x16x2_t t; };
static inline vu8 u8_load(const uint8_t* p) { return vld1q_u8(p); }
static inline void u8_store(uint8_t* p, vu8 v) { vst1q_u8(p, v); }
static inline vu8 u8_dup(uint8_t x) { return vdupq_n_u8(x); }
static inline vu8 u8_add(vu8 a, vu8 b) { return vaddq_u8(a, b); }
static inline vu8 u8_sub(vu8 a, vu8 b) { return vsubq_u8(a, b); }
static inline vu8 u8_qadd(vu8 a, vu8 b) { return vqaddq_u8(a, b); }
static inline vu8 u8_qsub(vu8 a, vu8 b) { return vqsubq_u8(a, b); }
static inline vu8 u8_max(vu8 a, vu8 b) { return vmaxq_u8(a, b); }
static inline vu8 u8_and(vu8 a, vu8 b) { return vandq_u8(a, b); }
static inline vu8 u8_lt(vu8 a, vu8 b) { return vcltq_u8(a, b); }
static inline vu8 s8_gt(vu8 a, vu8 b) { return vcgtq_s8(vreinterpretq_s8_u8(a), vreinterpretq_s8_u8(b)); }
static inline void tbl_make(Tbl32* t, const uint8_t* v32) { t->t.val[0] = vld1q_u8(v32); t->t.val[1] = vld1q_u8(v32 + 16); }
static inline vu8 tbl_lookup(const Tbl32& t, vu8 idx) { return vqtbl2q_u8(t.t, idx); }

static inline vs16 s16_load(const int16_t* p) { return vld1q_s16(p); }
static inline void s16_store(int16_t* p, vs16 v) { vst1q_s16(p, v); }
static inline vs16 s16_dup(int16_t x) { return vdupq_n_s16(x); }
static inline vs16 s16_qadd(vs16 a, vs16 b) { return vqaddq_s16(a, b); }
static inline vs16 s16_qsub(vs16 a, vs16 b) { return vqsubq_s16(a, b); }
static inline vs16 s16_max(vs16 a, vs16 b) { return vmaxq_s16(a, b); }
static inline vm16 s16_gt(vs16 a, vs16 b) { return vcgtq_s16(a, b); }
static inline vs16 s16_select(vm16 m, vs16 a, vs16 b) { return vbslq_s16(m, a, b); }
static inline vs16 s16_widen8(const int8_t* p) { return vmovl_s8(vld1_s8(p)); }
/* [prev[7], v0, ..., v6] */
static inline vs16 s16_shift_in(vs16 v, vs16 prev) { return vextq_s16(prev, v, 7); }
/* [v1, ..., v7, next[0]] */
static inline vs16 s16_shift_out(vs16 v, vs16 next) { return vextq_s16(v, next, 1); }
static inline vs16 s16_shift2_in(vs16 v, vs16 fill) { return vextq_s16(fill, v, 6); }
static inline vs16 s16_shift4_in(vs16 v, vs16 fill) { return vextq_s16(fill, v, 4); }
static inline vs16 s16_bcast7(vs16 v) { return vdupq_laneq_s16(v, 7); }
static inline int16_t s16_hmax(vs16 v) { return vmaxvq_s16(v); }
#else
typedef uint8_t vu8 __attribute__((vector_size(16)));
typedef int8_t vs8 __attribute__((vector_size(16)));
typedef int16_t vs16 __attribute__((vector_size(16)));
typedef int16_t vm16 __attribute__((vector_size(16)));
struct Tbl32 { uint8_t t[32]; };
static inline vu8 u8_load(const uint8_t* p) { vu8 v; memcpy(&v, p, 16); return v; }
static inline void u8_store(uint8_t* p, vu8 v) { memcpy(p, &v, 16); }
static inline vu8 u8_dup(uint8_t x) { vu8 v; for (int i = 0; i < 16; i++) v[i] = x; return v; }
static inline vu8 u8_add(vu8 a, vu8 b) { return a + b; }
static inline vu8 u8_sub(vu8 a, vu8 b) { return a - b; }
static inline vu8 u8_qadd(vu8 a, vu8 b) { vu8 s = a + b; return s | (vu8)(s < a); }
static inline vu8 u8_qsub(vu8 a, vu8 b) { return (a - b) & (vu8)(a >= b); }
static inline vu8 u8_max(vu8 a, vu8 b) { vu8 m = (vu8)(a > b); return (a & m) | (b & ~m); }
static inline vu8 u8_and(vu8 a, vu8 b) { return a & b; }
static inline vu8 u8_lt(vu8 a, vu8 b) { return (vu8)(a < b); }
static inline vu8 s8_gt(vu8 a, vu8 b) { return (vu8)((vs8)a > (vs8)b); }
static inline void tbl_make(Tbl32* t, const uint8_t* v32) { memcpy(t->t, v32, 32); }
static inline vu8 tbl_lookup(const Tbl32& t, vu8 idx) {
    vu8 r;
    for (int i = 0; i < 16; i++) r[i] = idx[i] < 32 ? t.t[idx[i]] : 0;
    return r;
}

static inline vs16 s16_load(const int16_t* p) { vs16 v; memcpy(&v, p, 16); return v; }
static inline void s16_store(int16_t* p, vs16 v) { memcpy(p, &v, 16); }
static inline vs16 s16_dup(int16_t x) { vs16 v; for (int i = 0; i < 8; i++) v[i] = x; return v; }
static inline int16_t sat16(int x) { return (int16_t)(x > 32767 ? 32767 : (x < -32768 ? -32768 : x)); }
static inline vs16 s16_qadd(vs16 a, vs16 b) { vs16 r; for (int i = 0; i < 8; i++) r[i] = sat16(a[i] + b[i]); return r; }
static inline vs16 s16_qsub(vs16 a, vs16 b) { vs16 r; for (int i = 0; i < 8; i++) r[i] = sat16(a[i] - b[i]); return r; }
static inline vs16 s16_max(vs16 a, vs16 b) { vm16 m = a > b; return (a & m) | (b & ~m); }
static inline vm16 s16_gt(vs16 a, vs16 b) { return a > b; }
static inline vs16 s16_select(vm16 m, vs16 a, vs16 b) { return (a & m) | (b & ~m); }
static inline vs16 s16_widen8(const int8_t* p) { vs16 v; for (int i = 0; i < 8; i++) v[i] = p[i]; return v; }
static inline vs16 s16_shift_in(vs16 v, vs16 prev) { return __builtin_shuffle(prev, v, (vs16){7, 8, 9, 10, 11, 12, 13, 14}); }
static inline vs16 s16_shift_out(vs16 v, vs16 next) { return __builtin_shuffle(v, next, (vs16){1, 2, 3, 4, 5, 6, 7, 8}); }
static inline vs16 s16_shift2_in(vs16 v, vs16 fill) { return __builtin_shuffle(fill, v, (vs16){6, 7, 8, 9, 10, 11, 12, 13}); }
static inline vs16 s16_shift4_in(vs16 v, vs16 fill) { return __builtin_shuffle(fill, v, (vs16){4, 5, 6, 7, 8, 9, 10, 11}); }
static inline vs16 s16_bcast7(vs16 v) { return s16_dup(v[7]); }
static inline int16_t s16_hmax(vs16 v) { int16_t m = v[0]; for (int i = 1; i < 8; i++) m = v[i] > m ? v[i] : m; return m; }
#endif

/* alphabet.rs:39-41: codes >= 24 score as X (22). */
static inline uint8_t code_index(uint8_t c) { return c < 24 ? c : 22; }

/* ------------------------------------------------------------------------
 * batch_u8 (band_simd8.rs:236-388): up to 32 banded jobs of one query.
 * ---------------------------------------------------------------------- */
const int U8_LANES = 32;
const int64_t U8_MAX_WIDTH = 126;
const uint8_t INVALID = 31; /* column outside a lane's subject */

struct U8Scratch {
    std::vector<uint8_t> cols; /* [column][32 lanes] residue codes */
    std::vector<uint8_t> h, e; /* [row][32 lanes] */
};

struct U8Lane {
    const uint8_t* s; /* subject window */
    int64_t n, lo, w; /* window length, clipped band lo and width hi - lo */
};

static void batch_u8(const uint8_t* qc, size_t m, const int8_t* bias, const U8Lane* lanes, int nl,
                     const Tbl32* tbl, uint8_t go, uint8_t ge, uint8_t off, U8Scratch& sc, uint8_t* maxes) {
    int64_t wmax = 0;
    for (int l = 0; l < nl; l++) wmax = std::max(wmax, lanes[l].w);
    const size_t ncols = m + (size_t)wmax;
    /* lane coordinates: column c of lane l is window column c + lo_l */
    sc.cols.assign(ncols * U8_LANES, INVALID);
    for (int l = 0; l < nl; l++) {
        int64_t c0 = std::max<int64_t>(-lanes[l].lo, 0);
        int64_t c1 = std::min<int64_t>(lanes[l].n - lanes[l].lo, (int64_t)ncols);
        for (int64_t c = c0; c < c1; c++) sc.cols[(size_t)c * U8_LANES + l] = code_index(lanes[l].s[c + lanes[l].lo]);
    }
    uint8_t wp1[U8_LANES];
    for (int l = 0; l < U8_LANES; l++) wp1[l] = l < nl ? (uint8_t)(lanes[l].w + 1) : 0;
    const vu8 wp1v[2] = {u8_load(wp1), u8_load(wp1 + 16)};
    sc.h.assign(m * U8_LANES, 0);
    sc.e.assign(m * U8_LANES, 0);
    const vu8 gov = u8_dup(go), gev = u8_dup(ge), offv = u8_dup(off), zero = u8_dup(0), one = u8_dup(1);
    const vu8 invalid = u8_dup(INVALID);
    vu8 maxh[2] = {zero, zero};
    vu8 prof[24][2];
    uint8_t* hp = sc.h.data();
    uint8_t* ep = sc.e.data();
    for (size_t c = 0; c < ncols; c++) {
        const size_t r0 = c > (size_t)wmax ? c - (size_t)wmax : 0;
        const size_t r1 = std::min(c, m - 1);
        if (r0 > r1) continue;
        vu8 colv[2];
        for (int hh = 0; hh < 2; hh++) {
            const vu8 rv = u8_load(&sc.cols[c * U8_LANES + 16 * hh]);
            colv[hh] = u8_lt(rv, invalid);
            for (int a = 0; a < 24; a++) prof[a][hh] = tbl_lookup(tbl[a], rv);
        }
        vu8 ul_h[2], u_h[2] = {zero, zero}, u_f[2] = {zero, zero};
        for (int hh = 0; hh < 2; hh++) ul_h[hh] = r0 > 0 ? u8_load(hp + (r0 - 1) * U8_LANES + 16 * hh) : zero;
        vu8 dv = u8_dup((uint8_t)(c - r0)); /* d = c - i, one less per row */
        for (size_t i = r0; i <= r1; i++) {
            const vu8 bv = u8_dup((uint8_t)(bias ? bias[i] : 0));
            const uint8_t a = qc[i];
            for (int hh = 0; hh < 2; hh++) {
                const vu8 valid = u8_and(colv[hh], s8_gt(wp1v[hh], dv));
                const vu8 p = u8_add(prof[a][hh], bv);
                uint8_t* hrow = hp + i * U8_LANES + 16 * hh;
                uint8_t* erow = ep + i * U8_LANES + 16 * hh;
                const vu8 ph = u8_load(hrow);
                const vu8 e = u8_and(u8_max(u8_qsub(ph, gov), u8_qsub(u8_load(erow), gev)), valid);
                const vu8 f = u8_and(u8_max(u8_qsub(u_h[hh], gov), u8_qsub(u_f[hh], gev)), valid);
                const vu8 diag = u8_qsub(u8_qadd(ul_h[hh], p), offv);
                const vu8 h = u8_and(u8_max(u8_max(e, f), diag), valid);
                maxh[hh] = u8_max(maxh[hh], h);
                ul_h[hh] = ph;
                u_h[hh] = h;
                u_f[hh] = f;
                u8_store(hrow, h);
                u8_store(erow, e);
            }
            dv = u8_sub(dv, one);
        }
    }
    u8_store(maxes, maxh[0]);
    u8_store(maxes + 16, maxh[1]);
}

/* ------------------------------------------------------------------------
 * banded_avx2_16 (banded_simd.rs:393-599), score only, 8 band cells per
 * chunk.  Returns false when the 16-bit range may not hold (the caller then
 * re-runs the job in 32 bits).
 * ---------------------------------------------------------------------- */
const int16_t NEG16 = -31000; /* banded_simd.rs:336 */

struct I16Scratch {
    std::vector<int16_t> hp, fp, hc, fc;
    std::vector<int8_t> prof;
    std::vector<uint8_t> codes;
};

/* tbl[a]: S(a, x) clamped to a signed byte, for x < 24 (banded_simd.rs:433-443) */
static void score_tables(const int32_t* matrix, Tbl32* tbl) {
    for (int a = 0; a < 24; a++) {
        uint8_t t[32] = {0};
        for (int x = 0; x < 24; x++) {
            const int32_t v = matrix[a * 24 + x];
            t[x] = (uint8_t)(int8_t)(v < -128 ? -128 : (v > 127 ? 127 : v));
        }
        tbl_make(&tbl[a], t);
    }
}

static bool banded16(const uint8_t* qc, size_t m, const uint8_t* s, size_t n, const int8_t* bias,
                     const Tbl32* tbl, int32_t go, int32_t ge, int64_t lo, int64_t w, I16Scratch& sc,
                     int32_t* score) {
    if (go < 0 || go > 1000 || ge < 0 || ge > 1000 || ge > go) return false;
    const int32_t limit = 32767 - 16 * ge - 192;
    const size_t wp = (size_t)w + 32;
    sc.hp.assign(wp, 0);
    sc.hc.assign(wp, 0);
    sc.fp.assign(wp, NEG16);
    sc.fc.assign(wp, NEG16);
    /* subject profile of the letters present: prof[a * stride + j] = S(a, s_j),
     * padded with S(a, '*') (code 23) past the subject */
    const size_t stride = (n + 32 + 15) & ~(size_t)15;
    uint32_t present = 0;
    for (size_t i = 0; i < m; i++) present |= 1u << qc[i];
    sc.prof.resize(24 * stride);
    sc.codes.resize(stride);
    for (size_t j = 0; j < stride; j++) sc.codes[j] = j < n ? code_index(s[j]) : 23;
    for (int a = 0; a < 24; a++) {
        if (!(present & (1u << a))) continue;
        uint8_t* row = reinterpret_cast<uint8_t*>(&sc.prof[(size_t)a * stride]);
        for (size_t j = 0; j < stride; j += 16) u8_store(row + j, tbl_lookup(tbl[a], u8_load(&sc.codes[j])));
    }
    int16_t* hp = sc.hp.data();
    int16_t* fp = sc.fp.data();
    int16_t* hc = sc.hc.data();
    int16_t* fc = sc.fc.data();
    const vs16 zero = s16_dup(0), negv = s16_dup(NEG16), gov = s16_dup((int16_t)go), gev = s16_dup((int16_t)ge);
    const vs16 ge8 = s16_dup((int16_t)(8 * ge));
    int16_t lane_i[8], ramp_i[8];
    for (int k = 0; k < 8; k++) { lane_i[k] = (int16_t)k; ramp_i[k] = (int16_t)(k * ge); }
    const vs16 lane = s16_load(lane_i), ramp = s16_load(ramp_i);
    int32_t best = 0;
    for (size_t i = 0; i < m; i++) {
        const int64_t ii = (int64_t)i;
        const int64_t kmin = std::max<int64_t>(-(ii + lo), 0);
        const int64_t kmax = std::min<int64_t>((int64_t)n - 1 - ii - lo, w - 1);
        if (kmin > kmax) {
            for (size_t k = 0; k < wp; k++) { hc[k] = (int64_t)k < kmin ? 0 : NEG16; fc[k] = NEG16; }
            std::swap(hp, hc);
            std::swap(fp, fc);
            continue;
        }
        for (int64_t k = 0; k < kmin; k++) { hc[k] = 0; fc[k] = NEG16; }
        const int8_t* prow = &sc.prof[(size_t)qc[i] * stride];
        const vs16 bv = s16_dup((int16_t)(bias ? bias[i] : 0));
        vs16 carry = negv, rowmax = zero;
        const int64_t base = ii + lo;
        int64_t k0 = kmin;
        vs16 hcur = s16_load(hp + k0), fcur = s16_load(fp + k0);
        while (k0 <= kmax) {
            const int64_t nvalid = std::min<int64_t>(kmax + 1 - k0, 8);
            const bool full = nvalid == 8;
            const vs16 sub = s16_widen8(prow + (base + k0));
            const vs16 hpk = hcur;
            const vs16 hnext = s16_load(hp + k0 + 8), fnext = s16_load(fp + k0 + 8);
            const vs16 hp1 = s16_shift_out(hpk, hnext), fp1 = s16_shift_out(fcur, fnext);
            hcur = hnext;
            fcur = fnext;
            const vs16 d = s16_qadd(s16_qadd(hpk, sub), bv);
            const vs16 f = s16_max(s16_qsub(hp1, gov), s16_qsub(fp1, gev));
            const vs16 hprime = s16_max(s16_max(d, f), zero);
            const vm16 valid = s16_gt(s16_dup((int16_t)nvalid), lane);
            const vs16 hprime_v = full ? hprime : s16_select(valid, hprime, negv);
            const vs16 open = s16_qsub(hprime_v, gov);
            /* E[k] = max_{k'<k} (H'[k'] - go - (k-1-k') ge), within the chunk */
            vs16 x = s16_qadd(s16_shift_in(open, negv), ramp);
            x = s16_max(x, s16_shift_in(x, negv));
            x = s16_max(x, s16_shift2_in(x, negv));
            x = s16_max(x, s16_shift4_in(x, negv));
            const vs16 e_loc = s16_qsub(x, ramp);
            const vs16 e = s16_max(e_loc, s16_qsub(carry, ramp));
            const vs16 h = s16_max(hprime, e);
            const vs16 h_v = full ? h : s16_select(valid, h, negv);
            const vs16 f_v = full ? f : s16_select(valid, f, negv);
            s16_store(hc + k0, h_v);
            s16_store(fc + k0, f_v);
            rowmax = s16_max(rowmax, h_v);
            if (full) {
                const vs16 a = s16_max(s16_qsub(hprime_v, gov), s16_qsub(e_loc, gev));
                carry = s16_max(s16_bcast7(a), s16_qsub(carry, ge8));
            }
            k0 += 8;
        }
        const int32_t rm = s16_hmax(rowmax);
        if (rm > limit) return false;
        if (rm > best) best = rm;
        /* cells right of the band that the next row reads (up to kmax + 16) */
        s16_store(hc + kmax + 1, negv);
        s16_store(hc + kmax + 9, negv);
        s16_store(fc + kmax + 1, negv);
        s16_store(fc + kmax + 9, negv);
        std::swap(hp, hc);
        std::swap(fp, fc);
    }
    *score = best;
    return true;
}

/* banded.rs:41-47 (Band::clip); false when the clipped band is empty. */
static bool clip_band(int64_t* lo, int64_t* hi, int64_t m, int64_t n) {
    if (m == 0 || n == 0 || *hi < *lo) return false;
    if (*lo < -(m - 1)) *lo = -(m - 1);
    if (*hi > n - 1) *hi = n - 1;
    return *hi >= *lo;
}

/* In-band cells as the reference counts them (banded.rs:123-131, 208). */
static uint64_t band_cells(int64_t m, int64_t n, int64_t lo, int64_t hi) {
    uint64_t cells = 0;
    for (int64_t d = lo; d <= hi; d++) {
        int64_t ilo = std::max<int64_t>(-d, 0), ihi = std::min<int64_t>(m, n - d);
        if (ihi > ilo) cells += (uint64_t)(ihi - ilo);
    }
    return cells;
}

struct Ctx {
    const uint8_t* residues;
    const uint8_t* qcodes;
    const uint64_t* qoffs;
    const int8_t* qbias;
    const orc_band_job* jobs;
    const int32_t* matrix;
    int32_t go, ge;
    int32_t* scores;
    int32_t smin, smax;
    Tbl32 tbl16[24]; /* signed-byte score tables of the 16-bit kernel's profiles */
};

struct Counts {
    uint64_t cells = 0, u8_jobs = 0, u8_overflows = 0, i16_jobs = 0, i32_jobs = 0;
};

/* score_banded_many (band_simd8.rs:78-185) for the jobs of one query. */
static void score_query(const Ctx& cx, uint32_t q, const uint64_t* idx, size_t nidx, U8Scratch& u8s,
                        I16Scratch& i16s, std::vector<uint8_t>& qcbuf, Counts& ct) {
    const size_t m = (size_t)(cx.qoffs[q + 1] - cx.qoffs[q]);
    qcbuf.resize(m + 1);
    for (size_t i = 0; i < m; i++) qcbuf[i] = code_index(cx.qcodes[cx.qoffs[q] + i]);
    const uint8_t* qc = qcbuf.data();
    const int8_t* bias = cx.qbias ? cx.qbias + cx.qoffs[q] : nullptr;
    struct J { uint64_t k; int64_t lo, hi, n; };
    std::vector<J> narrow, exact;
    for (size_t t = 0; t < nidx; t++) {
        const orc_band_job& jb = cx.jobs[idx[t]];
        int64_t lo = jb.band_lo, hi = jb.band_hi, n = jb.win_len;
        cx.scores[idx[t]] = 0;
        if (!clip_band(&lo, &hi, (int64_t)m, n)) continue;
        ct.cells += band_cells((int64_t)m, n, lo, hi);
        if (hi - lo <= U8_MAX_WIDTH) narrow.push_back({idx[t], lo, hi, n});
        else exact.push_back({idx[t], lo, hi, n});
    }
    int32_t bmin = 0, bmax = 0;
    if (bias && m) {
        bmin = bmax = bias[0];
        for (size_t i = 1; i < m; i++) { bmin = std::min<int32_t>(bmin, bias[i]); bmax = std::max<int32_t>(bmax, bias[i]); }
    }
    const int32_t off = -std::min(cx.smin + std::min(bmin, 0), 0);
    const int32_t pmax = cx.smax + std::max(bmax, 0) + off;
    const bool gaps_ok = cx.go >= 0 && cx.go <= 255 && cx.ge >= 0 && cx.ge <= 255;
    if (pmax < 128 && gaps_ok && off <= 127 && !narrow.empty()) {
        const int32_t limit = 255 - pmax;
        std::sort(narrow.begin(), narrow.end(), [](const J& a, const J& b) {
            if (a.hi - a.lo != b.hi - b.lo) return a.hi - a.lo < b.hi - b.lo;
            if (a.n != b.n) return a.n < b.n;
            return a.k < b.k;
        });
        Tbl32 tbl[24];
        for (int a = 0; a < 24; a++) {
            uint8_t t[32] = {0};
            for (int x = 0; x < 24; x++) t[x] = (uint8_t)(cx.matrix[a * 24 + x] + off);
            tbl_make(&tbl[a], t);
        }
        U8Lane lanes[U8_LANES];
        uint8_t maxes[U8_LANES];
        for (size_t c0 = 0; c0 < narrow.size(); c0 += U8_LANES) {
            const int nl = (int)std::min<size_t>(U8_LANES, narrow.size() - c0);
            for (int l = 0; l < nl; l++) {
                const J& jj = narrow[c0 + l];
                const orc_band_job& jb = cx.jobs[jj.k];
                lanes[l] = {cx.residues + jb.win_begin, jj.n, jj.lo, jj.hi - jj.lo};
            }
            batch_u8(qc, m, bias, lanes, nl, tbl, (uint8_t)cx.go, (uint8_t)cx.ge, (uint8_t)off, u8s, maxes);
            for (int l = 0; l < nl; l++) {
                if ((int32_t)maxes[l] >= limit) { exact.push_back(narrow[c0 + l]); ct.u8_overflows++; }
                else cx.scores[narrow[c0 + l].k] = maxes[l];
            }
            ct.u8_jobs += (uint64_t)nl;
        }
    } else {
        exact.insert(exact.end(), narrow.begin(), narrow.end());
    }
    for (const J& jj : exact) {
        const orc_band_job& jb = cx.jobs[jj.k];
        const uint8_t* s = cx.residues + jb.win_begin;
        int32_t sc = 0;
        if (banded16(qc, m, s, (size_t)jj.n, bias, cx.tbl16, cx.go, cx.ge, jj.lo, jj.hi - jj.lo + 1, i16s, &sc)) {
            ct.i16_jobs++;
        } else {
            orc_band_score r;
            orc_scheme sch = {cx.matrix, cx.go, cx.ge};
            orc_banded_score(cx.qcodes + cx.qoffs[q], m, s, (size_t)jj.n, bias, sch, jj.lo, jj.hi, &r);
            sc = r.score;
            ct.i32_jobs++;
        }
        cx.scores[jj.k] = sc;
    }
}

} // namespace

extern "C" int orc_simd_score_band_jobs(const uint8_t* residues, const uint8_t* qcodes, const uint64_t* qoffs,
                                        const int8_t* qbias, const orc_band_job* jobs, uint64_t njobs,
                                        const int32_t* matrix, int32_t gap_open, int32_t gap_extend,
                                        int32_t* scores, int threads, orc_simd_counters* counters) {
    if (threads < 1) threads = 1;
    uint32_t nq = 0;
    for (uint64_t k = 0; k < njobs; k++) nq = std::max(nq, jobs[k].query + 1);
    /* jobs grouped by query (input order within a query) */
    std::vector<uint64_t> start(nq + 1, 0), idx(njobs);
    for (uint64_t k = 0; k < njobs; k++) start[jobs[k].query + 1]++;
    for (uint32_t q = 0; q < nq; q++) start[q + 1] += start[q];
    {
        std::vector<uint64_t> fill(start.begin(), start.end() - 1);
        for (uint64_t k = 0; k < njobs; k++) idx[fill[jobs[k].query]++] = k;
    }
    std::vector<uint32_t> order;
    for (uint32_t q = 0; q < nq; q++)
        if (start[q + 1] > start[q]) order.push_back(q);
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        const uint64_t wa = (start[a + 1] - start[a]) * (qoffs[a + 1] - qoffs[a]);
        const uint64_t wb = (start[b + 1] - start[b]) * (qoffs[b + 1] - qoffs[b]);
        return wa != wb ? wa > wb : a < b;
    });
    Ctx cx{residues, qcodes, qoffs, qbias, jobs, matrix, gap_open, gap_extend, scores, 0, 0, {}};
    score_tables(matrix, cx.tbl16);
    cx.smin = cx.smax = matrix[0];
    for (int t = 0; t < 576; t++) { cx.smin = std::min(cx.smin, matrix[t]); cx.smax = std::max(cx.smax, matrix[t]); }
    std::atomic<size_t> next(0);
    std::vector<Counts> per(threads);
    auto work = [&](int tid) {
        U8Scratch u8s;
        I16Scratch i16s;
        std::vector<uint8_t> qcbuf;
        for (;;) {
            const size_t t = next.fetch_add(1);
            if (t >= order.size()) break;
            const uint32_t q = order[t];
            score_query(cx, q, &idx[start[q]], (size_t)(start[q + 1] - start[q]), u8s, i16s, qcbuf, per[tid]);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
    if (counters) {
        memset(counters, 0, sizeof(*counters));
        for (const Counts& c : per) {
            counters->cells += c.cells;
            counters->u8_jobs += c.u8_jobs;
            counters->u8_overflows += c.u8_overflows;
            counters->i16_jobs += c.i16_jobs;
            counters->i32_jobs += c.i32_jobs;
        }
    }
    return 0;
}
