// Scan schedule on the GPU: the seed scan of the database against a query
// batch's seed tables, the window filter, per-diagonal coverage with ungapped
// X-drop, and region clustering — Engine::search_scan up to the per-query
// candidate cap (src/search/engine/scan.rs:1261-1497).
//
// Database state (built once per database, seed alphabet and shape set):
//   sb[r]   seed byte of residue r: reduced letter, | 0x80 when masked from
//           seeding, 0x7F when not in the seed alphabet (scan.rs:123-141)
//   rem[r]  min(255, residues from r to the end of its subject)
//   dst[r]  min(255, residues from the start of its subject to r)
//   per shape: the bitmap of codes occurring more than the cap in the
//           database (scan.rs:1184-1238, cap = index.rs:329-336)
// Per call:
//   per shape: dense code -> batch-position table of the unmasked, not
//   frequent query seeds (count, scan, scatter; a presence bitmap in front),
//   then one thread per database position computes its seed code, looks it
//   up and runs the window filter on every hit; survivors (position, batch
//   position, shape) are appended to a device list.
//   Survivors are sorted into chains of one (subject, query, diagonal) in
//   (query position, shape) order — the order in which the reference visits
//   the hits of a pair (scan.rs:2158-2170) restricted to one diagonal, which
//   is all the coverage rule couples (scan.rs:2398-2425) — and one thread per
//   chain runs the coverage test and the X-drop extensions.  HSPs are sorted
//   by (subject, query, diagonal) and one thread per pair forms its regions
//   (scan.rs:2437-2474).  The per-query order and cap are applied on the host.
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include <algorithm>

#include "runtime.cuh"

namespace saber {

constexpr uint8_t kNonSeed = 0x7F;
constexpr uint8_t kMasked = 0x80;
constexpr uint8_t kQSent = 0xFE;
constexpr int kDBias = 1 << 19;  // diagonal offset in the chain keys

struct AlphaMap {
    uint8_t m[24];
};
struct ShapeDev {
    uint16_t off[16];
    uint32_t w, span;
};

// ---- database state --------------------------------------------------------
__global__ void k_seed_bytes(const uint8_t* __restrict__ res, const uint8_t* __restrict__ mask, uint64_t N,
                             AlphaMap am, uint8_t* __restrict__ sb) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t c = res[r];
        uint8_t v = (c < 24 && am.m[c] != 255) ? am.m[c] : kNonSeed;
        if (v != kNonSeed && mask && mask[r]) v |= kMasked;
        sb[r] = v;
    }
}

// distances to the end / from the start of the sequence holding position r
__global__ void k_dists(const uint64_t* __restrict__ offs, uint64_t nseq, uint64_t N, uint8_t* __restrict__ rem,
                        uint8_t* __restrict__ dst) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t lo = 0, hi = nseq;  // last s with offs[s] <= r
        while (hi - lo > 1) {
            uint64_t mid = (lo + hi) >> 1;
            if (offs[mid] <= r) lo = mid;
            else hi = mid;
        }
        const uint64_t a = r - offs[lo], b = offs[lo + 1] - r;
        rem[r] = (uint8_t)(b < 255 ? b : 255);
        dst[r] = (uint8_t)(a < 255 ? a : 255);
    }
}

// Adds a per-thread count to a global counter with one atomic per warp
// (every lane of the warp must call it).
__device__ __forceinline__ void count_add(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

__device__ __forceinline__ int64_t seed_code(const uint8_t* __restrict__ sr, const ShapeDev& sh, uint32_t asize) {
    uint32_t c = 0;
    // unrolled to the largest weight so that the offsets stay in registers
#pragma unroll
    for (uint32_t i = 0; i < 16; i++) {
        if (i >= sh.w) break;
        const uint8_t r = sr[sh.off[i]];
        if (r >= asize) return -1;
        c = c * asize + r;
    }
    return c;
}

__global__ void k_db_counts(const uint8_t* __restrict__ sb, const uint8_t* __restrict__ rem, uint64_t N, ShapeDev sh,
                            uint32_t asize, uint32_t* __restrict__ counts, unsigned long long* __restrict__ total) {
    unsigned long long t = 0;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (uint64_t)gridDim.x * blockDim.x) {
        if (rem[r] < sh.span) continue;
        const int64_t c = seed_code(sb + r, sh, asize);
        if (c < 0) continue;
        atomicAdd(&counts[c], 1u);
        t++;
    }
    count_add(total, t);
}

__global__ void k_freq_bits(const uint32_t* __restrict__ counts, uint64_t ncodes, uint64_t cap,
                            unsigned long long* __restrict__ bits) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncodes; c += (uint64_t)gridDim.x * blockDim.x)
        if (counts[c] > cap) atomicOr(&bits[c >> 6], 1ull << (c & 63));
}

// ---- query tables ------------------------------------------------------------
__global__ void k_query_bytes(const uint8_t* __restrict__ qcodes, const uint8_t* __restrict__ qmask, uint64_t QN,
                              AlphaMap am, uint8_t* __restrict__ qsb, uint8_t* __restrict__ qfull) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < QN; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint8_t c = qcodes[i];
        const uint8_t r = am.m[c < 24 ? c : 23];
        const bool ok = !(qmask && qmask[i]) && r != 255;
        qsb[i] = ok ? r : kQSent;
        qfull[i] = ok ? c : kQSent;
    }
}

__device__ __forceinline__ bool is_frequent(const unsigned long long* freq, uint32_t c) {
    return freq && ((freq[c >> 6] >> (c & 63)) & 1ull);
}

// Seed tables of one shape, rank-compressed: grp[c / 32] = {presence bits of
// codes c & ~31 .. c | 31, number of present codes before them}; the present
// code of rank k owns entries coff[k] .. coff[k + 1] of the batch positions.
// A present code's rank is grp.y + popc(grp.x & lanes below c % 32).
__device__ __forceinline__ bool code_rank(const uint2* __restrict__ grp, uint32_t c, uint32_t& k) {
    const uint2 g = grp[c >> 5];
    const uint32_t bit = 1u << (c & 31);
    k = g.y + __popc(g.x & (bit - 1u));
    return (g.x & bit) != 0;
}

// pass 0: count per code; pass 1: scatter batch positions through the ranks
// (cur = per-rank cursors)
template <int PASS>
__global__ void k_query_seeds(const uint8_t* __restrict__ qsb, const uint8_t* __restrict__ qrem, uint64_t QN,
                              ShapeDev sh, uint32_t asize, const unsigned long long* __restrict__ freq,
                              uint32_t* __restrict__ cnt, const uint2* __restrict__ grp,
                              const uint32_t* __restrict__ coff, uint32_t* __restrict__ ent,
                              unsigned long long* __restrict__ ctr) {
    unsigned long long kept = 0, skipped = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < QN; i += (uint64_t)gridDim.x * blockDim.x) {
        if (qrem[i] < sh.span) continue;
        const int64_t c = seed_code(qsb + i, sh, asize);
        if (c < 0) continue;
        if (is_frequent(freq, (uint32_t)c)) {
            skipped++;
            continue;
        }
        if (PASS == 0) {
            atomicAdd(&cnt[c], 1u);
            kept++;
        } else {
            uint32_t k;
            code_rank(grp, (uint32_t)c, k);
            const uint32_t slot = atomicAdd(&cnt[k], 1u);
            ent[coff[k] + slot] = (uint32_t)i;
        }
    }
    if (PASS == 0) {
        count_add(&ctr[0], kept);
        count_add(&ctr[1], skipped);
    }
}

// (first entry, entries) of each rank, the entries offset by the shape's base
__global__ void k_entry_ranges(const uint32_t* __restrict__ coff, uint64_t n, uint32_t base, uint2* __restrict__ rng) {
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        rng[k] = make_uint2(coff[k] + base, coff[k + 1] - coff[k]);
}

// presence bits and present-code counts of each 32-code group
__global__ void k_group_bits(const uint32_t* __restrict__ cnt, uint64_t ncodes, uint2* __restrict__ grp,
                             uint32_t* __restrict__ gcnt) {
    const int lane = threadIdx.x & 31;
    const uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t g = w0; g * 32 < ncodes; g += nw) {
        const uint64_t c = g * 32 + lane;
        const uint32_t b = __ballot_sync(0xffffffffu, c < ncodes && cnt[c] > 0);
        if (lane == 0) {
            grp[g] = make_uint2(b, 0u);
            gcnt[g] = __popc(b);
        }
    }
}

// ranks of the groups' first codes, and each present code's count at its rank
__global__ void k_group_ranks(const uint32_t* __restrict__ cnt, uint64_t ncodes, const uint32_t* __restrict__ grank,
                              uint2* __restrict__ grp, uint32_t* __restrict__ cntc) {
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncodes; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t g = (uint32_t)(c >> 5);
        if ((c & 31) == 0) grp[g].y = grank[g];
        const uint32_t n = cnt[c];
        if (n) {
            const uint32_t bits = grp[g].x;
            cntc[grank[g] + __popc(bits & ((1u << (c & 31)) - 1u))] = n;
        }
    }
}

// combined filter codes of the 256 residue values (comb_table)
struct CombTab {
    uint8_t t[256];
};

// ---- database scan with the window filter ---------------------------------------
constexpr int kMaxShapes = 32;
struct ScanArgs {
    const uint8_t *sb, *res, *rem, *dst;
    uint64_t N;
    const uint2* grp;                // rank-compressed presence tables of all shapes
    const uint2* rng;                // rank -> (first entry, entries) of all shapes
    const uint32_t* qent;            // batch positions of all shapes
    const uint4* qwin;               // per batch position: seed-letter window record (32 bytes)
    const uint4* qwinx;              // per batch position: full-code window record (32 bytes)
    const uint8_t* cb;               // combined filter codes of the database (combined mode)
    int cfil;
    uint32_t min_ids, kx;
    uint32_t s0, s1, asize;          // this pass's shapes [s0, s1)
    uint2* surv;
    unsigned long long* nsurv;  // counter (may exceed cap: overflow)
    uint64_t cap;
    unsigned long long* ctr;    // [2] hits, [3] filtered
    // per shape: care offsets, table / entry bases
    ShapeDev sh[kMaxShapes];
    uint64_t grp_off[kMaxShapes], rng_off[kMaxShapes];
};

// Lanes [lo, hi) of a 32-lane mask (0 <= lo, hi <= 32).
__device__ __forceinline__ uint32_t lane_range(int lo, int hi) {
    if (hi <= lo) return 0u;
    return (uint32_t)(((1ull << hi) - 1ull) & ~((1ull << lo) - 1ull));
}

// Bits 4w .. 4w + 3 of the result: which bytes of Q[w] ^ S[w] are zero (a
// carry-free zero-byte test, the four flags gathered with one multiply).
__device__ __forceinline__ uint32_t eq_bytes8(const uint32_t (&Q)[8], const uint32_t (&S)[8], uint32_t smask) {
    uint32_t E = 0;
#pragma unroll
    for (int w = 0; w < 8; w++) {
        const uint32_t x = Q[w] ^ (S[w] & smask);
        const uint32_t z = ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x | 0x7F7F7F7Fu);
        E |= (((z >> 7) * 0x10204080u) >> 28) << (4 * w);
    }
    return E;
}

__device__ __forceinline__ void ld256(uint32_t (&v)[8], const void* p) {
    asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "l"(p));
}

// 8 words of a staged byte buffer from byte `idx` on (9 aligned word reads
// and a funnel shift).
__device__ __forceinline__ void staged_words(const uint32_t* buf, int idx, uint32_t (&S)[8]) {
    const int wi = idx >> 2;
    const uint32_t sh = (uint32_t)(idx & 3) * 8u;
    uint32_t nx = buf[wi];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const uint32_t cur = nx;
        nx = buf[wi + j + 1];
        S[j] = __funnelshift_r(cur, nx, sh);
    }
}

// The shapes [s0, s1) over the database in one pass (the window filter is
// filter_scalar, scan.rs:1809-1856).  Each warp takes 32 consecutive
// positions [base, base + 32) and stages the subject's seed letters and
// residues of [base - 32, base + 96) in shared memory: every seed code and
// every filter window of those positions reads from there.  Four shapes at a
// time (their table lookups in flight together) the positions' seed codes go
// through the shapes' rank-compressed presence tables; positions with hits
// become (position, shape, entries) segments in a per-warp queue.  When the
// queue fills (and at the end of the 32 positions) the warp works through
// the queued hits, one per lane per round: the hit's query window is one
// aligned 32-byte record (letters outside the query are QSENT, which never
// equals a subject byte & 0x7F), the subject window comes from the staged
// bytes, restricted to lanes inside the subject.  Survivors collect in
// shared memory and go out 32 or more at a time.
constexpr int kSegCap = 192;
constexpr int kShapeUnroll = 4;
constexpr int kScanWarps = 8;
constexpr uint32_t kSurvStage = 64;

struct WarpScan {
    uint32_t* seg_n;   // kSegCap
    uint32_t* seg_eb;  // kSegCap: entry base (offset - first hit index)
    uint8_t* seg_rl;   // kSegCap: position - base
    uint8_t* seg_sh;   // kSegCap: shape
    uint2* sv;         // kSurvStage survivor records
    const uint32_t* sbw;   // 32 staged words: seed letters of [base - 32, base + 96)
    const uint32_t* resw;  // 32 staged words: residues of the same range
    uint32_t nsv;      // staged survivors (warp-uniform)
    uint32_t rd;       // this lane's position: rem | dst << 8
    uint64_t base;
};

__device__ __forceinline__ void surv_drain(const ScanArgs& a, int lane, WarpScan& ws) {
    __syncwarp();
    unsigned long long slot0 = 0;
    if (lane == 0) slot0 = atomicAdd(a.nsurv, (unsigned long long)ws.nsv);
    slot0 = __shfl_sync(0xffffffffu, slot0, 0);
    for (uint32_t i = lane; i < ws.nsv; i += 32)
        if (slot0 + i < a.cap) a.surv[slot0 + i] = ws.sv[i];
    __syncwarp();
    ws.nsv = 0;
}

// The queued segments' hits, 32 per round.  Each lane keeps kPer segments'
// starts in registers; a round's owners come from the bits of the segments
// that start inside it and the count of those that start before it.
template <bool COMB>
__device__ __forceinline__ void scan_flush(const ScanArgs& a, int lane, int nseg, WarpScan& ws,
                                           unsigned long long& hits, unsigned long long& filtered) {
    constexpr int kPer = kSegCap / 32;
    uint32_t st[kPer];
    uint32_t sum = 0;
#pragma unroll
    for (int t = 0; t < kPer; t++) {
        const int sidx = lane * kPer + t;
        st[t] = sum;
        sum += sidx < nseg ? ws.seg_n[sidx] : 0u;
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    const uint32_t lbase = incl - sum;
#pragma unroll
    for (int t = 0; t < kPer; t++) {
        const int sidx = lane * kPer + t;
        // segments past nseg never start inside a round
        st[t] = sidx < nseg ? lbase + st[t] : 0xFFFFFFFFu;
        if (sidx < nseg) ws.seg_eb[sidx] -= st[t];
    }
    __syncwarp();
    if (lane == 0) hits += total;
    for (uint32_t k0 = 0; k0 < total; k0 += 32) {
        uint32_t B = 0, before = 0;
#pragma unroll
        for (int t = 0; t < kPer; t++) {
            before += st[t] < k0;
            const uint32_t d = st[t] - k0;
            if (d < 32u) B |= 1u << d;
        }
        B = __reduce_or_sync(0xffffffffu, B);
        before = __reduce_add_sync(0xffffffffu, before);
        const uint32_t k = k0 + lane;
        const bool live = k < total;
        const uint32_t lanes_le = lane == 31 ? 0xFFFFFFFFu : ((2u << lane) - 1u);
        const uint32_t own = live ? before + __popc(B & lanes_le) - 1u : 0u;
        const int rl = ws.seg_rl[own];
        // the subject position's rem | dst from the lane that scanned it
        const uint32_t srd = __shfl_sync(0xffffffffu, ws.rd, rl);
        bool pass = false;
        uint32_t g = 0;
        if (live) {
            g = a.qent[ws.seg_eb[own] + k];
            if (a.min_ids == 0) {
                pass = true;
            } else if (COMB) {
                // one compare of combined codes: equal low nibbles are
                // reduced-letter identities, equal bytes exact ones; the
                // reference's decision (ids >= min_ids, else ids + kx * exact
                // >= min_ids) is ids + kx * exact >= min_ids since exact <= ids
                uint32_t Q[8], S[8];
                ld256(Q, a.qwin + 2 * (uint64_t)g);
                const int idx = rl + a.cfil + 16;  // staged byte of r + cfil - 16
                staged_words(ws.resw, idx, S);
                const int sdst = (int)(srd >> 8), srem = (int)(srd & 0xFFu);
                const uint32_t L = lane_range(max(0, 16 - a.cfil - sdst), min(32, srem + 16 - a.cfil));
                uint32_t Er = 0, Ee = 0;
#pragma unroll
                for (int w = 0; w < 8; w++) {
                    const uint32_t x = Q[w] ^ S[w];
                    const uint32_t zr = ~((x & 0x0F0F0F0Fu) + 0x0F0F0F0Fu) & 0x10101010u;
                    const uint32_t ze = ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
                    Er |= (((zr >> 4) * 0x10204080u) >> 28) << (4 * w);
                    Ee |= (((ze >> 7) * 0x10204080u) >> 28) << (4 * w);
                }
                pass = __popc(Er & L) + a.kx * __popc(Ee & L) >= a.min_ids;
            } else {
                uint32_t Q[8], S[8];
                ld256(Q, a.qwin + 2 * (uint64_t)g);
                const int idx = rl + a.cfil + 16;  // staged byte of r + cfil - 16
                staged_words(ws.sbw, idx, S);
                const int sdst = (int)(srd >> 8), srem = (int)(srd & 0xFFu);
                const uint32_t L = lane_range(max(0, 16 - a.cfil - sdst), min(32, srem + 16 - a.cfil));
                const uint32_t E = eq_bytes8(Q, S, 0x7F7F7F7Fu) & L;
                const uint32_t ids = __popc(E);
                if (ids >= a.min_ids) {
                    pass = true;
                } else if (a.kx != 0 && ids * (1 + a.kx) >= a.min_ids) {
                    ld256(Q, a.qwinx + 2 * (uint64_t)g);
                    staged_words(ws.resw, idx, S);
                    const uint32_t ex = __popc(E & eq_bytes8(Q, S, 0xFFFFFFFFu));
                    pass = ids + a.kx * ex >= a.min_ids;
                }
            }
            if (!pass) filtered++;
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, pass);
        if (pass)
            ws.sv[ws.nsv + __popc(bal & ((1u << lane) - 1u))] =
                make_uint2((uint32_t)(ws.base + rl), g | ((uint32_t)ws.seg_sh[own] << 27));
        ws.nsv += __popc(bal);
        if (ws.nsv >= 32) surv_drain(a, lane, ws);
    }
    __syncwarp();
}

// 4 bytes of buf at byte index i (4-aligned), `fill` outside [0, n)
__device__ __forceinline__ uint32_t stage_word(const uint8_t* __restrict__ buf, int64_t i, uint64_t n, uint8_t fill) {
    if (i >= 0 && (uint64_t)i + 4 <= n) return *reinterpret_cast<const uint32_t*>(buf + i);
    uint32_t v = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int64_t p = i + j;
        const uint32_t b = (p >= 0 && (uint64_t)p < n) ? buf[p] : fill;
        v |= b << (8 * j);
    }
    return v;
}

// Resident blocks per SM the scan and chain kernels are compiled for (a
// register budget); tuning constants.
#ifndef SABER_SCAN_MIN_BLOCKS
#define SABER_SCAN_MIN_BLOCKS 4
#endif
#ifndef SABER_CHAINS_MIN_BLOCKS
#define SABER_CHAINS_MIN_BLOCKS 4
#endif

template <bool COMB>
__global__ void __launch_bounds__(256, SABER_SCAN_MIN_BLOCKS) k_scan(ScanArgs a) {
    __shared__ uint32_t s_n[kScanWarps][kSegCap], s_eb[kScanWarps][kSegCap];
    __shared__ uint8_t s_rl[kScanWarps][kSegCap], s_sh[kScanWarps][kSegCap];
    __shared__ uint2 s_sv[kScanWarps][kSurvStage];
    __shared__ uint32_t s_sbw[kScanWarps][32], s_resw[kScanWarps][32];
    __shared__ ShapeDev s_shape[kMaxShapes];
    for (uint32_t i = threadIdx.x; i < a.s1; i += blockDim.x) s_shape[i] = a.sh[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t warp0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long hits = 0, filtered = 0;
    WarpScan ws{s_n[w], s_eb[w], s_rl[w], s_sh[w], s_sv[w], s_sbw[w], s_resw[w], 0u, 0u, 0u};
    const uint8_t* stb = reinterpret_cast<const uint8_t*>(s_sbw[w]) + 32 + lane;  // this lane's position
    for (uint64_t base = warp0 * 32; base < a.N; base += nwarps * 32) {
        const uint64_t r = base + lane;
        const int64_t wb = (int64_t)base - 32 + 4 * lane;
        __syncwarp();
        s_sbw[w][lane] = stage_word(a.sb, wb, a.N, kNonSeed);
        s_resw[w][lane] = COMB ? stage_word(a.cb, wb, a.N, 0xEEu) : stage_word(a.res, wb, a.N, 0xFFu);
        const int rem = r < a.N ? a.rem[r] : 0;
        ws.rd = r < a.N ? ((uint32_t)rem | ((uint32_t)a.dst[r] << 8)) : 0u;
        ws.base = base;
        __syncwarp();
        int nseg = 0;
        for (uint32_t s0 = a.s0; s0 < a.s1; s0 += kShapeUnroll) {
            uint32_t n[kShapeUnroll], e0[kShapeUnroll];
#pragma unroll
            for (int j = 0; j < kShapeUnroll; j++) {
                const uint32_t si = s0 + j;
                n[j] = 0;
                e0[j] = 0;
                if (si < a.s1 && rem >= (int)s_shape[si].span) {
                    const int64_t c = seed_code(stb, s_shape[si], a.asize);
                    uint32_t k;
                    if (c >= 0 && code_rank(a.grp + a.grp_off[si], (uint32_t)c, k)) {
                        const uint2 r = a.rng[a.rng_off[si] + k];
                        e0[j] = r.x;
                        n[j] = r.y;
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kShapeUnroll; j++) {
                const uint32_t bal = __ballot_sync(0xffffffffu, n[j] > 0);
                if (n[j] > 0) {
                    const int slot = nseg + __popc(bal & ((1u << lane) - 1u));
                    ws.seg_n[slot] = n[j];
                    ws.seg_eb[slot] = e0[j];
                    ws.seg_rl[slot] = (uint8_t)lane;
                    ws.seg_sh[slot] = (uint8_t)(s0 + j);
                }
                nseg += __popc(bal);
            }
            if (nseg > kSegCap - 32 * kShapeUnroll) {
                __syncwarp();
                scan_flush<COMB>(a, lane, nseg, ws, hits, filtered);
                nseg = 0;
            }
        }
        if (nseg) {
            __syncwarp();
            scan_flush<COMB>(a, lane, nseg, ws, hits, filtered);
        }
    }
    if (ws.nsv) surv_drain(a, lane, ws);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) filtered += __shfl_xor_sync(0xffffffffu, filtered, o);
    if (lane == 0) {
        atomicAdd(&a.ctr[2], hits);
        atomicAdd(&a.ctr[3], filtered);
    }
}

// Window records of the batch positions: record g holds the 32 letters at
// g + cfil - 16 + t (t < 32), QSENT where that position lies outside g's
// query (the filter's query-side lane bounds).
// With `comb` (a combined code table) a single record of combined codes is
// written to `win`: (group index << 4 | letter) where the letter counts, 0xFF
// elsewhere; `winx` is then unused.
__global__ void k_query_windows(const uint8_t* __restrict__ qsb, const uint8_t* __restrict__ qfull,
                                const uint8_t* __restrict__ qrem, const uint8_t* __restrict__ qdst, uint64_t QN,
                                int cfil, const CombTab* __restrict__ comb, uint8_t* __restrict__ win,
                                uint8_t* __restrict__ winx) {
    const uint64_t total = QN * 32;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t g = i >> 5;
        const int t = (int)(i & 31);
        const int lo = 16 - cfil - (int)qdst[g], hi = (int)qrem[g] + 16 - cfil;
        uint8_t v = kQSent, vx = kQSent;
        if (t >= lo && t < hi) {
            const uint64_t q = g + (uint64_t)(int64_t)(cfil - 16 + t);
            v = qsb[q];
            vx = qfull[q];
        }
        if (comb) {
            // letter from the seed byte, group index from the full code
            win[i] = v == kQSent ? (uint8_t)0xFF
                                 : (uint8_t)((vx < 24 ? (comb->t[vx] & 0xF0u) : 0xF0u) | (v & 0x0Fu));
        } else {
            win[i] = v;
            winx[i] = vx;
        }
    }
}

// Keys of the per-query region order (region_order, engine.rs:493-495:
// query, best descending, subject, d_min, d_max) for three stable radix
// passes, least significant first.
__global__ void k_region_keys(const saber_region* __restrict__ regs, uint32_t n, unsigned long long* __restrict__ k_lo,
                              uint32_t* __restrict__ k_sub, unsigned long long* __restrict__ k_hi,
                              uint32_t* __restrict__ idx) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const saber_region r = regs[i];
        k_lo[i] = ((unsigned long long)((uint32_t)r.d_min ^ 0x80000000u) << 32) | ((uint32_t)r.d_max ^ 0x80000000u);
        k_sub[i] = r.subject;
        k_hi[i] = ((unsigned long long)r.query << 32) | (0xFFFFFFFFu - ((uint32_t)r.best ^ 0x80000000u));
        idx[i] = i;
    }
}

__global__ void k_gather_u32_by(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx, uint32_t n,
                                uint32_t* __restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[idx[i]];
}

__global__ void k_gather_u64_by(const unsigned long long* __restrict__ src, const uint32_t* __restrict__ idx,
                                uint32_t n, unsigned long long* __restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[idx[i]];
}

__global__ void k_gather_uint4(const uint4* __restrict__ src, const uint32_t* __restrict__ idx, uint32_t n,
                               uint4* __restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[idx[i]];
}

__global__ void k_gather_regions(const saber_region* __restrict__ src, const uint32_t* __restrict__ idx, uint32_t n,
                                 saber_region* __restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[idx[i]];
}

// ---- chains ------------------------------------------------------------------------

// Bit layout of the chain keys: (query, subject, diagonal + dbias) above
// `low` bits.  In the composite layout the low bits hold (query position,
// shape), so one sort gives the chain order; otherwise (fields too wide for
// 64 bits) the keys are query << 44 | subject << 20 | diagonal + 2^19 and a
// first stable sort by (query position, shape) precedes.
struct KeyLayout {
    int low, bs, bd, bsh;  // bits below the chain key, of the subject, of the diagonal, of the shape
    int64_t dbias;
};

// Owner tables: blk[b] is the sequence holding position b * 256 of a
// concatenation with offsets offs[nseq + 1]; one thread per sequence writes
// the blocks that start inside it.
constexpr int kOwnerShift = 8;
__global__ void k_block_owner(const uint64_t* __restrict__ offs, uint64_t nseq, uint32_t* __restrict__ blk) {
    for (uint64_t sq = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; sq < nseq;
         sq += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b0 = (offs[sq] + (1ull << kOwnerShift) - 1) >> kOwnerShift;
        const uint64_t b1 = (offs[sq + 1] + (1ull << kOwnerShift) - 1) >> kOwnerShift;
        for (uint64_t b = b0; b < b1; b++) blk[b] = (uint32_t)sq;
    }
}

// The sequence holding position x (< offs[nseq]): the owner of x's block,
// then forward over the sequences that start later in the block.
__device__ __forceinline__ uint64_t owner_of(const uint64_t* offs, const uint32_t* blk, uint64_t x) {
    uint64_t sq = blk[x >> kOwnerShift];
    while (offs[sq + 1] <= x) sq++;
    return sq;
}

__global__ void k_surv_keys(const uint2* __restrict__ surv, uint32_t n, const uint64_t* __restrict__ soffs,
                            const uint32_t* __restrict__ sblk, const uint64_t* __restrict__ qoffs,
                            const uint32_t* __restrict__ qblk, KeyLayout L,
                            unsigned long long* __restrict__ key1, uint32_t* __restrict__ key2,
                            uint32_t* __restrict__ val) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint2 v = surv[i];
        const uint32_t g = v.y & ((1u << 27) - 1), shape = v.y >> 27;
        const uint64_t s = owner_of(soffs, sblk, v.x);
        const uint64_t q = owner_of(qoffs, qblk, g);
        const int64_t qp = (int64_t)g - (int64_t)qoffs[q], sp = (int64_t)v.x - (int64_t)soffs[s];
        const int64_t d = sp - qp;
        const unsigned long long ck =
            (((unsigned long long)q << L.bs | s) << L.bd) | (unsigned long long)(d + L.dbias);
        if (L.low) {
            key1[i] = (ck << L.low) | ((unsigned long long)qp << L.bsh) | shape;
        } else {
            key1[i] = ck;
            key2[i] = ((uint32_t)qp << 5) | shape;
        }
        val[i] = i;
    }
}

__global__ void k_gather_key1(const unsigned long long* __restrict__ key1, const uint32_t* __restrict__ val,
                              uint32_t n, unsigned long long* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = key1[val[i]];
}

__global__ void k_run_flags(const unsigned long long* __restrict__ key, uint32_t n, int shift,
                            uint8_t* __restrict__ flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        flag[i] = i == 0 || (key[i] >> shift) != (key[i - 1] >> shift);
}

struct ChainArgs {
    const uint2* surv;                // survivors in chain order
    const unsigned long long* key1s;  // sorted chain keys
    KeyLayout kl;
    const uint32_t* starts;           // chain starts
    const uint32_t* nchains;
    uint32_t nsurv;
    const uint64_t *soffs, *qoffs;
    const uint8_t* res;               // canonical residues
    uint64_t n_res;                   // residues (the buffer holds 64 more)
    const uint8_t* qcodes;            // query batch codes (16 bytes of padding)
    const int8_t* qbias;              // per batch position score bias, or null
    uint64_t qn;                      // batch positions
    const int32_t* matrix;            // 24 x 24 scores
    int thr, x;
    uint4* hsp;                       // (lo, hi, score, seed hits)
    unsigned long long* hkey;
    uint32_t* hval;
    unsigned long long* nhsp;
    uint64_t hcap;
    unsigned long long* ctr;          // [4] extensions, [5] avoided, [6] steps
    uint32_t* next;                   // chain work counter (zero at launch)
};

// Chains, one per lane (one subject, query and diagonal; hits in (query
// position, shape) order): the coverage test and the X-drop extensions of
// visit_scan (scan.rs:2384-2431), HSPs of at least thr appended with the
// number of the chain's seed hits they cover.  The ungapped X-drop
// (ungapped_xdrop, engine.rs:2460-2494; step count of xdrop_cat,
// scan.rs:859-904) runs as a per-lane state machine, 8 positions of each
// direction per warp iteration, the two directions side by side (they are
// independent: the HSP takes the sum of their bests and their extents):
// position t (0-based) of a direction scores
// P[s[sp + dir (t + off)]][qp + dir (t + off)] (off = 0 rightwards, 1
// leftwards); a strictly greater running sum is a new best and sets the
// extent to t + 1, a sum more than x below the best stops the direction
// after evaluating t.  So the warp's lanes stay converged whatever their
// chains' lengths, and lanes that finish a chain take the next one from a
// shared counter (chains are in query-major order, so a warp's lanes mostly
// read one query's profile).
constexpr int kXBlock = 8;

// 8 consecutive bytes of buf from byte index x on (bytes outside [0, limit)
// read as 0): two words, from three aligned loads when all are in range.
__device__ __forceinline__ uint2 load8(const uint8_t* __restrict__ buf, int64_t x, uint64_t limit) {
    if (x >= 0 && (uint64_t)x + 12 <= limit) {
        const uint32_t* w = reinterpret_cast<const uint32_t*>(buf + (x & ~(int64_t)3));
        const uint32_t sh = (uint32_t)(x & 3) * 8u;
        const uint32_t w0 = w[0], w1 = w[1], w2 = w[2];
        return make_uint2(__funnelshift_r(w0, w1, sh), __funnelshift_r(w1, w2, sh));
    }
    uint32_t v[2] = {0u, 0u};
#pragma unroll
    for (int b = 0; b < 8; b++) {
        const int64_t p = x + b;
        const uint32_t c = (p >= 0 && (uint64_t)p < limit) ? buf[p] : 0u;
        v[b >> 2] |= c << (8 * (b & 3));
    }
    return make_uint2(v[0], v[1]);
}

// One direction of an extension: position t of the next block, positions
// available n, running sum, best, extent, positions evaluated when it
// stopped, and whether it still runs.
struct XDir {
    int t, n, cur, best, xe, done;
    bool run;
};

// The block's 8 positions of one direction as byte runs of query codes,
// biases and subject residues (ascending addresses; leftwards reads them
// backwards).
struct XBlock {
    uint2 q, s, b;
};

__device__ __forceinline__ void xdrop_load(XBlock& L, const XDir& d, bool right, int64_t gq0, int64_t gs0,
                                           const ChainArgs& a) {
    const int64_t gq = gq0 + (right ? d.t : -(d.t + kXBlock));
    const int64_t gs = gs0 + (right ? d.t : -(d.t + kXBlock));
    L.q = load8(a.qcodes, gq, a.qn + 16);
    L.s = load8(a.res, gs, a.n_res + 64);
    L.b = a.qbias ? load8(reinterpret_cast<const uint8_t*>(a.qbias), gq, a.qn + 16) : make_uint2(0u, 0u);
}

// Scores S(q_i, s_j) + bias_i from the matrix in shared memory plus the
// query bias; then the X-drop rule.
__device__ __forceinline__ void xdrop_eval(XDir& d, const XBlock& L, bool right, const int32_t* smat, int x) {
    int sv[kXBlock];
#pragma unroll
    for (int u = 0; u < kXBlock; u++) {
        const int b = right ? u : kXBlock - 1 - u;  // byte of position t + u
        const uint32_t wq = b < 4 ? L.q.x : L.q.y, ws = b < 4 ? L.s.x : L.s.y, wb = b < 4 ? L.b.x : L.b.y;
        const int sh = 8 * (b & 3);
        int qcode = (int)((wq >> sh) & 0xFFu);
        qcode = qcode < 24 ? qcode : 22;
        const int scode = (int)((ws >> sh) & 0xFFu);
        const int bias = (int)(int8_t)((wb >> sh) & 0xFFu);
        sv[u] = smat[qcode * 24 + (scode < 24 ? scode : 22)] + bias;
    }
    bool stop = false;
    int done = 0;
#pragma unroll
    for (int u = 0; u < kXBlock; u++) {
        const int tt = d.t + u;
        if (!stop && tt < d.n) {
            d.cur += sv[u];
            if (d.cur > d.best) {
                d.best = d.cur;
                d.xe = tt + 1;
            } else if (d.cur < d.best - x) {
                stop = true;
                done = tt + 1;
            }
        }
    }
    d.t += kXBlock;
    if (stop || d.t >= d.n) {
        d.run = false;
        d.done = stop ? done : d.n;
    }
}

__global__ void __launch_bounds__(256, SABER_CHAINS_MIN_BLOCKS) k_chains(ChainArgs a) {
    __shared__ int32_t smat[576];
    for (int t = threadIdx.x; t < 576; t += blockDim.x) smat[t] = a.matrix[t];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t nch = *a.nchains;
    unsigned long long ext = 0, avoided = 0, steps = 0;
    uint32_t i = 0, e = 0;  // survivors left in this lane's chain
    bool retired = false;
    bool extending = false;  // an extension (both directions at once) is in progress
    unsigned long long hkey = 0;
    // positions fit 32 bits: queries and subjects are shorter than 2^19,
    // residue offsets below 2^32
    uint32_t q0 = 0;
    int qlen = 0, sl = 0, cover = 0;
    const uint8_t* subj = nullptr;
    int qp = 0, sp = 0;
    XDir R{0, 0, 0, 0, 0, 0, false}, Lf{0, 0, 0, 0, 0, 0, false};
    uint2 vnext = make_uint2(0, 0);
    bool have_next = false;  // vnext holds survivor i + 1 of this lane's chain
    const uint32_t m27 = (1u << 27) - 1u;
    while (true) {
        const bool need = !retired && !extending && i >= e;
        const uint32_t nb = __ballot_sync(0xffffffffu, need);
        if (nb) {
            const int leader = __ffs(nb) - 1;
            uint32_t c0 = 0;
            if (lane == leader) c0 = atomicAdd(a.next, (uint32_t)__popc(nb));
            c0 = __shfl_sync(0xffffffffu, c0, leader);
            if (need) {
                const uint32_t c = c0 + __popc(nb & ((1u << lane) - 1u));
                if (c >= nch) {
                    retired = true;
                } else {
                    i = a.starts[c];
                    e = c + 1 < nch ? a.starts[c + 1] : a.nsurv;
                    have_next = false;
                    const unsigned long long ck = a.key1s[i] >> a.kl.low;
                    const uint64_t q = ck >> (a.kl.bs + a.kl.bd);
                    const uint64_t s = (ck >> a.kl.bd) & ((1ull << a.kl.bs) - 1);
                    const int64_t d = (int64_t)(ck & ((1ull << a.kl.bd) - 1)) - a.kl.dbias;
                    hkey = (s << 40) | (q << 20) | (uint64_t)(d + kDBias);  // subject-major HSP key
                    q0 = (uint32_t)a.qoffs[q];
                    const uint64_t s0 = a.soffs[s];
                    qlen = (int)(a.qoffs[q + 1] - q0);
                    sl = (int)(a.soffs[s + 1] - s0);
                    subj = a.res + s0;
                    cover = 0;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, !retired) == 0) break;
        bool emit = false;
        uint4 hsp = make_uint4(0, 0, 0, 0);
        if (!retired) {
            if (!extending) {
                const uint2 v = have_next ? vnext : a.surv[i];
                // the chain's next survivor, for the coverage test at the end
                have_next = i + 1 < e;
                if (have_next) vnext = a.surv[i + 1];
                qp = (int)((v.y & m27) - q0);
                sp = (int)(v.x - (uint32_t)(subj - a.res));
                R = XDir{0, qlen - qp < sl - sp ? qlen - qp : sl - sp, 0, 0, 0, 0, true};
                Lf = XDir{0, qp < sp ? qp : sp, 0, 0, 0, 0, false};
                Lf.run = Lf.n > 0;
                extending = true;
            }
            // both directions advance a block per iteration: their loads are
            // issued together, then both are evaluated
            const int64_t gq0 = (int64_t)q0 + qp, gs0 = (int64_t)(subj - a.res) + sp;
            XBlock BR, BL;
            if (R.run) xdrop_load(BR, R, true, gq0, gs0, a);
            if (Lf.run) xdrop_load(BL, Lf, false, gq0, gs0, a);
            if (R.run) xdrop_eval(R, BR, true, smat, a.x);
            if (Lf.run) xdrop_eval(Lf, BL, false, smat, a.x);
            if (!R.run && !Lf.run) {
                steps += (uint64_t)(R.done + Lf.done);
                ext++;
                const int hi = qp + R.xe, lo = qp - Lf.xe;
                cover = hi;
                const int score = R.best + Lf.best;
                // the chain's next hits below hi are covered (query
                // positions ascend along the chain); the HSP counts them
                uint32_t j = i + 1;
                if (j < e && (int)((vnext.y & m27) - q0) < cover) {
                    j++;
                    have_next = false;
                    while (j < e && (int)((a.surv[j].y & m27) - q0) < cover) j++;
                }
                avoided += j - (i + 1);
                if (score >= a.thr) {
                    emit = true;
                    hsp = make_uint4((uint32_t)lo, (uint32_t)hi, (uint32_t)score, j - i);
                }
                i = j;
                extending = false;
            }
        }
        const uint32_t eb = __ballot_sync(0xffffffffu, emit);
        if (eb) {
            const int leader = __ffs(eb) - 1;
            unsigned long long slot0 = 0;
            if (lane == leader) slot0 = atomicAdd(a.nhsp, (unsigned long long)__popc(eb));
            slot0 = __shfl_sync(0xffffffffu, slot0, leader);
            if (emit) {
                const unsigned long long slot = slot0 + __popc(eb & ((1u << lane) - 1u));
                if (slot < a.hcap) {
                    a.hsp[slot] = hsp;
                    a.hkey[slot] = hkey;
                    a.hval[slot] = (uint32_t)slot;
                }
            }
        }
    }
    count_add(&a.ctr[4], ext);
    count_add(&a.ctr[5], avoided);
    count_add(&a.ctr[6], steps);
}

struct RegionArgs {
    const uint4* hsp;
    const uint32_t* order;            // HSPs sorted by (subject, query, diagonal)
    const unsigned long long* hkeys;  // sorted keys
    const uint32_t* starts;           // pair starts
    const uint32_t* npairs;
    uint32_t nhsp;
    const int32_t* region_thr;        // per query (NULL: hsp_threshold)
    int hsp_thr;
    int64_t join;
    uint32_t kmax;                    // max_regions_per_subject (<= 64)
    saber_region* out;
    uint4* rstat;                     // per region: HSPs, score sum, seed hits, 0
    unsigned long long* nout;
    uint64_t cap;
    unsigned long long* ctr;          // [7] hsps, [8] weak dropped
};

// Top list of one pair's regions by (best desc, d_min asc), with each
// region's HSP count, score sum and seed hits.  TopLocal holds up to 64 (the
// largest max_regions_per_subject) in local memory; TopReg holds up to K in
// registers, inserted by a compile-time network (the default cap is 4).  A
// new region goes after every entry that is not worse than it, as the
// reference's stable order does.
struct TopLocal {
    saber_region top[64];
    uint4 tst[64];
    uint32_t ntop = 0;
    __device__ __forceinline__ void insert(const saber_region& r, uint4 st, uint32_t kmax) {
        uint32_t pos = ntop;
        while (pos > 0 && (top[pos - 1].best < r.best || (top[pos - 1].best == r.best && top[pos - 1].d_min > r.d_min)))
            pos--;
        if (pos >= kmax) return;
        uint32_t last = ntop < kmax ? ntop : kmax - 1;
        for (uint32_t k = last; k > pos; k--) {
            top[k] = top[k - 1];
            tst[k] = tst[k - 1];
        }
        top[pos] = r;
        tst[pos] = st;
        if (ntop < kmax) ntop++;
    }
    __device__ __forceinline__ saber_region region(uint32_t k, uint32_t, uint32_t) const { return top[k]; }
    __device__ __forceinline__ uint4 stat(uint32_t k) const { return tst[k]; }
};

template <int K>
struct TopReg {
    int32_t dmin[K], dmax[K], best[K];
    uint4 tst[K];
    uint32_t ntop = 0;
    __device__ __forceinline__ void insert(const saber_region& r, uint4 st, uint32_t kmax) {
        uint32_t pos = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const bool worse = best[k] < r.best || (best[k] == r.best && dmin[k] > r.d_min);
            pos += ((uint32_t)k < ntop && !worse) ? 1u : 0u;
        }
        if (pos >= kmax) return;
#pragma unroll
        for (int k = K - 1; k > 0; k--) {
            if ((uint32_t)k > pos) {
                dmin[k] = dmin[k - 1];
                dmax[k] = dmax[k - 1];
                best[k] = best[k - 1];
                tst[k] = tst[k - 1];
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            if ((uint32_t)k == pos) {
                dmin[k] = r.d_min;
                dmax[k] = r.d_max;
                best[k] = r.best;
                tst[k] = st;
            }
        }
        if (ntop < kmax) ntop++;
    }
    __device__ __forceinline__ saber_region region(uint32_t k, uint32_t q, uint32_t s) const {
        saber_region r;
        r.query = q;
        r.subject = s;
        r.d_min = r.d_max = r.best = 0;
#pragma unroll
        for (int j = 0; j < K; j++)
            if ((uint32_t)j == k) {
                r.d_min = dmin[j];
                r.d_max = dmax[j];
                r.best = best[j];
            }
        return r;
    }
    __device__ __forceinline__ uint4 stat(uint32_t k) const {
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
        for (int j = 0; j < K; j++)
            if ((uint32_t)j == k) v = tst[j];
        return v;
    }
};

template <class Top>
__global__ void k_regions(RegionArgs a) {
    unsigned long long hsps = 0, weak = 0;
    const uint32_t np = *a.npairs;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const uint32_t b = a.starts[p];
        const uint32_t e = p + 1 < np ? a.starts[p + 1] : a.nhsp;
        const unsigned long long key = a.hkeys[b];
        const uint32_t s = (uint32_t)(key >> 40), q = (uint32_t)((key >> 20) & 0xFFFFF);
        const int thr = a.region_thr ? a.region_thr[q] : a.hsp_thr;
        hsps += e - b;
        // top kmax regions by (best desc, d_min asc)
        Top top;
        int64_t dmin = 0, dmax = 0;
        int best = 0;
        uint32_t evn = 0, evh = 0;
        int32_t evs = 0;
        bool open = false;
        auto close = [&]() {
            if (thr > a.hsp_thr && !(best >= thr || (evn >= 2 && evs >= thr))) {
                weak++;
                return;
            }
            saber_region r;
            r.query = q;
            r.subject = s;
            r.d_min = (int32_t)dmin;
            r.d_max = (int32_t)dmax;
            r.best = best;
            top.insert(r, make_uint4(evn, (uint32_t)evs, evh, 0u), a.kmax);
        };
        for (uint32_t i = b; i < e; i++) {
            const uint4 h = a.hsp[a.order[i]];
            const int64_t d = (int64_t)(a.hkeys[i] & 0xFFFFF) - kDBias;
            const int score = (int)h.z;
            if (open && d - dmax <= a.join) {
                if (d > dmax) dmax = d;
                if (score > best) best = score;
                evn++;
                evh += h.w;
                const int64_t sum = (int64_t)evs + score;
                evs = sum > INT32_MAX ? INT32_MAX : (int32_t)sum;
            } else {
                if (open) close();
                open = true;
                dmin = dmax = d;
                best = score;
                evn = 1;
                evh = h.w;
                evs = score;
            }
        }
        if (open) close();
        if (top.ntop) {
            const unsigned long long base = atomicAdd(a.nout, (unsigned long long)top.ntop);
            for (uint32_t k = 0; k < top.ntop; k++)
                if (base + k < a.cap) {
                    a.out[base + k] = top.region(k, q, s);
                    a.rstat[base + k] = top.stat(k);
                }
        }
    }
    count_add(&a.ctr[7], hsps);
    count_add(&a.ctr[8], weak);
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
static uint64_t ncodes_of(const saber_scan_params* p, uint32_t si) {
    uint64_t n = 1;
    for (uint32_t k = 0; k < p->shape_weight[si]; k++) n *= p->alpha_size;
    return n;
}

static ShapeDev shape_dev(const saber_scan_params* p, uint32_t si) {
    ShapeDev sh;
    memset(&sh, 0, sizeof(sh));
    for (uint32_t k = 0; k < p->shape_weight[si]; k++) sh.off[k] = p->shape_off[si][k];
    sh.w = p->shape_weight[si];
    sh.span = p->shape_span[si];
    return sh;
}

// auto_occ_cap (index.rs:329-336), host f64 as the reference computes it
static uint64_t auto_cap(uint64_t total, uint64_t ncodes, uint64_t db, uint64_t ref) {
    uint64_t fl = 256;
    if (ref > 0 && db > ref) fl = (uint64_t)std::ceil(256.0 * (double)db / (double)ref);
    uint64_t c = (uint64_t)std::ceil((double)total / (double)(ncodes ? ncodes : 1) * 64.0);
    return std::max(c, fl);
}

static uint64_t fingerprint(const saber_gpu* h, const saber_scan_params* p) {
    uint64_t f = 1469598103934665603ull;
    auto mix = [&](const void* d, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(d);
        for (size_t i = 0; i < n; i++) f = (f ^ b[i]) * 1099511628211ull;
    };
    mix(p->alpha_map, 24);
    mix(&p->alpha_size, 4);
    mix(&p->nshapes, 4);
    mix(p->shape_span, 4 * p->nshapes);
    mix(p->shape_weight, 4 * p->nshapes);
    mix(p->shape_off, sizeof(p->shape_off[0]) * p->nshapes);
    mix(&p->seed_max_occ, 8);
    mix(&p->ref_db_residues, 8);
    mix(&p->db_length, 8);
    mix(&h->main.n_res, 8);
    mix(&h->main.nsub, 8);
    const void* rp = h->main.res.p;
    mix(&rp, sizeof(rp));
    mix(&h->has_db_mask, 1);
    return f;
}

// Combined filter codes for alphabets of at most 14 letters whose groups
// hold at most 15 codes: byte = (index of the code within its letter's group)
// << 4 | letter, so that equal low nibbles are a reduced-letter identity and
// equal bytes an exact one.  Subject residues without a letter are 0xEE;
// query positions that never count are 0xFF; query codes >= 24 take group
// index 15, which no residue has.  Returns false when the alphabet does not
// fit (the filter then compares separate letter and residue records).
static bool comb_table(const saber_scan_params* p, uint8_t* tab /* 256 */) {
    if (p->alpha_size > 14) return false;
    int cnt[256] = {0};
    for (int c = 0; c < 256; c++) tab[c] = 0xEE;
    for (int c = 0; c < 24; c++) {
        const uint8_t L = p->alpha_map[c];
        if (L == 255) continue;
        if (L >= p->alpha_size) return false;
        if (cnt[L] >= 15) return false;
        tab[c] = (uint8_t)((cnt[L]++ << 4) | L);
    }
    return true;
}

__global__ void k_comb_bytes(const uint8_t* __restrict__ res, uint64_t N, CombTab tab, uint8_t* __restrict__ cb) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (uint64_t)gridDim.x * blockDim.x)
        cb[r] = tab.t[res[r]];
}

int scan_build_db(saber_gpu* h, const saber_scan_params* p) {
    const Dataset& ds = h->main;
    cudaStream_t s = h->stream;
    const uint64_t N = ds.n_res;
    AlphaMap am;
    memcpy(am.m, p->alpha_map, 24);
    {
        CombTab ct;
        h->sc_comb = comb_table(p, ct.t);
        if (h->sc_comb) {
            CUALLOC(h, h->sc_cb, N + 128);
            CU(h, cudaMemsetAsync(h->sc_cb.p, 0xEE, N + 128, s));
            if (N) k_comb_bytes<<<nblocks(N, 256, h->sm_count * 32), 256, 0, s>>>(ds.res.as<uint8_t>(), N, ct,
                                                                                 h->sc_cb.as<uint8_t>());
            CU(h, cudaGetLastError());
        }
    }
    CUALLOC(h, h->sc_sblk, ((N >> kOwnerShift) + 2) * 4);
    if (ds.nsub)
        k_block_owner<<<nblocks(ds.nsub, 256, h->sm_count * 32), 256, 0, s>>>(ds.soff.as<uint64_t>(), ds.nsub,
                                                                            h->sc_sblk.as<uint32_t>());
    CUALLOC(h, h->sc_sb, N + 128);
    CUALLOC(h, h->sc_rem, N + 64);
    CUALLOC(h, h->sc_dst, N + 64);
    CU(h, cudaMemsetAsync(h->sc_sb.p, kNonSeed, N + 128, s));
    CU(h, cudaMemsetAsync(h->sc_rem.p, 0, N + 64, s));
    CU(h, cudaMemsetAsync(h->sc_dst.p, 0, N + 64, s));
    if (N) {
        k_seed_bytes<<<nblocks(N, 256, h->sm_count * 32), 256, 0, s>>>(
            ds.res.as<uint8_t>(), h->has_db_mask ? h->db_mask.as<uint8_t>() : nullptr, N, am, h->sc_sb.as<uint8_t>());
        k_dists<<<nblocks(N, 256, h->sm_count * 32), 256, 0, s>>>(ds.soff.as<uint64_t>(), ds.nsub, N,
                                                                   h->sc_rem.as<uint8_t>(), h->sc_dst.as<uint8_t>());
        CU(h, cudaGetLastError());
    }
    // frequent codes per shape
    h->sc_caps.assign(p->nshapes, 0);
    h->sc_freq_off.assign(p->nshapes + 1, 0);
    uint64_t words = 0;
    for (uint32_t si = 0; si < p->nshapes; si++) {
        h->sc_freq_off[si] = words;
        words += (ncodes_of(p, si) + 63) / 64;
    }
    h->sc_freq_off[p->nshapes] = words;
    CUALLOC(h, h->sc_freq, words * 8 + 8);
    CU(h, cudaMemsetAsync(h->sc_freq.p, 0, words * 8 + 8, s));
    CUALLOC(h, h->sc_ctr, 32 * 8);
    for (uint32_t si = 0; si < p->nshapes; si++) {
        const uint64_t nc = ncodes_of(p, si);
        CUALLOC(h, h->sc_counts, nc * 4);
        CU(h, cudaMemsetAsync(h->sc_counts.p, 0, nc * 4, s));
        CU(h, cudaMemsetAsync(h->sc_ctr.p, 0, 8, s));
        if (N)
            k_db_counts<<<nblocks(N, 256, h->sm_count * 32), 256, 0, s>>>(
                h->sc_sb.as<uint8_t>(), h->sc_rem.as<uint8_t>(), N, shape_dev(p, si), p->alpha_size,
                h->sc_counts.as<uint32_t>(), h->sc_ctr.as<unsigned long long>());
        CU(h, cudaGetLastError());
        unsigned long long total = 0;
        CU(h, cudaMemcpyAsync(&total, h->sc_ctr.p, 8, cudaMemcpyDeviceToHost, s));
        CU(h, cudaStreamSynchronize(s));
        const uint64_t cap = p->seed_max_occ > 0 ? p->seed_max_occ
                                                 : auto_cap(total, nc, p->db_length, p->ref_db_residues);
        h->sc_caps[si] = cap;
        if (total > cap)
            k_freq_bits<<<nblocks(nc, 256, h->sm_count * 32), 256, 0, s>>>(
                h->sc_counts.as<uint32_t>(), nc, cap,
                h->sc_freq.as<unsigned long long>() + h->sc_freq_off[si]);
        CU(h, cudaGetLastError());
    }
    CU(h, cudaStreamSynchronize(s));
    h->sc_key = fingerprint(h, p);
    return SABER_OK;
}

static double ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// ---- the batch engine's regions: per-query cap and triage on the device ------
int triage_region_features(saber_gpu* h, const saber_region* d_reg, const uint4* d_rstat, const uint32_t* d_rq,
                           const uint32_t* d_rrank, const float4* d_qinfo, uint64_t n, float lambda, float logk);
int triage_predict(saber_gpu* h, DevBuf& model, DevBuf& wb, const float* d_X, uint64_t n, float* d_logit);

__global__ void k_query_count(const saber_region* __restrict__ reg, uint32_t n, uint32_t* __restrict__ qcnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&qcnt[reg[i].query], 1u);
}

// rank of each region within its query (regions are grouped by query) and
// whether it is within the query's first `cap`
__global__ void k_cap_flags(const saber_region* __restrict__ reg, uint32_t n, const uint32_t* __restrict__ qstart,
                            uint32_t cap, uint32_t* __restrict__ rank, uint8_t* __restrict__ flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t r = i - qstart[reg[i].query];
        rank[i] = r;
        flag[i] = r < cap;
    }
}

__global__ void k_gather_capped(const saber_region* __restrict__ reg, const uint4* __restrict__ rst,
                                const uint32_t* __restrict__ rank, const uint32_t* __restrict__ idx, uint32_t n,
                                saber_region* __restrict__ oreg, uint4* __restrict__ orst, uint32_t* __restrict__ orq,
                                uint32_t* __restrict__ orank) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = idx[i];
        const saber_region r = reg[k];
        oreg[i] = r;
        orst[i] = rst[k];
        orq[i] = r.query;
        orank[i] = rank[k];
    }
}

// per query: (length, region threshold, best of its first region, regions after the cap)
__global__ void k_query_info(const uint64_t* __restrict__ qoffs, const int32_t* __restrict__ rthr, int32_t thr0,
                             const uint32_t* __restrict__ qcnt, const uint32_t* __restrict__ qstart,
                             const saber_region* __restrict__ reg, uint32_t cap, uint32_t nq,
                             float4* __restrict__ qinfo) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const uint32_t c = qcnt[q];
        qinfo[q] = make_float4((float)(int64_t)(qoffs[q + 1] - qoffs[q]), (float)(rthr ? rthr[q] : thr0),
                               c ? (float)reg[qstart[q]].best : 0.f, (float)(c < cap ? c : cap));
    }
}

__global__ void k_keep_flags(const float* __restrict__ logit, uint32_t n, float thr, uint8_t* __restrict__ flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        flag[i] = logit[i] >= thr;
}

// the subject's first residue and length of each region (the host engine's
// windows and jobs need them for every region)
__global__ void k_region_subject_spans(const saber_region* __restrict__ reg, uint32_t n,
                                       const uint64_t* __restrict__ soffs, uint64_t* __restrict__ sbase,
                                       uint32_t* __restrict__ slen) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t sj = reg[i].subject;
        const uint64_t b = soffs[sj];
        sbase[i] = b;
        slen[i] = (uint32_t)(soffs[sj + 1] - b);
    }
}

__global__ void k_iota(uint32_t* __restrict__ v, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// Caps the sorted regions (sc_regions2 / sc_rstat2) at max_candidates per
// query, runs the learned triage on them when a model is installed (or
// collects their feature rows), and copies the kept regions with their
// positions in the capped list to pinned host memory.
static int region_sink(saber_gpu* h, const saber_scan_params* p, bool has_thr, uint64_t nregions, RegionSink& sk) {
    const QuerySet& qs = h->main.qs;
    cudaStream_t s = h->stream;
    const uint32_t nq = qs.nq;
    const uint32_t cap = std::max<uint32_t>(1, p->max_candidates);
    sk.n = sk.ncap = 0;
    sk.triaged = false;
    sk.collecting = h->tr_collect;
    if (h->tr_collect) {
        h->tr_rows.clear();
        h->tr_logits.clear();
        h->tr_labels.clear();
    }
    if (!nregions) return SABER_OK;
    const uint32_t n = (uint32_t)nregions;
    const saber_region* reg = h->sc_regions2.as<saber_region>();
    const uint4* rst = h->sc_rstat2.as<uint4>();
    CUALLOC(h, h->rg_qcnt, ((uint64_t)nq + 1) * 4);
    CUALLOC(h, h->rg_qstart, ((uint64_t)nq + 1) * 4);
    CUALLOC(h, h->rg_rank, (uint64_t)n * 4);
    CUALLOC(h, h->rg_flag, (uint64_t)n + 8);
    CUALLOC(h, h->rg_idx, (uint64_t)n * 4 + 8);
    CUALLOC(h, h->rg_idx2, (uint64_t)n * 4 + 8);
    uint32_t* qcnt = h->rg_qcnt.as<uint32_t>();
    uint32_t* qstart = h->rg_qstart.as<uint32_t>();
    uint32_t* nsel = h->sc_ctr.as<uint32_t>() + 44;
    CU(h, cudaMemsetAsync(qcnt, 0, ((uint64_t)nq + 1) * 4, s));
    k_query_count<<<nblocks(n, 256), 256, 0, s>>>(reg, n, qcnt);
    size_t t1 = 0, t2 = 0;
    CU(h, cub::DeviceScan::ExclusiveSum(nullptr, t1, qcnt, qstart, (int)nq + 1, s));
    CU(h, cub::DeviceSelect::Flagged(nullptr, t2, thrust::counting_iterator<uint32_t>(0), h->rg_flag.as<uint8_t>(),
                                     h->rg_idx.as<uint32_t>(), nsel, (int)n, s));
    CUALLOC(h, h->cub_tmp, std::max(t1, t2));
    size_t tb = h->cub_tmp.cap;
    CU(h, cub::DeviceScan::ExclusiveSum(h->cub_tmp.p, tb, qcnt, qstart, (int)nq + 1, s));
    k_cap_flags<<<nblocks(n, 256), 256, 0, s>>>(reg, n, qstart, cap, h->rg_rank.as<uint32_t>(), h->rg_flag.as<uint8_t>());
    tb = h->cub_tmp.cap;
    CU(h, cub::DeviceSelect::Flagged(h->cub_tmp.p, tb, thrust::counting_iterator<uint32_t>(0), h->rg_flag.as<uint8_t>(),
                                     h->rg_idx.as<uint32_t>(), nsel, (int)n, s));
    uint32_t ncap = 0;
    CU(h, cudaMemcpyAsync(&ncap, nsel, 4, cudaMemcpyDeviceToHost, s));
    CU(h, cudaStreamSynchronize(s));
    sk.ncap = ncap;
    if (!ncap) return SABER_OK;
    CUALLOC(h, h->tr_reg, (uint64_t)ncap * sizeof(saber_region));
    CUALLOC(h, h->tr_rstat, (uint64_t)ncap * sizeof(uint4));
    CUALLOC(h, h->tr_rq, (uint64_t)ncap * 4);
    CUALLOC(h, h->tr_rrank, (uint64_t)ncap * 4);
    k_gather_capped<<<nblocks(ncap, 256), 256, 0, s>>>(reg, rst, h->rg_rank.as<uint32_t>(), h->rg_idx.as<uint32_t>(),
                                                       ncap, h->tr_reg.as<saber_region>(), h->tr_rstat.as<uint4>(),
                                                       h->tr_rq.as<uint32_t>(), h->tr_rrank.as<uint32_t>());
    CU(h, cudaGetLastError());
    const saber_region* oreg = h->tr_reg.as<saber_region>();
    uint32_t nout = ncap;
    uint32_t* osrc = h->rg_idx2.as<uint32_t>();
    bool have_src = false;
    if (h->tr_on || h->tr_collect) {
        CUALLOC(h, h->tr_qinfo, std::max<uint64_t>(nq, 1) * sizeof(float4));
        if (nq)
            k_query_info<<<nblocks(nq, 256), 256, 0, s>>>(qs.offsets.as<uint64_t>(),
                                                          has_thr ? h->sc_rthr.as<int32_t>() : nullptr,
                                                          (int32_t)p->hsp_threshold, qcnt, qstart, reg, cap, nq,
                                                          h->tr_qinfo.as<float4>());
        int rc = triage_region_features(h, h->tr_reg.as<saber_region>(), h->tr_rstat.as<uint4>(),
                                        h->tr_rq.as<uint32_t>(), h->tr_rrank.as<uint32_t>(), h->tr_qinfo.as<float4>(),
                                        ncap, sk.lambda, sk.logk);
        if (rc != SABER_OK) return rc;
        if (h->tr_on) {
            rc = triage_predict(h, h->tr_model, h->tr_wb, h->tr_X.as<float>(), ncap, h->tr_logit.as<float>());
            if (rc != SABER_OK) return rc;
        }
        if (h->tr_collect) {
            h->tr_rows.resize((uint64_t)ncap * SABER_TRIAGE_ROW_FLOATS);
            CU(h, cudaMemcpyAsync(h->tr_rows.data(), h->tr_X.p, (uint64_t)ncap * SABER_TRIAGE_ROW_FLOATS * 4,
                                  cudaMemcpyDeviceToHost, s));
            h->tr_logits.assign(ncap, 0.f);
            if (h->tr_on)
                CU(h, cudaMemcpyAsync(h->tr_logits.data(), h->tr_logit.p, (uint64_t)ncap * 4, cudaMemcpyDeviceToHost,
                                      s));
            h->tr_labels.assign(ncap, 0);
        }
        if (h->tr_on) {
            k_keep_flags<<<nblocks(ncap, 256), 256, 0, s>>>(h->tr_logit.as<float>(), ncap, h->tr_threshold,
                                                           h->rg_flag.as<uint8_t>());
            tb = h->cub_tmp.cap;
            CU(h, cub::DeviceSelect::Flagged(h->cub_tmp.p, tb, thrust::counting_iterator<uint32_t>(0),
                                             h->rg_flag.as<uint8_t>(), osrc, nsel, (int)ncap, s));
            CU(h, cudaMemcpyAsync(&nout, nsel, 4, cudaMemcpyDeviceToHost, s));
            CU(h, cudaStreamSynchronize(s));
            CUALLOC(h, h->rg_out, (uint64_t)std::max<uint32_t>(nout, 1) * sizeof(saber_region));
            if (nout)
                k_gather_regions<<<nblocks(nout, 256), 256, 0, s>>>(h->tr_reg.as<saber_region>(), osrc, nout,
                                                                   h->rg_out.as<saber_region>());
            oreg = h->rg_out.as<saber_region>();
            have_src = true;
            sk.triaged = true;
        }
    }
    if (!have_src) k_iota<<<nblocks(nout, 256), 256, 0, s>>>(osrc, nout);
    CU(h, cudaGetLastError());
    CUALLOC(h, h->pin_reg, (uint64_t)std::max<uint32_t>(nout, 1) * sizeof(saber_region));
    CUALLOC(h, h->pin_src, (uint64_t)std::max<uint32_t>(nout, 1) * 4);
    CUALLOC(h, h->pin_sbase, (uint64_t)std::max<uint32_t>(nout, 1) * 8);
    CUALLOC(h, h->pin_slen, (uint64_t)std::max<uint32_t>(nout, 1) * 4);
    CUALLOC(h, h->rg_sbase, (uint64_t)std::max<uint32_t>(nout, 1) * 8);
    CUALLOC(h, h->rg_slen, (uint64_t)std::max<uint32_t>(nout, 1) * 4);
    if (nout) {
        k_region_subject_spans<<<nblocks(nout, 256), 256, 0, s>>>(oreg, nout, h->main.soff.as<uint64_t>(),
                                                                 h->rg_sbase.as<uint64_t>(),
                                                                 h->rg_slen.as<uint32_t>());
        CU(h, cudaGetLastError());
        CU(h, cudaMemcpyAsync(h->pin_reg.p, oreg, (uint64_t)nout * sizeof(saber_region), cudaMemcpyDeviceToHost, s));
        CU(h, cudaMemcpyAsync(h->pin_src.p, osrc, (uint64_t)nout * 4, cudaMemcpyDeviceToHost, s));
        CU(h, cudaMemcpyAsync(h->pin_sbase.p, h->rg_sbase.p, (uint64_t)nout * 8, cudaMemcpyDeviceToHost, s));
        CU(h, cudaMemcpyAsync(h->pin_slen.p, h->rg_slen.p, (uint64_t)nout * 4, cudaMemcpyDeviceToHost, s));
    }
    CU(h, cudaStreamSynchronize(s));
    sk.regs = h->pin_reg.as<saber_region>();
    sk.src = h->pin_src.as<uint32_t>();
    sk.sbase = h->pin_sbase.as<uint64_t>();
    sk.slen = h->pin_slen.as<uint32_t>();
    sk.n = nout;
    return SABER_OK;
}

int scan_regions(saber_gpu* h, const saber_scan_params* p, const uint8_t* q_mask, const int32_t* region_thr,
                 saber_region* out, uint64_t out_cap, uint64_t* n_out, saber_scan_stats* st, RegionSink* sink) {
    const Dataset& ds = h->main;
    const QuerySet& qs = ds.qs;
    if (!ds.has_db || !qs.has) return fail(h, SABER_ERR_STATE, "no database or query set loaded");
    if (!h->scheme.has) return fail(h, SABER_ERR_STATE, "no scoring scheme set");
    if (!p || p->nshapes == 0 || p->nshapes > 32 || p->alpha_size == 0 || p->alpha_size > 127)
        return fail(h, SABER_ERR_ARG, "invalid scan parameters");
    uint32_t minspan = 1u << 30;
    for (uint32_t si = 0; si < p->nshapes; si++) {
        if (p->shape_weight[si] < 1 || p->shape_weight[si] > 16 || p->shape_span[si] > 64 ||
            p->shape_span[si] < p->shape_weight[si])
            return fail(h, SABER_ERR_ARG, "invalid shape %u", si);
        if (ncodes_of(p, si) > (1ull << 31)) return fail(h, SABER_ERR_ARG, "shape %u has too many codes", si);
        minspan = std::min(minspan, p->shape_span[si]);
    }
    if (p->max_regions_per_subject > 64) return fail(h, SABER_ERR_ARG, "max_regions_per_subject must be <= 64");
    if (ds.max_len >= (uint64_t)kDBias)
        return fail(h, SABER_ERR_ARG, "subject too long for the seed scan (< 2^19 residues)");
    if (ds.n_res >= (1ull << 32))
        return fail(h, SABER_ERR_ARG, "database too large for one scan (residues < 2^32): split it into volumes");
    if (ds.nsub >= (1ull << 24) || qs.nq >= (1u << 20) || qs.offs[qs.nq] >= (1ull << 27))
        return fail(h, SABER_ERR_ARG, "scan batch too large (subjects < 2^24, queries < 2^20, residues < 2^27)");
    for (uint32_t q = 0; q < qs.nq; q++)
        if (qs.offs[q + 1] - qs.offs[q] >= (uint64_t)kDBias) return fail(h, SABER_ERR_ARG, "query too long");
    cudaStream_t s = h->stream;
    if (h->sc_key != fingerprint(h, p)) {
        int rc = scan_build_db(h, p);
        if (rc != SABER_OK) return rc;
    }
    saber_scan_stats local{};
    cudaEvent_t ev[5];
    for (int i = 0; i < 5; i++) CU(h, cudaEventCreate(&ev[i]));
    struct G {
        cudaEvent_t* e;
        ~G() {
            for (int i = 0; i < 5; i++) cudaEventDestroy(e[i]);
        }
    } g_{ev};
    CU(h, cudaEventRecord(ev[0], s));
    const uint64_t N = ds.n_res, QN = qs.offs[qs.nq];
    AlphaMap am;
    memcpy(am.m, p->alpha_map, 24);
    // query bytes and distances
    CUALLOC(h, h->sc_qsb, QN + 128);
    CUALLOC(h, h->sc_qfull, QN + 64);
    CUALLOC(h, h->sc_qrem, QN + 64);
    CUALLOC(h, h->sc_qdst, QN + 64);
    CUALLOC(h, h->sc_tmp, QN + 64);
    if (q_mask) CU(h, cudaMemcpyAsync(h->sc_tmp.p, q_mask, QN, cudaMemcpyHostToDevice, s));
    CU(h, cudaMemsetAsync(h->sc_qsb.p, kQSent, QN + 128, s));
    if (QN) {
        k_query_bytes<<<nblocks(QN, 256), 256, 0, s>>>(qs.codes.as<uint8_t>(), q_mask ? h->sc_tmp.as<uint8_t>() : nullptr,
                                                       QN, am, h->sc_qsb.as<uint8_t>(), h->sc_qfull.as<uint8_t>());
        k_dists<<<nblocks(QN, 256), 256, 0, s>>>(qs.offsets.as<uint64_t>(), qs.nq, QN, h->sc_qrem.as<uint8_t>(),
                                                 h->sc_qdst.as<uint8_t>());
        CU(h, cudaGetLastError());
    }
    if (region_thr) {
        CUALLOC(h, h->sc_rthr, (uint64_t)qs.nq * 4 + 4);
        CU(h, cudaMemcpyAsync(h->sc_rthr.p, region_thr, (uint64_t)qs.nq * 4, cudaMemcpyHostToDevice, s));
    }
    CUALLOC(h, h->sc_ctr, 32 * 8);
    unsigned long long* ctr = h->sc_ctr.as<unsigned long long>();
    CU(h, cudaMemsetAsync(ctr, 0, 32 * 8, s));
    // survivors buffer (grown and the scan redone on overflow)
    uint64_t scap = std::max<uint64_t>(1 << 20, h->sc_surv.cap / 8);
    uint64_t nsurv = 0;
    const int cfil = (int)(minspan / 2);
    // seed tables of all shapes, concatenated, rank-compressed: per shape the
    // 32-code groups (presence bits, rank), at most QN + 1 entry offsets and
    // QN batch positions -- sized by their bounds, so no host sync is needed
    const uint32_t nsh = p->nshapes;
    std::vector<uint64_t> gbase(nsh + 1, 0);
    uint64_t ncmax = 0;
    for (uint32_t si = 0; si < nsh; si++) {
        const uint64_t nc = ncodes_of(p, si);
        ncmax = std::max(ncmax, nc);
        gbase[si + 1] = gbase[si] + (nc + 31) / 32;
    }
    const uint64_t ngmax = (ncmax + 31) / 32;
    const uint64_t coff_n = QN + 1;
    CUALLOC(h, h->sc_qcnt, std::max(ncmax, coff_n) * 4);
    CUALLOC(h, h->sc_qpres, gbase[nsh] * 8 + 8);
    CUALLOC(h, h->sc_gcnt, ngmax * 4 + 4);
    CUALLOC(h, h->sc_grank, ngmax * 4 + 4);
    CUALLOC(h, h->sc_cntc, coff_n * 4);
    CUALLOC(h, h->sc_qoff, (uint64_t)nsh * coff_n * 4);
    CUALLOC(h, h->sc_qent, (uint64_t)nsh * QN * 4 + 4);
    CUALLOC(h, h->sc_qrng, (uint64_t)nsh * QN * 8 + 8);
    {
        size_t t1 = 0, t2 = 0;
        CU(h, cub::DeviceScan::ExclusiveSum(nullptr, t1, h->sc_gcnt.as<uint32_t>(), h->sc_grank.as<uint32_t>(),
                                            (int)ngmax, s));
        CU(h, cub::DeviceScan::ExclusiveSum(nullptr, t2, h->sc_cntc.as<uint32_t>(), h->sc_qoff.as<uint32_t>(),
                                            (int)coff_n, s));
        CUALLOC(h, h->cub_tmp, std::max(t1, t2));
    }
    uint32_t* cnt = h->sc_qcnt.as<uint32_t>();
    for (uint32_t si = 0; si < nsh; si++) {
        const uint64_t nc = ncodes_of(p, si), ng = (nc + 31) / 32;
        const ShapeDev sh = shape_dev(p, si);
        const unsigned long long* freq = h->sc_freq.as<unsigned long long>() + h->sc_freq_off[si];
        uint2* grp = h->sc_qpres.as<uint2>() + gbase[si];
        uint32_t* coff = h->sc_qoff.as<uint32_t>() + (uint64_t)si * coff_n;
        CU(h, cudaMemsetAsync(cnt, 0, nc * 4, s));
        CU(h, cudaMemsetAsync(h->sc_cntc.p, 0, coff_n * 4, s));
        if (QN)
            k_query_seeds<0><<<nblocks(QN, 256), 256, 0, s>>>(h->sc_qsb.as<uint8_t>(), h->sc_qrem.as<uint8_t>(), QN,
                                                              sh, p->alpha_size, freq, cnt, nullptr, nullptr,
                                                              nullptr, ctr);
        k_group_bits<<<nblocks(nc, 256, h->sm_count * 32), 256, 0, s>>>(cnt, nc, grp, h->sc_gcnt.as<uint32_t>());
        size_t tb = h->cub_tmp.cap;
        CU(h, cub::DeviceScan::ExclusiveSum(h->cub_tmp.p, tb, h->sc_gcnt.as<uint32_t>(), h->sc_grank.as<uint32_t>(),
                                            (int)ng, s));
        k_group_ranks<<<nblocks(nc, 256, h->sm_count * 32), 256, 0, s>>>(cnt, nc, h->sc_grank.as<uint32_t>(), grp,
                                                                         h->sc_cntc.as<uint32_t>());
        tb = h->cub_tmp.cap;
        CU(h, cub::DeviceScan::ExclusiveSum(h->cub_tmp.p, tb, h->sc_cntc.as<uint32_t>(), coff, (int)coff_n, s));
        if (QN)
            k_entry_ranges<<<nblocks(QN, 256), 256, 0, s>>>(coff, QN, (uint32_t)((uint64_t)si * QN),
                                                            h->sc_qrng.as<uint2>() + (uint64_t)si * QN);
        // pass 1: the counts' buffer becomes the per-rank cursors
        CU(h, cudaMemsetAsync(cnt, 0, coff_n * 4, s));
        if (QN)
            k_query_seeds<1><<<nblocks(QN, 256), 256, 0, s>>>(h->sc_qsb.as<uint8_t>(), h->sc_qrem.as<uint8_t>(), QN,
                                                              sh, p->alpha_size, freq, cnt, grp, coff,
                                                              h->sc_qent.as<uint32_t>() + (uint64_t)si * QN, ctr);
        CU(h, cudaGetLastError());
    }
    CU(h, cudaEventRecord(ev[1], s));
    ScanArgs a;
    a.sb = h->sc_sb.as<uint8_t>();
    a.res = ds.res.as<uint8_t>();
    a.rem = h->sc_rem.as<uint8_t>();
    a.dst = h->sc_dst.as<uint8_t>();
    a.N = N;
    a.grp = h->sc_qpres.as<uint2>();
    a.rng = h->sc_qrng.as<uint2>();
    a.qent = h->sc_qent.as<uint32_t>();
    CUALLOC(h, h->sc_qwin, QN * 32 + 32);
    CUALLOC(h, h->sc_qwinx, QN * 32 + 32);
    CombTab ctab;
    const bool comb = h->sc_comb && comb_table(p, ctab.t);
    CUALLOC(h, h->sc_combtab, sizeof(CombTab));
    if (comb) CU(h, cudaMemcpyAsync(h->sc_combtab.p, &ctab, sizeof(CombTab), cudaMemcpyHostToDevice, s));
    if (QN)
        k_query_windows<<<nblocks(QN * 32, 256), 256, 0, s>>>(
            h->sc_qsb.as<uint8_t>(), h->sc_qfull.as<uint8_t>(), h->sc_qrem.as<uint8_t>(), h->sc_qdst.as<uint8_t>(),
            QN, cfil, comb ? h->sc_combtab.as<CombTab>() : nullptr, h->sc_qwin.as<uint8_t>(),
            h->sc_qwinx.as<uint8_t>());
    a.cb = comb ? h->sc_cb.as<uint8_t>() : nullptr;
    a.qwin = h->sc_qwin.as<uint4>();
    a.qwinx = h->sc_qwinx.as<uint4>();
    a.cfil = cfil;
    a.min_ids = p->hit_filter_min_ids;
    a.kx = p->hit_filter_exact_weight;
    a.asize = p->alpha_size;
    a.nsurv = ctr + 10;
    a.ctr = ctr;
    for (uint32_t si = 0; si < nsh; si++) {
        a.sh[si] = shape_dev(p, si);
        a.grp_off[si] = gbase[si];
        a.rng_off[si] = (uint64_t)si * QN;
    }
    // passes over groups of shapes whose tables stay within the L2 budget:
    // as many shapes per pass as the largest shape's tables allow, rounded
    // down to whole unroll groups, and at least one unroll group: with fewer
    // shapes a lane has fewer table lookups in flight, which cost more than
    // the tables spilling from L2 (11,000 queries: 1 shape per pass 315 ms,
    // 4 shapes 298 ms; 2,000 queries: 4 shapes 65.8 ms, 8 or more 68 ms)
    uint64_t shape_bytes = 0;
    for (uint32_t si = 0; si < nsh; si++)
        shape_bytes = std::max(shape_bytes, (gbase[si + 1] - gbase[si]) * 8 + QN * 8 + QN * 4);
    uint64_t per_pass = std::max<uint64_t>(1, h->scan_table_bytes / std::max<uint64_t>(shape_bytes, 1));
    if (per_pass >= (uint64_t)kShapeUnroll) per_pass -= per_pass % kShapeUnroll;
    else per_pass = kShapeUnroll;
    std::vector<std::pair<uint32_t, uint32_t>> passes;
    for (uint32_t si = 0; si < nsh; si += (uint32_t)std::min<uint64_t>(per_pass, nsh))
        passes.push_back({si, (uint32_t)std::min<uint64_t>(nsh, si + per_pass)});
    int scan_bps = 0;
    CU(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&scan_bps, comb ? k_scan<true> : k_scan<false>,
                                                        kScanWarps * 32, 0));
    const unsigned scan_grid = (unsigned)std::max(1, scan_bps) * (unsigned)h->sm_count;
    for (int attempt = 0; attempt < 8; attempt++) {
        CUALLOC(h, h->sc_surv, scap * 8);
        CU(h, cudaMemsetAsync(ctr + 2, 0, 9 * 8, s));  // hits, filtered, ..., survivors
        if (QN && N) {
            a.surv = h->sc_surv.as<uint2>();
            a.cap = scap;
            for (const auto& ps : passes) {
                a.s0 = ps.first;
                a.s1 = ps.second;
                if (comb) k_scan<true><<<scan_grid, kScanWarps * 32, 0, s>>>(a);
                else k_scan<false><<<scan_grid, kScanWarps * 32, 0, s>>>(a);
            }
            CU(h, cudaGetLastError());
        }
        unsigned long long hc[16];
        CU(h, cudaMemcpyAsync(hc, ctr, 16 * 8, cudaMemcpyDeviceToHost, s));
        CU(h, cudaStreamSynchronize(s));
        nsurv = hc[10];
        local.seed_positions = hc[0];
        local.seeds_frequent_skipped = hc[1];
        local.hits = hc[2];
        local.hits_filtered = hc[3];
        if (nsurv <= scap) break;
        scap = nsurv + nsurv / 4 + 1024;
        if (attempt == 7) return fail(h, SABER_ERR_NOMEM, "survivor buffer did not converge");
    }
    if (nsurv >= (1ull << 31)) return fail(h, SABER_ERR_ARG, "too many survivors in one batch");
    const uint32_t ns = (uint32_t)nsurv;
    CU(h, cudaEventRecord(ev[2], s));
    uint64_t nregions = 0;
    std::vector<saber_region> regs;
    if (ns) {
        CUALLOC(h, h->sc_key1, (uint64_t)ns * 8);
        CUALLOC(h, h->sc_key1o, (uint64_t)ns * 8);
        CUALLOC(h, h->sc_val, (uint64_t)ns * 4);
        CUALLOC(h, h->sc_valo, (uint64_t)ns * 4);
        CUALLOC(h, h->sc_flags, (uint64_t)ns + 8);
        CUALLOC(h, h->sc_chains, (uint64_t)ns * 4 + 8);
        // chain order (query, subject, diagonal, query position, shape): one
        // sort of composite keys when the fields fit 64 bits, else two stable
        // sorts; the sorts cover only the keys' significant bits
        auto bits_for = [](uint64_t v) {
            int b = 1;
            while (b < 64 && (v >> b)) b++;
            return b;
        };
        uint64_t qmax = 1;
        for (uint32_t q = 0; q < qs.nq; q++) qmax = std::max<uint64_t>(qmax, qs.offs[q + 1] - qs.offs[q]);
        const uint64_t smax = std::max<uint64_t>(ds.max_len, 1);
        KeyLayout kl;
        {
            const int bq = bits_for(qs.nq ? qs.nq - 1 : 0), bs = bits_for(ds.nsub ? ds.nsub - 1 : 0);
            const int bd = bits_for(qmax + smax), bp = bits_for(qmax), bsh = bits_for(p->nshapes - 1);
            if (bq + bs + bd + bp + bsh <= 64) {
                kl = KeyLayout{bp + bsh, bs, bd, bsh, (int64_t)qmax};
            } else {
                kl = KeyLayout{0, 24, 20, 5, (int64_t)kDBias};
            }
        }
        if (!kl.low) {  // the second key of the two-sort layout
            CUALLOC(h, h->sc_key2, (uint64_t)ns * 4);
            CUALLOC(h, h->sc_key2o, (uint64_t)ns * 4);
        }
        const int chain_bits = bits_for(qs.nq ? qs.nq - 1 : 0) + kl.bs + kl.bd;
        // owner table of the batch positions (the database's is built with the scan state)
        CUALLOC(h, h->sc_qblk, ((QN >> kOwnerShift) + 2) * 4);
        if (qs.nq)
            k_block_owner<<<nblocks(qs.nq, 256), 256, 0, s>>>(qs.offsets.as<uint64_t>(), qs.nq,
                                                              h->sc_qblk.as<uint32_t>());
        k_surv_keys<<<nblocks(ns, 256), 256, 0, s>>>(h->sc_surv.as<uint2>(), ns, ds.soff.as<uint64_t>(),
                                                     h->sc_sblk.as<uint32_t>(), qs.offsets.as<uint64_t>(),
                                                     h->sc_qblk.as<uint32_t>(), kl,
                                                     kl.low ? h->sc_key1o.as<unsigned long long>()
                                                            : h->sc_key1.as<unsigned long long>(),
                                                     h->sc_key2.as<uint32_t>(),
                                                     kl.low ? h->sc_valo.as<uint32_t>() : h->sc_val.as<uint32_t>());
        const int k2_end = std::min(32, 5 + bits_for(qmax));
        const int k1_end = std::min(64, chain_bits + kl.low);
        size_t t1 = 0, t2 = 0, t3 = 0;
        if (!kl.low)
            CU(h, cub::DeviceRadixSort::SortPairs(nullptr, t1, h->sc_key2.as<uint32_t>(), h->sc_key2o.as<uint32_t>(),
                                                  h->sc_val.as<uint32_t>(), h->sc_valo.as<uint32_t>(), (int)ns, 0,
                                                  k2_end, s));
        CU(h, cub::DeviceRadixSort::SortPairs(nullptr, t2, h->sc_key1o.as<unsigned long long>(),
                                              h->sc_key1.as<unsigned long long>(), h->sc_valo.as<uint32_t>(),
                                              h->sc_val.as<uint32_t>(), (int)ns, 0, k1_end, s));
        CU(h, cub::DeviceSelect::Flagged(nullptr, t3, thrust::counting_iterator<uint32_t>(0), h->sc_flags.as<uint8_t>(),
                                         h->sc_chains.as<uint32_t>(), h->sc_ctr.as<uint32_t>() + 40, (int)ns, s));
        CUALLOC(h, h->cub_tmp, std::max(t1, std::max(t2, t3)));
        size_t tb = h->cub_tmp.cap;
        if (!kl.low) {
            CU(h, cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, tb, h->sc_key2.as<uint32_t>(),
                                                  h->sc_key2o.as<uint32_t>(), h->sc_val.as<uint32_t>(),
                                                  h->sc_valo.as<uint32_t>(), (int)ns, 0, k2_end, s));
            k_gather_key1<<<nblocks(ns, 256), 256, 0, s>>>(h->sc_key1.as<unsigned long long>(),
                                                           h->sc_valo.as<uint32_t>(), ns,
                                                           h->sc_key1o.as<unsigned long long>());
        }
        CU(h, cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, tb, h->sc_key1o.as<unsigned long long>(),
                                              h->sc_key1.as<unsigned long long>(), h->sc_valo.as<uint32_t>(),
                                              h->sc_val.as<uint32_t>(), (int)ns, 0, k1_end, s));
        // chains: runs of one (query, subject, diagonal)
        k_run_flags<<<nblocks(ns, 256), 256, 0, s>>>(h->sc_key1.as<unsigned long long>(), ns, kl.low,
                                                     h->sc_flags.as<uint8_t>());
        uint32_t* nchains = h->sc_ctr.as<uint32_t>() + 40;
        CU(h, cub::DeviceSelect::Flagged(h->cub_tmp.p, tb, thrust::counting_iterator<uint32_t>(0),
                                         h->sc_flags.as<uint8_t>(), h->sc_chains.as<uint32_t>(), nchains, (int)ns, s));
        // HSP buffers: at most one HSP per survivor, usually far fewer (7 % of
        // the survivors of a protein batch, 0.01 % in nn), so they start at an
        // eighth of the survivors (or what earlier calls needed) and are grown
        // and the chains rerun when an HSP count exceeds them
        uint64_t hcap = std::max<uint64_t>(std::max<uint64_t>(1u << 20, h->sc_hsp.cap / 16), (uint64_t)ns / 8);
        hcap = std::min<uint64_t>(hcap, std::max<uint64_t>(1024, ns));
        // survivors in chain order (one gather, so the chains read them directly)
        CUALLOC(h, h->sc_surv2, (uint64_t)ns * 8);
        k_gather_u64_by<<<nblocks(ns, 256), 256, 0, s>>>(
            reinterpret_cast<const unsigned long long*>(h->sc_surv.p), h->sc_val.as<uint32_t>(), ns,
            h->sc_surv2.as<unsigned long long>());
        ChainArgs c;
        c.surv = h->sc_surv2.as<uint2>();
        c.key1s = h->sc_key1.as<unsigned long long>();
        c.starts = h->sc_chains.as<uint32_t>();
        c.kl = kl;
        c.nchains = nchains;
        c.nsurv = ns;
        c.soffs = ds.soff.as<uint64_t>();
        c.qoffs = qs.offsets.as<uint64_t>();
        c.res = ds.res.as<uint8_t>();
        c.n_res = ds.n_res;
        c.qcodes = qs.codes.as<uint8_t>();
        c.qbias = qs.has_bias ? qs.bias.as<int8_t>() : nullptr;
        c.qn = qs.offs[qs.nq];
        c.matrix = h->scheme.d_matrix.as<int32_t>();
        c.thr = p->hsp_threshold;
        c.x = p->x_drop;
        c.nhsp = ctr + 11;
        c.ctr = ctr;
        c.next = reinterpret_cast<uint32_t*>(ctr + 14);
        int chain_bps = 0;
        CU(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&chain_bps, k_chains, 256, 0));
        unsigned long long nh = 0;
        for (int attempt = 0;; attempt++) {
            CUALLOC(h, h->sc_hsp, hcap * 16);
            CUALLOC(h, h->sc_hkey, hcap * 8);
            CUALLOC(h, h->sc_hkeyo, hcap * 8);
            CUALLOC(h, h->sc_hval, hcap * 4);
            CUALLOC(h, h->sc_hvalo, hcap * 4);
            c.hsp = h->sc_hsp.as<uint4>();
            c.hkey = h->sc_hkey.as<unsigned long long>();
            c.hval = h->sc_hval.as<uint32_t>();
            c.hcap = hcap;
            // extensions, avoided, steps; HSP count; chain work counter
            CU(h, cudaMemsetAsync(ctr + 4, 0, 3 * 8, s));
            CU(h, cudaMemsetAsync(ctr + 11, 0, 8, s));
            CU(h, cudaMemsetAsync(c.next, 0, 4, s));
            k_chains<<<(unsigned)std::max(1, chain_bps) * (unsigned)h->sm_count, 256, 0, s>>>(c);
            CU(h, cudaGetLastError());
            CU(h, cudaMemcpyAsync(&nh, ctr + 11, 8, cudaMemcpyDeviceToHost, s));
            CU(h, cudaStreamSynchronize(s));
            if (nh <= hcap) break;
            // the HSP count of a batch does not depend on the buffer: one rerun fits
            if (attempt >= 1) return fail(h, SABER_ERR_DEVICE, "HSP buffer overflow");
            hcap = nh + nh / 4 + 1024;
        }
        CU(h, cudaEventRecord(ev[3], s));
        const uint32_t nhsp = (uint32_t)nh;
        if (nhsp) {
            size_t t4 = 0;
            CU(h, cub::DeviceRadixSort::SortPairs(nullptr, t4, h->sc_hkey.as<unsigned long long>(),
                                                  h->sc_hkeyo.as<unsigned long long>(), h->sc_hval.as<uint32_t>(),
                                                  h->sc_hvalo.as<uint32_t>(), (int)nhsp, 0, 64, s));
            CUALLOC(h, h->cub_tmp, t4);
            tb = h->cub_tmp.cap;
            CU(h, cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, tb, h->sc_hkey.as<unsigned long long>(),
                                                  h->sc_hkeyo.as<unsigned long long>(), h->sc_hval.as<uint32_t>(),
                                                  h->sc_hvalo.as<uint32_t>(), (int)nhsp, 0, 64, s));
            CUALLOC(h, h->sc_pairs, (uint64_t)nhsp * 4 + 8);
            k_run_flags<<<nblocks(nhsp, 256), 256, 0, s>>>(h->sc_hkeyo.as<unsigned long long>(), nhsp, 20,
                                                           h->sc_flags.as<uint8_t>());
            uint32_t* npairs = h->sc_ctr.as<uint32_t>() + 42;
            CU(h, cub::DeviceSelect::Flagged(h->cub_tmp.p, tb, thrust::counting_iterator<uint32_t>(0),
                                             h->sc_flags.as<uint8_t>(), h->sc_pairs.as<uint32_t>(), npairs, (int)nhsp, s));
            uint64_t rcap = (uint64_t)nhsp + 16;
            CUALLOC(h, h->sc_regions, rcap * sizeof(saber_region));
            CUALLOC(h, h->sc_rstat, rcap * sizeof(uint4));
            RegionArgs r;
            r.hsp = h->sc_hsp.as<uint4>();
            r.order = h->sc_hvalo.as<uint32_t>();
            r.hkeys = h->sc_hkeyo.as<unsigned long long>();
            r.starts = h->sc_pairs.as<uint32_t>();
            r.npairs = npairs;
            r.nhsp = nhsp;
            r.region_thr = region_thr ? h->sc_rthr.as<int32_t>() : nullptr;
            r.hsp_thr = p->hsp_threshold;
            r.join = 2 * (int64_t)p->window_slack;
            r.kmax = std::max<uint32_t>(1, p->max_regions_per_subject);
            r.out = h->sc_regions.as<saber_region>();
            r.rstat = h->sc_rstat.as<uint4>();
            r.nout = ctr + 12;
            r.cap = rcap;
            r.ctr = ctr;
            if (r.kmax <= 4)
                k_regions<TopReg<4>><<<nblocks(nhsp, 128), 128, 0, s>>>(r);
            else
                k_regions<TopLocal><<<nblocks(nhsp, 128), 128, 0, s>>>(r);
            CU(h, cudaGetLastError());
            unsigned long long nr = 0;
            CU(h, cudaMemcpyAsync(&nr, ctr + 12, 8, cudaMemcpyDeviceToHost, s));
            CU(h, cudaStreamSynchronize(s));
            nregions = std::min<uint64_t>(nr, rcap);
            if (!sink) regs.resize(nregions);
            if (nregions) {
                // region_order on the device: stable passes by (d_min, d_max), subject, (query, best desc)
                const uint32_t nrg = (uint32_t)nregions;
                CUALLOC(h, h->sc_rk64a, (uint64_t)nrg * 8);
                CUALLOC(h, h->sc_rk64b, (uint64_t)nrg * 8);
                CUALLOC(h, h->sc_rk64c, (uint64_t)nrg * 8);
                CUALLOC(h, h->sc_rk32a, (uint64_t)nrg * 4);
                CUALLOC(h, h->sc_rk32b, (uint64_t)nrg * 4);
                CUALLOC(h, h->sc_ridxa, (uint64_t)nrg * 4);
                CUALLOC(h, h->sc_ridxb, (uint64_t)nrg * 4);
                CUALLOC(h, h->sc_regions2, (uint64_t)nrg * sizeof(saber_region));
                unsigned long long* klo = h->sc_rk64a.as<unsigned long long>();
                unsigned long long* khi = h->sc_rk64c.as<unsigned long long>();
                unsigned long long* k64o = h->sc_rk64b.as<unsigned long long>();
                uint32_t* ksub = h->sc_rk32a.as<uint32_t>();
                uint32_t* k32o = h->sc_rk32b.as<uint32_t>();
                uint32_t* ia = h->sc_ridxa.as<uint32_t>();
                uint32_t* ib = h->sc_ridxb.as<uint32_t>();
                k_region_keys<<<nblocks(nrg, 256), 256, 0, s>>>(h->sc_regions.as<saber_region>(), nrg, klo, ksub, khi, ia);
                size_t r1 = 0, r2 = 0;
                CU(h, cub::DeviceRadixSort::SortPairs(nullptr, r1, klo, k64o, ia, ib, (int)nrg, 0, 64, s));
                CU(h, cub::DeviceRadixSort::SortPairs(nullptr, r2, ksub, k32o, ia, ib, (int)nrg, 0, 32, s));
                CUALLOC(h, h->cub_tmp, std::max(r1, r2));
                size_t rb = h->cub_tmp.cap;
                // pass 1: (d_min, d_max); ib = order
                CU(h, cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, rb, klo, k64o, ia, ib, (int)nrg, 0, 64, s));
                // pass 2: subject, stable
                k_gather_u32_by<<<nblocks(nrg, 256), 256, 0, s>>>(ksub, ib, nrg, k32o);
                CU(h, cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, rb, k32o, ksub, ib, ia, (int)nrg, 0, 32, s));
                // pass 3: (query, best desc), stable
                k_gather_u64_by<<<nblocks(nrg, 256), 256, 0, s>>>(khi, ia, nrg, k64o);
                CU(h, cub::DeviceRadixSort::SortPairs(h->cub_tmp.p, rb, k64o, klo, ia, ib, (int)nrg, 0, 64, s));
                k_gather_regions<<<nblocks(nrg, 256), 256, 0, s>>>(h->sc_regions.as<saber_region>(), ib, nrg,
                                                                   h->sc_regions2.as<saber_region>());
                if (sink) {
                    CUALLOC(h, h->sc_rstat2, (uint64_t)nrg * sizeof(uint4));
                    k_gather_uint4<<<nblocks(nrg, 256), 256, 0, s>>>(h->sc_rstat.as<uint4>(), ib, nrg,
                                                                     h->sc_rstat2.as<uint4>());
                } else {
                    CU(h, cudaMemcpyAsync(regs.data(), h->sc_regions2.p, nregions * sizeof(saber_region),
                                          cudaMemcpyDeviceToHost, s));
                }
            }
        }
    } else {
        CU(h, cudaEventRecord(ev[3], s));
    }
    CU(h, cudaEventRecord(ev[4], s));
    unsigned long long hc[16];
    CU(h, cudaMemcpyAsync(hc, ctr, 16 * 8, cudaMemcpyDeviceToHost, s));
    CU(h, cudaStreamSynchronize(s));
    local.ungapped_extensions = hc[4];
    local.extensions_avoided = hc[5];
    local.xdrop_steps = hc[6];
    local.hsps = hc[7];
    local.regions_weak_dropped = hc[8];
    // per query in region_order (sorted on the device above), cap at max_candidates
    const uint64_t cap = std::max<uint32_t>(1, p->max_candidates);
    uint64_t w = 0;
    bool overflow = false;
    if (sink) {
        int rc = region_sink(h, p, region_thr != nullptr, nregions, *sink);
        if (rc != SABER_OK) return rc;
        w = sink->ncap;
        local.regions_dropped_by_cap = nregions - sink->ncap;
    } else {
        size_t i = 0;
        while (i < regs.size()) {
            size_t j = i;
            while (j < regs.size() && regs[j].query == regs[i].query) j++;
            const uint64_t take = std::min<uint64_t>(j - i, cap);
            local.regions_dropped_by_cap += (j - i) - take;
            for (uint64_t k = 0; k < take; k++) {
                if (w < out_cap) out[w] = regs[i + k];
                else overflow = true;
                w++;
            }
            i = j;
        }
    }
    local.regions = w;
    local.t_tables_ms = ev_ms(ev[0], ev[1]);
    local.t_scan_ms = ev_ms(ev[1], ev[2]);
    local.t_visit_ms = ev_ms(ev[2], ev[3]);
    local.t_regions_ms = ev_ms(ev[3], ev[4]);
    if (n_out) *n_out = w;
    if (st) *st = local;
    if (overflow) return fail(h, SABER_ERR_ARG, "region buffer too small: %llu regions", (unsigned long long)w);
    return SABER_OK;
}

}  // namespace saber
