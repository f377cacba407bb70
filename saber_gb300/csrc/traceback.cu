// Banded traceback on the GPU: direction bytes, first optimal cell, walk.
//
// k_band_align_warp computes, one job per warp in int32 (lanes across the
// band), the reference's banded_align_scalar (src/algorithm/banded.rs:227-332) — the same direction
// byte org | e_ext << 2 | f_ext << 3 per in-band cell, origin priority
// diagonal > E > F, extension bits only when strictly better — with the early
// exit of the dispatched kernel (rows after the first whose best reaches
// stop_at are not computed, banded_simd.rs:594-596), then follows the
// direction bytes from the first row-major optimal cell back to the start
// exactly as walk (banded.rs:336-403) does and writes the run-length encoded
// operations.  Direction bytes live in a pool in HBM (m x w bytes per job,
// row i at offset i*w, like the reference's dir buffer).  Without the
// direction pool (score-only requests) it returns the score and end cell of
// banded_score (banded.rs:134-224), which traceback_from_end needs.
//
// The widening driver of Engine::traceback / traceback_from_end
// (src/search/engine.rs:1328-1445) runs on the host below: every widening
// round of every unresolved region goes into one launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstring>
#include <vector>

#include "band_common.cuh"
#include "saber_gpu.h"

namespace saber {

struct AlignReq {
    const uint8_t* win;  // device window start
    const int16_t* prof; // device query profile (rows c, stride mpad)
    uint64_t dir_off;    // offset of this job's direction bytes in the pool (dir requests)
    uint64_t ops_off;    // offset of this job's op bytes / runs
    int32_t m, n, lo, w; // query length, window length, clipped band, width
    int32_t mpad;
    int32_t stop_at;
    int32_t want_dir;    // 1: direction bytes + walk; 0: score and end cell only
    int32_t pad_;
};

struct AlignOut {
    int32_t status;  // 1 alignment, 0 none
    int32_t score;
    uint32_t q_start, q_end, s_start, s_end;
    uint32_t n_ops;
    uint32_t pad_;
    uint64_t cells;
};

// The walk of one alignment from its best cell (banded.rs:336-403), run by
// one thread over the direction bytes (row stride w), then the run-length
// encoding in forward order.
__device__ void walk_runs(const uint8_t* dir, int64_t w, int64_t lo, int64_t bi, int64_t bk, uint8_t* ob,
                          uint32_t* rr, AlignOut& o) {
    uint32_t nop = 0;
    int state = 0;  // 0 = H, 1 = E (query gap, 'D'), 2 = F (subject gap, 'I')
    int64_t i = bi, k = bk;
    for (;;) {
        const uint8_t d = dir[(size_t)(i * w + k)];
        if (state == 0) {
            const uint8_t org = d & 3;
            if (org == 0) break;
            if (org == 1) {
                ob[nop++] = 'M';
                if (i == 0 || i + lo + k == 0) break;
                i -= 1;
            } else {
                state = org == 2 ? 1 : 2;
            }
        } else if (state == 1) {
            ob[nop++] = 'D';
            const bool ext = (d & 4) != 0;
            k -= 1;
            if (!ext) state = 0;
        } else {
            ob[nop++] = 'I';
            const bool ext = (d & 8) != 0;
            i -= 1;
            k += 1;
            if (!ext) state = 0;
        }
    }
    uint32_t qs = o.q_end, ss = o.s_end, nr = 0;
    for (uint32_t tt = 0; tt < nop; tt++) {
        const uint8_t op = ob[nop - 1 - tt];
        if (op == 'M') {
            qs--;
            ss--;
        } else if (op == 'I') {
            qs--;
        } else {
            ss--;
        }
        if (nr > 0 && (rr[nr - 1] & 0xFFu) == op) rr[nr - 1] += 0x100u;
        else rr[nr++] = 0x100u | op;
    }
    o.q_start = qs;
    o.s_start = ss;
    o.n_ops = nr;
}

// One warp per job: each row's band offsets k = 32c + lane in chunks of 32.
// F and the diagonal come from the previous row (coalesced loads from the
// warp's row buffers); E(i,k) = max over kmin <= j < k of
// H*(i,j) - go - (k-1-j) ge with H* = max(diag + S, F, 0), a warp max-scan of
// H* + j ge -- equal to the scalar recurrence of banded_align_scalar
// (banded.rs:227-332) when go >= ge, because opening a gap from an E-derived
// H never beats extending that E (set_scheme requires go >= ge).  Direction
// bytes, the first row-major best cell, stop_at and the walk are those of
// banded_align_scalar and walk.
__global__ void __launch_bounds__(128) k_band_align_warp(const AlignReq* __restrict__ reqs, uint32_t nreq,
                                                         uint8_t* __restrict__ dir_pool, uint8_t* __restrict__ opbytes,
                                                         uint32_t* __restrict__ runs, int32_t* __restrict__ slabs,
                                                         uint32_t slab_stride, int go, int ge,
                                                         AlignOut* __restrict__ outs) {
    const int NEG = INT32_MIN / 4;
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    int32_t* base = slabs + (size_t)warp * slab_stride * 4;
    for (uint32_t t = warp; t < nreq; t += nwarps) {
        const AlignReq rq = reqs[t];
        AlignOut o;
        o.status = 0;
        o.score = 0;
        o.q_start = o.q_end = o.s_start = o.s_end = 0;
        o.n_ops = 0;
        o.pad_ = 0;
        o.cells = 0;
        const int64_t m = rq.m, n = rq.n, lo = rq.lo, w = rq.w;
        if (w <= 0) {
            if (lane == 0) outs[t] = o;
            continue;
        }
        int32_t* hp = base;
        int32_t* fp = hp + slab_stride;
        int32_t* hc = fp + slab_stride;
        int32_t* fc = hc + slab_stride;
        for (int64_t k = lane; k <= w; k += 32) hp[k] = fp[k] = hc[k] = fc[k] = NEG;
        __syncwarp();
        uint8_t* dir = rq.want_dir ? dir_pool + rq.dir_off : nullptr;
        int32_t best = 0;
        int64_t bi = 0, bk = 0;
        uint64_t cells = 0;
        const int first_eext = (NEG - ge) > (NEG - go) ? 1 : 0;  // e_ext of a row's first cell
        for (int64_t i = 0; i < m; i++) {
            int64_t kmin = -(i + lo);
            if (kmin < 0) kmin = 0;
            int64_t kmax = n - 1 - i - lo;
            if (kmax > w - 1) kmax = w - 1;
            const int64_t bse = i + lo;
            int tmax = NEG;      // running max of H* + j ge over this row's earlier chunks
            int prevH = NEG, prevE = NEG;  // H and E at k - 1 for lane 0 (carry)
            int rowbest = 0;
            int64_t rowk = 0;
            // only the chunks that hold the row's window cells: the next row
            // reads this row's H and F at its own cells' k and k + 1, inside
            // [kmin - 1, kmax + 1]; at kmin - 1 only as the diagonal of column
            // 0, which is 0 by rule, and entry w stays NEG
            for (int64_t c0 = (kmin / 32) * 32; c0 <= kmax; c0 += 32) {
                const int64_t k = c0 + lane;
                const bool inb = k < w;
                const bool valid = inb && k >= kmin && k <= kmax;
                int f = NEG, hstar = NEG, h1 = 0, fe = 0, fo = 0;
                uint32_t c1 = 0;
                if (valid) {
                    const int64_t j = bse + k;
                    fo = hp[k + 1] - go;
                    fe = fp[k + 1] - ge;
                    f = i >= 1 ? max(fe, fo) : NEG;
                    const int32_t hd = (i >= 1 && j >= 1) ? hp[k] : 0;
                    const int32_t diag = hd + ((int32_t)rq.prof[(size_t)rq.win[j] * rq.mpad + i] - go);
                    c1 = diag > 0;
                    h1 = max(diag, 0);
                    hstar = max(h1, f);
                }
                // E via an exclusive max-scan of H* + k ge (carry from earlier chunks)
                int tv = valid ? hstar + (int)(k * ge) : NEG;
                int incl = tv;
#pragma unroll
                for (int o2 = 1; o2 < 32; o2 <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, incl, o2);
                    if (lane >= o2) incl = max(incl, u);
                }
                int excl = __shfl_up_sync(0xffffffffu, incl, 1);
                if (lane == 0) excl = NEG;
                excl = max(excl, tmax);
                int e = NEG;
                if (valid && k > kmin && excl > NEG) e = excl - go - (int)((k - 1) * ge);
                int h = NEG;
                uint8_t d = 0;
                if (valid) {
                    const uint32_t c2 = e > h1;
                    const int32_t h2 = max(h1, e);
                    const uint32_t c3 = f > h2;
                    h = max(h2, f);
                    d = (uint8_t)((c3 ? 3u : (c2 ? 2u : c1)) | ((uint32_t)(fe > fo) << 3));
                }
                // e_ext = E(k-1) - ge > H(k-1) - go (the previous cell of the row)
                int hl = __shfl_up_sync(0xffffffffu, h, 1);
                int el = __shfl_up_sync(0xffffffffu, e, 1);
                if (lane == 0) {
                    hl = prevH;
                    el = prevE;
                }
                if (valid) {
                    const uint32_t eext = k == kmin ? (uint32_t)first_eext : (uint32_t)((el - ge) > (hl - go));
                    d |= (uint8_t)(eext << 2);
                    if (dir) dir[(size_t)(i * w + k)] = d;
                }
                if (inb) {
                    hc[k] = valid ? h : NEG;
                    fc[k] = valid ? f : NEG;
                }
                // the first cell of the row's best
                const int cm = __reduce_max_sync(0xffffffffu, valid ? h : 0);
                if (cm > rowbest) {
                    rowbest = cm;
                    rowk = c0 + (__ffs(__ballot_sync(0xffffffffu, valid && h == cm)) - 1);
                }
                tmax = max(tmax, __shfl_sync(0xffffffffu, incl, 31));
                prevH = __shfl_sync(0xffffffffu, h, 31);
                prevE = __shfl_sync(0xffffffffu, e, 31);
            }
            if (kmin <= kmax) cells += (uint64_t)(kmax - kmin + 1);
            if (rowbest > best) {
                best = rowbest;
                bi = i;
                bk = rowk;
            }
            __syncwarp();
            int32_t* tmp = hp;
            hp = hc;
            hc = tmp;
            tmp = fp;
            fp = fc;
            fc = tmp;
            if (best >= rq.stop_at) break;
        }
        o.cells = cells;
        o.score = best;
        if (best > 0) {
            o.status = 1;
            o.q_end = (uint32_t)(bi + 1);
            o.s_end = (uint32_t)(bi + lo + bk + 1);
        }
        __syncwarp();
        if (lane == 0) {
            if (best > 0 && dir) walk_runs(dir, w, lo, bi, bk, opbytes + rq.ops_off, runs + rq.ops_off, o);
            outs[t] = o;
        }
        __syncwarp();
    }
}

cudaError_t launch_band_align(unsigned grid, cudaStream_t s, const AlignReq* reqs, uint32_t nreq, uint8_t* dir_pool,
                              uint8_t* opbytes, uint32_t* runs, int32_t* slabs, uint32_t slab_stride, int go, int ge,
                              AlignOut* outs) {
    // (set_scheme guarantees go >= ge, the condition of the warp kernel's E scan)
    k_band_align_warp<<<grid, 128, 0, s>>>(reqs, nreq, dir_pool, opbytes, runs, slabs, slab_stride, go, ge, outs);
    return cudaGetLastError();
}

}  // namespace saber
