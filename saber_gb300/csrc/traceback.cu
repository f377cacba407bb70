// Banded traceback on the GPU: direction bytes, first optimal cell, walk.
//
// k_band_align computes, one job per thread in int32, the reference's
// banded_align_scalar (src/algorithm/banded.rs:227-332) — the same direction
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

__global__ void __launch_bounds__(128) k_band_align(const AlignReq* __restrict__ reqs, uint32_t nreq,
                                                    uint8_t* __restrict__ dir_pool, uint8_t* __restrict__ opbytes,
                                                    uint32_t* __restrict__ runs, int32_t* __restrict__ slabs,
                                                    uint32_t slab_stride, int go, int ge,
                                                    AlignOut* __restrict__ outs) {
    const int NEG = INT32_MIN / 4;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    int32_t* hp0 = slabs + (size_t)tid * slab_stride * 4;
    for (uint32_t t = tid; t < nreq; t += nthreads) {
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
            outs[t] = o;
            continue;
        }
        int32_t* hp = hp0;
        int32_t* fp = hp + slab_stride;
        int32_t* hc = fp + slab_stride;
        int32_t* fc = hc + slab_stride;
        for (int64_t k = 0; k <= w; k++) hp[k] = fp[k] = hc[k] = fc[k] = NEG;
        uint8_t* dir = rq.want_dir ? dir_pool + rq.dir_off : nullptr;
        int32_t best = 0;
        int64_t bi = 0, bk = 0;
        uint64_t cells = 0;
        for (int64_t i = 0; i < m; i++) {
            int64_t kmin = -(i + lo);
            if (kmin < 0) kmin = 0;
            int64_t kmax = n - 1 - i - lo;
            if (kmax > w - 1) kmax = w - 1;
            if (kmin > kmax) {
                for (int64_t k = 0; k < w; k++) hc[k] = fc[k] = NEG;
            } else {
                int32_t e = NEG, h_left = NEG;
                const int64_t base = i + lo;
                uint8_t* drow = dir ? dir + (size_t)(i * w) : nullptr;
                for (int64_t k = kmin; k <= kmax; k++) {
                    const int64_t j = base + k;
                    const int32_t eo = h_left - go;
                    const int32_t ee = e - ge;
                    const uint32_t e_ext = ee > eo;
                    e = k > kmin ? max(ee, eo) : NEG;
                    const int32_t fo = hp[k + 1] - go;
                    const int32_t fe = fp[k + 1] - ge;
                    const uint32_t f_ext = fe > fo;
                    const int32_t f = i >= 1 ? max(fe, fo) : NEG;
                    const int32_t hd = (i >= 1 && j >= 1) ? hp[k] : 0;
                    const int32_t diag = hd + (int32_t)rq.prof[(size_t)rq.win[j] * rq.mpad + i];
                    const uint32_t c1 = diag > 0;
                    const int32_t h1 = max(diag, 0);
                    const uint32_t c2 = e > h1;
                    const int32_t h2 = max(h1, e);
                    const uint32_t c3 = f > h2;
                    const int32_t h = max(h2, f);
                    hc[k] = h;
                    fc[k] = f;
                    if (drow) drow[k] = (uint8_t)((c3 ? 3u : (c2 ? 2u : c1)) | (e_ext << 2) | (f_ext << 3));
                    h_left = h;
                    if (h > best) {
                        best = h;
                        bi = i;
                        bk = k;
                    }
                }
                cells += (uint64_t)(kmax - kmin + 1);
                for (int64_t k = 0; k < kmin; k++) hc[k] = fc[k] = NEG;
                for (int64_t k = kmax + 1; k < w; k++) hc[k] = fc[k] = NEG;
            }
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
        if (best > 0 && dir) {
            // walk (banded.rs:336-403): ops are produced last to first
            uint8_t* ob = opbytes + rq.ops_off;
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
            // start coordinates and run-length encoding in forward order
            uint32_t qs = o.q_end, ss = o.s_end, nr = 0;
            uint32_t* rr = runs + rq.ops_off;
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
        outs[t] = o;
    }
}

cudaError_t launch_band_align(unsigned grid, cudaStream_t s, const AlignReq* reqs, uint32_t nreq, uint8_t* dir_pool,
                              uint8_t* opbytes, uint32_t* runs, int32_t* slabs, uint32_t slab_stride, int go, int ge,
                              AlignOut* outs) {
    k_band_align<<<grid, 128, 0, s>>>(reqs, nreq, dir_pool, opbytes, runs, slabs, slab_stride, go, ge, outs);
    return cudaGetLastError();
}

}  // namespace saber
