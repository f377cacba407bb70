// Six-frame translation of nucleotide sequences into protein codes, for the
// translated modes: nx queries (each record searched as its six frames) and
// pn databases (each sequence stored as six frames, subject 6 * s + f),
// translation.rs:277-308, driver.rs:387-402, index.rs:1351-1368.
//
// Frame f < 3 reads the codons at f, f+3, ... while a whole codon remains;
// frames 3..5 read the reverse complement from the sequence end, offset
// f - 3 (complement of code c is 3 - c; codes above 3 stay).  A codon holding
// a code above 3 (N) is X; the others come from the 64-entry table of the
// genetic code.
//
// Byte work bound by HBM: one thread per output residue (three input bytes
// read through L1, one written).  The host lists chunks of 4,096 outputs of
// one frame (segment index, first output), so a block finds its frame
// without a search.
#include <cuda_runtime.h>

#include <vector>

#include "runtime.cuh"

namespace saber {

constexpr unsigned kTrThreads = 256;
constexpr unsigned kTrPerThread = 16;
constexpr uint64_t kTrChunk = kTrThreads * kTrPerThread;

__global__ void __launch_bounds__(kTrThreads) k_translate6(const uint8_t* __restrict__ nt,
                                                            const uint64_t* __restrict__ nt_offs,
                                                            const uint64_t* __restrict__ out_offs,
                                                            const uint2* __restrict__ chunks, uint64_t nchunks,
                                                            const uint8_t* __restrict__ aa64,
                                                            uint8_t* __restrict__ out) {
    __shared__ uint8_t aa[64];
    if (threadIdx.x < 64) aa[threadIdx.x] = aa64[threadIdx.x];
    __syncthreads();
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint2 ch = chunks[c];
        const uint32_t seg = ch.x, s = seg / 6, f = seg % 6;
        const uint8_t* x = nt + nt_offs[s];
        const int64_t n = (int64_t)(nt_offs[s + 1] - nt_offs[s]);
        const uint64_t o0 = out_offs[seg], len = out_offs[seg + 1] - o0;
#pragma unroll
        for (unsigned t = 0; t < kTrPerThread; t++) {
            const uint64_t j = (uint64_t)ch.y + t * kTrThreads + threadIdx.x;
            if (j >= len) break;
            uint32_t a, b, cc;
            if (f < 3) {
                const int64_t i = (int64_t)f + 3 * (int64_t)j;
                a = x[i];
                b = x[i + 1];
                cc = x[i + 2];
            } else {
                const int64_t k = (int64_t)(f - 3) + 3 * (int64_t)j;
                a = x[n - 1 - k];
                b = x[n - 2 - k];
                cc = x[n - 3 - k];
                a = a > 3 ? a : 3 - a;
                b = b > 3 ? b : 3 - b;
                cc = cc > 3 ? cc : 3 - cc;
            }
            out[o0 + j] = (a > 3 || b > 3 || cc > 3) ? (uint8_t)22 : aa[a * 16 + b * 4 + cc];
        }
    }
}

int translate6_host(saber_gpu* h, const uint8_t* nt, const uint64_t* nt_offsets, uint64_t nseq,
                    const uint8_t* codon64, uint8_t* out, uint64_t out_cap, uint64_t* out_offsets) {
    if (!nt_offsets || !codon64 || !out_offsets) return fail(h, SABER_ERR_ARG, "null argument");
    if (nseq > 0xffffffffull / 6) return fail(h, SABER_ERR_ARG, "too many sequences to translate");
    const uint64_t n0 = nseq ? nt_offsets[0] : 0, total_nt = nseq ? nt_offsets[nseq] - n0 : 0;
    std::vector<uint64_t> rel(nseq + 1);
    std::vector<uint2> chunks;
    out_offsets[0] = 0;
    for (uint64_t s = 0; s < nseq; s++) {
        if (nt_offsets[s + 1] < nt_offsets[s]) return fail(h, SABER_ERR_ARG, "offsets must be non-decreasing");
        rel[s] = nt_offsets[s] - n0;
        const uint64_t n = nt_offsets[s + 1] - nt_offsets[s];
        if (n / 3 >= 0xffffffffull) return fail(h, SABER_ERR_ARG, "sequence too long to translate");
        for (uint32_t f = 0; f < 6; f++) {
            const uint64_t off = f % 3, len = n >= off ? (n - off) / 3 : 0;
            const uint32_t seg = (uint32_t)(6 * s + f);
            out_offsets[seg + 1] = out_offsets[seg] + len;
            for (uint64_t j = 0; j < len; j += kTrChunk) chunks.push_back(make_uint2(seg, (uint32_t)j));
        }
    }
    rel[nseq] = total_nt;
    const uint64_t total = out_offsets[6 * nseq];
    if (total > out_cap) return fail(h, SABER_ERR_CAP, "translation needs %llu residues", (unsigned long long)total);
    if (total == 0) return SABER_OK;
    if (!nt || !out) return fail(h, SABER_ERR_ARG, "null sequence buffer");
    CUALLOC(h, h->tr_nt, total_nt + 16);
    CUALLOC(h, h->tr_offs, (nseq + 1) * sizeof(uint64_t));
    CUALLOC(h, h->tr_out_offs, (6 * nseq + 1) * sizeof(uint64_t));
    CUALLOC(h, h->tr_chunks, chunks.size() * sizeof(uint2));
    CUALLOC(h, h->tr_aa, 64);
    CUALLOC(h, h->tr_out, total);
    cudaStream_t st = h->stream;
    CU(h, cudaMemcpyAsync(h->tr_nt.p, nt + n0, total_nt, cudaMemcpyHostToDevice, st));
    CU(h, cudaMemcpyAsync(h->tr_offs.p, rel.data(), (nseq + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    CU(h, cudaMemcpyAsync(h->tr_out_offs.p, out_offsets, (6 * nseq + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                          st));
    CU(h, cudaMemcpyAsync(h->tr_chunks.p, chunks.data(), chunks.size() * sizeof(uint2), cudaMemcpyHostToDevice, st));
    CU(h, cudaMemcpyAsync(h->tr_aa.p, codon64, 64, cudaMemcpyHostToDevice, st));
    const unsigned grid = (unsigned)std::min<uint64_t>(chunks.size(), (uint64_t)h->sm_count * 8);
    k_translate6<<<grid, kTrThreads, 0, st>>>((const uint8_t*)h->tr_nt.p, (const uint64_t*)h->tr_offs.p,
                                              (const uint64_t*)h->tr_out_offs.p, (const uint2*)h->tr_chunks.p,
                                              chunks.size(), (const uint8_t*)h->tr_aa.p, (uint8_t*)h->tr_out.p);
    CU(h, cudaGetLastError());
    CU(h, cudaMemcpyAsync(out, h->tr_out.p, total, cudaMemcpyDeviceToHost, st));
    CU(h, cudaStreamSynchronize(st));
    return SABER_OK;
}

}  // namespace saber
