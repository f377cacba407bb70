// Internal runtime types shared by the library's translation units: device
// buffers, datasets, schemes, the handle and the error helpers.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "band_common.cuh"
#include "region_sink.h"
#include "saber_gpu.h"

namespace saber {

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    // grow-only; contents are not preserved
    cudaError_t reserve(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

// Pinned host memory (grow-only, 25 % slack; contents are not preserved).
struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    HostBuf() = default;
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
    ~HostBuf() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t reserve(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(bytes + bytes / 4, 4096);
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

struct QuerySet {
    uint32_t nq = 0;
    std::vector<uint64_t> offs;  // host copy
    std::vector<uint64_t> poff;  // host copy of the profile offsets
    std::vector<uint32_t> pmpad; // host copy of the profile row strides
    DevBuf codes, offsets, bias, prof, prof_off, prof_mpad;
    DevBuf prof8;              // int8 copy of prof, valid when p8
    uint64_t prof_elems = 0;   // entries of prof
    int bias_min = 0, bias_max = 0;
    bool has = false;
    bool has_bias = false;
    bool p8 = false;           // every profile entry fits in [-127, 127]
};

// Residues + subject offsets + a query set with profiles for one scheme.
struct Dataset {
    DevBuf res, soff;
    uint64_t n_res = 0, nsub = 0;
    uint64_t max_len = 0;  // longest subject
    bool has_db = false;
    QuerySet qs;
};

// Key of a captured scoring graph: sizes, settings and every buffer it reads
// or writes (a reallocated buffer means a new capture).
struct GraphKey {
    uint64_t npad, wcap, n_res;
    int32_t rows, go, ge;
    uint32_t pair_steps, nq, long_steps;
    const void* ptrs[16];
    const void* prof8;
    bool operator==(const GraphKey& o) const { return std::memcmp(this, &o, sizeof(GraphKey)) == 0; }
};
struct GraphEntry {
    cudaGraphExec_t exec;
    const void* extra;
};

struct Scheme {
    int32_t matrix[576];
    int32_t go = 11, ge = 1;
    bool has = false;
    DevBuf d_matrix;
};

}  // namespace saber

struct saber_gpu {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    std::string err;
    int sm_count = 0;
    int strip_rows = saber::kStripRows;  // tuning: rows per strip of the int16 kernel
    uint32_t pair_steps = saber::kPairStepsDefault;  // tuning: paired-strip threshold
    uint32_t long_steps = saber::kLongStepsDefault;  // tuning: lane sweeps longer than this go to the warp kernel
    // captured scoring graphs (saber_gpu_score_band_jobs with graphs on)
    bool use_graphs = true;
    uint64_t graph_captures = 0;
    saber::DevBuf g_nreal, g_wmax;
    std::vector<std::pair<saber::GraphKey, saber::GraphEntry>> graphs;
    // the handle's scheme and dataset (set_scheme / load_db / load_queries)
    saber::Scheme scheme;
    saber::Dataset main;
    // per-call scheme and dataset of the one-query entry points
    saber::Scheme eph_scheme;
    saber::Dataset eph;
    // per-call scratch
    saber::DevBuf keys_in, keys_out, vals_in, vals_out, counts, stats, cub_tmp, bufs, slabs, list, jobs_dev,
        scores_dev;
    // scan state: per-residue seed bytes / distances of the database, the
    // database mask, per-shape frequent-code bitmaps, and per-call buffers
    saber::DevBuf sc_sblk, sc_qblk;  // owner tables of 256-position blocks (database, batch)
    saber::DevBuf db_mask, sc_sb, sc_rem, sc_dst, sc_freq, sc_counts, sc_qsb, sc_qfull, sc_qrem, sc_qdst,
        sc_qcnt, sc_qoff, sc_qent, sc_qpres, sc_surv, sc_key1, sc_key2, sc_val, sc_key1o, sc_key2o, sc_valo,
        sc_chains, sc_hsp, sc_hkey, sc_hkeyo, sc_hval, sc_hvalo, sc_pairs, sc_regions, sc_rthr, sc_ctr, sc_tmp,
        sc_rk64a, sc_rk64b, sc_rk64c, sc_rk32a, sc_rk32b, sc_ridxa, sc_ridxb, sc_regions2, sc_rstat, sc_rstat2,
        sc_flags, sc_gcnt, sc_grank, sc_cntc, sc_qwin, sc_qwinx, sc_surv2, sc_qrng, sc_cb, sc_combtab;
    bool sc_comb = false;  // the database's combined filter codes (sc_cb) are built
    uint64_t scan_table_bytes = 48ull << 20;  // tuning: seed-table bytes per scan pass (L2 budget)
    bool has_db_mask = false;
    // learned triage: installed model, per-call feature buffers, collection
    saber::DevBuf tr_model, tr_wb, tr_sfeat, tr_qfeat, tr_reg, tr_rstat, tr_rq, tr_rrank, tr_qinfo, tr_X, tr_logit;
    bool tr_on = false, tr_sfeat_ok = false;
    uint64_t tr_sfeat_key = 0;
    float tr_threshold = 0.f;
    bool tr_collect = false;
    std::vector<float> tr_rows, tr_logits;
    std::vector<uint8_t> tr_labels;
    uint64_t sc_key = 0;            // fingerprint of the database state built
    std::vector<uint64_t> sc_caps;  // per shape
    std::vector<uint64_t> sc_freq_off;
    // device-side region cap / triage / compaction, pinned host staging
    saber::DevBuf rg_qcnt, rg_qstart, rg_rank, rg_flag, rg_idx, rg_idx2, rg_out, rg_sbase, rg_slen;
    saber::HostBuf pin_reg, pin_src, pin_sbase, pin_slen;
    saber::HostBuf pin_scratch[4];  // the batch engine's staging (pinned_scratch)
    saber::DevBuf mask_runs;  // database mask runs being expanded
    // six-frame translation scratch
    saber::DevBuf tr_nt, tr_offs, tr_out_offs, tr_chunks, tr_aa, tr_out;
    // tantan masking scratch
    saber::DevBuf tt_ord, tt_base, tt_F, tt_BS, tt_count, tt_codes, tt_offs, tt_mask, tt_probs;
    std::vector<int32_t> tt_lambda_matrix;  // the matrix whose implied lambda is cached
    double tt_lambda = 0.0;
    // traceback scratch
    saber::DevBuf al_reqs, al_outs, al_dir, al_opbytes, al_runs, al_slabs, al_packed, al_pack_off;
};

namespace saber {

static int fail(saber_gpu* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->err = buf;
    return code;
}

#define CU(h, call)                                                                       \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return ::saber::fail((h), SABER_ERR_CUDA, "%s: %s (%s:%d)", #call,            \
                                 cudaGetErrorString(e_), __FILE__, __LINE__);             \
    } while (0)
#define CUALLOC(h, buf, bytes)                                                            \
    do {                                                                                  \
        cudaError_t e_ = (buf).reserve(bytes);                                            \
        if (e_ != cudaSuccess)                                                            \
            return ::saber::fail((h), SABER_ERR_NOMEM, "device allocation of %zu bytes: %s", \
                                 (size_t)(bytes), cudaGetErrorString(e_));                \
    } while (0)


int scan_regions(saber_gpu* h, const saber_scan_params* p, const uint8_t* q_mask, const int32_t* region_thr,
                 saber_region* out, uint64_t out_cap, uint64_t* n_out, saber_scan_stats* st,
                 RegionSink* sink = nullptr);

static inline unsigned nblocks(uint64_t n, unsigned t, unsigned cap = 65535u * 16u) {
    uint64_t b = (n + t - 1) / t;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

}  // namespace saber
