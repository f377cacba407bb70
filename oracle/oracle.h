/*
 * CPU oracle for the seed-and-extend scoring path — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference (SABER 1.4.0, Rust) scalar
 * algorithms that the GPU path must reproduce bit for bit.  It is used by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and
 * only as the checker or as the timed CPU reference — never by the product
 * library.  Every function cites the reference file:line it follows (paths
 * relative to the reference crate root).
 *
 * Pinning: the full-window SW score is pinned against the reference's own
 * compiled kernel (src/gpu/kernels/sw.cu, built here by oracle/Makefile into
 * oracle/_ref) on the reference's test-vector generator
 * (examples/gpu_vectors.rs), committed as tests/golden/sw_vectors.json, and
 * against the known answers of the reference unit tests
 * (reference.rs:128-146, banded.rs:716-731, gpu/mod.rs:178-182).
 */
#ifndef SABER_ORACLE_H
#define SABER_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scoring scheme: 24x24 matrix in NCBI order (row = query code, column =
 * subject code), SABER gap convention (a gap of length k costs
 * open + (k-1)*extend).  banded.rs:21-27. */
typedef struct {
    const int32_t* matrix; /* 576 entries, row-major */
    int32_t gap_open;
    int32_t gap_extend;
} orc_scheme;

/* banded.rs:90-99 */
typedef struct {
    int32_t score;
    uint64_t q_end;  /* exclusive end of the first (row-major) optimal cell */
    uint64_t s_end;
    uint64_t cells;  /* evaluated in-band cells */
} orc_band_score;

/* banded.rs:101-113.  ops are (op, len) run-length pairs, op in 'M','I','D'. */
typedef struct {
    int32_t score;
    uint64_t q_start, q_end, s_start, s_end; /* 0-based, half open */
    uint64_t cells;
    uint32_t n_ops;
} orc_alignment;

/* reference.rs:15-52: full-matrix Gotoh SW in i64; first row-major maximum. */
int64_t orc_sw_reference(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                         const int32_t* matrix, const int8_t* bias,
                         int64_t gap_open, int64_t gap_extend,
                         uint64_t* q_end, uint64_t* s_end);

/* reference.rs:58-103.  Returns 0 and fills score/ends, or -1 when the ops
 * run past a sequence end or hold an unknown op. */
int orc_score_alignment(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                        uint64_t q_start, uint64_t s_start,
                        const uint8_t* ops, const uint32_t* lens, uint32_t n_ops,
                        const int32_t* matrix, const int8_t* bias,
                        int64_t gap_open, int64_t gap_extend,
                        int64_t* score, uint64_t* q_end, uint64_t* s_end);

/* banded.rs:134-224 (banded_score_scalar).  Band is lo <= j - i <= hi. */
void orc_banded_score(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                      const int8_t* bias, orc_scheme sc, int64_t lo, int64_t hi,
                      orc_band_score* out);

/* banded.rs:227-332 + walk banded.rs:336-403, with the stop_at early exit of
 * the dispatched kernel (banded_simd.rs:594-596: rows after the first whose
 * best reaches stop_at are not computed; the alignment is unchanged, only
 * `cells` shrinks).
 * Returns 1 and fills `out`/ops on an alignment, 0 when the best score is
 * 0 (Ok(None)), -2 when m*w exceeds max_dir_bytes (Err(need)), -3 when the
 * ops buffer is too small.  ops/lens receive at most ops_cap runs. */
int orc_banded_align(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                     const int8_t* bias, orc_scheme sc, int64_t lo, int64_t hi,
                     uint64_t max_dir_bytes, int32_t stop_at,
                     orc_alignment* out, uint8_t* ops, uint32_t* lens, uint32_t ops_cap);

/* Direction bytes of the scalar traceback kernel (banded.rs:287-313), for
 * tests that compare per-cell origins: dir receives m*w bytes (row i, band
 * offset k at dir[i*w+k]); cells outside the row range are left 0xFF.
 * Returns the clipped width w (0 when empty). */
uint64_t orc_banded_dir(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                        const int8_t* bias, orc_scheme sc, int64_t lo, int64_t hi,
                        uint8_t* dir, uint64_t dir_cap, int64_t* clipped_lo);

/* engine.rs:2460-2494 (ungapped_xdrop): returns score; q range [*q_lo, *q_hi). */
int32_t orc_ungapped_xdrop(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                           uint64_t qp, uint64_t sp, const int32_t* matrix,
                           const int8_t* bias, int32_t x,
                           uint64_t* q_lo, uint64_t* q_hi);

/* ---- batched banded jobs (CPU baseline and parity driver) ---------------
 * Same job layout as the GPU library (include/saber_gpu.h, saber_band_job). */
typedef struct {
    uint32_t query;     /* index into the query set */
    uint32_t subject;   /* subject id (informational) */
    uint64_t win_begin; /* absolute residue offset of the window start */
    uint32_t win_len;   /* window length n */
    int32_t band_lo;    /* band relative to the window, j - i */
    int32_t band_hi;
    uint32_t flags;
} orc_band_job;

/* Scores every job with orc_banded_score (score only; score_banded_many's
 * contract, band_simd8.rs:75-185) using `threads` POSIX threads.
 * cells_out (optional) receives the total in-band cells. */
int orc_score_band_jobs(const uint8_t* residues, const uint8_t* qcodes,
                        const uint64_t* qoffs, const int8_t* qbias,
                        const orc_band_job* jobs, uint64_t njobs,
                        const int32_t* matrix, int32_t gap_open, int32_t gap_extend,
                        int32_t* scores, int threads, uint64_t* cells_out);


/* ---- SIMD-class restatement of the reference's CPU scoring (simd_band.cpp) ----
 * score_banded_many (band_simd8.rs:78-185) per query: the inter-sequence
 * unsigned 8-bit kernel batch_u8 (band_simd8.rs:236-388) for bands of width
 * <= 126, the 16-bit row kernel banded_avx2_16 (banded_simd.rs:393-599) for
 * wider bands and 8-bit overflows, and 32 bits (orc_banded_score) where the
 * 16-bit range may not hold.  Same jobs and scores as orc_score_band_jobs;
 * queries are spread over `threads` threads. */
typedef struct {
    uint64_t cells;        /* in-band cells of all jobs */
    uint64_t u8_jobs;      /* jobs run through the 8-bit kernel */
    uint64_t u8_overflows; /* of those, re-scored because the lane may have saturated */
    uint64_t i16_jobs;     /* jobs finished by the 16-bit kernel */
    uint64_t i32_jobs;     /* jobs re-run in 32 bits */
} orc_simd_counters;

int orc_simd_score_band_jobs(const uint8_t* residues, const uint8_t* qcodes,
                             const uint64_t* qoffs, const int8_t* qbias,
                             const orc_band_job* jobs, uint64_t njobs,
                             const int32_t* matrix, int32_t gap_open, int32_t gap_extend,
                             int32_t* scores, int threads, orc_simd_counters* counters);

/* ---- scan schedule: seeds -> hits -> window filter -> X-drop -> regions ----
 * Restates Engine::search_scan for one query batch (src/search/engine/scan.rs:
 * build_scan_db 1066-1257, build_batch 1500-1596, scan_hits 1603-1804,
 * filter_scalar 1809-1856, visit_chunk_inner 2084-2225, visit_scan 2384-2431,
 * finish_subject_into 2437-2474; index.rs:329-336 auto_occ_cap; the per-query
 * candidate cap under region_order, engine.rs:493-495). */
typedef struct {
    uint8_t alpha_map[24];      /* reduced letter per code, 255 = not seedable */
    uint32_t alpha_size;
    uint32_t nshapes;
    uint32_t shape_span[32];
    uint32_t shape_weight[32];
    uint16_t shape_off[32][16];
    uint32_t hit_filter_min_ids; /* 0 = no window filter */
    uint32_t hit_filter_exact_weight;
    int32_t hsp_threshold;
    int32_t x_drop;
    int32_t window_slack;
    uint32_t max_regions_per_subject;
    uint32_t max_candidates;
    uint64_t seed_max_occ;       /* 0 = automatic cap */
    uint64_t ref_db_residues;
    uint64_t db_length;          /* database residues of the statistics */
} orc_scan_params;

typedef struct {
    uint32_t query, subject;
    int32_t d_min, d_max, best;
} orc_region;

typedef struct {
    uint64_t seed_positions, seeds_frequent_skipped, hits, hits_filtered, ungapped_extensions,
        extensions_avoided, xdrop_steps, hsps, regions, regions_weak_dropped, regions_dropped_by_cap;
} orc_scan_counters;

/* Returns the number of regions written to `out` (capacity out_cap; -1 when
 * too small), ordered by query, then region_order.  db_mask / q_mask: one
 * byte per residue, nonzero = masked from seeding (NULL = none). */
int64_t orc_scan_regions(const uint8_t* res, const uint64_t* soffs, uint64_t nsub, const uint8_t* db_mask,
                         const uint8_t* qcodes, const uint64_t* qoffs, uint32_t nq, const int8_t* qbias,
                         const uint8_t* q_mask, const int32_t* region_thr, const int32_t* matrix,
                         const orc_scan_params* p, orc_region* out, uint64_t out_cap,
                         orc_scan_counters* ctr);

/* orc_scan_regions with the subjects (counting and hit passes) and the
 * (subject, query) pairs (coverage, X-drop, regions) spread over `threads`
 * threads; the output does not depend on the thread count. */
int64_t orc_scan_regions_mt(const uint8_t* res, const uint64_t* soffs, uint64_t nsub, const uint8_t* db_mask,
                            const uint8_t* qcodes, const uint64_t* qoffs, uint32_t nq, const int8_t* qbias,
                            const uint8_t* q_mask, const int32_t* region_thr, const int32_t* matrix,
                            const orc_scan_params* p, orc_region* out, uint64_t out_cap,
                            orc_scan_counters* ctr, int threads);

/* auto_occ_cap (src/search/index.rs:329-336). */
uint64_t orc_auto_occ_cap(uint64_t total, uint64_t ncodes, uint64_t db_residues, uint64_t ref_residues);

/* ---- tantan seed masking (oracle/tantan.c) ---- */

/* TantanParams (masking.rs:36-49); defaults 0.005, 0.05, 50, 0.9, 0.5. */
typedef struct {
    double repeat_start, repeat_end;
    uint32_t max_period;
    double decay, min_prob;
} orc_tantan_params;

/* implied_lambda (masking.rs:531-583); NaN when no root is found. */
double orc_tantan_lambda(const int32_t* matrix576);
/* Tantan::with_params tables (masking.rs:162-179); returns the lambda used. */
double orc_tantan_tables(const int32_t* matrix576, const orc_tantan_params* p, double lambda, float* lr768,
                         float* b2f);
/* compute_body (masking.rs:429-529) for one sequence. */
int orc_tantan_probs(const uint8_t* seq, size_t n, const float* lr768, const float* b2f, const orc_tantan_params* p,
                     float* post);
/* Tantan::mask (masking.rs:191-196) over offsets[nseq + 1]; returns the
 * number of masked positions (-1 on allocation failure). */
int64_t orc_tantan_mask(const uint8_t* codes, const uint64_t* offsets, uint64_t nseq, const int32_t* matrix576,
                        const orc_tantan_params* p, double lambda, uint8_t* mask, float* probs);

/* ---- six-frame translation (oracle/translate.c) ---- */

/* CodonTable::translate_codes (translation.rs:277-299): frame 0..5 of
 * nucleotide codes (0..3, 4 = N) into protein codes; returns the count. */
size_t orc_translate_codes(const uint8_t* nt, size_t n, unsigned frame, const uint8_t* aa64, uint8_t* out);

#ifdef __cplusplus
}
#endif
#endif
