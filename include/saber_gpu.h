/*
 * saber_gpu.h — C ABI of the GB300 seed-and-extend scoring library
 * (libsaber_gb300.so).
 *
 * Plain C types only: opaque handle, caller-owned buffers, int status codes
 * (0 = ok, negative = error; the message is in saber_gpu_last_error).  No
 * exception crosses the ABI.  One CUDA stream per handle; calls on one handle
 * are serialised by an internal mutex (as the reference's CUDA backend
 * serialises launches, src/gpu/cuda.rs:37,144); separate handles are
 * independent.  There is no CPU fallback: a call that cannot run on the GPU
 * returns an error.
 *
 * Encodings and conventions (src/gpu/mod.rs:9-26):
 *   - residues are canonical alignment codes (protein ARNDCQEGHILKMFPSTWYVBZX*
 *     -> 0..23, nucleotide ACGTN -> 0..4); codes >= 24 are scored as X (22);
 *   - substitution matrix: 24x24 int32, row = query code, column = subject code;
 *   - gaps (SABER convention): a gap of length k costs open + (k-1)*extend;
 *   - bias[i] (int8) is added to every aligned column of query position i;
 *   - scores are exact int32, never saturated.
 *
 * Bands are diagonal bands lo <= j - i <= hi in window coordinates (i query
 * position, j position in the subject window), as src/algorithm/banded.rs:29-54.
 */
#ifndef SABER_GPU_H
#define SABER_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SABER_OK 0
#define SABER_ERR_ARG (-1)      /* invalid argument */
#define SABER_ERR_CUDA (-2)     /* CUDA runtime / launch error */
#define SABER_ERR_NOMEM (-3)    /* device allocation failed */
#define SABER_ERR_STATE (-4)    /* missing prerequisite (no DB, no queries, ...) */
#define SABER_ERR_CAP (-5)      /* traceback direction matrix over the byte cap */
#define SABER_ERR_DEVICE (-6)   /* a device-side check failed (error word set) */

typedef struct saber_gpu saber_gpu;

/* One banded scoring job: the query, a subject window inside the loaded
 * database and the band its alignment must stay in.  Mirrors the reference's
 * BandJob (src/algorithm/band_simd8.rs:27-33) plus the query/window
 * addressing that Engine::score_windows does per region
 * (src/search/engine.rs:1045-1054).  32 bytes. */
typedef struct {
    uint32_t query;     /* index into the loaded query set */
    uint32_t subject;   /* subject id (informational; not read by the kernels) */
    uint64_t win_begin; /* absolute residue offset of the window start in the DB */
    uint32_t win_len;   /* window length n */
    int32_t band_lo;    /* band, relative to the window: band_lo <= j - i <= band_hi */
    int32_t band_hi;
    uint32_t flags;     /* reserved, 0 */
} saber_band_job;

/* Work counters of the last scoring call (names follow the reference's
 * Counters, src/search/engine.rs:205-282, where they exist). */
typedef struct {
    uint64_t jobs;            /* jobs scored */
    uint64_t banded_cells;    /* in-band cells, counted as banded.rs:123-131 */
    uint64_t fast_cells;      /* the part of banded_cells in jobs of the packed int16 kernel */
    uint64_t fast_jobs;       /* jobs taken by the packed int16 kernel */
    uint64_t generic_jobs;    /* jobs scored directly in int32 (narrow bands) */
    uint64_t i16_rescored;    /* int16 results at the overflow limit, rescored in int32 */
    uint64_t empty_jobs;      /* empty band / window / query: score 0 */
    uint64_t kernel_launches; /* this library's own kernels launched by the call */
    uint64_t library_launches;/* CUB sort / scan / select kernels launched by the call */
    double t_prep_ms;         /* device time: classify, sort, pairing (CUDA events) */
    double t_fast_ms;         /* device time of the packed int16 kernel */
    double t_generic_ms;      /* device time of the int32 kernel */
    uint64_t prof8;           /* 1: the packed kernel read the int8 copy of the query profiles (every
                                 S + bias + go of the query set in [-127, 127]), 0: the int16 profiles */
} saber_score_stats;

/* ---- handle ---------------------------------------------------------- */

/* Opens device `device` and creates the handle's stream.  Replaces
 * try_init_backend / CudaBackend::new_on_device (src/gpu/mod.rs:63-77,
 * src/gpu/cuda.rs:45-51). */
int saber_gpu_open(int device, saber_gpu** out);
int saber_gpu_close(saber_gpu* h);
/* Last error message of this handle ("" when none).  Valid until the next call. */
const char* saber_gpu_last_error(const saber_gpu* h);
/* The CUDA stream (cudaStream_t) all work of this handle runs on. */
void* saber_gpu_stream(saber_gpu* h);

/* Scoring scheme for the following calls.  Replaces the `matrix` and `gaps`
 * arguments of ScoreBackend::score_windows (src/gpu/mod.rs:51-58) and the
 * banded Scheme (src/algorithm/banded.rs:21-27).  Requires
 * 0 <= gap_extend <= gap_open <= 1000. */
int saber_gpu_set_scheme(saber_gpu* h, const int32_t* matrix576, int32_t gap_open,
                         int32_t gap_extend);

/* Uploads the database residues (codes) and subject offsets (nsub + 1
 * entries, offsets[0] = 0).  Replaces the residue access of SeedIndex
 * (src/search/index.rs:644,701-717) for the device path. */
int saber_gpu_load_db(saber_gpu* h, const uint8_t* residues, uint64_t n_residues,
                      const uint64_t* offsets, uint64_t nsub);

/* Uploads a query set: codes, offsets (nq + 1 entries) and the per-position
 * composition bias (same offsets; NULL = no bias).  Builds the device query
 * profiles for the current scheme.  Replaces the per-query QueryPrep inputs
 * (src/search/engine.rs:497-510) that the scoring stage reads. */
int saber_gpu_load_queries(saber_gpu* h, const uint8_t* codes, const uint64_t* offsets,
                           const int8_t* bias, uint32_t nq);

/* ---- banded scoring (score only) -------------------------------------
 * Exact score of every job, identical to the reference's banded_score /
 * score_banded_many (src/algorithm/banded.rs:408-449,
 * src/algorithm/band_simd8.rs:78-185): the optimal local alignment inside
 * the clipped band; 0 for an empty band, window or query. */

/* Host buffers: copies the jobs in and the scores out on the handle's stream
 * (end-to-end path). */
int saber_gpu_score_band_jobs(saber_gpu* h, const saber_band_job* jobs, uint64_t njobs,
                              int32_t* scores, saber_score_stats* stats);

/* Device buffers: d_jobs and d_scores are device pointers; the call enqueues
 * on the handle's stream and returns after the work is queued and its
 * bookkeeping read back (one small device-to-host read). */
int saber_gpu_score_band_jobs_dev(saber_gpu* h, const saber_band_job* d_jobs, uint64_t njobs,
                                  int32_t* d_scores, saber_score_stats* stats);

/* One query against many banded subject windows, host buffers, caller order:
 * the signature of score_banded_many (src/algorithm/band_simd8.rs:78-86) in C.
 * subjects: concatenated windows with offsets (njobs + 1); bands: lo/hi per job. */
int saber_gpu_score_banded_many(saber_gpu* h, const uint8_t* query, uint32_t m,
                                const int8_t* bias, const uint8_t* subjects,
                                const uint64_t* sub_offsets, const int64_t* band_lo,
                                const int64_t* band_hi, uint64_t njobs, int32_t* scores);

/* ScoreBackend::score_windows (src/gpu/mod.rs:51-58, src/gpu/cuda.rs:112-155):
 * full-window local SW score of one query against every window, in input
 * order, with its own matrix and gaps (the handle's scheme is not changed). */
int saber_gpu_score_windows(saber_gpu* h, const uint8_t* query, uint32_t m,
                            const int8_t* bias, const uint8_t* windows,
                            const uint64_t* win_offsets, uint32_t nwin,
                            const int32_t* matrix576, int32_t gap_open, int32_t gap_extend,
                            int32_t* scores);

/* ---- scan schedule: seeds, hits, window filter, X-drop, regions ------------ */

/* Seeding scheme and heuristics of the scan schedule (ScanSeeds,
 * src/search/engine/scan.rs:28-33, and the SearchParams fields it reads,
 * src/search/engine.rs:60-159).  Shapes are given by their care offsets. */
typedef struct {
    uint8_t alpha_map[24];         /* reduced letter per residue code, 255 = not seedable */
    uint32_t alpha_size;           /* letters of the seed alphabet */
    uint32_t nshapes;              /* <= 32 */
    uint32_t shape_span[32];
    uint32_t shape_weight[32];     /* <= 16 */
    uint16_t shape_off[32][16];    /* care offsets of every shape */
    uint32_t hit_filter_min_ids;   /* window filter threshold, 0 = off */
    uint32_t hit_filter_exact_weight;
    int32_t hsp_threshold;         /* minimum ungapped HSP score */
    int32_t x_drop;                /* ungapped X-drop */
    int32_t window_slack;          /* HSPs within 2 x slack diagonals form one region */
    uint32_t max_regions_per_subject;
    uint32_t max_candidates;       /* regions kept per query */
    uint64_t seed_max_occ;         /* 0 = automatic frequent-seed cap */
    uint64_t ref_db_residues;      /* reference database size of the automatic cap */
    uint64_t db_length;            /* database residues of the statistics */
} saber_scan_params;

/* A candidate region: subject, diagonal range d = j - i, best HSP score
 * (Region, src/search/engine.rs:467-473). */
typedef struct {
    uint32_t query;
    uint32_t subject;
    int32_t d_min, d_max;
    int32_t best;
} saber_region;

/* Work counters of one scan (names of Counters, src/search/engine.rs:205-282). */
typedef struct {
    uint64_t seed_positions, seeds_frequent_skipped, hits, hits_filtered, ungapped_extensions,
        extensions_avoided, xdrop_steps, hsps, regions, regions_weak_dropped, regions_dropped_by_cap;
    double t_tables_ms, t_scan_ms, t_visit_ms, t_regions_ms;
} saber_scan_stats;

/* Database seed mask: one byte per residue of the loaded database, nonzero =
 * masked from seeding (the tantan runs of the index, index.rs mask_runs;
 * scan.rs:123-141 applies them).  NULL clears the mask. */
int saber_gpu_load_db_mask(saber_gpu* h, const uint8_t* mask, uint64_t n_residues);
/* The same mask given as nruns sorted half-open runs [runs[2r], runs[2r+1])
 * of database residues, as a SABERIDX index stores it (section "maskruns",
 * index.rs:613-617); expanded on the device. */
int saber_gpu_load_db_mask_runs(saber_gpu* h, const uint64_t* runs, uint64_t nruns);

/* ---- tantan seed masking (masking.rs) -----------------------------------------
 *
 * Tantan's HMM (Frith 2011): posterior probability that each residue lies in
 * a tandem repeat, from a scaled forward-backward pass in f32 that rounds
 * every operation as the reference's scalar body does (masking.rs:429-529);
 * positions with posterior >= min_prob are masked from seeding.  Model
 * parameters follow TantanParams (masking.rs:36-49); lambda <= 0 derives it
 * from the matrix (implied_lambda, masking.rs:531-583). */
typedef struct {
    double repeat_start;  /* r, default 0.005 */
    double repeat_end;    /* e, default 0.05 */
    uint32_t max_period;  /* W repeat states, default 50, at most 64 */
    uint32_t pad_;
    double decay;         /* d, default 0.9 */
    double min_prob;      /* mask threshold, default 0.5 */
    double lambda;        /* <= 0: implied by the matrix */
} saber_tantan_params;

/* The lambda implied by a 24x24 matrix (its 20 standard letters); NaN when
 * no root exists.  Host only (masking.rs:531-583). */
double saber_tantan_implied_lambda(const int32_t* matrix576);
/* Tantan::mask over a batch of sequences (masking.rs:191-196), computed on
 * the GPU: codes / offsets[nseq + 1] on the host; mask[i] = 1 where the
 * posterior >= min_prob (indexed like codes); probs (NULL = not wanted)
 * receives the posteriors.  *n_masked = masked positions; *lambda_out
 * (nullable) = the lambda used.  The reference masks queries with BLOSUM62
 * (engine.rs:575-577). */
int saber_gpu_tantan_mask(saber_gpu* h, const saber_tantan_params* params, const int32_t* matrix576,
                          const uint8_t* codes, const uint64_t* offsets, uint64_t nseq, uint8_t* mask,
                          float* probs, uint64_t* n_masked, double* lambda_out);
/* Masks the loaded database on the device and installs the result as its
 * seed mask (as saber_gpu_load_db_mask would): the reference's scan database
 * with tantan recomputed (scan.rs:1078-1123). */
int saber_gpu_tantan_mask_db(saber_gpu* h, const saber_tantan_params* params, const int32_t* matrix576,
                             uint64_t* n_masked, double* lambda_out);

/* ---- six-frame translation (translation.rs) ------------------------------------
 *
 * Frames 0..5 of every nucleotide sequence (codes 0..3 = ACGT, 4 = N; frames
 * 3..5 on the reverse complement, read from the sequence end) translated with
 * a 64-entry codon table (protein codes, index a*16 + b*4 + c), codons
 * holding N give X (CodonTable::translate_codes, translation.rs:277-308).
 * out receives frame f of sequence s as segment 6*s + f (the reference's
 * translated database order, index.rs:1351-1368; a query's frames in
 * driver.rs:387-402); out_offsets[6*nseq + 1] its bounds.  At most
 * 2 x (nucleotides) residues; SABER_ERR_CAP when out_cap is smaller. */
int saber_gpu_translate6(saber_gpu* h, const uint8_t* nt, const uint64_t* nt_offsets, uint64_t nseq,
                         const uint8_t* codon64, uint8_t* out, uint64_t out_cap, uint64_t* out_offsets);

/* Engine::search_scan's candidate regions for the loaded query set against
 * the loaded database (scan.rs:1261-1497 up to the per-query candidate cap):
 * seed tables of the batch, database scan with the window filter,
 * per-diagonal coverage and ungapped X-drop, region clustering, per-subject
 * and per-query caps.  q_mask: one byte per query residue, nonzero = masked
 * from seeding (NULL = none); region_thr: the per-query region threshold
 * (Engine::hsp_threshold_for, engine.rs:729-736; NULL = hsp_threshold).
 * Regions are written ordered by query, then region_order (engine.rs:493). */
int saber_gpu_scan(saber_gpu* h, const saber_scan_params* params, const uint8_t* q_mask,
                   const int32_t* region_thr, saber_region* out, uint64_t out_cap,
                   uint64_t* n_out, saber_scan_stats* stats);

/* ---- banded traceback ---------------------------------------------------- */

/* One banded alignment job: window of the loaded database, band relative to
 * the window, and stop_at (rows after the first whose best cell reaches it
 * are not computed; INT32_MAX = none).  The arguments of banded_align_until
 * (src/algorithm/banded.rs:472-521) per job. */
typedef struct {
    uint32_t query;
    uint32_t subject;   /* informational */
    uint64_t win_begin;
    uint32_t win_len;
    int32_t band_lo, band_hi;
    int32_t stop_at;
} saber_align_job;

/* Result of one alignment (LocalAlignment, banded.rs:101-113, plus status).
 * Coordinates are 0-based half-open in window coordinates; the operations are
 * n_ops run-length words at ops[ops_offset..]: (run length << 8) | op with op
 * the ASCII 'M', 'I' (query residue vs gap) or 'D' (subject residue vs gap). */
typedef struct {
    int32_t status;  /* banded_align: 1 alignment, 0 none (best 0), SABER_ERR_CAP over
                        the byte cap; traceback: 1 exact, 2 inexact (band capped), 0 none */
    int32_t score;
    uint32_t q_start, q_end, s_start, s_end;
    uint32_t n_ops, ops_offset;
    uint64_t cells;
} saber_alignment;

/* Banded SW with traceback for every job (banded_align_until,
 * banded.rs:472-521, with walk banded.rs:336-403); a job whose direction
 * matrix (m x band width bytes) exceeds max_dir_bytes gets status
 * SABER_ERR_CAP, as the reference returns Err(bytes). */
int saber_gpu_banded_align(saber_gpu* h, const saber_align_job* jobs, uint64_t njobs,
                           uint64_t max_dir_bytes, saber_alignment* out, uint32_t* ops,
                           uint64_t ops_cap);

/* banded_align_until for one query / subject pair given as host arrays, with
 * the handle's scheme (parity mirror of banded.rs:472). */
int saber_gpu_banded_align_one(saber_gpu* h, const uint8_t* query, uint32_t m,
                               const int8_t* bias, const uint8_t* subject, uint32_t n,
                               int64_t band_lo, int64_t band_hi, uint64_t max_dir_bytes,
                               int32_t stop_at, saber_alignment* out, uint32_t* ops,
                               uint64_t ops_cap);

/* One region to trace back (the arguments of Engine::traceback,
 * src/search/engine.rs:1328-1337): its diagonals relative to the window
 * start (region d_min - lo, d_max - lo), the exact score of the window
 * (want) and the scoring band of its plan (limit, flags bit 1).  flags bit 0:
 * full band (exhaustive search or a region with best == 0). */
typedef struct {
    uint32_t query;
    uint32_t subject;   /* informational */
    uint64_t win_begin;
    uint32_t win_len;
    int32_t d_min, d_max;
    int32_t limit_lo, limit_hi;
    int32_t want;
    uint32_t flags;
    uint32_t reserved;  /* 0; pads the struct to 48 bytes */
} saber_traceback_job;

typedef struct {
    uint64_t tracebacks;      /* banded_align calls (Counters::tracebacks) */
    uint64_t band_widenings;  /* Counters::band_widenings */
    uint64_t end_anchored;    /* Counters::end_anchored_tracebacks */
    uint64_t band_capped;     /* Counters::band_capped */
    uint64_t banded_cells;    /* cells of all passes */
    uint64_t launches;        /* widening rounds (one launch each) */
} saber_traceback_stats;

/* The widening band traceback that reproduces the window score
 * (Engine::traceback + traceback_from_end, src/search/engine.rs:1328-1445),
 * batched: band = region diagonals +- pad, pad = max(band_pad, 4) doubling,
 * clipped to the limit, until the score reaches want or the band covers; a
 * band over the byte cap falls back to the end-anchored search. */
int saber_gpu_traceback(saber_gpu* h, const saber_traceback_job* jobs, uint64_t njobs,
                        int32_t band_pad, uint64_t max_dir_bytes, saber_alignment* out,
                        uint32_t* ops, uint64_t ops_cap, saber_traceback_stats* stats);

/* ---- the batch search (host engine over the device stages) ---------------
 *
 * saber_gpu_search runs Engine::search_scan for one query batch end to end
 * (src/search/engine/scan.rs:1261-1497 with the shared Engine stages of
 * src/search/engine.rs): query preparation (composition bias, statistics,
 * floors, engine.rs:714-786), the scan (saber_gpu_scan), window plans
 * (engine.rs:1223-1324), two-stage banded scoring of the whole batch
 * (engine.rs:1021-1099), finish with E-values, ordering, per-subject and
 * per-query caps and the widening traceback (engine.rs:1127-1221,1328-1445),
 * and make_hit (engine.rs:1447-1530).  The f64 statistics run on the host
 * in the operation order of src/scoring/stats.rs. */
typedef struct {
    /* SearchParams (engine.rs:60-201) */
    double evalue;                 /* -E; <= 0 or inf: no cut */
    double min_bitscore;           /* NaN: none */
    uint32_t max_target_seqs, max_hsps;
    double min_identity, min_query_cover, min_subject_cover;
    int32_t hsp_threshold;
    double hsp_floor_fraction;
    int32_t band_pad, window_slack, score_band, score_prefilter_band;
    double score_prefilter_frac;
    uint32_t comp_bias;            /* 1: composition-bias correction (protein) */
    uint32_t exhaustive;           /* --preset exhaustive: every subject, full rectangle */
    uint64_t traceback_max_bytes;
    uint64_t ref_db_residues;
    uint32_t evalue_model;         /* 0 per-subject, 1 database */
    uint32_t is_protein;
    /* gapped Karlin-Altschul parameters of the scheme (stats.rs:277-310) */
    double lambda, k, h, alpha, beta;
    uint32_t even_scores_only;
    uint32_t pad_;
    /* the scan; its db_length is the database length of the statistics (the
     * residues; a translated database: its nucleotides / 3, driver.rs:575-583) */
    saber_scan_params scan;
    /* sequences of the statistics; 0 = the loaded subjects (a translated
     * database: its nucleotide sequences, driver.rs:575-583) */
    uint64_t stats_num_seqs;
} saber_search_params;

/* One reported alignment (Hit, engine.rs:310-357): 1-based inclusive
 * coordinates; n_ops run-length words (len << 8 | op) at ops[ops_offset..]. */
typedef struct {
    uint32_t query, subject;
    int32_t score;
    uint32_t exact;
    double evalue, bitscore;
    uint32_t q_start, q_end, s_start, s_end;
    uint32_t columns, matches, mismatches, positives, gap_opens, gap_columns;
    uint32_t q_len, s_len;
    uint32_t n_ops, pad_;
    uint64_t ops_offset;
} saber_hit;

typedef struct {
    saber_scan_stats scan;
    saber_traceback_stats traceback;
    uint64_t regions;             /* candidate regions after the per-query caps */
    uint64_t triage_dropped;      /* regions dropped by the learned triage */
    uint64_t band_scored_regions, band_rescored, banded_cells, score_launches;
    uint64_t alignments;
    double t_prep_ms, t_scan_ms, t_triage_ms, t_plan_ms, t_score_ms, t_finish_ms, t_total_ms;  /* host wall clock */
    /* inside t_score_ms: wall clock of the scoring calls (copies, kernels,
     * synchronisation) and the device time of their kernels */
    double t_score_calls_ms, t_score_device_ms;
    /* inside t_finish_ms: wall clock of the traceback calls */
    double t_finish_tb_ms;
    /* the scoring calls' device time by part (saber_score_stats) */
    double t_score_prep_ms, t_score_fast_ms, t_score_generic_ms;
    /* host parts: inside t_score_ms, building the first-stage jobs and the
     * second-stage decisions and jobs; inside t_finish_ms, the per-query
     * E-value order */
    double t_score_build_ms, t_score_stage2_ms, t_finish_order_ms;
} saber_search_stats;

/* Hits of every query of the batch, ordered by query, then (E-value, score
 * desc, subject, s_start) as the reference reports them.  db_res / db_offsets:
 * the host copy of the loaded database (make_hit reads residues); q_mask:
 * one byte per query residue masked from seeding (NULL = none).  Returns
 * SABER_ERR_CAP with *n_hits / *n_ops set when hits_cap or ops_cap is too
 * small (nothing else is written then). */
int saber_gpu_search(saber_gpu* h, const saber_search_params* params, const uint8_t* db_res,
                     const uint64_t* db_offsets, uint64_t nsub, const uint8_t* q_codes,
                     const uint64_t* q_offsets, uint32_t nq, const uint8_t* q_mask, saber_hit* hits,
                     uint64_t hits_cap, uint64_t* n_hits, uint32_t* ops, uint64_t ops_cap, uint64_t* n_ops,
                     saber_search_stats* stats);

/* ---- learned triage of candidate regions ------------------------------------
 *
 * A 3-layer MLP (24 region features -> 256 -> 256 -> 1 logit, ReLU) with
 * bf16 weights and fp32 accumulation, trained on the GPU by this library's
 * own forward / backward / Adam kernels, on labels that the plain search
 * produces (the region yields a reported hit).  Installed on a handle, the
 * batch engine (saber_gpu_search) drops the candidate regions whose logit is
 * below the threshold before window planning and banded scoring; every
 * surviving region is still scored exactly.  No reference counterpart.
 *
 * Model: SABER_TRIAGE_MODEL_FLOATS floats: W1[32][256] (input-major; rows
 * 24..31 unused), b1[256], W2[256][256], b2[256], W3[256], b3, mu[32],
 * isd[32] (input normalisation x' = (x - mu) * isd, not trained).  Feature
 * rows are 32 floats (24 used). */
#define SABER_TRIAGE_MODEL_FLOATS 74561
#define SABER_TRIAGE_ROW_FLOATS 32

typedef struct {
    uint32_t epochs, batch;
    float lr, pos_weight, weight_decay;
    uint32_t pad_;
    uint64_t seed;
} saber_triage_train_cfg;

typedef struct {
    uint64_t steps;
    double final_loss;   /* mean batch loss of the last epoch */
} saber_triage_train_stats;

/* One forward + backward pass over n rows: gradients of the mean weighted
 * binary cross-entropy (positives weighted by pos_weight) in the model
 * layout (zeros for mu / isd), and the loss. */
int saber_gpu_triage_grads(saber_gpu* h, const float* model, const float* rows, const uint8_t* labels, uint32_t n,
                           float pos_weight, float* grads, double* loss);
/* Adam training (seeded shuffles, mini-batches) starting from and
 * overwriting model. */
int saber_gpu_triage_train(saber_gpu* h, float* model, const float* rows, const uint8_t* labels, uint64_t n,
                           const saber_triage_train_cfg* cfg, saber_triage_train_stats* stats);
/* Logits of n feature rows (the inference kernel the engine runs). */
int saber_gpu_triage_predict(saber_gpu* h, const float* model, const float* rows, uint64_t n, float* logits);
/* Install (model != NULL) or remove the triage model of the batch engine:
 * regions with logit < threshold are dropped. */
int saber_gpu_set_triage(saber_gpu* h, const float* model, float threshold);
/* Collect, on the next saber_gpu_search calls, every candidate region's
 * feature row and label (1 = it produced a reported hit), regions in the
 * engine's order (query, then region order); with triage installed, the
 * rows of the regions kept and the logits of all.  collect = 0 stops. */
int saber_gpu_collect_regions(saber_gpu* h, int32_t collect);
int saber_gpu_collected_regions(saber_gpu* h, float* rows, uint8_t* labels, float* logits, uint64_t cap,
                                uint64_t* n);

/* Tuning: rows per strip of the packed int16 scoring kernel (8 or 16,
 * default 16).  Results do not depend on it.  No reference counterpart (the
 * reference's AVX2 kernels have fixed vector widths). */
int saber_gpu_set_strip_rows(saber_gpu* h, int32_t strip_rows);
int32_t saber_gpu_get_strip_rows(saber_gpu* h);

/* Tuning: with 16-row strips, a job of width > 32 whose sweep as 16-row
 * strips takes more than `steps` column steps (strips x (width + 15)) is
 * swept by a whole lane as paired strips (32 rows, half the critical path);
 * 0xFFFFFFFF disables pairing.  Default 2048.  Results do not depend on it.
 * No reference counterpart. */
int saber_gpu_set_pair_steps(saber_gpu* h, uint32_t steps);
uint32_t saber_gpu_get_pair_steps(saber_gpu* h);

/* Tuning: a job whose sweep in one lane would take more than `steps` column
 * steps (strips x the steps of a strip, window columns only) is scored by
 * the int32 kernel instead, which pipelines a long job's strips over a
 * warp's lanes, so one long job does not set the launch's length.
 * 0xFFFFFFFF keeps every job on the int16 lanes; 0xFFFFFFFE (the default)
 * picks, per call, the power of two at or above four times the sweep steps
 * of one int16 lane if the batch's in-band cells were spread evenly over
 * the lanes (32 cells per step), and at least 2048.  Results do not depend
 * on it.
 * No reference counterpart. */
int saber_gpu_set_long_steps(saber_gpu* h, uint32_t steps);
uint32_t saber_gpu_get_long_steps(saber_gpu* h);

/* Tuning: bytes of seed tables (rank-compressed presence groups, entry
 * offsets, batch positions) that one database pass of saber_gpu_scan looks
 * up; the shapes are split into passes of at most this many bytes (at least
 * one shape per pass) so that the tables stay resident in L2.  Default 48 MiB.
 * Results do not depend on it.  No reference counterpart (the reference
 * scans shape by shape on the CPU). */
int saber_gpu_set_scan_table_bytes(saber_gpu* h, uint64_t bytes);
uint64_t saber_gpu_get_scan_table_bytes(saber_gpu* h);

/* Captured scoring graphs (default on): saber_gpu_score_band_jobs (and so
 * the batch engine's scoring stages) runs classify -> radix sort -> int16
 * kernels -> int32 kernel as one CUDA graph with every count kept on the
 * device, job count padded to a power of two and scratch sized for the
 * widest band rounded up to a power of two; a graph is captured once per
 * size bucket and buffer set and replayed.  Off: the step-by-step launches
 * (which also report per-stage device times).  Results do not depend on it.
 * saber_gpu_graph_captures counts the captures of the handle. */
int saber_gpu_set_graphs(saber_gpu* h, int32_t on);
int32_t saber_gpu_get_graphs(saber_gpu* h);
uint64_t saber_gpu_graph_captures(saber_gpu* h);

/* Allocation-free variant of saber_gpu_score_band_jobs_dev.  No counterpart
 * in the reference.  It exists for callers that cannot allocate GPU memory at
 * scoring time: a process whose device memory is held by another allocator or
 * reserved up front in a fixed budget, or a latency-bound path where the
 * device synchronisation of a cudaMalloc is not acceptable.  It makes no
 * cudaMalloc/cudaFree and calls no allocating library routine: it reads the
 * handle's resident database, query set and scheme and the caller's device
 * buffers d_jobs / d_scores, and uses a fixed 16 MiB scratch array compiled
 * into the library (held by every GPU that loads the library until the
 * process exits).  Scores equal those of the other entry points (int32
 * recurrence of banded.rs:134-224).
 * max_band_width bounds the clipped band width of every job (1..4096; larger
 * is rejected with SABER_ERR_ARG; a job wider than it, or one outside the
 * loaded queries or database, makes the call return SABER_ERR_ARG with the
 * job's index in the message).  The scratch holds (16 MiB - 256 B) /
 * (16 (max_band_width + 1)) scoring threads, about 4,000 at 257 and 255 at
 * 4096, so a smaller max_band_width scores faster.
 * The call runs on the handle's stream, which is not ordered after the
 * caller's streams: finish writing d_jobs before the call.  It returns once
 * d_scores is written (it reads a status word back and waits for the stream).
 * The first call on a device looks up the scratch array's device address;
 * make it before any stream capture.  Every call shares the scratch and it
 * keeps the last call's contents (the status word is cleared by each call);
 * calls that overlap on the GPU race on it. */
int saber_gpu_score_band_jobs_noalloc(saber_gpu* h, const saber_band_job* d_jobs, uint64_t njobs,
                                      int32_t max_band_width, int32_t* d_scores);

/* Measures the integer-pipe peak of this GPU for the roofline: throughput of
 * the DPX packed-int16 max/add-max instructions the scoring kernel uses
 * (lane-instructions per second; each does two 16-bit operations) and of plain
 * int32 max instructions.  No reference counterpart (measurement utility). */
int saber_gpu_probe_int_peak(saber_gpu* h, double* dpx_s16x2_lane_ops_per_s,
                             double* i32_lane_ops_per_s);

/* Lane-instructions per second of the packed cell's instructions, each timed
 * alone in independent chains: rates[0] DPX fused add-max (viaddmax s16x2),
 * rates[1] DPX three-input max with relu, rates[2] packed add (vadd2),
 * rates[3] byte permute, rates[4] a fused add-max chain and a packed-add
 * chain side by side (together, when they issue to different pipes, above
 * either alone).  Measurement utility; no reference counterpart. */
int saber_gpu_probe_pipe_rates(saber_gpu* h, double rates[5]);

/* In-band cell count of one job after clipping the band to the m x n
 * rectangle, counted as the reference counts banded cells (the row_range span
 * summed over rows, src/algorithm/banded.rs:123-131,208).  Host-only helper;
 * needs no GPU. */
uint64_t saber_band_cells(uint64_t m, uint64_t n, int64_t band_lo, int64_t band_hi);

#ifdef __cplusplus
}
#endif
#endif
