/*
 * CPU oracle (test infrastructure only) — see oracle.h for scope and pinning.
 * Restates the reference's scalar algorithms; each function cites the
 * reference file:line it follows.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* alphabet.rs:39-41: codes >= 24 are scored as X (22). */
static inline int code_index(uint8_t c) { return c < 24 ? (int)c : 22; }

/* banded.rs:121 */
#define NEG32 (INT32_MIN / 4)

static inline int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }
static inline int32_t max32(int32_t a, int32_t b) { return a > b ? a : b; }

int64_t orc_sw_reference(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                         const int32_t* matrix, const int8_t* bias,
                         int64_t go, int64_t ge, uint64_t* q_end, uint64_t* s_end) {
    /* reference.rs:15-52 */
    *q_end = 0;
    *s_end = 0;
    if (m == 0 || n == 0) return 0;
    const int64_t neg = INT64_MIN / 4;
    size_t w = n + 1;
    int64_t* h = (int64_t*)calloc((m + 1) * w, sizeof(int64_t));
    int64_t* e = (int64_t*)malloc((m + 1) * w * sizeof(int64_t));
    int64_t* f = (int64_t*)malloc((m + 1) * w * sizeof(int64_t));
    for (size_t t = 0; t < (m + 1) * w; t++) { e[t] = neg; f[t] = neg; }
    int64_t best = 0;
    uint64_t bi = 0, bj = 0;
    for (size_t i = 1; i <= m; i++) {
        int qi = code_index(q[i - 1]);
        int64_t b = bias ? (int64_t)bias[i - 1] : 0;
        for (size_t j = 1; j <= n; j++) {
            int sj = code_index(s[j - 1]);
            int64_t ee = max64(h[i * w + j - 1] - go, e[i * w + j - 1] - ge);
            int64_t ff = max64(h[(i - 1) * w + j] - go, f[(i - 1) * w + j] - ge);
            int64_t dd = h[(i - 1) * w + j - 1] + (int64_t)matrix[qi * 24 + sj] + b;
            int64_t v = max64(max64(max64(0, ee), ff), dd);
            e[i * w + j] = ee;
            f[i * w + j] = ff;
            h[i * w + j] = v;
            if (v > best) { best = v; bi = i; bj = j; }
        }
    }
    free(h); free(e); free(f);
    *q_end = bi;
    *s_end = bj;
    return best;
}

int orc_score_alignment(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                        uint64_t q_start, uint64_t s_start,
                        const uint8_t* ops, const uint32_t* lens, uint32_t n_ops,
                        const int32_t* matrix, const int8_t* bias,
                        int64_t go, int64_t ge,
                        int64_t* score, uint64_t* q_end, uint64_t* s_end) {
    /* reference.rs:58-103 */
    uint64_t i = q_start, j = s_start;
    int64_t sc = 0;
    for (uint32_t t = 0; t < n_ops; t++) {
        uint64_t len = lens[t];
        switch (ops[t]) {
        case 'M':
            for (uint64_t k = 0; k < len; k++) {
                if (i >= m || j >= n) return -1;
                int64_t b = bias ? (int64_t)bias[i] : 0;
                sc += (int64_t)matrix[code_index(q[i]) * 24 + code_index(s[j])] + b;
                i++; j++;
            }
            break;
        case 'I':
            if (len == 0 || i + len > m) return -1;
            sc -= go + ((int64_t)len - 1) * ge;
            i += len;
            break;
        case 'D':
            if (len == 0 || j + len > n) return -1;
            sc -= go + ((int64_t)len - 1) * ge;
            j += len;
            break;
        default:
            return -1;
        }
    }
    *score = sc;
    *q_end = i;
    *s_end = j;
    return 0;
}

/* banded.rs:45-47 (Band::clip) and 41-43 (width). */
static void band_clip(int64_t* lo, int64_t* hi, size_t m, size_t n) {
    int64_t l = *lo, h = *hi;
    if (l < -((int64_t)m - 1)) l = -((int64_t)m - 1);
    if (h > (int64_t)n - 1) h = (int64_t)n - 1;
    *lo = l;
    *hi = h;
}

/* banded.rs:123-131 (row_range): k in [kmin, kmax], j = i + lo + k. */
static int row_range(int64_t i, int64_t lo, int64_t w, int64_t n, int64_t* kmin, int64_t* kmax) {
    int64_t a = -(i + lo);
    if (a < 0) a = 0;
    int64_t b = n - 1 - i - lo;
    if (b > w - 1) b = w - 1;
    *kmin = a;
    *kmax = b;
    return a <= b;
}

void orc_banded_score(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                      const int8_t* bias, orc_scheme sc, int64_t lo, int64_t hi,
                      orc_band_score* out) {
    /* banded.rs:134-224 */
    out->score = 0; out->q_end = 0; out->s_end = 0; out->cells = 0;
    if (m == 0 || n == 0 || hi < lo) return;
    band_clip(&lo, &hi, m, n);
    int64_t w = hi - lo + 1;
    if (w <= 0) return;
    int32_t* hp = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    int32_t* fp = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    int32_t* hc = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    int32_t* fc = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    for (int64_t k = 0; k <= w; k++) { hp[k] = fp[k] = hc[k] = fc[k] = NEG32; }
    const int32_t go = sc.gap_open, ge = sc.gap_extend;
    uint64_t cells = 0;
    int32_t best = 0;
    uint64_t bq = 0, bs = 0;
    for (int64_t i = 0; i < (int64_t)m; i++) {
        int64_t kmin, kmax;
        if (!row_range(i, lo, w, (int64_t)n, &kmin, &kmax)) {
            for (int64_t k = 0; k < w; k++) { hc[k] = NEG32; fc[k] = NEG32; }
        } else {
            const int32_t* row = sc.matrix + code_index(q[i]) * 24;
            int32_t b = bias ? (int32_t)bias[i] : 0;
            int32_t e = NEG32, h_left = NEG32;
            int64_t base = i + lo;
            for (int64_t k = kmin; k <= kmax; k++) {
                int64_t j = base + k;
                int32_t ecand = max32(h_left - go, e - ge);
                e = k > kmin ? ecand : NEG32;
                int32_t f = i >= 1 ? max32(hp[k + 1] - go, fp[k + 1] - ge) : NEG32;
                int32_t hd = (i >= 1 && j >= 1) ? hp[k] : 0;
                int32_t diag = hd + row[code_index(s[j])] + b;
                int32_t h = max32(max32(max32(diag, e), f), 0);
                hc[k] = h;
                fc[k] = f;
                h_left = h;
                if (h > best) { best = h; bq = (uint64_t)i + 1; bs = (uint64_t)j + 1; }
            }
            cells += (uint64_t)(kmax - kmin + 1);
            for (int64_t k = 0; k < kmin; k++) { hc[k] = NEG32; fc[k] = NEG32; }
            for (int64_t k = kmax + 1; k < w; k++) { hc[k] = NEG32; fc[k] = NEG32; }
        }
        int32_t* t;
        t = hp; hp = hc; hc = t;
        t = fp; fp = fc; fc = t;
    }
    out->score = best;
    out->q_end = bq;
    out->s_end = bs;
    out->cells = cells;
    free(hp); free(fp); free(hc); free(fc);
}

/* Shared DP of banded_align_scalar (banded.rs:250-326); fills dir, returns
 * best (score, i, k) and cells.  stop_at: banded_simd.rs:594-596. */
static void banded_dir_dp(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                          const int8_t* bias, orc_scheme sc, int64_t lo, int64_t w,
                          uint8_t* dir, int32_t stop_at,
                          int32_t* best_score, int64_t* best_i, int64_t* best_k, uint64_t* cells_out) {
    int32_t* hp = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    int32_t* fp = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    int32_t* hc = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    int32_t* fc = (int32_t*)malloc((size_t)(w + 1) * sizeof(int32_t));
    for (int64_t k = 0; k <= w; k++) { hp[k] = fp[k] = hc[k] = fc[k] = NEG32; }
    const int32_t go = sc.gap_open, ge = sc.gap_extend;
    int32_t bsc = 0;
    int64_t bi = 0, bk = 0;
    uint64_t cells = 0;
    for (int64_t i = 0; i < (int64_t)m; i++) {
        int64_t kmin, kmax;
        if (!row_range(i, lo, w, (int64_t)n, &kmin, &kmax)) {
            for (int64_t k = 0; k < w; k++) { hc[k] = NEG32; fc[k] = NEG32; }
        } else {
            const int32_t* row = sc.matrix + code_index(q[i]) * 24;
            int32_t b = bias ? (int32_t)bias[i] : 0;
            int32_t e = NEG32, h_left = NEG32;
            int64_t base = i + lo;
            uint8_t* dirrow = dir + (size_t)(i * w);
            for (int64_t k = kmin; k <= kmax; k++) {
                int64_t j = base + k;
                int32_t eo = h_left - go;
                int32_t ee = e - ge;
                uint8_t e_ext = ee > eo;
                e = k > kmin ? max32(ee, eo) : NEG32;
                int32_t fo = hp[k + 1] - go;
                int32_t fe = fp[k + 1] - ge;
                uint8_t f_ext = fe > fo;
                int32_t f = i >= 1 ? max32(fe, fo) : NEG32;
                int32_t hd = (i >= 1 && j >= 1) ? hp[k] : 0;
                int32_t diag = hd + row[code_index(s[j])] + b;
                uint8_t c1 = diag > 0;
                int32_t h1 = max32(diag, 0);
                uint8_t c2 = e > h1;
                int32_t h2 = max32(h1, e);
                uint8_t c3 = f > h2;
                int32_t h = max32(h2, f);
                uint8_t org = c3 ? 3 : (c2 ? 2 : c1);
                hc[k] = h;
                fc[k] = f;
                dirrow[k] = (uint8_t)(org | (e_ext << 2) | (f_ext << 3));
                h_left = h;
                if (h > bsc) { bsc = h; bi = i; bk = k; }
            }
            cells += (uint64_t)(kmax - kmin + 1);
            for (int64_t k = 0; k < kmin; k++) { hc[k] = NEG32; fc[k] = NEG32; }
            for (int64_t k = kmax + 1; k < w; k++) { hc[k] = NEG32; fc[k] = NEG32; }
        }
        int32_t* t;
        t = hp; hp = hc; hc = t;
        t = fp; fp = fc; fc = t;
        if (bsc >= stop_at) break;
    }
    *best_score = bsc;
    *best_i = bi;
    *best_k = bk;
    *cells_out = cells;
    free(hp); free(fp); free(hc); free(fc);
}

uint64_t orc_banded_dir(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                        const int8_t* bias, orc_scheme sc, int64_t lo, int64_t hi,
                        uint8_t* dir, uint64_t dir_cap, int64_t* clipped_lo) {
    if (m == 0 || n == 0 || hi < lo) return 0;
    band_clip(&lo, &hi, m, n);
    int64_t w = hi - lo + 1;
    if (w <= 0 || (uint64_t)(m * (uint64_t)w) > dir_cap) return 0;
    memset(dir, 0xFF, (size_t)(m * (uint64_t)w));
    int32_t bsc; int64_t bi, bk; uint64_t cells;
    banded_dir_dp(q, m, s, n, bias, sc, lo, w, dir, INT32_MAX, &bsc, &bi, &bk, &cells);
    *clipped_lo = lo;
    return (uint64_t)w;
}

int orc_banded_align(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                     const int8_t* bias, orc_scheme sc, int64_t lo, int64_t hi,
                     uint64_t max_dir_bytes, int32_t stop_at,
                     orc_alignment* out, uint8_t* ops, uint32_t* lens, uint32_t ops_cap) {
    /* banded.rs:227-332 */
    memset(out, 0, sizeof(*out));
    if (m == 0 || n == 0 || hi < lo) return 0;
    band_clip(&lo, &hi, m, n);
    int64_t w = hi - lo + 1;
    if (w <= 0) return 0;
    uint64_t need = (uint64_t)m * (uint64_t)w;
    if (need > max_dir_bytes) return -2;
    uint8_t* dir = (uint8_t*)calloc((size_t)need, 1);
    int32_t bsc; int64_t bi, bk; uint64_t cells;
    banded_dir_dp(q, m, s, n, bias, sc, lo, w, dir, stop_at, &bsc, &bi, &bk, &cells);
    if (bsc <= 0) { free(dir); out->cells = cells; return 0; }

    /* walk, banded.rs:336-403 */
    uint64_t q_end = (uint64_t)bi + 1;
    uint64_t s_end = (uint64_t)(bi + lo + bk) + 1;
    size_t cap = (size_t)(m + n + 2);
    uint8_t* opbuf = (uint8_t*)malloc(cap);
    size_t nop = 0;
    int state = 0; /* 0 = H, 1 = E (query gap, 'D'), 2 = F (subject gap, 'I') */
    int64_t i = bi, k = bk;
    for (;;) {
        uint8_t d = dir[(size_t)(i * w + k)];
        if (state == 0) {
            uint8_t org = d & 3;
            if (org == 0) break;
            if (org == 1) {
                opbuf[nop++] = 'M';
                int64_t j = i + lo + k;
                if (i == 0 || j == 0) break;
                i -= 1;
            } else if (org == 2) {
                state = 1;
            } else {
                state = 2;
            }
        } else if (state == 1) {
            opbuf[nop++] = 'D';
            int ext = (d & 4) != 0;
            k -= 1;
            if (!ext) state = 0;
        } else {
            opbuf[nop++] = 'I';
            int ext = (d & 8) != 0;
            i -= 1;
            k += 1;
            if (!ext) state = 0;
        }
    }
    /* reverse, derive start coordinates, run-length encode */
    uint64_t qs = q_end, ss = s_end;
    uint32_t runs = 0;
    uint8_t* rop = (uint8_t*)malloc(nop + 1);
    uint32_t* rlen = (uint32_t*)malloc((nop + 1) * sizeof(uint32_t));
    for (size_t t = 0; t < nop; t++) {
        uint8_t op = opbuf[nop - 1 - t];
        if (op == 'M') { qs--; ss--; }
        else if (op == 'I') qs--;
        else ss--;
        if (runs > 0 && rop[runs - 1] == op) {
            rlen[runs - 1]++;
        } else {
            rop[runs] = op;
            rlen[runs] = 1;
            runs++;
        }
    }
    int rc = 1;
    if (runs > ops_cap || !ops || !lens) {
        rc = -3;
    } else {
        memcpy(ops, rop, runs);
        memcpy(lens, rlen, runs * sizeof(uint32_t));
    }
    free(rop);
    free(rlen);
    free(opbuf);
    free(dir);
    out->score = bsc;
    out->q_start = qs;
    out->q_end = q_end;
    out->s_start = ss;
    out->s_end = s_end;
    out->cells = cells;
    out->n_ops = runs;
    return rc;
}

int32_t orc_ungapped_xdrop(const uint8_t* q, size_t m, const uint8_t* s, size_t n,
                           uint64_t qp, uint64_t sp, const int32_t* matrix,
                           const int8_t* bias, int32_t x,
                           uint64_t* q_lo, uint64_t* q_hi) {
    /* engine.rs:2460-2494 */
    int32_t best_r = 0, cur = 0;
    uint64_t end = qp;
    uint64_t i = qp, j = sp;
    while (i < m && j < n) {
        cur += matrix[code_index(q[i]) * 24 + code_index(s[j])] + (bias ? (int32_t)bias[i] : 0);
        i++; j++;
        if (cur > best_r) { best_r = cur; end = i; }
        else if (cur < best_r - x) break;
    }
    int32_t best_l = 0;
    cur = 0;
    uint64_t start = qp;
    int64_t ii = (int64_t)qp - 1, jj = (int64_t)sp - 1;
    while (ii >= 0 && jj >= 0) {
        cur += matrix[code_index(q[ii]) * 24 + code_index(s[jj])] + (bias ? (int32_t)bias[ii] : 0);
        if (cur > best_l) { best_l = cur; start = (uint64_t)ii; }
        else if (cur < best_l - x) break;
        ii--; jj--;
    }
    *q_lo = start;
    *q_hi = end > qp ? end : qp;
    return best_r + best_l;
}

/* ---- batched jobs ------------------------------------------------------ */

typedef struct {
    const uint8_t* residues;
    const uint8_t* qcodes;
    const uint64_t* qoffs;
    const int8_t* qbias;
    const orc_band_job* jobs;
    uint64_t njobs;
    orc_scheme sc;
    int32_t* scores;
    uint64_t next;          /* shared work counter (atomic) */
    uint64_t cells;         /* summed under atomic add */
} batch_ctx;

static void* batch_worker(void* arg) {
    batch_ctx* c = (batch_ctx*)arg;
    uint64_t local_cells = 0;
    for (;;) {
        uint64_t b = __atomic_fetch_add(&c->next, 64, __ATOMIC_RELAXED);
        if (b >= c->njobs) break;
        uint64_t e = b + 64 < c->njobs ? b + 64 : c->njobs;
        for (uint64_t t = b; t < e; t++) {
            const orc_band_job* jb = &c->jobs[t];
            uint64_t q0 = c->qoffs[jb->query], q1 = c->qoffs[jb->query + 1];
            orc_band_score o;
            orc_banded_score(c->qcodes + q0, (size_t)(q1 - q0),
                             c->residues + jb->win_begin, jb->win_len,
                             c->qbias ? c->qbias + q0 : NULL, c->sc,
                             jb->band_lo, jb->band_hi, &o);
            c->scores[t] = o.score;
            local_cells += o.cells;
        }
    }
    __atomic_fetch_add(&c->cells, local_cells, __ATOMIC_RELAXED);
    return NULL;
}

int orc_score_band_jobs(const uint8_t* residues, const uint8_t* qcodes,
                        const uint64_t* qoffs, const int8_t* qbias,
                        const orc_band_job* jobs, uint64_t njobs,
                        const int32_t* matrix, int32_t gap_open, int32_t gap_extend,
                        int32_t* scores, int threads, uint64_t* cells_out) {
    batch_ctx c;
    c.residues = residues; c.qcodes = qcodes; c.qoffs = qoffs; c.qbias = qbias;
    c.jobs = jobs; c.njobs = njobs; c.scores = scores;
    c.sc.matrix = matrix; c.sc.gap_open = gap_open; c.sc.gap_extend = gap_extend;
    c.next = 0; c.cells = 0;
    if (threads < 1) threads = 1;
    if (threads > 512) threads = 512;
    pthread_t tid[512];
    int started = 0;
    for (int t = 1; t < threads; t++) {
        if (pthread_create(&tid[t], NULL, batch_worker, &c) == 0) started = t;
        else break;
    }
    batch_worker(&c);
    for (int t = 1; t <= started; t++) pthread_join(tid[t], NULL);
    if (cells_out) *cells_out = c.cells;
    return 0;
}

/* ======================================================================== */
/* scan schedule                                                             */
/* ======================================================================== */
#include <math.h>

#define NONSEED 0x7F
#define MASKED 0x80

uint64_t orc_auto_occ_cap(uint64_t total, uint64_t ncodes, uint64_t db_residues, uint64_t ref_residues) {
    /* index.rs:329-336 */
    uint64_t floor_ = 256;
    if (ref_residues > 0 && db_residues > ref_residues)
        floor_ = (uint64_t)ceil(256.0 * (double)db_residues / (double)ref_residues);
    uint64_t c = (uint64_t)ceil((double)total / (double)(ncodes > 0 ? ncodes : 1) * 64.0);
    return c > floor_ ? c : floor_;
}

typedef struct { uint32_t code; uint32_t q; uint32_t p; } seed_t;
typedef struct { uint32_t subject, query, qp, sp, shape; } surv_t;
typedef struct { int64_t diag; uint32_t q_lo, q_hi; int32_t score; } hsp_t;

static int cmp_seed(const void* a, const void* b) {
    const seed_t* x = (const seed_t*)a; const seed_t* y = (const seed_t*)b;
    if (x->code != y->code) return x->code < y->code ? -1 : 1;
    if (x->q != y->q) return x->q < y->q ? -1 : 1;
    return x->p < y->p ? -1 : (x->p > y->p);
}
/* (subject, query) groups in order; within a pair (qp, shape, sp):
 * scan.rs:2158-2170 (survivors in (shape, position) order, stable by position) */
static int cmp_surv(const void* a, const void* b) {
    const surv_t* x = (const surv_t*)a; const surv_t* y = (const surv_t*)b;
    if (x->subject != y->subject) return x->subject < y->subject ? -1 : 1;
    if (x->query != y->query) return x->query < y->query ? -1 : 1;
    if (x->qp != y->qp) return x->qp < y->qp ? -1 : 1;
    if (x->shape != y->shape) return x->shape < y->shape ? -1 : 1;
    return x->sp < y->sp ? -1 : (x->sp > y->sp);
}
static int cmp_hsp(const void* a, const void* b) {
    const hsp_t* x = (const hsp_t*)a; const hsp_t* y = (const hsp_t*)b;
    return x->diag < y->diag ? -1 : (x->diag > y->diag);
}
/* region_order, engine.rs:493-495 (within one query) */
static int cmp_region(const void* a, const void* b) {
    const orc_region* x = (const orc_region*)a; const orc_region* y = (const orc_region*)b;
    if (x->query != y->query) return x->query < y->query ? -1 : 1;
    if (x->best != y->best) return x->best > y->best ? -1 : 1;
    if (x->subject != y->subject) return x->subject < y->subject ? -1 : 1;
    if (x->d_min != y->d_min) return x->d_min < y->d_min ? -1 : 1;
    return x->d_max < y->d_max ? -1 : (x->d_max > y->d_max);
}

/* seed code of the care positions (scan.rs:841-856): -1 when invalid */
static int64_t code_at(const uint8_t* sr, const uint16_t* offs, uint32_t w, uint32_t asize) {
    uint32_t c = 0;
    for (uint32_t i = 0; i < w; i++) {
        uint8_t r = sr[offs[i]];
        if (r >= asize) return -1;
        c = c * asize + r;
    }
    return c;
}

/* Work split of the scan oracle over host threads.  Subjects (counting and
 * hit passes) and (subject, query) pairs (the visit) are independent units;
 * per-thread outputs are merged and put in the total orders the sequential
 * statement uses (cmp_surv, cmp_region), so the result does not depend on
 * the thread count. */
typedef struct {
    void (*fn)(void* ctx, uint64_t b, uint64_t e, int tid);
    void* ctx;
    uint64_t n, chunk, next;
    int tid_next;
} par_ctx;

static void* par_worker(void* arg) {
    par_ctx* p = (par_ctx*)arg;
    int tid = __atomic_fetch_add(&p->tid_next, 1, __ATOMIC_RELAXED);
    for (;;) {
        uint64_t b = __atomic_fetch_add(&p->next, p->chunk, __ATOMIC_RELAXED);
        if (b >= p->n) break;
        uint64_t e = b + p->chunk < p->n ? b + p->chunk : p->n;
        p->fn(p->ctx, b, e, tid);
    }
    return NULL;
}

static void par_for(uint64_t n, uint64_t chunk, int threads, void (*fn)(void*, uint64_t, uint64_t, int), void* ctx) {
    par_ctx p = {fn, ctx, n, chunk ? chunk : 1, 0, 0};
    pthread_t tid[256];
    int started = 0;
    for (int t = 1; t < threads && t < 256; t++) {
        if (pthread_create(&tid[started], NULL, par_worker, &p) != 0) break;
        started++;
    }
    par_worker(&p);
    for (int t = 0; t < started; t++) pthread_join(tid[t], NULL);
}

typedef struct {
    surv_t* v;
    size_t n, cap;
    orc_scan_counters c;
    orc_region* r;
    size_t nr, rcap;
} scan_local;

typedef struct {
    const uint8_t* res; const uint64_t* soffs; const uint8_t* sb;
    const uint8_t* qred; const uint8_t* qfull; const uint8_t* qcodes; const uint64_t* qoffs;
    const int8_t* qbias; const int32_t* region_thr; const int32_t* matrix;
    const orc_scan_params* P;
    uint32_t span, w, asize;
    const uint16_t* offs;
    int64_t cfil;
    uint32_t* cnt;       /* code counts of the counting pass (atomic adds) */
    uint64_t total;      /* valid positions of the counting pass (atomic add) */
    const seed_t* seeds; /* batch seeds of the shape, code order */
    size_t nseed;
    uint32_t shape;
    const surv_t* sv;    /* sorted survivors (visit pass) */
    const size_t* grp;   /* (subject, query) group starts, ngrp + 1 entries */
    scan_local* loc;
} scan_ctx;

/* frequent codes: counts of the database's valid codes (scan.rs:1184-1238) */
static void scan_count(void* vc, uint64_t b0, uint64_t e0, int tid) {
    scan_ctx* c = (scan_ctx*)vc;
    uint64_t total = 0;
    for (uint64_t s = b0; s < e0; s++) {
        uint64_t b = c->soffs[s], e = c->soffs[s + 1];
        if (e - b < c->span) continue;
        for (uint64_t p = b; p + c->span <= e; p++) {
            int64_t code = code_at(c->sb + p, c->offs, c->w, c->asize);
            if (code >= 0) { __atomic_fetch_add(&c->cnt[code], 1u, __ATOMIC_RELAXED); total++; }
        }
    }
    __atomic_fetch_add(&c->total, total, __ATOMIC_RELAXED);
}

/* database positions: hits and window filter (scan.rs:1603-1856) */
static void scan_hits(void* vc, uint64_t b0, uint64_t e0, int tid) {
    scan_ctx* c = (scan_ctx*)vc;
    scan_local* L = &c->loc[tid];
    const orc_scan_params* P = c->P;
    for (uint64_t s = b0; s < e0; s++) {
        uint64_t b = c->soffs[s], e = c->soffs[s + 1];
        const int64_t sl = (int64_t)(e - b);
        if ((uint64_t)sl < c->span) continue;
        for (int64_t p = 0; p + (int64_t)c->span <= sl; p++) {
            int64_t code = code_at(c->sb + b + p, c->offs, c->w, c->asize);
            if (code < 0) continue;
            /* entries of the code */
            size_t lo = 0, hi = c->nseed;
            while (lo < hi) { size_t mid = (lo + hi) / 2; if (c->seeds[mid].code < (uint32_t)code) lo = mid + 1; else hi = mid; }
            for (size_t k = lo; k < c->nseed && c->seeds[k].code == (uint32_t)code; k++) {
                const uint32_t q = c->seeds[k].q, qp = c->seeds[k].p;
                L->c.hits++;
                if (P->hit_filter_min_ids > 0) {
                    const int64_t ss = p + c->cfil - 16;
                    const int64_t qs = (int64_t)qp + c->cfil - 16;
                    const int64_t qlen = (int64_t)(c->qoffs[q + 1] - c->qoffs[q]);
                    uint32_t r = 0, ex = 0;
                    for (int t = 0; t < 32; t++) {
                        int64_t j = ss + t, i = qs + t;
                        if (j < 0 || j >= sl) continue;
                        if (i < 0 || i >= qlen) continue;
                        uint8_t qr = c->qred[c->qoffs[q] + i];
                        if (qr != 0xFE && qr == (c->sb[b + j] & 0x7F)) {
                            r++;
                            if (P->hit_filter_exact_weight > 0 && c->qfull[c->qoffs[q] + i] == c->res[b + j]) ex++;
                        }
                    }
                    if (r + P->hit_filter_exact_weight * ex < P->hit_filter_min_ids) {
                        L->c.hits_filtered++;
                        continue;
                    }
                }
                if (L->n == L->cap) { L->cap = L->cap ? 2 * L->cap : 1024; L->v = (surv_t*)realloc(L->v, L->cap * sizeof(surv_t)); }
                surv_t* o = &L->v[L->n++];
                o->subject = (uint32_t)s; o->query = q; o->qp = qp; o->sp = (uint32_t)p; o->shape = c->shape;
            }
        }
    }
}

static void push_region(scan_local* L, orc_region r) {
    if (L->nr == L->rcap) { L->rcap = L->rcap ? 2 * L->rcap : 1024; L->r = (orc_region*)realloc(L->r, L->rcap * sizeof(orc_region)); }
    L->r[L->nr++] = r;
}

/* one (subject, query) pair: coverage + X-drop -> HSPs -> regions
 * (visit_chunk_inner / visit_scan / finish_subject_into, scan.rs:2084-2474) */
static void scan_visit(void* vc, uint64_t g0, uint64_t g1, int tid) {
    scan_ctx* c = (scan_ctx*)vc;
    scan_local* L = &c->loc[tid];
    const orc_scan_params* P = c->P;
    const int32_t* matrix = c->matrix;
    const surv_t* sv = c->sv;
    for (uint64_t g = g0; g < g1; g++) {
        const size_t i = c->grp[g], j = c->grp[g + 1];
        const uint32_t q = sv[i].query, s = sv[i].subject;
        const uint8_t* qc = c->qcodes + c->qoffs[q];
        const int8_t* qb = c->qbias ? c->qbias + c->qoffs[q] : NULL;
        const uint64_t qlen = c->qoffs[q + 1] - c->qoffs[q];
        const uint8_t* sc = c->res + c->soffs[s];
        const uint64_t sl = c->soffs[s + 1] - c->soffs[s];
        uint32_t* cover = (uint32_t*)calloc(qlen + sl + 1, sizeof(uint32_t));
        size_t nh = 0;
        hsp_t* hs = (hsp_t*)malloc((j - i) * sizeof(hsp_t));
        for (size_t k = i; k < j; k++) {
            const uint32_t qp = sv[k].qp, sp = sv[k].sp;
            const int64_t d = (int64_t)sp - (int64_t)qp;
            const size_t di = (size_t)(d + (int64_t)qlen);
            if (qp < cover[di]) { L->c.extensions_avoided++; continue; }
            L->c.ungapped_extensions++;
            uint64_t lo, hi;
            int32_t score = orc_ungapped_xdrop(qc, qlen, sc, sl, qp, sp, matrix, qb, P->x_drop, &lo, &hi);
            {
                /* steps of xdrop_cat (scan.rs:904): right steps + left steps */
                uint64_t nrt = qlen - qp < sl - sp ? qlen - qp : sl - sp;
                uint64_t nlt = qp < sp ? qp : sp;
                int32_t best = 0, cur = 0; uint64_t tr = 0;
                while (tr < nrt) {
                    cur += matrix[(qc[qp + tr] < 24 ? qc[qp + tr] : 22) * 24 + (sc[sp + tr] < 24 ? sc[sp + tr] : 22)] + (qb ? qb[qp + tr] : 0);
                    tr++;
                    if (cur > best) best = cur;
                    if (cur < best - P->x_drop) break;
                }
                int32_t bl = 0, cl = 0; uint64_t tl = 1;
                if (nlt > 0) {
                    for (;;) {
                        cl += matrix[(qc[qp - tl] < 24 ? qc[qp - tl] : 22) * 24 + (sc[sp - tl] < 24 ? sc[sp - tl] : 22)] + (qb ? qb[qp - tl] : 0);
                        if (cl > bl) bl = cl;
                        tl++;
                        if (!(tl <= nlt && cl >= bl - P->x_drop)) break;
                    }
                }
                L->c.xdrop_steps += tr + tl - 1;
            }
            cover[di] = (uint32_t)hi;
            if (score >= P->hsp_threshold) {
                hs[nh].diag = d; hs[nh].q_lo = (uint32_t)lo; hs[nh].q_hi = (uint32_t)hi; hs[nh].score = score;
                nh++;
            }
        }
        free(cover);
        if (nh) {
            /* finish_subject_into (scan.rs:2437-2474) */
            L->c.hsps += nh;
            qsort(hs, nh, sizeof(hsp_t), cmp_hsp);
            const int64_t join = 2 * (int64_t)P->window_slack;
            orc_region* rg = (orc_region*)malloc(nh * sizeof(orc_region));
            uint32_t* ev_n = (uint32_t*)malloc(nh * sizeof(uint32_t));
            int32_t* ev_s = (int32_t*)malloc(nh * sizeof(int32_t));
            size_t ng = 0;
            for (size_t k = 0; k < nh; k++) {
                if (ng > 0 && hs[k].diag - rg[ng - 1].d_max <= join) {
                    if (hs[k].diag > rg[ng - 1].d_max) rg[ng - 1].d_max = (int32_t)hs[k].diag;
                    if (hs[k].score > rg[ng - 1].best) rg[ng - 1].best = hs[k].score;
                    ev_n[ng - 1]++;
                    int64_t sum = (int64_t)ev_s[ng - 1] + hs[k].score;
                    ev_s[ng - 1] = sum > INT32_MAX ? INT32_MAX : (sum < INT32_MIN ? INT32_MIN : (int32_t)sum);
                } else {
                    rg[ng].query = q; rg[ng].subject = s;
                    rg[ng].d_min = rg[ng].d_max = (int32_t)hs[k].diag; rg[ng].best = hs[k].score;
                    ev_n[ng] = 1; ev_s[ng] = hs[k].score;
                    ng++;
                }
            }
            const int32_t thr = c->region_thr ? c->region_thr[q] : P->hsp_threshold;
            size_t kept = ng;
            if (thr > P->hsp_threshold) {
                kept = 0;
                for (size_t k = 0; k < ng; k++)
                    if (rg[k].best >= thr || (ev_n[k] >= 2 && ev_s[k] >= thr)) rg[kept++] = rg[k];
                L->c.regions_weak_dropped += ng - kept;
            }
            /* sort by (best desc, d_min asc), keep max_regions_per_subject */
            for (size_t a = 1; a < kept; a++) {
                orc_region x = rg[a];
                size_t b2 = a;
                while (b2 > 0 && (rg[b2 - 1].best < x.best || (rg[b2 - 1].best == x.best && rg[b2 - 1].d_min > x.d_min))) {
                    rg[b2] = rg[b2 - 1];
                    b2--;
                }
                rg[b2] = x;
            }
            size_t keep = kept < P->max_regions_per_subject ? kept : (P->max_regions_per_subject ? P->max_regions_per_subject : 1);
            if (keep > kept) keep = kept;
            for (size_t k = 0; k < keep; k++) push_region(L, rg[k]);
            free(rg); free(ev_n); free(ev_s);
        }
        free(hs);
    }
}

static void add_counters(orc_scan_counters* a, const orc_scan_counters* b) {
    a->seed_positions += b->seed_positions; a->seeds_frequent_skipped += b->seeds_frequent_skipped;
    a->hits += b->hits; a->hits_filtered += b->hits_filtered; a->ungapped_extensions += b->ungapped_extensions;
    a->extensions_avoided += b->extensions_avoided; a->xdrop_steps += b->xdrop_steps; a->hsps += b->hsps;
    a->regions += b->regions; a->regions_weak_dropped += b->regions_weak_dropped;
    a->regions_dropped_by_cap += b->regions_dropped_by_cap;
}

int64_t orc_scan_regions(const uint8_t* res, const uint64_t* soffs, uint64_t nsub, const uint8_t* db_mask,
                         const uint8_t* qcodes, const uint64_t* qoffs, uint32_t nq, const int8_t* qbias,
                         const uint8_t* q_mask, const int32_t* region_thr, const int32_t* matrix,
                         const orc_scan_params* P, orc_region* out, uint64_t out_cap,
                         orc_scan_counters* ctr) {
    return orc_scan_regions_mt(res, soffs, nsub, db_mask, qcodes, qoffs, nq, qbias, q_mask, region_thr, matrix, P,
                               out, out_cap, ctr, 1);
}

int64_t orc_scan_regions_mt(const uint8_t* res, const uint64_t* soffs, uint64_t nsub, const uint8_t* db_mask,
                            const uint8_t* qcodes, const uint64_t* qoffs, uint32_t nq, const int8_t* qbias,
                            const uint8_t* q_mask, const int32_t* region_thr, const int32_t* matrix,
                            const orc_scan_params* P, orc_region* out, uint64_t out_cap,
                            orc_scan_counters* ctr, int threads) {
    memset(ctr, 0, sizeof(*ctr));
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    const uint64_t N = soffs[nsub];
    const uint32_t asize = P->alpha_size;
    /* database seed bytes (scan.rs:123-141, seed_map at 1072-1077) */
    uint8_t* sb = (uint8_t*)malloc(N + 1);
    for (uint64_t r = 0; r < N; r++) {
        uint8_t c = res[r];
        uint8_t v = (c < 24 && P->alpha_map[c] != 255) ? P->alpha_map[c] : NONSEED;
        if (v != NONSEED && db_mask && db_mask[r]) v |= MASKED;
        sb[r] = v;
    }
    /* query reduced bytes and window bytes (build_batch, scan.rs:1514-1530) */
    const uint64_t QN = qoffs[nq];
    uint8_t* qred = (uint8_t*)malloc(QN + 1); /* reduced letter or 0xFE */
    uint8_t* qfull = (uint8_t*)malloc(QN + 1); /* alignment code or 0xFE */
    for (uint64_t i = 0; i < QN; i++) {
        uint8_t c = qcodes[i];
        uint8_t r = P->alpha_map[c < 24 ? c : 23];
        int ok = !(q_mask && q_mask[i]) && r != 255;
        qred[i] = ok ? r : 0xFE;
        qfull[i] = ok ? c : 0xFE;
    }
    uint32_t cmin = 1u << 30;
    for (uint32_t s = 0; s < P->nshapes; s++) if (P->shape_span[s] < cmin) cmin = P->shape_span[s];

    scan_local* loc = (scan_local*)calloc((size_t)threads, sizeof(scan_local));
    scan_ctx cx;
    memset(&cx, 0, sizeof(cx));
    cx.res = res; cx.soffs = soffs; cx.sb = sb; cx.qred = qred; cx.qfull = qfull; cx.qcodes = qcodes;
    cx.qoffs = qoffs; cx.qbias = qbias; cx.region_thr = region_thr; cx.matrix = matrix; cx.P = P;
    cx.asize = asize; cx.cfil = cmin / 2; cx.loc = loc;
    const uint64_t sub_chunk = 256;
    for (uint32_t si = 0; si < P->nshapes; si++) {
        const uint32_t span = P->shape_span[si], w = P->shape_weight[si];
        const uint16_t* offs = P->shape_off[si];
        uint64_t ncodes = 1;
        for (uint32_t k = 0; k < w; k++) ncodes *= asize;
        cx.span = span; cx.w = w; cx.offs = offs; cx.shape = si;
        /* frequent codes (scan.rs:1184-1238) */
        cx.cnt = (uint32_t*)calloc(ncodes, sizeof(uint32_t));
        cx.total = 0;
        par_for(nsub, sub_chunk, threads, scan_count, &cx);
        uint64_t cap = P->seed_max_occ > 0 ? P->seed_max_occ
                                           : orc_auto_occ_cap(cx.total, ncodes, P->db_length, P->ref_db_residues);
        uint8_t* freq = (uint8_t*)calloc(ncodes, 1);
        if (cx.total > cap)
            for (uint64_t c = 0; c < ncodes; c++) freq[c] = cx.cnt[c] > cap;
        free(cx.cnt);
        cx.cnt = NULL;
        /* query seeds (scan.rs:1541-1562) */
        size_t nseed = 0, seed_cap = 1024;
        seed_t* seeds = (seed_t*)malloc(seed_cap * sizeof(seed_t));
        for (uint32_t q = 0; q < nq; q++) {
            uint64_t b = qoffs[q], e = qoffs[q + 1];
            if (e - b < span) continue;
            for (uint64_t p = b; p + span <= e; p++) {
                int64_t c = code_at(qred + p, offs, w, asize);
                if (c < 0) continue;
                if (freq[c]) { ctr->seeds_frequent_skipped++; continue; }
                if (nseed == seed_cap) { seed_cap *= 2; seeds = (seed_t*)realloc(seeds, seed_cap * sizeof(seed_t)); }
                seeds[nseed].code = (uint32_t)c; seeds[nseed].q = q; seeds[nseed].p = (uint32_t)(p - b);
                nseed++;
            }
        }
        free(freq);
        ctr->seed_positions += nseed;
        qsort(seeds, nseed, sizeof(seed_t), cmp_seed);
        cx.seeds = seeds;
        cx.nseed = nseed;
        if (nseed) par_for(nsub, sub_chunk, threads, scan_hits, &cx);
        free(seeds);
    }
    free(sb);
    /* survivors of all threads, in the (subject, query, qp, shape, sp) order */
    size_t ns = 0;
    for (int t = 0; t < threads; t++) ns += loc[t].n;
    surv_t* sv = (surv_t*)malloc((ns ? ns : 1) * sizeof(surv_t));
    {
        size_t o = 0;
        for (int t = 0; t < threads; t++) {
            if (loc[t].n) memcpy(sv + o, loc[t].v, loc[t].n * sizeof(surv_t));
            o += loc[t].n;
            free(loc[t].v);
            loc[t].v = NULL;
        }
    }
    qsort(sv, ns, sizeof(surv_t), cmp_surv);
    /* (subject, query) groups, visited on all threads */
    size_t ngrp = 0;
    size_t* grp = (size_t*)malloc((ns + 1) * sizeof(size_t));
    for (size_t i = 0; i < ns;) {
        size_t j = i + 1;
        while (j < ns && sv[j].subject == sv[i].subject && sv[j].query == sv[i].query) j++;
        grp[ngrp++] = i;
        i = j;
    }
    grp[ngrp] = ns;
    cx.sv = sv;
    cx.grp = grp;
    par_for(ngrp, 64, threads, scan_visit, &cx);
    free(sv);
    free(grp);
    free(qred);
    free(qfull);
    size_t nr = 0;
    for (int t = 0; t < threads; t++) { nr += loc[t].nr; add_counters(ctr, &loc[t].c); }
    orc_region* regs_all = (orc_region*)malloc((nr ? nr : 1) * sizeof(orc_region));
    {
        size_t o = 0;
        for (int t = 0; t < threads; t++) {
            if (loc[t].nr) memcpy(regs_all + o, loc[t].r, loc[t].nr * sizeof(orc_region));
            o += loc[t].nr;
            free(loc[t].r);
        }
    }
    free(loc);
    /* per query: region_order, cap at max_candidates */
    qsort(regs_all, nr, sizeof(orc_region), cmp_region);
    uint64_t w = 0;
    size_t a = 0;
    const uint64_t cap = P->max_candidates ? P->max_candidates : 1;
    while (a < nr) {
        size_t b2 = a;
        while (b2 < nr && regs_all[b2].query == regs_all[a].query) b2++;
        size_t take = (b2 - a) > cap ? cap : (b2 - a);
        ctr->regions_dropped_by_cap += (b2 - a) - take;
        for (size_t k = 0; k < take; k++) {
            if (w >= out_cap) { free(regs_all); return -1; }
            out[w++] = regs_all[a + k];
        }
        a = b2;
    }
    ctr->regions = w;
    free(regs_all);
    return (int64_t)w;
}
