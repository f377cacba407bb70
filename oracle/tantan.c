/*
 * CPU oracle of tantan seed masking — TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Restates the reference's scalar masker, masking.rs (SABER 1.4.0):
 *   - the model tables of Tantan::with_params (masking.rs:162-179),
 *   - implied_lambda / invert20 (masking.rs:531-612),
 *   - the scaled forward-backward of compute_body (masking.rs:429-529) with
 *     sum8 / dot8's eight accumulators and combination tree
 *     (masking.rs:121-152),
 *   - the >= min_prob mask of Tantan::mask (masking.rs:191-196).
 * Built with -ffp-contract=off: every f32 / f64 operation rounds on its own,
 * as Rust evaluates them (no fused multiply-add).
 *
 * Pinning: implied_lambda of BLOSUM62 reproduces the value the reference
 * publishes (0.32403216734804396, bench/results/v1.2.0/masking_f32_vs_f64.txt);
 * the posteriors are checked against the reference's masking tests
 * (masking.rs:640-706: poly-Q masked, diverse head not, probabilities in
 * [0, 1]) and its CLI test (tests/cli.rs:118-133: > 900 of the 980 repeat
 * residues masked).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* Integer power by binary exponentiation, as Rust's f64::powi lowers to
 * (LLVM's powi: multiply by the running square for every set bit). */
static double powi_bin(double a, int b) {
    int recip = b < 0;
    if (recip) b = -b;
    double r = 1.0;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return recip ? 1.0 / r : r;
}

/* masking.rs:586-612: Gauss-Jordan inverse with partial pivoting.  Returns 0
 * when a pivot is below 1e-300. */
static int invert20(double a[20][20], double inv[20][20]) {
    for (int i = 0; i < 20; i++)
        for (int j = 0; j < 20; j++) inv[i][j] = i == j ? 1.0 : 0.0;
    for (int col = 0; col < 20; col++) {
        int piv = col;
        for (int r = col + 1; r < 20; r++)
            if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
        if (fabs(a[piv][col]) < 1e-300) return 0;
        if (piv != col) {
            for (int j = 0; j < 20; j++) {
                double t = a[col][j];
                a[col][j] = a[piv][j];
                a[piv][j] = t;
                t = inv[col][j];
                inv[col][j] = inv[piv][j];
                inv[piv][j] = t;
            }
        }
        double d = a[col][col];
        for (int j = 0; j < 20; j++) {
            a[col][j] /= d;
            inv[col][j] /= d;
        }
        for (int r = 0; r < 20; r++) {
            if (r == col) continue;
            double f = a[r][col];
            if (f != 0.0) {
                for (int j = 0; j < 20; j++) {
                    a[r][j] -= f * a[col][j];
                    inv[r][j] -= f * inv[col][j];
                }
            }
        }
    }
    return 1;
}

/* masking.rs:535-553: (sum of the entries of (e^{lambda S})^-1) - 1 over the
 * 20 standard letters, and whether every row and column sum is positive.
 * Returns 0 when the matrix is singular. */
static int lambda_f(const int32_t* m, double l, double* v, int* positive) {
    double a[20][20], inv[20][20];
    for (int i = 0; i < 20; i++)
        for (int j = 0; j < 20; j++) a[i][j] = exp(l * (double)m[i * 24 + j]);
    if (!invert20(a, inv)) return 0;
    double total = 0.0;
    int pos = 1;
    for (int i = 0; i < 20; i++) {
        double rs = 0.0, cs = 0.0;
        for (int k = 0; k < 20; k++) rs += inv[i][k];
        for (int k = 0; k < 20; k++) cs += inv[k][i];
        if (rs <= 0.0 || cs <= 0.0) pos = 0;
        total += rs;
    }
    *v = total - 1.0;
    *positive = pos;
    return 1;
}

/* masking.rs:531-583: scan lambda = 0.02, 0.03, ... < 3 for a sign change of
 * lambda_f, bisect it 80 times, accept the root if its implied frequencies are
 * positive.  Returns NAN when no root is found. */
double orc_tantan_lambda(const int32_t* matrix576) {
    int have_prev = 0;
    double pl = 0.0, pv = 0.0;
    for (double l = 0.02; l < 3.0; l += 0.01) {
        double v;
        int pos;
        if (!lambda_f(matrix576, l, &v, &pos)) continue;
        if (have_prev && ((pv > 0.0) != (v > 0.0))) {
            double lo = pl, hi = l, vlo = pv;
            for (int it = 0; it < 80; it++) {
                double mid = 0.5 * (lo + hi), vm;
                int pm;
                if (!lambda_f(matrix576, mid, &vm, &pm)) return NAN;
                if ((vm > 0.0) == (vlo > 0.0)) {
                    lo = mid;
                    vlo = vm;
                } else {
                    hi = mid;
                }
            }
            double root = 0.5 * (lo + hi), vr;
            int pr;
            if (lambda_f(matrix576, root, &vr, &pr) && pr) return root;
        }
        have_prev = 1;
        pl = l;
        pv = v;
    }
    return NAN;
}

/* masking.rs:162-179: lr[a][b] = (f32) exp(lambda * S(a, b)) for a, b < 24
 * (columns 24..31 zero), b2f[i] = (f32) (r * first * d^i) with
 * first = (1 - d) / (1 - d^W) (1 / W when d == 1).  lambda <= 0 or NaN
 * derives it from the matrix (0.3176 when no root exists).  Returns the
 * lambda used. */
double orc_tantan_tables(const int32_t* matrix576, const orc_tantan_params* p, double lambda, float* lr768,
                         float* b2f) {
    if (!(lambda > 0.0)) {
        lambda = orc_tantan_lambda(matrix576);
        if (isnan(lambda)) lambda = 0.3176;
    }
    for (int a = 0; a < 24; a++)
        for (int b = 0; b < 32; b++)
            lr768[a * 32 + b] = b < 24 ? (float)exp(lambda * (double)matrix576[a * 24 + b]) : 0.0f;
    int w = p->max_period > 0 ? (int)p->max_period : 1;
    double first = fabs(p->decay - 1.0) < 1e-12 ? 1.0 / (double)w
                                                : (1.0 - p->decay) / (1.0 - powi_bin(p->decay, w));
    for (int i = 0; i < w; i++) b2f[i] = (float)(p->repeat_start * first * powi_bin(p->decay, i));
    return lambda;
}

/* masking.rs:121-138 */
static float sum8(const float* v, int n) {
    float a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int c = n / 8;
    for (int j = 0; j < c; j++)
        for (int k = 0; k < 8; k++) a[k] += v[8 * j + k];
    float t = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    for (int i = 8 * c; i < n; i++) t += v[i];
    return t;
}

/* masking.rs:139-152 */
static float dot8(const float* x, const float* y, int n) {
    float a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int c = n / 8;
    for (int j = 0; j < c; j++)
        for (int k = 0; k < 8; k++) a[k] += x[8 * j + k] * y[8 * j + k];
    float t = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
    for (int i = 8 * c; i < n; i++) t += x[i] * y[i];
    return t;
}

/* masking.rs:429-529: posterior repeat probability of every position of one
 * sequence (codes clamped to 23).  lr768 / b2f from orc_tantan_tables. */
int orc_tantan_probs(const uint8_t* seq, size_t n, const float* lr768, const float* b2f, const orc_tantan_params* p,
                     float* post) {
    if (n == 0) return 0;
    int w = p->max_period > 0 ? (int)p->max_period : 1;
    int ns = w + 1;
    float b2b = (float)(1.0 - p->repeat_start);
    float f2f = (float)(1.0 - p->repeat_end);
    float f2b = (float)p->repeat_end;
    uint8_t* codes = (uint8_t*)malloc(n);
    float* emit = (float*)malloc(n * (size_t)w * sizeof(float));
    float* fwd = (float*)malloc(n * (size_t)ns * sizeof(float));
    float* scale = (float*)malloc(n * sizeof(float));
    float* vec = (float*)malloc(5 * (size_t)w * sizeof(float));
    if (!codes || !emit || !fwd || !scale || !vec) {
        free(codes), free(emit), free(fwd), free(scale), free(vec);
        return -1;
    }
    for (size_t i = 0; i < n; i++) codes[i] = seq[i] < 23 ? seq[i] : 23;
    for (size_t q = 0; q < n; q++) {
        const float* row = lr768 + 32 * codes[q];
        size_t maxi = q < (size_t)w ? q : (size_t)w;
        for (size_t i = 0; i < (size_t)w; i++) emit[q * w + i] = i < maxi ? row[codes[q - 1 - i]] : 0.0f;
    }
    float* prev_f = vec;
    float* cur_f = vec + w;
    memset(prev_f, 0, (size_t)w * sizeof(float));
    float prev_b = 1.0f;
    for (size_t q = 0; q < n; q++) {
        const float* e = emit + q * w;
        float sum_f = sum8(prev_f, w);
        float cur_b = prev_b * b2b + sum_f * f2b;
        for (int i = 0; i < w; i++) cur_f[i] = (prev_b * b2f[i] + prev_f[i] * f2f) * e[i];
        float tot = cur_b + sum8(cur_f, w);
        float s = tot > 0.0f ? 1.0f / tot : 1.0f;
        scale[q] = s;
        float* row = fwd + q * ns;
        row[0] = cur_b * s;
        for (int i = 0; i < w; i++) row[1 + i] = cur_f[i] * s;
        prev_b = row[0];
        memcpy(prev_f, row + 1, (size_t)w * sizeof(float));
    }
    float* nf = vec + 2 * w;
    float* nnf = vec + 3 * w;
    float* be = vec + 4 * w;
    for (int i = 0; i < w; i++) nf[i] = f2b;
    float nb = 1.0f;
    for (size_t q = n; q-- > 0;) {
        const float* row = fwd + q * ns;
        float pb = row[0] * nb;
        float pf = dot8(row + 1, nf, w);
        float z = pb + pf;
        post[q] = z > 0.0f ? pf / z : 0.0f;
        if (q == 0) break;
        const float* e = emit + q * w;
        float s = scale[q];
        for (int i = 0; i < w; i++) be[i] = e[i] * nf[i];
        float to_fg = dot8(b2f, be, w);
        float fb = f2b * nb;
        for (int i = 0; i < w; i++) nnf[i] = (f2f * be[i] + fb) * s;
        nb = (b2b * nb + to_fg) * s;
        float* t = nf;
        nf = nnf;
        nnf = t;
    }
    free(codes), free(emit), free(fwd), free(scale), free(vec);
    return 0;
}

/* masking.rs:191-196 over a batch of sequences (offsets[nseq + 1]): mask[i] =
 * (f64) post[i] >= min_prob; probs (optional) receives the posteriors.
 * Returns the number of masked positions, or -1 on allocation failure. */
int64_t orc_tantan_mask(const uint8_t* codes, const uint64_t* offsets, uint64_t nseq, const int32_t* matrix576,
                        const orc_tantan_params* p, double lambda, uint8_t* mask, float* probs) {
    int w = p->max_period > 0 ? (int)p->max_period : 1;
    float lr[24 * 32];
    float* b2f = (float*)malloc((size_t)w * sizeof(float));
    if (!b2f) return -1;
    orc_tantan_tables(matrix576, p, lambda, lr, b2f);
    int64_t masked = 0;
    size_t maxn = 0;
    for (uint64_t s = 0; s < nseq; s++)
        if (offsets[s + 1] - offsets[s] > maxn) maxn = offsets[s + 1] - offsets[s];
    float* post = (float*)malloc((maxn ? maxn : 1) * sizeof(float));
    if (!post) {
        free(b2f);
        return -1;
    }
    for (uint64_t s = 0; s < nseq; s++) {
        size_t n = offsets[s + 1] - offsets[s];
        if (orc_tantan_probs(codes + offsets[s], n, lr, b2f, p, post) != 0) {
            masked = -1;
            break;
        }
        for (size_t i = 0; i < n; i++) {
            uint8_t m = (double)post[i] >= p->min_prob;
            mask[offsets[s] + i] = m;
            masked += m;
            if (probs) probs[offsets[s] + i] = post[i];
        }
    }
    free(post);
    free(b2f);
    return masked;
}
