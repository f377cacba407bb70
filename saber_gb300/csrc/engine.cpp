// Host engine of the batch search: Engine::search_scan for one query batch
// (src/search/engine/scan.rs:1261-1497) with the shared Engine stages of
// src/search/engine.rs, over the device stages of this library (scan,
// banded scoring, widening traceback).  The host keeps what the reference
// keeps on its host: query preparation, window plans, the two-stage scoring
// bookkeeping, the f64 Karlin-Altschul statistics (in the operation order of
// src/scoring/stats.rs, glibc libm, no contraction: this file is compiled
// with -ffp-contract=off), finish and make_hit.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <atomic>
#include <limits>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

#include "region_sink.h"

namespace saber {
// Pinned host staging owned by the handle (slot 0..3, grow-only, contents
// not preserved); null when the allocation fails.  saber_gpu.cu
void* pinned_scratch(saber_gpu* h, int slot, size_t bytes);
}  // namespace saber

#include <cuda_runtime.h>  // float4, uint4

#include "saber_gpu.h"

namespace {

constexpr double kRegionFloorEvalue = 10.0;     // engine.rs:518
constexpr int64_t kBandScoreMinCells = 1 << 20;  // engine.rs:401
constexpr int64_t kBandCostRatio = 12;           // engine.rs:402
constexpr int64_t kBandBridge = 1024;            // engine.rs:404
constexpr int64_t kI32Max = 2147483647;
constexpr int64_t kI64Max = std::numeric_limits<int64_t>::max();
const double kLn2 = std::log(2.0);
const double kInf = std::numeric_limits<double>::infinity();

// Robinson & Robinson background frequencies per 1000 (src/scoring/bias.rs:32-53)
constexpr double kRobinson[20] = {78.05, 51.29, 44.87, 53.64, 19.25, 42.64, 62.95, 73.77, 21.99, 51.42,
                                  90.19, 57.44, 22.43, 38.56, 52.03, 71.20, 58.41, 13.30, 32.16, 64.41};

// Runs f(i) for i in [0, n) on the host cores (chunks taken from an atomic
// counter); the per-query stages of the engine are independent.
template <class F>
void parallel_for(size_t n, F f) {
    unsigned hw = std::thread::hardware_concurrency();
    size_t nt = std::min<size_t>(hw ? hw : 1, (n + 7) / 8);
    if (nt <= 1) {
        for (size_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (;;) {
            const size_t b = next.fetch_add(8);
            if (b >= n) return;
            for (size_t i = b; i < std::min(n, b + 8); i++) f(i);
        }
    };
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; t++) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Memo of a pure function of the subject length (per query): direct-mapped,
// so a collision only recomputes.
struct LenMemo {
    // a query's candidate subjects have up to a few thousand distinct lengths
    static constexpr int kSlots = 8192;
    int64_t key[kSlots];
    double val[kSlots];
    LenMemo() {
        for (int i = 0; i < kSlots; i++) key[i] = -1;
    }
    template <class F>
    double get(int64_t n, F f) {
        const int i = (int)(((uint64_t)n * 0x9E3779B97F4A7C15ull) >> 51);
        if (key[i] != n) {
            key[i] = n;
            val[i] = f();
        }
        return val[i];
    }
};

// ---- statistics (src/scoring/stats.rs) ------------------------------------

// BLAST_ComputeLengthAdjustment (stats.rs:458-520)
int64_t length_adjustment(double k, double log_k, double adl, double beta, int64_t query_length, int64_t db_length,
                          int64_t db_num_seqs) {
    const double m = (double)query_length, n = (double)db_length, nn = (double)db_num_seqs;
    double ell_min = 0.0, ell_next = 0.0;
    bool converged = false;
    const double a = nn;
    const double mb = m * nn + n;
    const double c = n * m - std::max(m, n) / k;
    if (c < 0.0) return 0;
    double ell_max = 2.0 * c / (mb + std::sqrt(mb * mb - 4.0 * a * c));
    for (int i = 1; i <= 20; i++) {
        const double ell = ell_next;
        const double ss = (m - ell) * (n - nn * ell);
        const double ell_bar = adl * (log_k + std::log(ss)) + beta;
        if (ell_bar >= ell) {
            ell_min = ell;
            if (ell_bar - ell_min <= 1.0) {
                converged = true;
                break;
            }
            if (ell_min == ell_max) break;
        } else {
            ell_max = ell;
        }
        if (ell_min <= ell_bar && ell_bar <= ell_max) ell_next = ell_bar;
        else ell_next = i == 1 ? ell_max : (ell_min + ell_max) / 2.0;
    }
    if (converged) {
        int64_t adj = (int64_t)ell_min;
        const double ell = std::ceil(ell_min);
        if (ell <= ell_max) {
            const double ss = (m - ell) * (n - nn * ell);
            if (adl * (log_k + std::log(ss)) + beta >= ell) adj = (int64_t)ell;
        }
        return adj;
    }
    return (int64_t)ell_min;
}

struct Karlin {
    double lambda, k, log_k, adl, beta;
    bool even;
};

// QueryStatistics (stats.rs:646-760)
struct QStats {
    Karlin p;
    bool database_model;
    int64_t query_len;
    double num_seqs, search_space;

    double adj_score(int64_t raw) const { return (double)(p.even && raw % 2 != 0 ? raw - 1 : raw); }
    double space_for(int64_t subject_len) const {
        if (database_model) return search_space;
        const int64_t m = std::max<int64_t>(query_len, 1), n = std::max<int64_t>(subject_len, 1);
        int64_t adj = length_adjustment(p.k, p.log_k, p.adl, p.beta, m, n, 1);
        const int64_t min_l = (int64_t)std::ceil(1.0 / p.k);
        adj = std::max<int64_t>(std::min(std::min(adj, std::max<int64_t>(m - min_l, 0)), std::max<int64_t>(n - min_l, 0)),
                                0);
        return num_seqs * (double)std::max<int64_t>(m - adj, 1) * (double)std::max<int64_t>(n - adj, 1);
    }
    double space_lower_bound(int64_t subject_len) const {
        if (database_model) return search_space;
        const double m = (double)std::max<int64_t>(query_len, 1), n = (double)std::max<int64_t>(subject_len, 1);
        const double up = std::ceil(std::max(p.adl * (p.log_k + std::log(m * n)) + p.beta, 0.0));
        return num_seqs * std::max(m - up, 1.0) * std::max(n - up, 1.0);
    }
    double floor_lower_bound(double evalue_cut, bool has_bits, double min_bits, int64_t subject_len,
                             int64_t db_floor) const {
        if (database_model) return (double)db_floor;
        double f = 1.0;
        if (evalue_cut > 0.0 && std::isfinite(evalue_cut))
            f = std::max(f, std::log(p.k * space_lower_bound(subject_len) / evalue_cut) / p.lambda);
        if (has_bits) f = std::max(f, (min_bits * kLn2 + p.log_k) / p.lambda);
        if (p.even) f -= 1.0;
        return f;
    }
    double evalue_in(int64_t raw, double space) const {
        if (raw <= 0) return kInf;
        const double s = adj_score(raw);
        const double e = p.k * space * std::exp(-p.lambda * s);
        return e == 0.0 ? 2.2250738585072014e-308 : e;
    }
    double evalue_for(int64_t raw, int64_t subject_len) const { return evalue_in(raw, space_for(subject_len)); }
    double evalue(int64_t raw) const {
        if (raw <= 0) return kInf;
        const double s = adj_score(raw);
        const double e = p.k * search_space * std::exp(-p.lambda * s);
        return e == 0.0 ? 2.2250738585072014e-308 : e;
    }
    double bitscore(int64_t raw) const {
        if (raw <= 0) return 0.0;
        return (p.lambda * adj_score(raw) - p.log_k) / kLn2;
    }
    bool passes(int64_t s, double ecut, bool has_bits, double bits) const {
        return evalue(s) <= ecut && (!has_bits || bitscore(s) >= bits);
    }
    int64_t min_score(double ecut, bool has_bits, double bits) const {
        double floor = 1.0;
        if (ecut > 0.0 && std::isfinite(ecut)) floor = std::max(floor, std::log((p.k * search_space) / ecut) / p.lambda);
        if (has_bits) floor = std::max(floor, (bits * kLn2 + p.log_k) / p.lambda);
        if (!std::isfinite(floor)) return 1;
        int64_t s = (int64_t)std::max(std::ceil(floor), 1.0);
        while (s > 1 && passes(s - 1, ecut, has_bits, bits)) s--;
        while (!passes(s, ecut, has_bits, bits) && s < kI64Max / 2) s++;
        return s;
    }
};

// SearchStatistics::for_query (stats.rs:581-645)
QStats for_query(const Karlin& kp, bool database_model, int64_t db_length, int64_t db_num_seqs, int64_t qlen) {
    const int64_t dbl = std::max<int64_t>(db_length, 1), dbn = std::max<int64_t>(db_num_seqs, 1);
    const int64_t m = std::max<int64_t>(qlen, 1);
    int64_t adj = length_adjustment(kp.k, kp.log_k, kp.adl, kp.beta, m, dbl, dbn);
    const int64_t min_q = (int64_t)std::ceil(1.0 / kp.k);
    if (m - adj < min_q) adj = std::max<int64_t>(m - min_q, 0);
    const double eff_q = std::max((double)(m - adj), 1.0);
    const double eff_db = std::max((double)dbl - (double)dbn * (double)adj, 1.0);
    QStats q;
    q.p = kp;
    q.database_model = database_model;
    q.query_len = m;
    q.num_seqs = (double)dbn;
    q.search_space = eff_q * eff_db;
    return q;
}

// ---- composition bias (src/scoring/bias.rs:64-122) -------------------------
void composition_bias(const uint8_t* q, int64_t n, const int32_t* mat, int8_t* out) {
    std::fill(out, out + n, (int8_t)0);
    if (n < 2) return;
    double s = 0.0;
    for (int a = 0; a < 20; a++) s += kRobinson[a];
    double p[20], bg[20];
    for (int a = 0; a < 20; a++) p[a] = kRobinson[a] / s;
    for (int r = 0; r < 20; r++) {
        double acc = 0.0;
        for (int a = 0; a < 20; a++) acc += p[a] * (double)mat[r * 24 + a];
        bg[r] = acc;
    }
    // prefix sums of S(r, q_j) for r < 20 (codes >= 24 index column 23)
    std::vector<int64_t> csum((size_t)20 * (n + 1), 0);
    for (int r = 0; r < 20; r++) {
        int64_t* c = &csum[(size_t)r * (n + 1)];
        for (int64_t j = 0; j < n; j++) c[j + 1] = c[j] + mat[r * 24 + std::min<int>(q[j], 23)];
    }
    const int64_t half = 20;
    for (int64_t i = 0; i < n; i++) {
        const int r = q[i];
        if (r >= 20) continue;
        const int64_t hi = std::min(i + half + 1, n), lo = std::max<int64_t>(i - half, 0);
        const int64_t w = hi - lo;
        if (w < 2) continue;
        const int64_t* c = &csum[(size_t)r * (n + 1)];
        const int64_t acc = c[hi] - c[lo];
        const int64_t own = mat[r * 24 + r];
        const double neigh = (double)(acc - own) / (double)(w - 1);
        const double f = bg[r] - neigh;
        const int64_t v = f < 0.0 ? (int64_t)(f - 0.5) : (int64_t)(f + 0.5);
        out[i] = (int8_t)std::max<int64_t>(-127, std::min<int64_t>(127, v));
    }
}

// ---- the batch ----------------------------------------------------------------
struct Region {
    uint32_t subject;
    int64_t dmin, dmax, best;
    uint64_t src;    // index among the scan's regions of the batch
    uint64_t sbase;  // the subject's first residue in the database
    int64_t sl;      // the subject's length
};
struct Plan {
    int64_t lo, hi;
    bool band;
    int64_t blo, bhi;
};
struct Prep {
    QStats qs;
    int64_t floor, region_floor, region_thr;
};
struct Aln {
    bool present = false;
    int32_t status = 0, score = 0;
    uint32_t q_start = 0, q_end = 0, s_start = 0, s_end = 0;
    std::vector<uint32_t> runs;
};
struct HitRec {
    saber_hit h;
    std::vector<uint32_t> runs;
};

inline void band_clip(int64_t& lo, int64_t& hi, int64_t m, int64_t n) {
    lo = std::max(lo, -(m - 1));
    hi = std::min(hi, n - 1);
}
inline bool band_covers(int64_t lo, int64_t hi, int64_t m, int64_t n) { return lo <= -(m - 1) && hi >= n - 1; }
inline int64_t band_width(int64_t lo, int64_t hi) { return std::max<int64_t>(hi - lo + 1, 0); }

struct Engine {
    saber_gpu* h;
    const saber_search_params& P;
    const uint8_t* db;
    const uint64_t* soff;
    uint64_t nsub;
    int32_t mat[576];
    Karlin kp;
    bool has_bits;
    saber_search_stats st{};

    Engine(saber_gpu* h_, const saber_search_params& p, const uint8_t* db_, const uint64_t* soff_, uint64_t nsub_,
           const int32_t* m)
        : h(h_), P(p), db(db_), soff(soff_), nsub(nsub_) {
        std::memcpy(mat, m, sizeof(mat));
        kp.lambda = p.lambda;
        kp.k = p.k;
        kp.log_k = std::log(p.k);
        kp.adl = p.alpha / p.lambda;
        kp.beta = p.beta;
        kp.even = p.even_scores_only != 0;
        has_bits = !std::isnan(p.min_bitscore);
    }

    int64_t slen(uint32_t s) const { return (int64_t)(soff[s + 1] - soff[s]); }

    double region_evalue() const {
        const double e = std::max(P.evalue, kRegionFloorEvalue);
        const double r = (double)P.ref_db_residues;
        const double dbl = (double)std::max<uint64_t>(P.scan.db_length, 1);
        if (P.ref_db_residues > 0 && dbl > r) return e * (dbl / r);
        return e;
    }

    // engine.rs:759-786
    Prep prepare(int64_t qlen) const {
        Prep pr;
        const int64_t nseq = P.stats_num_seqs ? (int64_t)P.stats_num_seqs : (int64_t)nsub;
        pr.qs = for_query(kp, P.evalue_model == 1, (int64_t)P.scan.db_length, nseq, std::max<int64_t>(qlen, 1));
        pr.floor = pr.qs.min_score(P.evalue, has_bits, P.min_bitscore);
        const double re = region_evalue();
        if (re == P.evalue && !has_bits) pr.region_floor = pr.floor;
        else pr.region_floor = pr.qs.min_score(re, false, 0.0);
        const double f = P.hsp_floor_fraction;
        if (f > 0.0 && pr.region_floor > 0) {
            const double v = std::min(std::ceil((double)pr.region_floor * f), (double)kI32Max);
            pr.region_thr = std::max<int64_t>(P.hsp_threshold, (int64_t)v);
        } else {
            pr.region_thr = P.hsp_threshold;
        }
        return pr;
    }

    // engine.rs:1223-1234
    void window(int64_t dmin, int64_t dmax, int64_t sl, int64_t qlen, int64_t& lo, int64_t& hi) const {
        const int64_t slack = P.window_slack;
        lo = std::min(std::max<int64_t>(dmin - slack, 0), sl);
        hi = std::max(std::min(qlen + dmax + slack, sl), lo);
        if ((hi - lo) * 4 >= sl * 3) {
            lo = 0;
            hi = sl;
        }
    }

    // engine.rs:1247-1324
    std::vector<Plan> plan_windows(const std::vector<Region>& regs, int64_t qlen) const {
        const size_t n = regs.size();
        // per-thread work buffers (a query's regions are planned on one thread)
        thread_local std::vector<int64_t> span_lo, span_hi;
        thread_local std::vector<uint32_t> by, tmp;
        thread_local std::vector<size_t> idx;
        span_lo.resize(n);
        span_hi.resize(n);
        for (size_t i = 0; i < n; i++) {
            span_lo[i] = regs[i].dmin;
            span_hi[i] = regs[i].dmax;
        }
        // group by subject, stable (the index breaks ties): 12-bit counting
        // passes over the subject ids, least significant digit first
        by.resize(n);
        tmp.resize(n);
        uint32_t smax = 0;
        for (size_t i = 0; i < n; i++) {
            by[i] = (uint32_t)i;
            smax = std::max(smax, regs[i].subject);
        }
        for (int sh = 0; sh == 0 || (sh < 32 && (smax >> sh) != 0); sh += 12) {
            uint32_t cnt[4097] = {0};
            for (size_t i = 0; i < n; i++) cnt[((regs[by[i]].subject >> sh) & 4095u) + 1]++;
            for (int b = 0; b < 4096; b++) cnt[b + 1] += cnt[b];
            for (size_t i = 0; i < n; i++) tmp[cnt[(regs[by[i]].subject >> sh) & 4095u]++] = by[i];
            std::swap(by, tmp);
        }
        for (size_t a = 0; a < n;) {
            size_t b = a;
            while (b < n && regs[by[b]].subject == regs[by[a]].subject) b++;
            int64_t top = std::numeric_limits<int64_t>::min();
            for (size_t t = a; t < b; t++) top = std::max(top, regs[by[t]].best);
            const int64_t strong = std::max<int64_t>(2 * (int64_t)P.hsp_threshold, top / 4);
            idx.clear();
            for (size_t t = a; t < b; t++)
                if (regs[by[t]].best >= strong) idx.push_back(by[t]);
            std::sort(idx.begin(), idx.end(), [&](size_t x, size_t y) {
                if (regs[x].dmin != regs[y].dmin) return regs[x].dmin < regs[y].dmin;
                if (regs[x].dmax != regs[y].dmax) return regs[x].dmax < regs[y].dmax;
                return x < y;
            });
            size_t start = 0;
            while (start < idx.size()) {
                int64_t lo = regs[idx[start]].dmin, hi = regs[idx[start]].dmax;
                size_t end = start + 1;
                while (end < idx.size() && regs[idx[end]].dmin - hi <= kBandBridge) {
                    hi = std::max(hi, regs[idx[end]].dmax);
                    end++;
                }
                for (size_t t = start; t < end; t++) {
                    span_lo[idx[t]] = lo;
                    span_hi[idx[t]] = hi;
                }
                start = end;
            }
            a = b;
        }
        std::vector<Plan> plans(n);
        for (size_t ri = 0; ri < n; ri++) {
            const Region& r = regs[ri];
            int64_t lo, hi;
            window(r.dmin, r.dmax, r.sl, qlen, lo, hi);
            Plan own{lo, hi, false, 0, 0};
            if (P.exhaustive || r.best == 0 || (int64_t)P.window_slack >= kI64Max / 8) {
                plans[ri] = own;
                continue;
            }
            if (P.score_band > 0) {
                const int64_t w = P.score_band, dmin = span_lo[ri], dmax = span_hi[ri], sl = r.sl;
                const int64_t lo2 = std::min(std::max<int64_t>(dmin - w, 0), sl);
                const int64_t hi2 = std::max(std::min(qlen + dmax + w, sl), lo2);
                const int64_t nn = hi2 - lo2;
                int64_t blo = dmin - w - lo2, bhi = dmax + w - lo2;
                band_clip(blo, bhi, qlen, nn);
                if (nn == 0 || band_covers(blo, bhi, qlen, nn)) plans[ri] = Plan{lo2, hi2, false, 0, 0};
                else plans[ri] = Plan{lo2, hi2, true, blo, bhi};
                continue;
            }
            if (qlen * (hi - lo) < kBandScoreMinCells) {
                plans[ri] = own;
                continue;
            }
            int64_t ulo, uhi;
            window(span_lo[ri], span_hi[ri], r.sl, qlen, ulo, uhi);
            const int64_t nn = uhi - ulo;
            int64_t blo = span_lo[ri] - ulo - P.window_slack, bhi = span_hi[ri] - ulo + P.window_slack;
            band_clip(blo, bhi, qlen, nn);
            if (band_covers(blo, bhi, qlen, nn)) {
                plans[ri] = own;
                continue;
            }
            const int64_t rows = std::min(qlen, nn + band_width(blo, bhi));
            const int64_t rect = qlen * nn;
            if (band_width(blo, bhi) * rows * kBandCostRatio < rect) plans[ri] = Plan{ulo, uhi, true, blo, bhi};
            else plans[ri] = own;
        }
        return plans;
    }

    saber_band_job job(uint32_t qi, const Region& r, int64_t lo, int64_t hi, int64_t blo, int64_t bhi) const {
        saber_band_job j{};
        j.query = qi;
        j.subject = r.subject;
        j.win_begin = r.sbase + (uint64_t)lo;
        j.win_len = (uint32_t)(hi - lo);
        j.band_lo = (int32_t)std::max<int64_t>(std::min(blo, kI32Max), -kI32Max - 1);
        j.band_hi = (int32_t)std::max<int64_t>(std::min(bhi, kI32Max), -kI32Max - 1);
        j.flags = 0;
        return j;
    }

    // Scores of n jobs into the handle's pinned staging slot `slot` (fast
    // copies, no zero fill); *out stays valid until the slot is reused.
    int score(const saber_band_job* jobs, size_t n, int slot, const int32_t** out) {
        int32_t* sc = static_cast<int32_t*>(saber::pinned_scratch(h, slot, n * sizeof(int32_t)));
        if (!sc) return SABER_ERR_NOMEM;
        *out = sc;
        if (n == 0) return SABER_OK;
        saber_score_stats ss{};
        const double t0 = now_ms();
        int rc = saber_gpu_score_band_jobs(h, jobs, n, sc, &ss);
        if (rc != SABER_OK) return rc;
        st.t_score_calls_ms += now_ms() - t0;
        st.t_score_device_ms += ss.t_prep_ms + ss.t_fast_ms + ss.t_generic_ms;
        st.t_score_prep_ms += ss.t_prep_ms;
        st.t_score_fast_ms += ss.t_fast_ms;
        st.t_score_generic_ms += ss.t_generic_ms;
        st.banded_cells += ss.banded_cells;
        st.score_launches += 1;
        return SABER_OK;
    }

    // engine.rs:1021-1099, batched over the queries.  The jobs are built in
    // the handle's pinned staging buffers (no zero-fill, fast copies), every
    // per-region loop runs over the queries in parallel.
    int score_windows(const std::vector<Prep>& preps, const std::vector<std::vector<Region>>& per_q,
                      const std::vector<std::vector<Plan>>& plans, const std::vector<int64_t>& qlens,
                      std::vector<std::vector<int64_t>>& scores) {
        const int64_t wn = P.score_prefilter_band, full_band = P.score_band;
        struct Ref {
            uint32_t qi, ri;
            int kind;  // 0 full, 1 narrow, 2 band
        };
        const size_t nq = per_q.size();
        const double tb0 = now_ms();
        scores.resize(nq);
        std::vector<size_t> base(nq + 1, 0);
        for (size_t qi = 0; qi < nq; qi++) base[qi + 1] = base[qi] + per_q[qi].size();
        const size_t n1 = base[nq];
        saber_band_job* s1 = static_cast<saber_band_job*>(saber::pinned_scratch(h, 0, n1 * sizeof(saber_band_job)));
        if (n1 && !s1) return SABER_ERR_NOMEM;
        std::unique_ptr<Ref[]> r1(new Ref[n1 ? n1 : 1]);
        std::vector<uint64_t> banded(nq, 0);
        parallel_for(nq, [&](size_t q) {
            const uint32_t qi = (uint32_t)q;
            scores[qi].assign(per_q[qi].size(), 0);
            const int64_t m = qlens[qi];
            for (uint32_t ri = 0; ri < per_q[qi].size(); ri++) {
                const Region& r = per_q[qi][ri];
                const Plan& pl = plans[qi][ri];
                const int64_t n = pl.hi - pl.lo;
                const size_t k = base[qi] + ri;
                if (!pl.band) {
                    s1[k] = job(qi, r, pl.lo, pl.hi, -m, n);
                    r1[k] = {qi, ri, 0};
                } else if (0 < wn && wn < full_band) {
                    int64_t blo = r.dmin - wn - pl.lo, bhi = r.dmax + wn - pl.lo;
                    band_clip(blo, bhi, m, n);
                    s1[k] = job(qi, r, pl.lo, pl.hi, blo, bhi);
                    r1[k] = {qi, ri, 1};
                    banded[qi]++;
                } else {
                    s1[k] = job(qi, r, pl.lo, pl.hi, pl.blo, pl.bhi);
                    r1[k] = {qi, ri, 2};
                    banded[qi]++;
                }
            }
        });
        for (uint64_t v : banded) st.band_scored_regions += v;
        st.t_score_build_ms += now_ms() - tb0;
        const int32_t* sc1 = nullptr;
        int rc = score(s1, n1, 2, &sc1);
        if (rc != SABER_OK) return rc;
        const double ts0 = now_ms();
        // stage-2 decision per region (f64 threshold of the region's subject length)
        const double re = region_evalue();
        std::vector<uint8_t> again(n1, 0);
        std::vector<size_t> n2q(nq + 1, 0);
        parallel_for(nq, [&](size_t q) {
            size_t c = 0;
            LenMemo memo;  // the threshold depends on the query and the subject length only
            for (size_t k = base[q]; k < base[q + 1]; k++) {
                const Ref& x = r1[k];
                if (x.kind != 1) {
                    scores[x.qi][x.ri] = sc1[k];
                    continue;
                }
                const Region& r = per_q[x.qi][x.ri];
                const Prep& pr = preps[x.qi];
                const int64_t sl = r.sl;
                const double thr = memo.get(sl, [&]() {
                    return P.score_prefilter_frac * pr.qs.floor_lower_bound(re, false, 0.0, sl, pr.region_floor);
                });
                if ((double)sc1[k] >= thr) {
                    again[k] = 1;
                    c++;
                } else {
                    scores[x.qi][x.ri] = sc1[k];
                }
            }
            n2q[q + 1] = c;
        });
        for (size_t q = 0; q < nq; q++) n2q[q + 1] += n2q[q];
        const size_t n2 = n2q[nq];
        saber_band_job* s2 = static_cast<saber_band_job*>(saber::pinned_scratch(h, 1, n2 * sizeof(saber_band_job)));
        if (n2 && !s2) return SABER_ERR_NOMEM;
        std::unique_ptr<Ref[]> r2(new Ref[n2 ? n2 : 1]);
        parallel_for(nq, [&](size_t q) {
            size_t w = n2q[q];
            for (size_t k = base[q]; k < base[q + 1]; k++) {
                if (!again[k]) continue;
                const Ref& x = r1[k];
                const Region& r = per_q[x.qi][x.ri];
                const Plan& pl = plans[x.qi][x.ri];
                s2[w] = job(x.qi, r, pl.lo, pl.hi, pl.blo, pl.bhi);
                r2[w] = x;
                w++;
            }
        });
        st.t_score_stage2_ms += now_ms() - ts0;
        const int32_t* sc2 = nullptr;
        rc = score(s2, n2, 3, &sc2);
        if (rc != SABER_OK) return rc;
        for (size_t k = 0; k < n2; k++) scores[r2[k].qi][r2[k].ri] = sc2[k];
        st.band_rescored += n2;
        return SABER_OK;
    }

    // engine.rs:1447-1530
    HitRec make_hit(const uint8_t* q, int64_t qlen, uint32_t subject, int64_t s_off, const Aln& al,
                    const QStats& qs) const {
        const uint8_t* s_full = db + soff[subject];
        const int64_t s_len = slen(subject);
        const uint8_t* s = s_full + s_off;
        int64_t i = al.q_start, j = al.s_start;
        uint64_t matches = 0, mism = 0, pos = 0, gopen = 0, gcols = 0, cols = 0;
        const int lim = P.is_protein ? 20 : 4;
        for (uint32_t run : al.runs) {
            const char op = (char)(run & 0xFF);
            const int64_t l = run >> 8;
            cols += l;
            if (op == 'M') {
                for (int64_t t = 0; t < l; t++) {
                    const int a = q[i + t], b = s[j + t];
                    const bool ident = a == b && a < lim;
                    const int sc = mat[(a < 24 ? a : 22) * 24 + (b < 24 ? b : 22)];
                    matches += ident;
                    pos += ident || sc > 0;
                }
                mism += l;
                i += l;
                j += l;
            } else if (op == 'I') {
                gopen++;
                gcols += l;
                i += l;
            } else {
                gopen++;
                gcols += l;
                j += l;
            }
        }
        mism -= matches;
        HitRec r;
        saber_hit& x = r.h;
        std::memset(&x, 0, sizeof(x));
        x.subject = subject;
        x.score = al.score;
        x.exact = al.status == 1;
        x.bitscore = qs.bitscore(al.score);
        x.evalue = qs.evalue_for(al.score, s_len);
        x.q_start = al.q_start + 1;
        x.q_end = al.q_end;
        x.s_start = (uint32_t)(al.s_start + s_off + 1);
        x.s_end = (uint32_t)(al.s_end + s_off);
        x.columns = (uint32_t)cols;
        x.matches = (uint32_t)matches;
        x.mismatches = (uint32_t)mism;
        x.positives = (uint32_t)pos;
        x.gap_opens = (uint32_t)gopen;
        x.gap_columns = (uint32_t)gcols;
        x.q_len = (uint32_t)qlen;
        x.s_len = (uint32_t)s_len;
        r.runs = al.runs;
        return r;
    }

    static double identity(const saber_hit& x) { return x.columns == 0 ? 0.0 : 100.0 * x.matches / x.columns; }
    static double query_cover(const saber_hit& x) {
        return x.q_len == 0 ? 0.0 : 100.0 * ((double)x.q_end + 1 - x.q_start) / x.q_len;
    }
    static double subject_cover(const saber_hit& x) {
        return x.s_len == 0 ? 0.0 : 100.0 * ((double)x.s_end + 1 - x.s_start) / x.s_len;
    }
    // engine.rs:2415-2417
    static bool overlaps(const saber_hit& a, const saber_hit& b) {
        return a.q_start <= b.q_end && b.q_start <= a.q_end && a.s_start <= b.s_end && b.s_start <= a.s_end;
    }

    struct QState {
        size_t pos = 0;
        std::vector<HitRec> out;
        std::vector<uint64_t> hit_src;
        std::unordered_map<uint32_t, uint32_t> per_subject;
        uint32_t reported = 0;
        bool done = false;
    };

    static uint64_t key(uint32_t qi, uint32_t ri) { return ((uint64_t)qi << 32) | ri; }

    // engine.rs:1127-1221: E-value cut and order, then speculative batched
    // tracebacks (a traceback depends only on its region) for the next chunk
    // of candidates of every unfinished query, and the reporting steps
    int finish(const uint8_t* q_codes, const uint64_t* q_offsets, const std::vector<Prep>& preps,
               const std::vector<std::vector<Region>>& per_q, const std::vector<std::vector<Plan>>& plans,
               const std::vector<std::vector<int64_t>>& scores, std::vector<std::vector<HitRec>>& result,
               std::vector<uint64_t>* hit_src) {
        const double ecut = (P.evalue > 0.0 && std::isfinite(P.evalue)) ? P.evalue : kInf;
        const size_t nq = per_q.size();
        const double to0 = now_ms();
        std::vector<std::vector<std::pair<double, uint32_t>>> orders(nq);
        parallel_for(nq, [&](size_t qi) {
            const QStats& qs = preps[qi].qs;
            auto& order = orders[qi];
            const auto& regs = per_q[qi];
            LenMemo lb, sp;  // search spaces depend on the query and the subject length only
            for (uint32_t i = 0; i < regs.size(); i++) {
                const int64_t sc = scores[qi][i];
                if (qs.database_model) {
                    if (sc >= preps[qi].floor) order.push_back({qs.evalue(sc), i});
                    continue;
                }
                if (sc <= 0 || (has_bits && qs.bitscore(sc) < P.min_bitscore)) continue;
                const int64_t n = regs[i].sl;
                if (qs.evalue_in(sc, lb.get(n, [&]() { return qs.space_lower_bound(n); })) > ecut) continue;
                const double e = qs.evalue_in(sc, sp.get(n, [&]() { return qs.space_for(n); }));
                if (e <= ecut) order.push_back({e, i});
            }
            const auto& sc_ = scores[qi];
            std::stable_sort(order.begin(), order.end(), [&](const std::pair<double, uint32_t>& a,
                                                             const std::pair<double, uint32_t>& b) {
                if (a.first != b.first) return a.first < b.first;
                const int64_t sa = sc_[a.second], sb = sc_[b.second];
                if (sa != sb) return sa > sb;
                const Region& x = regs[a.second];
                const Region& y = regs[b.second];
                if (x.best != y.best) return x.best > y.best;
                if (x.subject != y.subject) return x.subject < y.subject;
                if (x.dmin != y.dmin) return x.dmin < y.dmin;
                return x.dmax < y.dmax;
            });
        });
        st.t_finish_order_ms += now_ms() - to0;
        std::unordered_map<uint64_t, Aln> tb;
        std::vector<QState> state(nq);
        for (size_t qi = 0; qi < nq; qi++) state[qi].done = orders[qi].empty();
        tb.reserve(nq * std::max<size_t>(4, (size_t)P.max_target_seqs * P.max_hsps) + 16);
        // speculative tracebacks per query and round: as many candidates as
        // the report can take (more rounds follow only where candidates
        // fail, are duplicates or repeat a subject)
        const size_t chunk = std::max<size_t>(4, (size_t)P.max_target_seqs * P.max_hsps);
        for (;;) {
            std::vector<std::pair<uint32_t, uint32_t>> need;
            for (uint32_t qi = 0; qi < nq; qi++) {
                if (state[qi].done) continue;
                const size_t k = state[qi].pos;
                for (size_t t = k; t < std::min(orders[qi].size(), k + chunk); t++) {
                    const uint32_t ri = orders[qi][t].second;
                    if (!tb.count(key(qi, ri))) need.push_back({qi, ri});
                }
            }
            if (!need.empty()) {
                int rc = traceback(need, per_q, plans, scores, q_offsets, tb);
                if (rc != SABER_OK) return rc;
            }
            std::vector<uint8_t> moved(nq, 0);
            parallel_for(nq, [&](size_t q) {
                const uint32_t qi = (uint32_t)q;
                if (state[qi].done) return;
                moved[qi] = finish_steps(qi, state[qi], orders[qi], per_q[qi], plans[qi], tb, preps[qi],
                                         q_codes + q_offsets[qi], (int64_t)(q_offsets[qi + 1] - q_offsets[qi]), ecut);
            });
            bool progress = false;
            for (uint8_t v : moved) progress |= v != 0;
            bool all = true;
            for (const QState& s : state) all &= s.done;
            if (all) break;
            if (need.empty() && !progress) break;
        }
        result.assign(nq, {});
        for (uint32_t qi = 0; qi < nq; qi++) {
            auto& hits = state[qi].out;
            std::stable_sort(hits.begin(), hits.end(), [](const HitRec& a, const HitRec& b) {
                if (a.h.evalue != b.h.evalue) return a.h.evalue < b.h.evalue;
                if (a.h.score != b.h.score) return a.h.score > b.h.score;
                if (a.h.subject != b.h.subject) return a.h.subject < b.h.subject;
                return a.h.s_start < b.h.s_start;
            });
            for (auto& x : hits) x.h.query = qi;
            if (hit_src) hit_src->insert(hit_src->end(), state[qi].hit_src.begin(), state[qi].hit_src.end());
            st.alignments += hits.size();
            result[qi] = std::move(hits);
        }
        return SABER_OK;
    }

    bool finish_steps(uint32_t qi, QState& stt, const std::vector<std::pair<double, uint32_t>>& order,
                      const std::vector<Region>& regs, const std::vector<Plan>& plans,
                      const std::unordered_map<uint64_t, Aln>& tb, const Prep& prep, const uint8_t* q, int64_t qlen,
                      double ecut) {
        bool moved = false;
        while (stt.pos < order.size()) {
            const uint32_t ri = order[stt.pos].second;
            const uint32_t s = regs[ri].subject;
            auto it = stt.per_subject.find(s);
            if (stt.reported >= P.max_target_seqs && it == stt.per_subject.end()) {
                stt.done = true;
                return true;
            }
            const uint32_t cnt = it == stt.per_subject.end() ? 0 : it->second;
            if (cnt >= P.max_hsps) {
                stt.pos++;
                moved = true;
                continue;
            }
            auto t = tb.find(key(qi, ri));
            if (t == tb.end()) return moved;
            stt.pos++;
            moved = true;
            const Aln& al = t->second;
            if (!al.present) continue;
            HitRec hit = make_hit(q, qlen, s, plans[ri].lo, al, prep.qs);
            if (cnt > 0) {
                bool dup = false;
                for (const HitRec& o : stt.out)
                    if (o.h.subject == hit.h.subject && overlaps(o.h, hit.h)) {
                        dup = true;
                        break;
                    }
                if (dup) continue;
            }
            bool passes;
            if (prep.qs.database_model) passes = hit.h.score >= prep.floor;
            else passes = hit.h.evalue <= ecut && (!has_bits || hit.h.bitscore >= P.min_bitscore);
            if (identity(hit.h) < P.min_identity || query_cover(hit.h) < P.min_query_cover ||
                subject_cover(hit.h) < P.min_subject_cover || !passes)
                continue;
            if (cnt == 0) stt.reported++;
            stt.per_subject[s] = cnt + 1;
            stt.out.push_back(std::move(hit));
            stt.hit_src.push_back(regs[ri].src);
        }
        stt.done = true;
        return true;
    }

    // engine.rs:1328-1445 through the batched widening traceback
    int traceback(const std::vector<std::pair<uint32_t, uint32_t>>& need, const std::vector<std::vector<Region>>& per_q,
                  const std::vector<std::vector<Plan>>& plans, const std::vector<std::vector<int64_t>>& scores,
                  const uint64_t* q_offsets, std::unordered_map<uint64_t, Aln>& tb) {
        std::vector<saber_traceback_job> jobs(need.size());
        uint64_t cap = 64;
        for (size_t k = 0; k < need.size(); k++) {
            const uint32_t qi = need[k].first, ri = need[k].second;
            const Region& r = per_q[qi][ri];
            const Plan& pl = plans[qi][ri];
            const bool full = P.exhaustive || r.best == 0;
            saber_traceback_job& j = jobs[k];
            std::memset(&j, 0, sizeof(j));
            j.query = qi;
            j.subject = r.subject;
            j.win_begin = r.sbase + (uint64_t)pl.lo;
            j.win_len = (uint32_t)(pl.hi - pl.lo);
            j.d_min = (int32_t)(r.dmin - pl.lo);
            j.d_max = (int32_t)(r.dmax - pl.lo);
            j.limit_lo = pl.band ? (int32_t)pl.blo : 0;
            j.limit_hi = pl.band ? (int32_t)pl.bhi : 0;
            j.want = (int32_t)scores[qi][ri];
            j.flags = (full ? 1u : 0u) | (pl.band ? 2u : 0u);
            cap += (uint64_t)j.win_len + (q_offsets[qi + 1] - q_offsets[qi]) + 2;
        }
        std::vector<saber_alignment> out(need.size());
        // the library writes only the runs it returns: no zero fill of the bound
        std::unique_ptr<uint32_t[]> ops(new uint32_t[cap]);
        saber_traceback_stats ts{};
        const double t0 = now_ms();
        int rc = saber_gpu_traceback(h, jobs.data(), jobs.size(), P.band_pad, P.traceback_max_bytes, out.data(),
                                     ops.get(), cap, &ts);
        if (rc != SABER_OK) return rc;
        st.t_finish_tb_ms += now_ms() - t0;
        st.traceback.tracebacks += ts.tracebacks;
        st.traceback.band_widenings += ts.band_widenings;
        st.traceback.end_anchored += ts.end_anchored;
        st.traceback.band_capped += ts.band_capped;
        st.traceback.banded_cells += ts.banded_cells;
        st.traceback.launches += ts.launches;
        for (size_t k = 0; k < need.size(); k++) {
            Aln a;
            const saber_alignment& o = out[k];
            a.present = o.status != 0;
            a.status = o.status;
            a.score = o.score;
            a.q_start = o.q_start;
            a.q_end = o.q_end;
            a.s_start = o.s_start;
            a.s_end = o.s_end;
            if (a.present) a.runs.assign(ops.get() + o.ops_offset, ops.get() + o.ops_offset + o.n_ops);
            tb.insert_or_assign(key(need[k].first, need[k].second), std::move(a));
        }
        return SABER_OK;
    }
};

}  // namespace

extern "C" int saber_gpu_search(saber_gpu* h, const saber_search_params* params, const uint8_t* db_res,
                                const uint64_t* db_offsets, uint64_t nsub, const uint8_t* q_codes,
                                const uint64_t* q_offsets, uint32_t nq, const uint8_t* q_mask, saber_hit* hits,
                                uint64_t hits_cap, uint64_t* n_hits, uint32_t* ops, uint64_t ops_cap, uint64_t* n_ops,
                                saber_search_stats* stats);

namespace saber {
int scheme_matrix(saber_gpu* h, int32_t* out576);  // saber_gpu.cu
int scan_search_regions(saber_gpu* h, const saber_scan_params* p, const uint8_t* q_mask, const int32_t* region_thr,
                        RegionSink& sink, saber_scan_stats* st);  // saber_gpu.cu
void triage_set_labels(saber_gpu* h, const std::vector<uint64_t>& hit_regions);
}

extern "C" int saber_gpu_search(saber_gpu* h, const saber_search_params* params, const uint8_t* db_res,
                                const uint64_t* db_offsets, uint64_t nsub, const uint8_t* q_codes,
                                const uint64_t* q_offsets, uint32_t nq, const uint8_t* q_mask, saber_hit* hits,
                                uint64_t hits_cap, uint64_t* n_hits, uint32_t* ops, uint64_t ops_cap, uint64_t* n_ops,
                                saber_search_stats* stats) {
    if (!h || !params || !db_offsets || (nq && (!q_codes || !q_offsets)) || !n_hits || !n_ops) return SABER_ERR_ARG;
    if (nsub && !db_res) return SABER_ERR_ARG;
    const double t0 = now_ms();
    int32_t mat[576];
    int rc = saber::scheme_matrix(h, mat);
    if (rc != SABER_OK) return rc;
    Engine E(h, *params, db_res, db_offsets, nsub, mat);
    const saber_search_params& P = *params;

    // query preparation (engine.rs:759-786)
    std::vector<int64_t> qlens(nq);
    std::vector<Prep> preps(nq);
    std::vector<int8_t> bias(nq ? q_offsets[nq] : 0, 0);
    parallel_for(nq, [&](size_t qi) {
        qlens[qi] = (int64_t)(q_offsets[qi + 1] - q_offsets[qi]);
        if (P.comp_bias && P.is_protein)
            composition_bias(q_codes + q_offsets[qi], qlens[qi], mat, bias.data() + q_offsets[qi]);
        preps[qi] = E.prepare(qlens[qi]);
    });
    rc = saber_gpu_load_queries(h, q_codes, q_offsets, bias.data(), nq);
    if (rc != SABER_OK) return rc;
    const double t1 = now_ms();

    // candidate regions
    std::vector<std::vector<Region>> per_q(nq);
    double t_scan_end = 0;
    bool collecting = false;
    if (P.exhaustive) {
        for (uint32_t qi = 0; qi < nq; qi++)
            if (qlens[qi] > 0)
                for (uint32_t s = 0; s < nsub; s++)
                    per_q[qi].push_back({s, -qlens[qi], E.slen(s), 0, 0, db_offsets[s], E.slen(s)});
    } else if (nq && nsub) {
        std::vector<int32_t> thr(nq);
        for (uint32_t qi = 0; qi < nq; qi++) thr[qi] = (int32_t)preps[qi].region_thr;
        // candidate regions, capped per query and triaged (a no-op without a
        // model or collection) on the device; the kept ones arrive grouped by
        // query in region order, each with its position in the capped list
        saber::RegionSink sink;
        sink.lambda = (float)P.lambda;
        sink.logk = (float)std::log(P.k);
        rc = saber::scan_search_regions(h, &P.scan, q_mask, thr.data(), sink, &E.st.scan);
        if (rc != SABER_OK) return rc;
        t_scan_end = now_ms();
        collecting = sink.collecting;
        if (sink.triaged) E.st.triage_dropped += sink.ncap - sink.n;
        const saber_region* R = sink.regs;
        const uint32_t* src = sink.src;
        const uint64_t* sbase = sink.sbase;
        const uint32_t* slen = sink.slen;
        const uint64_t nr = sink.n;
        parallel_for(nq, [&](size_t qi) {
            auto by_query = [](const saber_region& r, uint64_t q) { return r.query < q; };
            const uint64_t b = (uint64_t)(std::lower_bound(R, R + nr, (uint64_t)qi, by_query) - R);
            const uint64_t e = (uint64_t)(std::lower_bound(R + b, R + nr, (uint64_t)qi + 1, by_query) - R);
            auto& v = per_q[qi];
            v.reserve(e - b);
            for (uint64_t t = b; t < e; t++)
                v.push_back({R[t].subject, R[t].d_min, R[t].d_max, R[t].best, src[t], sbase[t], (int64_t)slen[t]});
        });
    }
    for (uint32_t qi = 0; qi < nq; qi++) {
        if (qlens[qi] == 0) per_q[qi].clear();
        E.st.regions += per_q[qi].size();
    }
    const double t2 = now_ms();
    if (t_scan_end == 0) t_scan_end = t2;

    std::vector<std::vector<Plan>> plans(nq);
    parallel_for(nq, [&](size_t qi) { plans[qi] = E.plan_windows(per_q[qi], qlens[qi]); });
    const double t3 = now_ms();
    std::vector<std::vector<int64_t>> scores;
    rc = E.score_windows(preps, per_q, plans, qlens, scores);
    if (rc != SABER_OK) return rc;
    const double t4 = now_ms();
    std::vector<std::vector<HitRec>> result;
    std::vector<uint64_t> hit_src;
    rc = E.finish(q_codes, q_offsets, preps, per_q, plans, scores, result, collecting ? &hit_src : nullptr);
    if (rc != SABER_OK) return rc;
    if (collecting) saber::triage_set_labels(h, hit_src);
    const double t5 = now_ms();

    uint64_t nh = 0, no = 0;
    for (const auto& v : result)
        for (const HitRec& x : v) {
            nh++;
            no += x.runs.size();
        }
    *n_hits = nh;
    *n_ops = no;
    E.st.t_prep_ms = t1 - t0;
    E.st.t_scan_ms = t_scan_end - t1;
    E.st.t_triage_ms = t2 - t_scan_end;
    E.st.t_plan_ms = t3 - t2;
    E.st.t_score_ms = t4 - t3;
    E.st.t_finish_ms = t5 - t4;
    E.st.t_total_ms = t5 - t0;
    if (stats) *stats = E.st;
    if (nh > hits_cap || no > ops_cap || (nh && !hits) || (no && !ops)) return SABER_ERR_CAP;
    uint64_t k = 0, o = 0;
    for (const auto& v : result)
        for (const HitRec& x : v) {
            hits[k] = x.h;
            hits[k].ops_offset = o;
            hits[k].n_ops = (uint32_t)x.runs.size();
            std::copy(x.runs.begin(), x.runs.end(), ops + o);
            o += x.runs.size();
            k++;
        }
    return SABER_OK;
}
