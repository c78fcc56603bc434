// Seeded synthetic rating matrices (see include/cdmf_synth.h).
//
// Every random draw comes from a counter-based hash of (seed, stream, index),
// so rows can be generated in parallel and the result does not depend on the
// thread count.  Steps:
//   1. row degrees: capped Zipf rank weights over a hashed permutation of the
//      rows, scaled so the capped, integerised degrees sum to nnz_total
//      (largest-remainder rounding), or uniform degrees (row_mode 1);
//   2. column sampling weights: capped Zipf over a hashed permutation of the
//      columns, or Beta inclusion weights (col_mode 1);
//   3. optional forced entries so that every column is non-empty;
//   4. per row, distinct columns drawn by weight: rejection sampling from the
//      inverse CDF for sparse rows, Efraimidis-Spirakis keys for dense rows;
//   5. values from a planted low-rank model plus Gaussian noise, rounded to a
//      quantum and clamped;
//   6. a uniform hold-out of nnz_test entries (the smallest hash keys), the
//      rest compacted into the train CSR, and CSC by a stable counting sort.
#include <cdmf_synth.h>
#include <cdmf_cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>
#include <omp.h>

namespace {

inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
inline uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t i) {
    return mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) ^ (i * 0x9E3779B97F4A7C15ull + stream));
}
// uniform in (0, 1)
inline double u01(uint64_t seed, uint64_t stream, uint64_t i) {
    return ((double)(hash3(seed, stream, i) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
inline double normal(uint64_t seed, uint64_t stream, uint64_t i) {
    double a = u01(seed, stream, 2 * i), b = u01(seed, stream, 2 * i + 1);
    return std::sqrt(-2.0 * std::log(a)) * std::cos(6.283185307179586 * b);
}
// Marsaglia-Tsang gamma(shape >= 1) with a bounded number of tries.
double gamma_draw(double shape, uint64_t seed, uint64_t stream, uint64_t i) {
    double boost = 1.0;
    if (shape < 1.0) {
        boost = std::pow(u01(seed, stream + 7, i), 1.0 / shape);
        shape += 1.0;
    }
    const double d = shape - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
    for (uint64_t tr = 0; tr < 64; ++tr) {
        double x = normal(seed, stream, i * 64 + tr);
        double v = 1.0 + c * x;
        if (v <= 0) continue;
        v = v * v * v;
        double u = u01(seed, stream + 3, i * 64 + tr);
        if (std::log(u) < 0.5 * x * x + d - d * v + d * std::log(v)) return boost * d * v;
    }
    return boost * d;
}

enum : uint64_t {
    S_RPERM = 1, S_CPERM, S_RDEG, S_FORCE, S_ROW, S_U, S_V, S_NOISE, S_TEST, S_BETA_A, S_BETA_B = S_BETA_A + 16
};

// Rank of every element under a hashed permutation.
std::vector<int64_t> hashed_ranks(int64_t count, uint64_t seed, uint64_t stream) {
    std::vector<uint64_t> key(count);
    std::vector<int64_t> order(count);
    for (int64_t i = 0; i < count; ++i) { key[i] = hash3(seed, stream, i); order[i] = i; }
    std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return key[a] != key[b] ? key[a] < key[b] : a < b;
    });
    std::vector<int64_t> rank(count);
    for (int64_t r = 0; r < count; ++r) rank[order[r]] = r;
    return rank;
}

// Integer degrees clamp(s * w_i, lo, hi) summing to `total` (largest remainder).
bool capped_degrees(const std::vector<double>& w, int64_t lo, int64_t hi, int64_t total,
                    std::vector<int64_t>& deg) {
    const int64_t count = (int64_t)w.size();
    if (count == 0) return total == 0;
    if (lo * count > total || hi * count < total) return false;
    auto mass = [&](double s) {
        double acc = 0;
        for (double x : w) acc += std::min<double>(hi, std::max<double>(lo, s * x));
        return acc;
    };
    double a = 0, b = 1;
    while (mass(b) < (double)total) b *= 2;
    for (int it = 0; it < 200; ++it) {
        double mid = 0.5 * (a + b);
        (mass(mid) < (double)total ? a : b) = mid;
    }
    deg.assign(count, 0);
    std::vector<double> frac(count);
    int64_t acc = 0;
    for (int64_t i = 0; i < count; ++i) {
        double x = std::min<double>(hi, std::max<double>(lo, b * w[i]));
        deg[i] = (int64_t)std::floor(x);
        frac[i] = x - (double)deg[i];
        acc += deg[i];
    }
    std::vector<int64_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) {
        return frac[x] != frac[y] ? frac[x] > frac[y] : x < y;
    });
    // add where there is room (below hi), remove where there is slack (above lo)
    int64_t diff = total - acc;
    for (int64_t q = 0; diff > 0 && q < count; ++q)
        if (deg[order[q]] < hi) { deg[order[q]]++; diff--; }
    for (int64_t q = count - 1; diff < 0 && q >= 0; --q)
        if (deg[order[q]] > lo) { deg[order[q]]--; diff++; }
    for (int64_t i = 0; diff > 0 && i < count; ++i)
        while (diff > 0 && deg[i] < hi) { deg[i]++; diff--; }
    return diff == 0;
}

}  // namespace

struct cdmf_synth {
    int64_t m = 0, n = 0, nnz = 0, nnz_test = 0;
    std::vector<uint32_t> csr_ptr, csr_idx, csc_ptr, csc_idx, te_row, te_col;
    std::vector<float> csr_val, csc_val, te_val;
};

extern "C" int cdmf_csr_to_csc(int64_t m, int64_t n, int64_t nnz, const uint32_t* csr_row_ptr,
                               const uint32_t* csr_col_idx, const float* csr_val, uint32_t* csc_col_ptr,
                               uint32_t* csc_row_idx, float* csc_val, uint32_t* perm) {
    if (m < 0 || n < 0 || nnz < 0 || nnz > (int64_t)UINT32_MAX) return CDMF_ERR_INVALID;
    if (!csr_row_ptr || !csc_col_ptr || (nnz > 0 && (!csr_col_idx || !csc_row_idx))) return CDMF_ERR_INVALID;
    if ((int64_t)csr_row_ptr[m] != nnz) return CDMF_ERR_INVALID;
    std::vector<uint64_t> cnt(n + 1, 0);
    for (int64_t p = 0; p < nnz; ++p) {
        if (csr_col_idx[p] >= (uint64_t)n) return CDMF_ERR_INVALID;
        cnt[csr_col_idx[p] + 1]++;
    }
    for (int64_t j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
    for (int64_t j = 0; j <= n; ++j) csc_col_ptr[j] = (uint32_t)cnt[j];
    for (int64_t i = 0; i < m; ++i) {
        if (csr_row_ptr[i] > csr_row_ptr[i + 1]) return CDMF_ERR_INVALID;
        for (uint32_t p = csr_row_ptr[i]; p < csr_row_ptr[i + 1]; ++p) {
            uint64_t q = cnt[csr_col_idx[p]]++;
            csc_row_idx[q] = (uint32_t)i;
            if (csc_val && csr_val) csc_val[q] = csr_val[p];
            if (perm) perm[q] = p;
        }
    }
    return CDMF_OK;
}

extern "C" int cdmf_synth_create(const cdmf_synth_spec* sp, int threads, cdmf_synth** out) {
    if (!sp || !out) return CDMF_ERR_INVALID;
    *out = nullptr;
    const int64_t m = sp->m, n = sp->n;
    if (m <= 0 || n <= 0 || m > (int64_t)UINT32_MAX || n > (int64_t)UINT32_MAX) return CDMF_ERR_INVALID;
    if (sp->rank < 0 || sp->row_min < 0 || sp->row_max < sp->row_min || sp->row_max > n) return CDMF_ERR_INVALID;
    if (threads > 0) omp_set_num_threads(threads);
    const uint64_t seed = sp->seed;

    // 1. row degrees
    std::vector<int64_t> deg;
    if (sp->row_mode == 0) {
        std::vector<int64_t> rr = hashed_ranks(m, seed, S_RPERM);
        std::vector<double> w(m);
        for (int64_t i = 0; i < m; ++i) w[i] = std::pow((double)(rr[i] + 1), -sp->row_alpha);
        if (!capped_degrees(w, sp->row_min, sp->row_max, sp->nnz_total, deg)) return CDMF_ERR_INVALID;
    } else {
        deg.resize(m);
        const int64_t span = sp->row_max - sp->row_min + 1;
        for (int64_t i = 0; i < m; ++i)
            deg[i] = sp->row_min + std::min<int64_t>(span - 1, (int64_t)(u01(seed, S_RDEG, i) * (double)span));
    }

    // 2. column weights
    std::vector<double> cw(n);
    if (sp->col_mode == 0) {
        std::vector<int64_t> cr = hashed_ranks(n, seed, S_CPERM);
        for (int64_t j = 0; j < n; ++j) cw[j] = std::pow((double)(cr[j] + 1), -sp->col_alpha);
        if (sp->col_cap > 0) {
            // scale so the expected degrees sum to nnz_total, then cap
            double tot = 0;
            for (double x : cw) tot += x;
            double a = 0, b = (double)sp->nnz_total / tot * 4 + 1;
            auto mass = [&](double s) {
                double acc = 0;
                for (double x : cw) acc += std::min<double>((double)sp->col_cap, s * x);
                return acc;
            };
            if (mass(b * 1e6) >= (double)sp->nnz_total) {
                while (mass(b) < (double)sp->nnz_total) b *= 2;
                for (int it = 0; it < 200; ++it) {
                    double mid = 0.5 * (a + b);
                    (mass(mid) < (double)sp->nnz_total ? a : b) = mid;
                }
                for (double& x : cw) x = std::min<double>((double)sp->col_cap, b * x);
            }
        }
    } else {
        for (int64_t j = 0; j < n; ++j) {
            double x = gamma_draw(sp->col_beta_a, seed, S_BETA_A, j);
            double y = gamma_draw(sp->col_beta_b, seed, S_BETA_B, j);
            cw[j] = std::max(1e-6, x / (x + y));
        }
    }
    std::vector<double> cdf(n);
    {
        double acc = 0;
        for (int64_t j = 0; j < n; ++j) { acc += cw[j]; cdf[j] = acc; }
        for (int64_t j = 0; j < n; ++j) cdf[j] /= acc;
        cdf[n - 1] = 1.0;
    }

    // 3. forced entries: column j is guaranteed a row f_j
    std::vector<std::vector<uint32_t>> forced(m);
    if (sp->col_min_one) {
        for (int64_t j = 0; j < n; ++j) {
            int64_t f = (int64_t)(hash3(seed, S_FORCE, j) % (uint64_t)m);
            forced[f].push_back((uint32_t)j);
        }
        // rows whose forced set exceeds the degree grow; the largest rows give the difference back
        int64_t extra = 0;
        for (int64_t i = 0; i < m; ++i)
            if ((int64_t)forced[i].size() > deg[i]) { extra += (int64_t)forced[i].size() - deg[i]; deg[i] = (int64_t)forced[i].size(); }
        if (sp->row_mode == 0 && extra > 0) {
            std::vector<int64_t> order(m);
            std::iota(order.begin(), order.end(), 0);
            std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return deg[a] != deg[b] ? deg[a] > deg[b] : a < b; });
            for (int64_t q = 0; extra > 0; q = (q + 1) % m) {
                int64_t i = order[q];
                if (deg[i] > std::max<int64_t>((int64_t)forced[i].size(), sp->row_min)) { deg[i]--; extra--; }
            }
        }
    }
    int64_t total = 0;
    std::vector<uint64_t> ptr(m + 1, 0);
    for (int64_t i = 0; i < m; ++i) { ptr[i + 1] = ptr[i] + (uint64_t)deg[i]; }
    total = (int64_t)ptr[m];
    if (total > (int64_t)UINT32_MAX) return CDMF_ERR_INVALID;

    // 4. per-row distinct columns
    std::vector<uint32_t> cols;
    try { cols.resize(total); } catch (...) { return CDMF_ERR_ALLOC; }
    const int64_t dense_cut = std::max<int64_t>(1, n / 4);
#pragma omp parallel
    {
        std::vector<char> mark(n, 0);
        std::vector<uint32_t> pick;
        std::vector<std::pair<double, uint32_t>> keys;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < m; ++i) {
            const int64_t d = deg[i];
            pick.clear();
            for (uint32_t j : forced[i]) { mark[j] = 1; pick.push_back(j); }
            int64_t need = d - (int64_t)pick.size();
            bool dense = d >= dense_cut || sp->col_mode == 1;
            uint64_t ctr = 0;
            if (!dense) {
                const uint64_t limit = (uint64_t)need * 50 + 1000;
                while (need > 0 && ctr < limit) {
                    double u = u01(seed, S_ROW, ((uint64_t)i << 24) ^ ctr);
                    ++ctr;
                    int64_t j = std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin();
                    if (j >= n) j = n - 1;
                    if (!mark[j]) { mark[j] = 1; pick.push_back((uint32_t)j); --need; }
                }
            }
            if (need > 0) {
                // Efraimidis-Spirakis: the `need` largest log(u)/w among the unmarked columns
                keys.clear();
                for (int64_t j = 0; j < n; ++j)
                    if (!mark[j]) keys.emplace_back(std::log(u01(seed, S_ROW + 100, (uint64_t)i * (uint64_t)n + j)) / cw[j], (uint32_t)j);
                std::nth_element(keys.begin(), keys.begin() + (need - 1), keys.end(),
                                 [](const std::pair<double, uint32_t>& a, const std::pair<double, uint32_t>& b) {
                                     return a.first != b.first ? a.first > b.first : a.second < b.second;
                                 });
                for (int64_t q = 0; q < need; ++q) { mark[keys[q].second] = 1; pick.push_back(keys[q].second); }
            }
            std::sort(pick.begin(), pick.end());
            for (size_t q = 0; q < pick.size(); ++q) { cols[ptr[i] + q] = pick[q]; mark[pick[q]] = 0; }
        }
    }

    // 5. values from the planted model
    const int r = sp->rank;
    std::vector<float> U((size_t)m * r), V((size_t)n * r);
    for (int64_t q = 0; q < (int64_t)m * r; ++q) U[q] = (float)(sp->factor_std * normal(seed, S_U, q));
    for (int64_t q = 0; q < (int64_t)n * r; ++q) V[q] = (float)(sp->factor_std * normal(seed, S_V, q));
    double scale = 1.0;
    if (sp->planted_std > 0 && r > 0 && sp->factor_std > 0)
        scale = sp->planted_std / (sp->factor_std * sp->factor_std * std::sqrt((double)r));
    std::vector<float> vals(total);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < m; ++i) {
        for (uint64_t p = ptr[i]; p < ptr[i + 1]; ++p) {
            const uint32_t j = cols[p];
            double dot = 0;
            for (int t = 0; t < r; ++t) dot += (double)U[(size_t)i * r + t] * (double)V[(size_t)j * r + t];
            double x = dot * scale + sp->offset + sp->noise_std * normal(seed, S_NOISE, ((uint64_t)i << 32) | j);
            if (sp->quantum > 0) x = std::floor(x / sp->quantum + 0.5) * sp->quantum;
            x = std::min(sp->vmax, std::max(sp->vmin, x));
            vals[p] = (float)x;
        }
    }

    // 6. hold-out
    int64_t nt = sp->nnz_test >= 0 ? sp->nnz_test : (int64_t)std::llround(sp->test_fraction * (double)total);
    if (nt < 0 || nt > total) return CDMF_ERR_INVALID;
    std::vector<char> is_test(total, 0);
    if (nt > 0) {
        std::vector<uint64_t> key(total);
#pragma omp parallel for
        for (int64_t p = 0; p < total; ++p) key[p] = hash3(seed, S_TEST, (uint64_t)p);
        std::vector<uint64_t> sorted_keys(key);
        std::nth_element(sorted_keys.begin(), sorted_keys.begin() + (nt - 1), sorted_keys.end());
        const uint64_t thr = sorted_keys[nt - 1];
        int64_t c = 0;
        for (int64_t p = 0; p < total; ++p)
            if (key[p] < thr) { is_test[p] = 1; ++c; }
        for (int64_t p = 0; p < total && c < nt; ++p)
            if (key[p] == thr && !is_test[p]) { is_test[p] = 1; ++c; }
    }
    cdmf_synth* s = new (std::nothrow) cdmf_synth();
    if (!s) return CDMF_ERR_ALLOC;
    try {
        s->m = m;
        s->n = n;
        s->nnz = total - nt;
        s->nnz_test = nt;
        s->csr_ptr.assign(m + 1, 0);
        s->csr_idx.resize(s->nnz);
        s->csr_val.resize(s->nnz);
        s->te_row.resize(nt);
        s->te_col.resize(nt);
        s->te_val.resize(nt);
        int64_t q = 0, e = 0;
        for (int64_t i = 0; i < m; ++i) {
            for (uint64_t p = ptr[i]; p < ptr[i + 1]; ++p) {
                if (is_test[p]) {
                    s->te_row[e] = (uint32_t)i; s->te_col[e] = cols[p]; s->te_val[e] = vals[p]; ++e;
                } else {
                    s->csr_idx[q] = cols[p]; s->csr_val[q] = vals[p]; ++q;
                }
            }
            s->csr_ptr[i + 1] = (uint32_t)q;
        }
        s->csc_ptr.resize(n + 1);
        s->csc_idx.resize(s->nnz);
        s->csc_val.resize(s->nnz);
    } catch (...) {
        delete s;
        return CDMF_ERR_ALLOC;
    }
    int st = cdmf_csr_to_csc(m, n, s->nnz, s->csr_ptr.data(), s->csr_idx.data(), s->csr_val.data(),
                             s->csc_ptr.data(), s->csc_idx.data(), s->csc_val.data(), nullptr);
    if (st) { delete s; return st; }
    *out = s;
    return CDMF_OK;
}

extern "C" int cdmf_synth_info(const cdmf_synth* s, int64_t* m, int64_t* n, int64_t* nnz, int64_t* nnz_test) {
    if (!s) return CDMF_ERR_INVALID;
    if (m) *m = s->m;
    if (n) *n = s->n;
    if (nnz) *nnz = s->nnz;
    if (nnz_test) *nnz_test = s->nnz_test;
    return CDMF_OK;
}

template <class T>
static void copy_out(T* dst, const std::vector<T>& src) {
    if (dst && !src.empty()) std::memcpy(dst, src.data(), sizeof(T) * src.size());
}

extern "C" int cdmf_synth_copy(const cdmf_synth* s, uint32_t* csr_row_ptr, uint32_t* csr_col_idx, float* csr_val,
                               uint32_t* csc_col_ptr, uint32_t* csc_row_idx, float* csc_val, uint32_t* test_row,
                               uint32_t* test_col, float* test_val) {
    if (!s) return CDMF_ERR_INVALID;
    copy_out(csr_row_ptr, s->csr_ptr);
    copy_out(csr_col_idx, s->csr_idx);
    copy_out(csr_val, s->csr_val);
    copy_out(csc_col_ptr, s->csc_ptr);
    copy_out(csc_row_idx, s->csc_idx);
    copy_out(csc_val, s->csc_val);
    copy_out(test_row, s->te_row);
    copy_out(test_col, s->te_col);
    copy_out(test_val, s->te_val);
    return CDMF_OK;
}

extern "C" void cdmf_synth_destroy(cdmf_synth* s) { delete s; }

extern "C" void cdmf_initial_col(float* X, uint32_t k, uint32_t n) {
    srand(0u);
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t t = 0; t < k; ++t)
            X[(size_t)t * n + i] = 0.1f * ((float)rand() / RAND_MAX) + 0.001f;
}
