/*
 * CPU model of the engine's 16-bit residual mode -- TEST INFRASTRUCTURE ONLY.
 *
 * The engine can store both residual copies in BF16 or FP16 while the
 * factors and all sums stay FP32.  This file models that mode on the host so
 * its error can be explained and bounded without a GPU:
 *   - the residual lives in one array (CSR order; the engine's two copies
 *     hold the same values) and every write rounds it to the storage type,
 *     round to nearest even, as __float2bfloat16_rn / __float2half_rn do;
 *   - the subtract of feature t is applied together with the add-back of
 *     feature t+1 in one read-modify-write, as the engine's first sweep of a
 *     feature does: r <- store(r - a*b + c*d), two FP32 roundings, one store;
 *   - at the start of every outer iteration after the first, the residual
 *     is recomputed from the FP32 ratings and factors (r = store(R - W.H),
 *     the dot product in t order with fmaf), as the engine's refresh does;
 *   - refresh_every > 0 adds the same refresh every refresh_every features
 *     of the first outer iteration, or of every outer iteration with
 *     refresh_all (schedules the engine does not run; the model measures
 *     what they would buy).
 * Line sums are sequential in index order with separate roundings, as in the
 * reference (src/cdmf_ref.cpp:7-17), so with FP32 storage the model is the
 * reference's arithmetic and reproduces oracle/ccdpp_oracle.c bit for bit
 * (the fused subtract and add-back round exactly as the reference's two
 * passes, src/cdmf_ref.cpp:86-89,120-121).  The test RMSE is
 * src/tools.cpp:543-582 as in the oracle.
 *
 * Only tests/ and oracle/ use it.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int64_t m, n, nnz;
    const uint32_t *csr_row_ptr, *csr_col_idx;
    const float *csr_val;
    const uint32_t *csc_col_ptr, *csc_row_idx;
    const float *csc_val;
    int64_t nnz_test;
    const uint32_t *test_row, *test_col;
    const float *test_val;
} model_problem;

static float store_bf16(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) {            /* Inf stays, NaN stays NaN */
        if (u & 0x007fffffu) u |= 0x00400000u;
        u &= 0xffff0000u;
    } else {
        u += 0x7fffu + ((u >> 16) & 1u);                /* round to nearest even */
        u &= 0xffff0000u;
    }
    memcpy(&x, &u, 4);
    return x;
}

/* The binary16 value nearest to x (ties to even), as a float: 10 mantissa
 * bits for normal results, multiples of 2^-24 below 2^-14, infinity from
 * 65520 up.  Written out rather than through a compiler half type so that it
 * builds the same everywhere. */
static float store_f16(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    const uint32_t sign = u & 0x80000000u, a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) return x;                                  /* Inf, NaN */
    if (a >= 0x477ff000u) {                                          /* >= 65520 */
        u = sign | 0x7f800000u;
        memcpy(&x, &u, 4);
        return x;
    }
    if (a < 0x38800000u) {                                           /* < 2^-14: subnormal */
        const float q = nearbyintf(fabsf(x) * 0x1p24f) * 0x1p-24f;
        return sign ? -q : q;
    }
    uint32_t r = (a + 0xfffu + ((a >> 13) & 1u)) & ~0x1fffu;        /* drop 13 of 23 bits */
    r |= sign;
    memcpy(&x, &r, 4);
    return x;
}

static float store(float x, int storage) {
    if (storage == 1) return store_bf16(x);
    if (storage == 2) return store_f16(x);
    return x;
}

static void refresh(const model_problem *P, int storage, uint32_t k, const float *W, const float *H, float *r) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < P->m; ++i)
        for (uint32_t p = P->csr_row_ptr[i]; p < P->csr_row_ptr[i + 1]; ++p) {
            const uint32_t j = P->csr_col_idx[p];
            float dot = 0.0f;
            for (uint32_t t = 0; t < k; ++t) dot = fmaf(W[(size_t)t * P->m + i], H[(size_t)t * P->n + j], dot);
            r[p] = store(P->csr_val[p] - dot, storage);
        }
}

static double test_rmse(const model_problem *P, uint32_t k, const float *W, const float *H) {
    double sum = 0;
    for (int64_t e = 0; e < P->nnz_test; ++e) {
        const uint32_t i = P->test_row[e], j = P->test_col[e];
        double pred = 0;
        for (uint32_t t = 0; t < k; ++t) pred += W[(size_t)t * P->m + i] * H[(size_t)t * P->n + j];
        const double d = (pred - (double)P->test_val[e]) * (pred - (double)P->test_val[e]);
        if (!isnan(d)) sum += d;
    }
    return P->nnz_test ? sqrt(sum / (double)P->nnz_test) : -1.0;
}

/* W (k x m) in/out, H (k x n) out (zeroed first), rmse[maxiter].  storage:
 * 0 = FP32, 1 = BF16, 2 = FP16; refresh_every / refresh_all: the extra
 * refreshes above (0 / 0: the engine's schedule).  Returns 0, or -1 when the CSC arrays are not
 * the canonical transpose of the CSR arrays or memory runs out. */
int mixed_model_ccdpp(const model_problem *P, uint32_t k, double lambda_d, int maxiter, int maxinner, int storage,
                      int refresh_every, int refresh_all, int threads, float *W, float *H, double *rmse) {
    const int64_t m = P->m, n = P->n, N = P->nnz;
    const float lambda = (float)lambda_d;
    if (threads > 0) omp_set_num_threads(threads);
    float *r = (float *)malloc(sizeof(float) * (size_t)(N > 0 ? N : 1));
    uint32_t *from_csc = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(N > 0 ? N : 1));
    uint32_t *next = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    if (!r || !from_csc || !next) { free(r); free(from_csc); free(next); return -1; }
    /* CSC position -> CSR position (rows ascend inside a column) */
    memcpy(next, P->csc_col_ptr, sizeof(uint32_t) * (size_t)n);
    for (int64_t i = 0; i < m; ++i)
        for (uint32_t p = P->csr_row_ptr[i]; p < P->csr_row_ptr[i + 1]; ++p) {
            const uint32_t j = P->csr_col_idx[p], q = next[j]++;
            if (q >= P->csc_col_ptr[j + 1] || P->csc_row_idx[q] != (uint32_t)i) {
                free(r); free(from_csc); free(next);
                return -1;
            }
            from_csc[q] = p;
        }
    free(next);
    for (int64_t p = 0; p < N; ++p) r[p] = store(P->csr_val[p], storage);
    memset(H, 0, sizeof(float) * (size_t)k * (size_t)n);
    int pending = -1, since_refresh = 0;
    for (int oiter = 1; oiter <= maxiter; ++oiter) {
        if (oiter > 1 && storage != 0) {
            refresh(P, storage, k, W, H, r);
            pending = -1;
            since_refresh = 0;
        }
        for (uint32_t t = 0; t < k; ++t) {
            if ((oiter == 1 || refresh_all) && storage != 0 && refresh_every > 0 && since_refresh >= refresh_every) {
                refresh(P, storage, k, W, H, r);
                pending = -1;
                since_refresh = 0;
            }
            float *Wt = W + (size_t)t * m, *Ht = H + (size_t)t * n;
            const float *Wp = pending >= 0 ? W + (size_t)pending * m : NULL;
            const float *Hp = pending >= 0 ? H + (size_t)pending * n : NULL;
#pragma omp parallel for schedule(dynamic, 256)
            for (int64_t i = 0; i < m; ++i)
                for (uint32_t p = P->csr_row_ptr[i]; p < P->csr_row_ptr[i + 1]; ++p) {
                    const uint32_t j = P->csr_col_idx[p];
                    float x = r[p];
                    if (Wp) x = x - Wp[i] * Hp[j];
                    if (oiter > 1) x = x + Wt[i] * Ht[j];
                    r[p] = store(x, storage);
                }
            for (int it = 0; it < maxinner; ++it) {
#pragma omp parallel for schedule(dynamic, 64)
                for (int64_t j = 0; j < n; ++j) {
                    const uint32_t b = P->csc_col_ptr[j], e = P->csc_col_ptr[j + 1];
                    if (b == e) { Ht[j] = 0.0f; continue; }
                    float g = 0.0f, h = lambda * (float)(e - b);
                    for (uint32_t q = b; q < e; ++q) {
                        const float y = Wt[P->csc_row_idx[q]];
                        g += y * r[from_csc[q]];
                        h += y * y;
                    }
                    Ht[j] = g / h;
                }
#pragma omp parallel for schedule(dynamic, 256)
                for (int64_t i = 0; i < m; ++i) {
                    const uint32_t b = P->csr_row_ptr[i], e = P->csr_row_ptr[i + 1];
                    if (b == e) { Wt[i] = 0.0f; continue; }
                    float g = 0.0f, h = lambda * (float)(e - b);
                    for (uint32_t p = b; p < e; ++p) {
                        const float y = Ht[P->csr_col_idx[p]];
                        g += y * r[p];
                        h += y * y;
                    }
                    Wt[i] = g / h;
                }
            }
            pending = (int)t;
            since_refresh++;
        }
        if (rmse) rmse[oiter - 1] = test_rmse(P, k, W, H);
    }
    free(r);
    free(from_csc);
    return 0;
}
