/*
 * CPU oracle for the CCD++ hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the algorithm of the reference's OpenMP
 * engine `cdmf_ref` (src/cdmf_ref.cpp) and of its test-RMSE helper
 * `calculate_rmse_directly` (src/tools.cpp:543-582).  The parity tests,
 * `__graft_entry__.smoke()` and the `cpu_baseline` leg of `bench.py` compare
 * the CUDA engine against it.  Nothing in the product
 * (the `cdmf_gb300` package, `libcdmf_cuda.so`, the `cdmf` CLI) links or
 * calls it.
 *
 * Build: `make -C oracle` gives liboracle_f32.so (VT = float, the reference's
 * `-DVALUE_TYPE=float`, CMakeLists.txt:15) and liboracle_f64.so (VT = double:
 * the FP64 oracle; inputs are read as float32 and widened, which is what the
 * stock FP64 build of the reference fails to do, src/pmf_util.h:92,137).
 * Always compiled with -ffp-contract=off: the reference's x86-64 build has no
 * FMA instructions (baseline ISA), so every `a += b * c` there rounds twice;
 * the flag keeps that rounding on aarch64 hosts too, where GCC would
 * otherwise contract to FMA.
 *
 * Pinned against the reference itself: oracle/build_ref.sh compiles the
 * reference's own src/cdmf_ref.cpp + src/tools.cpp into oracle/_ref, and
 * tests/golden/make_golden.py checks this restatement bit for bit against it
 * and stores the reference's outputs as golden vectors under tests/golden/.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#ifndef ORACLE_VT
#define ORACLE_VT float
#endif
typedef ORACLE_VT VT;

/* Same field order as `cdmf_problem` in include/cdmf_cuda.h. */
typedef struct {
    int64_t m, n, nnz;
    const uint32_t *csr_row_ptr, *csr_col_idx;
    const float *csr_val;
    const uint32_t *csc_col_ptr, *csc_row_idx;
    const float *csc_val;
    int64_t nnz_test;
    const uint32_t *test_row, *test_col;
    const float *test_val;
} oracle_problem;

/* One sweep line: src/cdmf_ref.cpp:7-17 (RankOneUpdate).  `lam` is already
 * lambda * nnz_j (src/cdmf_ref.cpp:98,106); h starts from it and the squares
 * are added in index order. */
static VT rank_one_update(const uint32_t *ptr, const uint32_t *idx, const VT *val,
                          int64_t j, const VT *u, VT lam) {
    VT g = 0, h = lam;
    if (ptr[j + 1] == ptr[j]) return 0;
    for (uint32_t p = ptr[j]; p < ptr[j + 1]; ++p) {
        uint32_t i = idx[p];
        g += u[i] * val[p];
        h += u[i] * u[i];
    }
    return g / h;
}

/* src/cdmf_ref.cpp:19-44 (UpdateRating): val[p] +=/-= Wt[idx[p]] * Ht[c] over
 * every line c of a compressed copy.  The loss it also returns is unused by
 * the reference, so it is not computed here. */
static void update_rating(const uint32_t *ptr, const uint32_t *idx, VT *val, int64_t lines,
                          const VT *Wt, const VT *Ht, int add) {
    if (add) {
#pragma omp parallel for schedule(dynamic, 500)
        for (int64_t c = 0; c < lines; ++c) {
            VT Htc = Ht[c];
            for (uint32_t p = ptr[c]; p < ptr[c + 1]; ++p) val[p] += Wt[idx[p]] * Htc;
        }
    } else {
#pragma omp parallel for schedule(dynamic, 500)
        for (int64_t c = 0; c < lines; ++c) {
            VT Htc = Ht[c];
            for (uint32_t p = ptr[c]; p < ptr[c + 1]; ++p) val[p] -= Wt[idx[p]] * Htc;
        }
    }
}

/* One outer iteration of src/cdmf_ref.cpp:74-125 on an explicit state.
 * W: k x m and H: k x n, feature-major (MatData X[t][i], src/pmf_util.h:8).
 * res_csc is R.csc_val_ (the residual in CSC order), res_csr is R.csr_val_
 * (= Rt.csc_val_ of the shallow transpose, src/pmf_util.h:38-53).
 * rank_s / update_s receive the reference's two phase timers. */
int oracle_outer_iteration(const oracle_problem *P, uint32_t k, double lambda_d, int maxinner,
                           int oiter, int threads, VT *W, VT *H, VT *res_csc, VT *res_csr,
                           double *rank_s, double *update_s) {
    const int64_t m = P->m, n = P->n;
    const VT lambda = (VT)lambda_d;
    if (threads > 0) omp_set_num_threads(threads);
    VT *u = (VT *)malloc(sizeof(VT) * (size_t)(m > 0 ? m : 1));
    VT *v = (VT *)malloc(sizeof(VT) * (size_t)(n > 0 ? n : 1));
    if (!u || !v) { free(u); free(v); return -1; }
    double t_rank = 0, t_update = 0;
    for (uint32_t t = 0; t < k; ++t) {
        double start = omp_get_wtime();
        VT *Wt = W + (size_t)t * m;
        VT *Ht = H + (size_t)t * n;
#pragma omp parallel for
        for (int64_t i = 0; i < m; ++i) u[i] = Wt[i];
#pragma omp parallel for
        for (int64_t i = 0; i < n; ++i) v[i] = Ht[i];
        if (oiter > 1) {                               /* src/cdmf_ref.cpp:86-89 */
            update_rating(P->csc_col_ptr, P->csc_row_idx, res_csc, n, Wt, Ht, 1);
            update_rating(P->csr_row_ptr, P->csr_col_idx, res_csr, m, Ht, Wt, 1);
        }
        t_update += omp_get_wtime() - start;
        for (int iter = 1; iter <= maxinner; ++iter) {  /* src/cdmf_ref.cpp:93-110 */
            start = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 500)
            for (int64_t c = 0; c < n; ++c) {
                VT lam = lambda * (VT)(P->csc_col_ptr[c + 1] - P->csc_col_ptr[c]);
                v[c] = rank_one_update(P->csc_col_ptr, P->csc_row_idx, res_csc, c, u, lam);
            }
            t_rank += omp_get_wtime() - start;
            start = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 500)
            for (int64_t c = 0; c < m; ++c) {
                VT lam = lambda * (VT)(P->csr_row_ptr[c + 1] - P->csr_row_ptr[c]);
                u[c] = rank_one_update(P->csr_row_ptr, P->csr_col_idx, res_csr, c, v, lam);
            }
            t_rank += omp_get_wtime() - start;
        }
        start = omp_get_wtime();
#pragma omp parallel for
        for (int64_t i = 0; i < m; ++i) Wt[i] = u[i];
#pragma omp parallel for
        for (int64_t i = 0; i < n; ++i) Ht[i] = v[i];
        update_rating(P->csc_col_ptr, P->csc_row_idx, res_csc, n, u, v, 0);   /* :120 */
        update_rating(P->csr_row_ptr, P->csr_col_idx, res_csr, m, v, u, 0);   /* :121 */
        t_update += omp_get_wtime() - start;
    }
    free(u);
    free(v);
    if (rank_s) *rank_s = t_rank;
    if (update_s) *update_s = t_update;
    return 0;
}

/* src/tools.cpp:543-582 (calculate_rmse_directly, CCD layout): float
 * products W[t][i]*H[t][j] summed in double in t order, NaN terms skipped but
 * counted.  Returns -1 for an empty test set (the reference exits there). */
double oracle_rmse(const oracle_problem *P, uint32_t k, const VT *W, const VT *H) {
    double rmse = 0;
    int64_t num = 0;
    for (int64_t e = 0; e < P->nnz_test; ++e) {
        uint32_t i = P->test_row[e], j = P->test_col[e];
        double v = P->test_val[e];
        double pred = 0;
        for (uint32_t t = 0; t < k; ++t) pred += W[(size_t)t * P->m + i] * H[(size_t)t * P->n + j];
        double tmp = (pred - v) * (pred - v);
        if (!isnan(tmp)) rmse += tmp;
        num++;
    }
    if (num == 0) return -1.0;
    return sqrt(rmse / (double)num);
}

/* The whole engine, src/cdmf_ref.cpp:47-140.  W (k x m) is in/out, H (k x n)
 * is output only (zeroed first, :57-61).  Optional outputs: rmse[maxiter]
 * (the value of the :135 log line), W_hist/H_hist (maxiter snapshots of
 * W/H after each outer iteration), res_csc/res_csr (the final residuals),
 * times[2*maxiter] (rank_time, update_time per outer iteration). */
int oracle_ccdpp(const oracle_problem *P, uint32_t k, double lambda, int maxiter, int maxinner,
                 int threads, VT *W, VT *H, double *rmse, VT *W_hist, VT *H_hist,
                 VT *res_csc_out, VT *res_csr_out, double *times) {
    const int64_t m = P->m, n = P->n, N = P->nnz;
    VT *rc = res_csc_out, *rr = res_csr_out;
    VT *own_c = NULL, *own_r = NULL;
    if (!rc) rc = own_c = (VT *)malloc(sizeof(VT) * (size_t)(N > 0 ? N : 1));
    if (!rr) rr = own_r = (VT *)malloc(sizeof(VT) * (size_t)(N > 0 ? N : 1));
    if (!rc || !rr) { free(own_c); free(own_r); return -1; }
    for (int64_t p = 0; p < N; ++p) { rc[p] = (VT)P->csc_val[p]; rr[p] = (VT)P->csr_val[p]; }
    for (size_t q = 0; q < (size_t)k * n; ++q) H[q] = 0;
    int rc_status = 0;
    for (int oiter = 1; oiter <= maxiter; ++oiter) {
        double tr = 0, tu = 0;
        if (oracle_outer_iteration(P, k, lambda, maxinner, oiter, threads, W, H, rc, rr, &tr, &tu)) {
            rc_status = -1;
            break;
        }
        if (times) { times[2 * (oiter - 1)] = tr; times[2 * (oiter - 1) + 1] = tu; }
        if (rmse) rmse[oiter - 1] = P->nnz_test > 0 ? oracle_rmse(P, k, W, H) : -1.0;
        if (W_hist) memcpy(W_hist + (size_t)(oiter - 1) * k * m, W, sizeof(VT) * (size_t)k * m);
        if (H_hist) memcpy(H_hist + (size_t)(oiter - 1) * k * n, H, sizeof(VT) * (size_t)k * n);
    }
    free(own_c);
    free(own_r);
    return rc_status;
}

/* Widening helper for the FP64 build: copies float32 factors into VT. */
void oracle_widen(const float *src, VT *dst, int64_t count) {
    for (int64_t q = 0; q < count; ++q) dst[q] = (VT)src[q];
}

int oracle_value_bytes(void) { return (int)sizeof(VT); }
