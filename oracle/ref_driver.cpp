// Driver that exposes the reference's own CPU engine through a C entry
// point -- oracle build only (oracle/_ref/libcdmf_ref.so).
//
// It is compiled together with the reference's unmodified src/cdmf_ref.cpp
// and src/tools.cpp (see oracle/build_ref.sh) and does what src/main.cpp:
// 28-36 and :82-90 do, except that the initial W is injected instead of
// drawn by initial_col, so both the oracle and the CUDA engine start from
// the same factors.
#include "tools.h"
#include "cdmf.h"

extern "C" int ref_dims(const char* dir, long* m, long* n, unsigned long* nnz, unsigned long* nnz_test) {
    SparseMatrix R;
    TestData T;
    load(dir, R, T);                      // src/tools.cpp:271
    *m = R.rows;
    *n = R.cols;
    *nnz = R.nnz;
    *nnz_test = T.nnz;
    return 0;
}

// Runs cdmf_ref (src/cdmf_ref.cpp:47) on the cdmf-format directory `dir`.
// W_init/W_out: k*m feature-major, H_out: k*n.  rmse_out receives
// calculate_rmse_directly of the final factors (src/tools.cpp:543), which is
// the RMSE the reference prints after its last outer iteration.
// res_csc_out/res_csr_out (nullable) receive the final residual copies.
extern "C" int ref_run(const char* dir, unsigned k, float lambda, int maxiter, int maxinner, int threads,
                       const float* W_init, float* W_out, float* H_out, double* rmse_out,
                       float* res_csc_out, float* res_csr_out) {
    SparseMatrix R;
    TestData T;
    load(dir, R, T);
    parameter param;
    param.k = k;
    param.lambda = lambda;
    param.maxiter = maxiter;
    param.maxinneriter = maxinner;
    param.threads = threads;
    MatData W(k, VecData(R.rows)), H(k, VecData(R.cols));
    for (unsigned t = 0; t < k; ++t)
        for (long i = 0; i < R.rows; ++i) W[t][i] = W_init[(size_t)t * R.rows + i];
    cdmf_ref(R, W, H, T, param);
    for (unsigned t = 0; t < k; ++t) {
        for (long i = 0; i < R.rows; ++i) W_out[(size_t)t * R.rows + i] = W[t][i];
        for (long j = 0; j < R.cols; ++j) H_out[(size_t)t * R.cols + j] = H[t][j];
    }
    if (rmse_out) *rmse_out = T.nnz ? calculate_rmse_directly(W, H, T, k, false) : -1.0;
    if (res_csc_out)
        for (unsigned long p = 0; p < R.nnz; ++p) res_csc_out[p] = R.get_csc_val()[p];
    if (res_csr_out)
        for (unsigned long p = 0; p < R.nnz; ++p) res_csr_out[p] = R.get_csr_val()[p];
    return 0;
}

// The reference's own initial_col (src/tools.cpp:349): srand(0) then
// 0.1*rand()/RAND_MAX + 0.001, i outer, t inner.
extern "C" void ref_initial_col(float* X, unsigned k, unsigned n) {
    MatData M;
    initial_col(M, k, n);
    for (unsigned t = 0; t < k; ++t)
        for (unsigned i = 0; i < n; ++i) X[(size_t)t * n + i] = M[t][i];
}
