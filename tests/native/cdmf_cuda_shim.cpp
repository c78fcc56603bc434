// cdmf_cuda_shim.cpp -- the translation unit a maintainer of cdmf adds as
// src/cdmf_cuda_shim.cpp; links against libcdmf_cuda.so.  It keeps the shape of
// the reference's engine calls (src/cdmf.h:4-10) and prints the reference's
// per-iteration log line (src/cdmf_ocl_1.cpp:380).
#include "tools.h"
#include "cdmf.h"
#include <cdmf_cuda.h>

void cdmf_cuda(SparseMatrix& R, MatData& W_c, MatData& H_c, TestData& T, parameter& param) {
    cdmf_problem p;
    p.m = R.rows;  p.n = R.cols;  p.nnz = (int64_t)R.nnz;
    p.csr_row_ptr = R.get_csr_row_ptr();  p.csr_col_idx = R.get_csr_col_indx();  p.csr_val = R.get_csr_val();
    p.csc_col_ptr = R.get_csc_col_ptr();  p.csc_row_idx = R.get_csc_row_indx();  p.csc_val = R.get_csc_val();
    p.nnz_test = (int64_t)T.nnz;
    p.test_row = T.getTestRow();  p.test_col = T.getTestCol();  p.test_val = T.getTestVal();
    cdmf_opts o;
    cdmf_opts_default(&o);
    o.k = param.k;  o.lambda = param.lambda;  o.maxiter = param.maxiter;
    o.maxinneriter = param.maxinneriter;  o.version = param.version;
    std::vector<float> W((size_t)param.k * R.rows), H((size_t)param.k * R.cols);
    for (unsigned t = 0; t < param.k; ++t)
        std::copy(W_c[t].begin(), W_c[t].end(), W.begin() + (size_t)t * R.rows);
    int st = cdmf_cuda_train(&p, &o, W.data(), H.data(), nullptr,
        [](int it, double rmse, double ms, void*) {
            printf("[-INFO-] iteration num %d \trank_time %.4lf|%.4lf s \tupdate_time %.4lf|%.4lfs \tRMSE=%f time:%fs\n",
                   it, 0.0, ms / 1e3, 0.0, 0.0, rmse, 0.0);
        }, nullptr);
    if (st != CDMF_OK) { fprintf(stderr, "%s\n", cdmf_cuda_strerror(st)); exit(EXIT_FAILURE); }
    for (unsigned t = 0; t < param.k; ++t) {
        std::copy(W.begin() + (size_t)t * R.rows, W.begin() + (size_t)(t + 1) * R.rows, W_c[t].begin());
        std::copy(H.begin() + (size_t)t * R.cols, H.begin() + (size_t)(t + 1) * R.cols, H_c[t].begin());
    }
}
