// `cdmf` -- the reference's command-line driver (src/main.cpp:7-122) on the
// GB300 engine.  Same flags, same log lines (scripts/grep_it.sh parses the
// "OCL Training time" and "Test RMSE" lines); -V 1/2/3 all reach the CUDA
// engine through include/cdmf_cuda.h.  -r 1 re-runs the engine in the
// reference's summation order (bit-identical to src/cdmf_ref.cpp) and runs
// the reference's 10 % golden_compare on the two results.
#include "cdmf_host.h"

#include <cdmf_cuda.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>

namespace {

struct LogState {
    double prev_ms = 0;
};

void log_outer(int oiter, double rmse, double ms_so_far, void* user) {
    LogState* s = (LogState*)user;
    const double step = (ms_so_far - s->prev_ms) / 1e3;
    s->prev_ms = ms_so_far;
    // rank_time holds the fused sweep time; the residual updates are fused
    // into the sweeps, so update_time is 0 (src/cdmf_ocl_1.cpp:380 format)
    printf("[-INFO-] iteration num %d \trank_time %.4lf|%.4lf s \tupdate_time %.4lf|%.4lfs \tRMSE=%f time:%fs\n",
           oiter, step, ms_so_far / 1e3, 0.0, 0.0, rmse, 0.0);
}

// Flattens MatData (as src/cdmf_ocl_1.cpp:70-82 does), trains, copies back.
int cdmf_cuda(SparseMatrix& R, MatData& W, MatData& H, TestData& T, parameter& param, int reduce) {
    cdmf_problem p;
    p.m = R.rows;
    p.n = R.cols;
    p.nnz = (int64_t)R.nnz;
    p.csr_row_ptr = R.csr_row_ptr.data();
    p.csr_col_idx = R.csr_col_indx.data();
    p.csr_val = R.csr_val.data();
    p.csc_col_ptr = R.csc_col_ptr.data();
    p.csc_row_idx = R.csc_row_indx.data();
    p.csc_val = R.csc_val.data();
    p.nnz_test = (int64_t)T.nnz;
    p.test_row = T.test_row.data();
    p.test_col = T.test_col.data();
    p.test_val = T.test_val.data();
    cdmf_opts o;
    cdmf_opts_default(&o);
    o.k = param.k;
    o.lambda = param.lambda;
    o.maxiter = param.maxiter;
    o.maxinneriter = param.maxinneriter;
    o.version = param.version;
    o.residual = param.residual;
    o.reduce = reduce;
    o.use_graph = param.graph;
    o.device = (int)param.platform_id;
    o.verbose = param.verbose;
    o.rmse_each_outer = T.nnz > 0;
    const unsigned k = param.k;
    std::vector<float> Wf((size_t)k * R.rows), Hf((size_t)k * R.cols, 0.0f);
    for (unsigned t = 0; t < k; ++t)
        for (long i = 0; i < R.rows; ++i) Wf[(size_t)t * R.rows + i] = W[t][i];
    LogState ls;
    auto t1 = std::chrono::high_resolution_clock::now();
    int st = cdmf_cuda_train(&p, &o, Wf.data(), Hf.data(), nullptr, log_outer, &ls);
    auto t2 = std::chrono::high_resolution_clock::now();
    if (st != CDMF_OK) {
        fprintf(stderr, "[FAILED] cdmf_cuda_train: %s\n", cdmf_cuda_strerror(st));
        return st;
    }
    std::chrono::duration<double> d = t2 - t1;
    printf("[INFO] OCL Training time: %lf s\n", d.count());
    // throughput of the whole call (upload, create, outer iterations, download)
    printf("[INFO] Rank-one updates/s: %.1f, outer iterations/s: %.2f (whole call)\n",
           (double)k * param.maxiter / d.count(), (double)param.maxiter / d.count());
    for (unsigned t = 0; t < k; ++t) {
        for (long i = 0; i < R.rows; ++i) W[t][i] = Wf[(size_t)t * R.rows + i];
        for (long j = 0; j < R.cols; ++j) H[t][j] = Hf[(size_t)t * R.cols + j];
    }
    return CDMF_OK;
}

}  // namespace

int main(int argc, char** argv) {
    auto t7 = std::chrono::high_resolution_clock::now();
    parameter param = parse_command_line(argc, argv);
    std::cout << "------------------------------------------------------" << std::endl;
    std::cout << "[info] Loading R matrix..." << std::endl;
    auto t3 = std::chrono::high_resolution_clock::now();
    SparseMatrix R;
    TestData T;
    if (!load(param.scr_dir, R, T)) return EXIT_FAILURE;
    auto t4 = std::chrono::high_resolution_clock::now();
    std::chrono::duration<double> d34 = t4 - t3;
    std::cout << "[info] Loading rating data time: " << d34.count() << "s.\n";
    std::cout << "------------------------------------------------------" << std::endl;
    MatData W, H, W_ref, H_ref;
    initial_col(W, param.k, R.rows);
    initial_col(H, param.k, R.cols);
    initial_col(W_ref, param.k, R.rows);
    initial_col(H_ref, param.k, R.cols);
    switch (param.version) {
        case 1: std::cout << "[info] Picked Version 1: Native" << std::endl; break;
        case 2:   // the binned sweeps of version 1; the line keeps the reference's prefix for its scripts
            std::cout << "[info] Picked Version 2: Thread Batching (the binned sweeps of version 1)" << std::endl;
            break;
        case 3: std::cout << "[info] Picked Version 3: Load Balancing" << std::endl; break;
        default: printf("[FAILED] Wrong version"); return EXIT_FAILURE;
    }
    if (cdmf_cuda(R, W, H, T, param, param.reduce) != CDMF_OK) return EXIT_FAILURE;
    if (param.do_predict == 1) {
        std::cout << "------------------------------------------------------" << std::endl;
        auto t5 = std::chrono::high_resolution_clock::now();
        if (!calculate_rmse(W, H, param.scr_dir, param.k, (int)param.platform_id)) return EXIT_FAILURE;
        auto t6 = std::chrono::high_resolution_clock::now();
        std::chrono::duration<double> d = t6 - t5;
        std::cout << "[info] OCL Predict Time: " << d.count() << " s.\n";
    }
    if (param.do_ref == 1) {
        std::cout << "------------------------------------------------------" << std::endl;
        std::cout << "[info] Computing cdmf results in the reference summation order." << std::endl;
        auto t9 = std::chrono::high_resolution_clock::now();
        if (cdmf_cuda(R, W_ref, H_ref, T, param, CDMF_REDUCE_SEQUENTIAL) != CDMF_OK) return EXIT_FAILURE;
        auto t10 = std::chrono::high_resolution_clock::now();
        std::chrono::duration<double> d = t10 - t9;
        std::cout << "[info] OMP Training Time: " << d.count() << " s.\n";
        std::cout << "------------------------------------------------------" << std::endl;
        std::cout << "[info] validate the results." << std::endl;
        golden_compare(W, W_ref, param.k, R.rows);
        golden_compare(H, H_ref, param.k, R.cols);
    }
    std::cout << "------------------------------------------------------" << std::endl;
    auto t8 = std::chrono::high_resolution_clock::now();
    std::chrono::duration<double> d78 = t8 - t7;
    std::cout << "Total Time: " << d78.count() << " s.\n";
    return EXIT_SUCCESS;
}
