/*
 * cdmf_cuda.h -- C ABI of the GB300 (sm_103a) CCD++ engine.
 *
 * Drop-in for the reference's OpenCL engines (src/cdmf.h:4-10):
 *   void cdmf_ocl_01(SparseMatrix& R, MatData& W, MatData& H, TestData& T,
 *                    parameter& p, char filename[]);          src/cdmf.h:8
 *   void cdmf_ocl_02(...same...);                              src/cdmf.h:6
 *   void cdmf_csr5(SparseMatrix& R, MatData& W, MatData& H,
 *                  parameter& p, char filename[]);             src/cdmf.h:10
 * called from src/main.cpp:43,50,57.  The C++ types become plain pointers:
 *   SparseMatrix (src/pmf_util.h:13-114)  -> cdmf_problem CSR + CSC arrays
 *   TestData     (src/pmf_util.h:117-161) -> cdmf_problem test COO arrays
 *   MatData W, H (src/pmf_util.h:8)       -> float[k*m], float[k*n], feature-major
 *                                            (W[t*m + i] == W_c[t][i], as the
 *                                            reference flattens it, src/cdmf_ocl_1.cpp:70-82)
 *   parameter    (src/pmf.h:4-26)         -> cdmf_opts
 *
 * Semantics kept from the reference:
 *   - host R is never modified (the GPU engines copy it, src/cdmf_ocl_1.cpp:101-133);
 *   - W is in/out, H is output only and starts from zero (src/cdmf_ocl_1.cpp:64-68);
 *   - the test set is read-only; the test RMSE after each outer iteration is
 *     the value of the reference's "[-INFO-] iteration num" line
 *     (src/cdmf_ref.cpp:130-136, src/cdmf_ocl_1.cpp:357-381).
 * Changed on purpose: errors are returned as negative status codes instead of
 * abort()/exit() (src/util.h:20-22, src/main.cpp:60-63); the library never
 * terminates the process.
 *
 * Threading: a handle belongs to the thread that uses it; distinct handles
 * may be used from distinct threads.  All pointers passed to create/train are
 * borrowed for the duration of the call only.
 */
#ifndef CDMF_CUDA_H
#define CDMF_CUDA_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: 0 = OK, negative = error. */
#define CDMF_OK 0
#define CDMF_ERR_INVALID (-1)      /* bad argument or inconsistent sparse structure */
#define CDMF_ERR_ALLOC (-2)        /* host or device allocation failed */
#define CDMF_ERR_CUDA (-3)         /* CUDA runtime error (see cdmf_cuda_last_error) */
#define CDMF_ERR_NO_DEVICE (-4)    /* no usable CUDA device */
#define CDMF_ERR_EMPTY_TEST (-5)   /* RMSE asked for with an empty test set (src/tools.cpp:576 exits) */
#define CDMF_ERR_NUMERIC (-6)      /* residual drift / non-finite factors reported by a device check */
#define CDMF_ERR_UNSUPPORTED (-7)  /* option combination not supported */
#define CDMF_ERR_TOO_LARGE (-8)    /* size beyond a stated limit */

/* Residual storage precision (cdmf_opts.residual). */
#define CDMF_RES_F32 0
#define CDMF_RES_BF16 1
#define CDMF_RES_F16 2

/* Reduction order (cdmf_opts.reduce). */
#define CDMF_REDUCE_TREE 0        /* parallel, deterministic fixed-shape tree */
#define CDMF_REDUCE_SEQUENTIAL 1  /* every line summed by one thread in index order:
                                     the reference's order (src/cdmf_ref.cpp:10-14) */

/* SparseMatrix + TestData (src/pmf_util.h:13-161) as plain arrays.
 * CSR: csr_row_ptr[m+1], csr_col_idx[nnz], csr_val[nnz];
 * CSC: csc_col_ptr[n+1], csc_row_idx[nnz], csc_val[nnz] -- the same matrix;
 * indices inside a line ascending (scipy canonical order).
 * Test COO: test_row/test_col/test_val[nnz_test], 0-based. */
typedef struct {
    int64_t m, n, nnz;
    const uint32_t *csr_row_ptr, *csr_col_idx;
    const float *csr_val;
    const uint32_t *csc_col_ptr, *csc_row_idx;
    const float *csc_val;
    int64_t nnz_test;
    const uint32_t *test_row, *test_col;
    const float *test_val;
} cdmf_problem;

/* parameter (src/pmf.h:4-26) plus the engine's own knobs. */
typedef struct {
    uint32_t k;               /* rank (-k, default 10) */
    float lambda;             /* regularisation (-l, default 0.1) */
    int32_t maxiter;          /* outer iterations (-t, default 5) */
    int32_t maxinneriter;     /* inner iterations (-T, default 5) */
    int32_t version;          /* -V: 1 and 2 = row-length-binned sweeps, 3 = nnz-balanced tiles */
    int32_t residual;         /* CDMF_RES_* */
    int32_t reduce;           /* CDMF_REDUCE_* */
    int32_t rmse_each_outer;  /* 1: test RMSE after every outer iteration, as the reference */
    int32_t use_graph;        /* 1: replay each outer iteration as one CUDA graph */
    int32_t threads_per_block;/* -nThreadsPerBlock; 0 = engine default (256) */
    int32_t device;           /* CUDA device ordinal */
    int32_t verbose;
    int32_t relabel;          /* 1: renumber rows and columns by degree inside the engine
                                 (tree order only; results come back in the caller's numbering),
                                 built on the GPU for the line layout; 2: the same numbering
                                 built on the host */
    int32_t autotune;         /* 1: pick the bin thresholds by timing candidates on this matrix
                                 at create (cached per matrix shape in the process) */
    int32_t layout;           /* CDMF_LAYOUT_*: how the residual copies are stored (tree order) */
} cdmf_opts;

/* Residual copy layout (cdmf_opts.layout). */
#define CDMF_LAYOUT_LINES 0    /* CSR / CSC as given; row-length-binned sweeps */
#define CDMF_LAYOUT_BLOCKED 1  /* cross-index blocks: gather tables staged in shared memory,
                                  16-bit indices; used with tree order only */

/* Line-length bin thresholds of the binned sweeps (versions 1/2), in
 * nonzeros: <= thread_max one thread per line, <= group_max 8 lanes,
 * <= warp_max a warp, <= cta_max a CTA, above: split in chunks of `chunk`. */
typedef struct {
    uint32_t thread_max, group_max, warp_max, cta_max, chunk;
} cdmf_bincfg;

/* Engine timings and counters of the most recent cdmf_cuda_run/train. */
typedef struct {
    double train_ms;          /* CUDA-event time of the whole run on the engine stream */
    double sweep_csc_ms;      /* sum of CSC (h_t) sweep kernel times   (profiling on) */
    double sweep_csr_ms;      /* sum of CSR (w_t) sweep kernel times   (profiling on) */
    double rmse_ms;           /* sum of test-RMSE kernel times         (profiling on) */
    double refresh_ms;        /* sum of residual refresh kernel times  (profiling on) */
    int64_t launches;         /* kernels launched by the run */
    int64_t sweep_csc_launches, sweep_csr_launches, rmse_launches, refresh_launches;
    int64_t updates;          /* rank-one updates performed (outer iterations x k) */
    double bytes_per_update;  /* compulsory HBM bytes of one rank-one update */
    double drift_rms;         /* 16-bit modes: RMS of (exact - stored) residual at the last refresh, FP64 */
    int64_t nonfinite;        /* 16-bit modes: non-finite residuals found at the last refresh */
} cdmf_stats;

typedef struct cdmf_handle cdmf_handle;

/* Called after every outer iteration: the reference's log-line values.
 * train_ms_so_far: device time since the first outer iteration started. */
typedef void (*cdmf_outer_cb)(int oiter, double rmse, double train_ms_so_far, void* user);

/* The reference's defaults (src/pmf.h:4-26: k 10, lambda 0.1, 5 x 5
 * iterations, version 1) and the engine's for the rest. */
void cdmf_opts_default(cdmf_opts* o);
const char* cdmf_cuda_strerror(int status);
int cdmf_cuda_version(void);

/* One call = the reference engine call (cdmf_ocl_01 / cdmf_ocl_02 / cdmf_csr5,
 * src/cdmf.h:6-10, called at src/main.cpp:43,50,57): upload, H := 0
 * (src/cdmf_ocl_1.cpp:64-68), maxiter outer iterations from the given W,
 * download W and H.  Each outer iteration is queued before the previous
 * one's RMSE is read back, so cb runs while the GPU works on the next one.
 * rmse_out (nullable) receives maxiter values when opts->rmse_each_outer.
 * A non-finite residual met by a refresh ends the call with
 * CDMF_ERR_NUMERIC; W and H are then left as they were. */
int cdmf_cuda_train(const cdmf_problem* p, const cdmf_opts* o, float* W, float* H,
                    double* rmse_out, cdmf_outer_cb cb, void* user);

/* Test RMSE of given factors over a test COO with double values: the
 * reference's calculate_rmse of the text test file (src/tools.cpp:489-541,
 * values parsed with %lf, indices already 0-based).  Host pointers; the
 * prediction and reduction run on `device`.  nan_count (nullable) receives
 * the number of NaN terms, which are skipped in the sum but counted in the
 * mean, as the reference does. */
int cdmf_cuda_rmse_coo(uint32_t k, int64_t m, int64_t n, const float* W, const float* H, int64_t nnz_test,
                       const uint32_t* test_row, const uint32_t* test_col, const double* test_val, int device,
                       double* rmse, int64_t* nan_count);

/* Test RMSE on device arrays without any allocation by the library.  It has
 * no counterpart in the reference.  It serves callers that cannot let a
 * library call cudaMalloc: a serving process that hands out every byte of
 * device memory from its own pool (a library allocation would sit outside
 * that pool's accounting and can fail once the pool holds the memory), or a
 * runtime whose device memory budget is fixed when it starts.  W (k x m),
 * H (k x n), test_row/test_col/test_val (nnz_test) are DEVICE pointers the
 * caller owns, indices 0-based and in range; rmse and nan_count are host
 * pointers.  Same arithmetic and result as cdmf_cuda_rmse_coo.  The kernel's
 * scratch is a fixed file-scope device array of about 5 KB (608 block
 * partials and three counters), held by every device that loads the library
 * until exit and shared by all calls: calls that overlap on the GPU race on
 * it, so the caller serialises them.  The first call on a device looks up the
 * array's device address and keeps it; do not call again on a device after
 * resetting it (cudaDeviceReset), which moves the array.  Test sets larger than
 * CDMF_NOALLOC_MAX_TEST entries (the reference counts entries in an int) are
 * rejected with CDMF_ERR_TOO_LARGE.  stream: a cudaStream_t, or NULL for the
 * default stream; the call copies the result to host memory and waits for
 * its own work before it returns. */
#define CDMF_NOALLOC_MAX_TEST 2147483647LL
int cdmf_cuda_rmse_coo_noalloc(uint32_t k, int64_t m, int64_t n, const float* W, const float* H, int64_t nnz_test,
                               const uint32_t* test_row, const uint32_t* test_col, const double* test_val,
                               void* stream, double* rmse, int64_t* nan_count);

/* Handle API: the same engine split into upload / run / read-back.  No single
 * reference counterpart: the reference's engine functions (src/cdmf.h:6-10)
 * do all of this in one call; the split serves one-step parity checks,
 * repeated runs on one upload, and the benchmark. */
int cdmf_cuda_create(const cdmf_problem* p, const cdmf_opts* o, cdmf_handle** out);
void cdmf_cuda_destroy(cdmf_handle* h);
const char* cdmf_cuda_last_error(const cdmf_handle* h);
/* Starts a fresh factorisation: W := W0, H := H0 (NULL = zero, as the
 * reference), both residual copies := the ratings, next outer iteration = 1. */
int cdmf_cuda_set_factors(cdmf_handle* h, const float* W0, const float* H0);
/* Runs n_outer further outer iterations.  rmse_out (nullable) gets one value
 * per iteration when rmse_each_outer is set. */
int cdmf_cuda_run(cdmf_handle* h, int n_outer, double* rmse_out);
int cdmf_cuda_get_factors(cdmf_handle* h, float* W, float* H);
/* Test RMSE of the current factors (src/tools.cpp:543-582). */
int cdmf_cuda_rmse(cdmf_handle* h, double* rmse);
/* FP64 training objective of the current state, a convergence monitor:
 * sq_residual = sum of r_ij^2 over the training nonzeros (the `loss` that
 * UpdateRating computes and discards, src/cdmf_ref.cpp:20-43), regularizer =
 * lambda * (sum_i nnz_i |w_i|^2 + sum_j nnz_j |h_j|^2) (the lambda scaling of
 * RankOneUpdate, src/cdmf_ref.cpp:7-17), objective = their sum.  Any output
 * may be NULL.  Applies a deferred subtract first, as get_state does. */
int cdmf_cuda_objective(cdmf_handle* h, double* sq_residual, double* regularizer, double* objective);
/* Full engine state for one-step parity: factors, both residual copies (in
 * CSC and CSR order, widened to float) and the next outer iteration number. */
int cdmf_cuda_get_state(cdmf_handle* h, float* W, float* H, float* res_csc, float* res_csr, int* next_oiter);
int cdmf_cuda_set_state(cdmf_handle* h, const float* W, const float* H, const float* res_csc,
                        const float* res_csr, int next_oiter);
int cdmf_cuda_set_profiling(cdmf_handle* h, int on);
int cdmf_cuda_stats(const cdmf_handle* h, cdmf_stats* s);
/* Bin thresholds: read (the CSR copy's), set (re-plans the bins of both
 * copies), or pick by timing three steady-state features per candidate on
 * this matrix (coordinate search over group_max, warp_max, cta_max and chunk,
 * first one plan for both copies, then the CSC copy's alone, and over the
 * lanes per group-bin line).  A new plan drops the outer iterations already
 * captured as CUDA graphs.  Autotuning uses the factors and residual as
 * scratch and leaves a fresh state (as cdmf_cuda_set_factors(h, NULL, NULL)).
 * Picks are kept per process for each (shape, residual type, numbering,
 * device).  Handles whose sweeps do not use the bins (reduce = sequential,
 * version 3, the blocked layout) are left as they are, with *best_ms = 0. */
int cdmf_cuda_get_bincfg(const cdmf_handle* h, cdmf_bincfg* c);
int cdmf_cuda_set_bincfg(cdmf_handle* h, const cdmf_bincfg* c);
int cdmf_cuda_autotune(cdmf_handle* h, cdmf_bincfg* chosen, double* best_ms);
/* Canonical CSR and CSC of a COO rating list, built on the GPU: the arrays
 * the reference's data/a/a_compress.py:130-155 writes with scipy's
 * tocsr()/tocsc() and src/tools.cpp:271-347 loads.  Entries are sorted by
 * (row, column); duplicate (row, column) pairs are summed in FP64 in input
 * order and stored as float; the CSC lists rows ascending inside each column.
 * All arrays are host memory.  csr_idx, csr_val, csc_idx and csc_val must hold
 * nnz entries; *nnz_out receives the number of distinct entries (<= nnz).
 * An index outside [0, m) x [0, n) returns CDMF_ERR_INVALID. */
int cdmf_cuda_compress(int64_t m, int64_t n, int64_t nnz, const uint32_t* rows, const uint32_t* cols,
                       const double* vals, int device, uint32_t* csr_ptr, uint32_t* csr_idx, float* csr_val,
                       uint32_t* csc_ptr, uint32_t* csc_idx, float* csc_val, int64_t* nnz_out);
/* Dual SpMV handle for callers of the reference's CSR5 library
 * (anonymouslibHandle, src/anonymouslib_opencl.h:11-26, as driven by
 * src/cdmf_csr5.cpp:205-286).  All matrix and vector arrays are the caller's
 * device memory and must stay alive while the handle uses them.
 *   cdmf_spmv_create(m, n)                 anonymouslibHandle(m, n) + device
 *   cdmf_spmv_input_csr(nnz, ptr, idx, val)  inputCSR (row pointers checked)
 *   cdmf_spmv_as_csr5 / cdmf_spmv_as_csr    asCSR5 (plans the load-balanced
 *                                          work, checks column indices) / asCSR
 *   cdmf_spmv_set_x(x)                     setX
 *   cdmf_spmv_run(alpha, y_t, y_b, ms)     spmv: y_t[i] = sum_j val_ij x[col_j],
 *                                          y_b[i] = sum_j x[col_j]^2; alpha is not
 *                                          applied, as in the reference kernel
 *                                          (csr5_spmv.cl:135-147); returns
 *                                          CDMF_ERR_UNSUPPORTED in CSR form, as the
 *                                          reference returns ANONYMOUSLIB_UNSUPPORTED_CSR_SPMV.
 * Sums run in a fixed order: repeated calls give identical bits. */
typedef struct cdmf_spmv cdmf_spmv;
int cdmf_spmv_create(int64_t m, int64_t n, int device, cdmf_spmv** out);
void cdmf_spmv_destroy(cdmf_spmv* s);
const char* cdmf_spmv_last_error(const cdmf_spmv* s);
int cdmf_spmv_input_csr(cdmf_spmv* s, int64_t nnz, const uint32_t* row_ptr, const uint32_t* col_idx,
                        const float* val);
int cdmf_spmv_as_csr5(cdmf_spmv* s);
int cdmf_spmv_as_csr(cdmf_spmv* s);
int cdmf_spmv_set_x(cdmf_spmv* s, const float* x);
int cdmf_spmv_run(cdmf_spmv* s, float alpha, float* y_t, float* y_b, double* ms);
/* Page-locked host memory for inputs and outputs of cdmf_cuda_train /
 * create / get_factors (copies from it run at full link speed).  NULL on
 * failure. */
void* cdmf_cuda_host_alloc(uint64_t bytes);
void cdmf_cuda_host_free(void* p);
/* Row-length bins of the two sweeps: counts[5] of lines per bin
 * (thread, 8-lane group, warp, CTA, split) and nnz[5] for CSR (which=0) or
 * CSC (which=1). */
int cdmf_cuda_bins(const cdmf_handle* h, int which, int64_t counts[5], int64_t nnz[5]);

/* ---- Batches of independent factorisations --------------------------------
 * No counterpart in the reference (which runs one problem per process).
 * nprob problems of uneven sizes, each with its own k and lambda, each run by
 * its own engine on its own CUDA stream with its single-problem schedule; a
 * batched run issues all problems' outer iterations together so that the GPU
 * overlaps their kernels, and with opts[0].use_graph it is captured once as
 * one CUDA graph (a branch per problem) and replayed after.  Results are
 * bit-identical to running each problem alone.  All problems must share
 * device, residual, reduce and maxinneriter.  W0/W/H are arrays of nprob
 * pointers (k_q x m_q, k_q x n_q).  rmse_out holds nprob x n_outer values
 * (problem-major). */
typedef struct cdmf_batch cdmf_batch;
int cdmf_cuda_batch_create(const cdmf_problem* probs, const cdmf_opts* opts, int nprob, cdmf_batch** out);
void cdmf_cuda_batch_destroy(cdmf_batch* b);
const char* cdmf_cuda_batch_last_error(const cdmf_batch* b);
int cdmf_cuda_batch_set_factors(cdmf_batch* b, const float* const* W0);
int cdmf_cuda_batch_run(cdmf_batch* b, int n_outer, double* rmse_out);
/* The same problems run one after another through their own handles (each
 * run finished before the next starts, launches issued eagerly), timed on the
 * host clock of the batch stream: the comparison point for
 * cdmf_cuda_batch_run. */
int cdmf_cuda_batch_run_sequential(cdmf_batch* b, int n_outer, double* rmse_out, double* ms_out);
int cdmf_cuda_batch_get_factors(cdmf_batch* b, float* const* W, float* const* H);
int cdmf_cuda_batch_stats(const cdmf_batch* b, cdmf_stats* s);

#ifdef __cplusplus
}
#endif
#endif
