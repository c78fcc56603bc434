/*
 * cdmf_synth.h -- seeded synthetic rating matrices in cdmf's in-memory layout.
 *
 * Replaces the reference's unseeded data generators and COO->CSR/CSC
 * converters (the data/a, data/b, data/c generator scripts and the
 * *_compress.py converters, data/a/a_compress.py:130-155).  The output
 * is the structure the reference's loader fills (src/pmf_util.h:18-36,
 * 121-144): CSR and CSC of the training matrix with 32-bit unsigned indices
 * and float32 values, row indices ascending inside each CSC column and
 * column indices ascending inside each CSR row (scipy's canonical order,
 * which data/a/a_compress.py:147-148 writes), plus the held-out test set as
 * COO in row-major order.
 *
 * Results depend only on the spec (seed included), not on the thread count
 * or the host architecture's integer behaviour.
 */
#ifndef CDMF_SYNTH_H
#define CDMF_SYNTH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t m, n;            /* users (rows) x items (columns) */
    int64_t nnz_total;       /* distinct nonzeros before the test split (row_mode 0) */
    int64_t nnz_test;        /* entries held out; < 0: use test_fraction */
    double test_fraction;
    int32_t row_mode;        /* 0: capped Zipf degrees summing to nnz_total; 1: uniform in [row_min,row_max] */
    double row_alpha;        /* Zipf exponent of the row rank weights (row_mode 0) */
    int64_t row_min, row_max;
    int32_t col_mode;        /* 0: capped Zipf column weights; 1: Beta(col_beta_a, col_beta_b) inclusion weights */
    double col_alpha;
    int64_t col_cap;         /* cap on a column's expected degree (col_mode 0) */
    double col_beta_a, col_beta_b;
    int32_t col_min_one;     /* 1: every column receives at least one entry */
    int32_t rank;            /* planted model rank */
    double factor_std;       /* std of the planted U and V entries */
    double planted_std;      /* > 0: rescale the planted dot products to this std */
    double offset, noise_std;
    double quantum;          /* > 0: round values to multiples of this */
    double vmin, vmax;       /* clamp range */
    uint64_t seed;
} cdmf_synth_spec;

typedef struct cdmf_synth cdmf_synth;

/* Generates the matrix.  Returns 0 or a negative cdmf status (cdmf_cuda.h). */
int cdmf_synth_create(const cdmf_synth_spec* spec, int threads, cdmf_synth** out);
/* Sizes of the generated train matrix and test set. */
int cdmf_synth_info(const cdmf_synth* s, int64_t* m, int64_t* n, int64_t* nnz_train, int64_t* nnz_test);
/* Copies the arrays out; any pointer may be NULL to skip that array. */
int cdmf_synth_copy(const cdmf_synth* s, uint32_t* csr_row_ptr, uint32_t* csr_col_idx, float* csr_val,
                    uint32_t* csc_col_ptr, uint32_t* csc_row_idx, float* csc_val,
                    uint32_t* test_row, uint32_t* test_col, float* test_val);
void cdmf_synth_destroy(cdmf_synth* s);

/* CSR -> CSC by a stable counting sort (row indices stay ascending inside a
 * column), the transposition scipy's tocsc performs.  perm (nullable) gets,
 * for every CSC position, the CSR position it came from. */
int cdmf_csr_to_csc(int64_t m, int64_t n, int64_t nnz, const uint32_t* csr_row_ptr,
                    const uint32_t* csr_col_idx, const float* csr_val, uint32_t* csc_col_ptr,
                    uint32_t* csc_row_idx, float* csc_val, uint32_t* perm);

/* The reference's factor initialisation initial_col (src/tools.cpp:349-357):
 * srand(0), then X[t][i] = 0.1f * (float(rand()) / RAND_MAX) + 0.001f with i
 * outer and t inner, through the C library's rand().  X is k x n, feature-major. */
void cdmf_initial_col(float* X, uint32_t k, uint32_t n);

#ifdef __cplusplus
}
#endif
#endif
