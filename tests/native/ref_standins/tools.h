// Stand-in for the reference's src/tools.h with the members the shim uses
// (src/pmf_util.h: SparseMatrix accessors, MatData, TestData; src/pmf.h:
// parameter), so the shim compiles without the reference tree.
#pragma once
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>
typedef std::vector<std::vector<float> > MatData;
struct SparseMatrix {
    long rows, cols, nnz;
    unsigned *csr_row_ptr_, *csr_col_indx_, *csc_col_ptr_, *csc_row_indx_;
    float *csr_val_, *csc_val_;
    unsigned* get_csr_row_ptr() { return csr_row_ptr_; }
    unsigned* get_csr_col_indx() { return csr_col_indx_; }
    float* get_csr_val() { return csr_val_; }
    unsigned* get_csc_col_ptr() { return csc_col_ptr_; }
    unsigned* get_csc_row_indx() { return csc_row_indx_; }
    float* get_csc_val() { return csc_val_; }
};
struct TestData {
    long nnz;
    unsigned *row, *col;
    float* val;
    unsigned* getTestRow() { return row; }
    unsigned* getTestCol() { return col; }
    float* getTestVal() { return val; }
};
struct parameter {
    unsigned k;
    float lambda;
    int maxiter, maxinneriter, version;
};
