// Host-side data model and helpers of the `cdmf` command-line driver.
//
// Mirrors the reference's surface so scripts and users see the same thing:
//   parameter    -- src/pmf.h:4-26 (same fields and defaults)
//   SparseMatrix -- src/pmf_util.h:13-114 (CSR + CSC, 32-bit unsigned indices)
//   TestData     -- src/pmf_util.h:117-161 (COO)
//   MatData      -- src/pmf_util.h:8 (vector<vector<float>>, X[t][i])
// The engine itself is reached only through include/cdmf_cuda.h.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

using VecData = std::vector<float>;
using MatData = std::vector<VecData>;

class parameter {
public:
    int threads = 16;
    int nBlocks = 1;
    int nThreadsPerBlock = 32;
    int do_ref = 0;
    int do_predict = 0;
    int maxinneriter = 5;
    int maxiter = 5;
    unsigned k = 10;
    float lambda = 0.1f;
    unsigned platform_id = 0;
    int verbose = 0;
    int version = 1;
    char device_type[4] = {'g', 'p', 'u', '\0'};
    char scr_dir[1024] = "../data/simple";
    char kcode_path[1024] = "../kcode";
    // engine knobs (long flags)
    int residual = 0;   // -residual f32|bf16|f16
    int reduce = 0;     // -reduce tree|sequential
    int graph = 0;      // -graph 0|1
};

struct SparseMatrix {
    long rows = 0, cols = 0;
    unsigned long nnz = 0, max_row_nnz = 0, max_col_nnz = 0;
    std::vector<uint32_t> csr_row_ptr, csr_col_indx, csc_col_ptr, csc_row_indx;
    std::vector<float> csr_val, csc_val;
};

struct TestData {
    unsigned long rows = 0, cols = 0, nnz = 0;
    std::vector<uint32_t> test_row, test_col;
    std::vector<float> test_val;
};

// src/tools.cpp:271-347; returns false (after printing) where the reference exits.
bool load(const char* srcdir, SparseMatrix& R, TestData& T);
// src/tools.cpp:349-357 through cdmf_initial_col (the C library's rand()).
void initial_col(MatData& X, unsigned k, unsigned n);
// src/tools.cpp:378-465; exits with the help text on bad flags like the reference.
parameter parse_command_line(int argc, char** argv);
// src/tools.cpp:467-487.
void golden_compare(const MatData& W, const MatData& W_ref, unsigned k, unsigned m);
// src/tools.cpp:489-541 with the prediction done by the engine's RMSE kernel.
bool calculate_rmse(const MatData& W, const MatData& H, const char* srcdir, unsigned k, int device);
