// Degree relabelling of a cdmf_problem (see relabel.cpp).
#pragma once
#include <cdmf_cuda.h>

#include <cstdint>
#include <vector>

namespace cdmf {

struct Relabel {
    std::vector<uint32_t> row_old, row_new, col_old, col_new;   // new id -> caller id, caller id -> new id
    std::vector<uint32_t> csr_ptr, csr_idx, csc_ptr, csc_idx;   // structure in the new numbering
    std::vector<float> csr_val, csc_val;
    std::vector<uint32_t> csr_pos, csc_pos;   // new position -> caller's position (CSR, CSC)
    std::vector<uint32_t> csc_from_csr;       // new CSC position -> new CSR position
    std::vector<uint32_t> te_row, te_col;     // test set in the new numbering
};

// false: the CSC arrays are not the transpose of the CSR arrays, or out of memory
bool relabel(const cdmf_problem& p, Relabel& r);

}  // namespace cdmf
