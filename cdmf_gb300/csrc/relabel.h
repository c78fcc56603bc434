// Degree relabelling of a cdmf_problem (see relabel.cpp).
#pragma once
#include <cdmf_cuda.h>

#include <cstdint>
#include <memory>
#include <utility>
#include <vector>

namespace cdmf {

// std::vector whose resize leaves elements uninitialised (every element is
// written by a later parallel pass; this saves a serial zero fill of
// gigabytes).
template <class T>
struct DefaultInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = DefaultInitAlloc<U>; };
    DefaultInitAlloc() = default;
    template <class U> DefaultInitAlloc(const DefaultInitAlloc<U>&) {}
    template <class U> void construct(U* p) { ::new ((void*)p) U; }
    template <class U, class... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};
template <class T> using uvec = std::vector<T, DefaultInitAlloc<T>>;

struct Relabel {
    uvec<uint32_t> row_old, row_new, col_old, col_new;   // new id -> caller id, caller id -> new id
    uvec<uint32_t> csr_ptr, csr_idx, csc_idx;            // structure in the new numbering
    std::vector<uint32_t> csc_ptr;
    uvec<float> csr_val, csc_val;
    uvec<uint32_t> csr_pos, csc_pos;   // new position -> caller's position (CSR; CSC filled on demand)
    uvec<uint32_t> csc_from_csr;       // new CSC position -> new CSR position
    uvec<uint32_t> te_row, te_col;     // test set in the new numbering
};

// Builds both copies from the caller's CSR (the CSC arrays must hold the
// same matrix; they are read only by relabel_csc_positions).  false: out of
// memory or an inconsistent structure.
bool relabel(const cdmf_problem& p, Relabel& r);
// New CSC position -> caller's CSC position, from the caller's CSR
// structure (its CSC being the stable transposition of it), needed only to
// move residual state across the boundary.
bool relabel_csc_positions(int64_t m, int64_t n, const uint32_t* ucsr_ptr, const uint32_t* ucsr_idx,
                           const uvec<uint32_t>& csr_pos, const uvec<uint32_t>& csc_from_csr, uvec<uint32_t>& csc_pos);

}  // namespace cdmf
