// Device-side builds of the engine's sparse structures (compress.cu).
#pragma once
#include <cdmf_cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "relabel.h"

namespace cdmf {

// Degree relabelling of a caller's CSR, built on the GPU: the same arrays as
// relabel() in relabel.cpp (rows and columns by decreasing degree, ties by
// id; entries of a row by new column; CSC the stable transposition), left on
// the device.  Device arrays are cudaMalloc'd into `allocs` (the caller frees
// them); the structure scratch is freed before return.
struct GpuRelabel {
    uint32_t *csr_ptr = nullptr, *csr_idx = nullptr, *csc_ptr = nullptr, *csc_idx = nullptr;
    float *csr_val = nullptr, *csc_val = nullptr;
    uint32_t* csr_pos = nullptr;        // new CSR position -> caller's CSR position
    uint32_t* csc_from_csr = nullptr;   // new CSC position -> new CSR position
    uint32_t* to_csc = nullptr;         // new CSR position -> new CSC position
    uint32_t *uptr = nullptr, *uidx = nullptr;   // the caller's CSR structure (device copy)
    uint32_t *d_row_old = nullptr, *d_col_old = nullptr;   // new id -> caller id (device)
    uvec<uint32_t> row_old, col_old;    // new id -> caller id (host)
    std::vector<uint32_t> hptr_r, hptr_c;   // new row / column pointers (host)
};

// CDMF_OK or a CDMF_ERR_* status.  p must hold a valid CSR with nnz > 0.
int gpu_relabel(const cdmf_problem& p, cudaStream_t s, GpuRelabel& out, std::vector<void*>& allocs);

}  // namespace cdmf
