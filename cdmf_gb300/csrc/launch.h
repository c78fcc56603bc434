// Host-side launchers of the templated sweep and refresh kernels.
//
// Every launcher is a template on the residual type RT (0 = FP32, 1 = BF16,
// 2 = FP16) and picks the kernel instantiation for the sweep mode and the
// residual writes (sub = pending subtract, add = add-back) at run time.  The
// definitions are in launch.cu, which the build compiles once per residual
// type and kernel family (CDMF_LAUNCH_RT, CDMF_LAUNCH_PART), so the kernel
// instantiations are spread over translation units that compile in parallel.
// The engine only declares them here.
#pragma once
#include "sweep_kernels.cuh"
#include "tile_kernels.cuh"
#include "blocked_kernels.cuh"
#include "refresh_kernels.cuh"

#include <cuda_runtime.h>

#include <mutex>
#include <set>
#include <utility>

namespace cdmf {

// Function attributes belong to the device they were set on, so the
// launchers set them once per (device, kernel).
inline std::pair<int, const void*> attr_key(const void* kernel) {
    int dev = 0;
    cudaGetDevice(&dev);
    return {dev, kernel};
}

// The sweeps use almost no shared memory; give the unified L1/shared
// storage to L1, which holds the gather tables.
template <class K>
void prefer_l1(K kernel) {
    static std::mutex mu;
    static std::set<std::pair<int, const void*>> done;
    std::lock_guard<std::mutex> lk(mu);
    if (done.insert(attr_key((const void*)kernel)).second)
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
}

// Opts a kernel into `bytes` of dynamic shared memory (beyond the default
// 48 KB including static) with the unified storage split toward shared memory.
template <class K>
void allow_smem(K kernel, size_t bytes) {
    static std::mutex mu;
    static std::set<std::pair<int, const void*>> done;
    std::lock_guard<std::mutex> lk(mu);
    if (done.insert(attr_key((const void*)kernel)).second) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
}

// --- family 0 (launch.cu, CDMF_LAUNCH_PART 0): the length-binned sweeps ---

// sweep_kernel over the bins; mode M_PLAIN, M_CSC, M_CSCP, M_CSCQ, M_CSR or M_CSR16.
template <int RT>
void launch_rt(const SweepArgs& A, int mode, bool sub, bool add, unsigned grid, cudaStream_t s);

// Sets the dynamic shared memory limit of every sweep_smemq_kernel of RT.
template <int RT>
void smemq_attrs(int bytes);

// sweep_smemq_kernel (first CSR sweep, cross table in shared memory);
// i16 selects the 16-bit column indices.
template <int RT>
void smemq_rt(const SweepArgs& A, bool i16, bool sub, bool add, unsigned grid, size_t smem, uint32_t nb,
              uint32_t* queue, cudaStream_t s);

// The dual SpMV (M_DUAL, FP32 values only).
void launch_dual(const SweepArgs& A, unsigned grid, cudaStream_t s);

// --- family 1 (launch.cu, CDMF_LAUNCH_PART 1): tiles, blocks, refresh ---

// tile_sweep_kernel (nonzero-balanced tiles); mode M_PLAIN, M_CSC or M_CSR.
template <int RT>
void tile_rt(const TileArgs& T, int mode, bool sub, bool add, unsigned grid, cudaStream_t s);

// blocked_sweep_kernel (cross table blocks in shared memory).
template <int RT>
void blocked_rt(const BlockedArgs& B, int mode, bool sub, bool add, unsigned grid, cudaStream_t s);

// refresh_warp_kernel over one problem; D.slices picks the instantiation
// (1, 2, 4, 8 slices of the rank, 0 = any rank).  RT is 1 or 2.
template <int RT>
void launch_refresh_rt(const RefreshDesc& D, unsigned grid, cudaStream_t s);

}  // namespace cdmf
