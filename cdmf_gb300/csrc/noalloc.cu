// Test RMSE without any allocation by the library (cdmf_cuda_rmse_coo_noalloc).
//
// Some callers cannot let a library call cudaMalloc: a serving process that
// hands out all of its device memory from its own pool (an allocation made
// behind the pool's back is not in its accounting, and fails once the pool
// holds the memory), or an embedded runtime whose memory budget is fixed at
// start-up.  This entry point computes the same test RMSE as
// cdmf_cuda_rmse_coo, on device arrays the caller already holds, and keeps
// the kernel's scratch (per-block partial sums, the result slot, the NaN
// count and the arrival counter) in a fixed file-scope device array instead
// of allocating it.
//
// The array lives in every device that loads the library, until the process
// exits.  It is shared by all calls: calls that overlap on the GPU (from
// several streams or threads at once) race on it and must be serialised by
// the caller.  Its device address is looked up once per device, on the first
// call made with that device current, and kept.  A device reset moves the
// array, so a caller that resets a device does not call this entry point on
// it again.
#include <cdmf_cuda.h>

#include "sweep_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

namespace {

// Grid cap of the RMSE kernel: the scratch holds one partial per block.
constexpr int kNoAllocBlocks = 4 * 152;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    double part[kNoAllocBlocks];
    double out;
    unsigned long long nans;
    uint32_t counter;
};

static __device__ __align__(256) NoAllocScratch g_rmse_scratch;

NoAllocScratch* g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

// Device address of g_rmse_scratch on the current device (looked up once).
cudaError_t scratch_on_current_device(NoAllocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_rmse_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = (NoAllocScratch*)p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int cdmf_cuda_rmse_coo_noalloc(uint32_t k, int64_t m, int64_t n, const float* W, const float* H,
                                          int64_t nnz_test, const uint32_t* test_row, const uint32_t* test_col,
                                          const double* test_val, void* stream, double* rmse, int64_t* nan_count) {
    if (k == 0 || m <= 0 || n <= 0 || nnz_test < 0 || !W || !H || !rmse) return CDMF_ERR_INVALID;
    if (nnz_test == 0) return CDMF_ERR_EMPTY_TEST;
    if (!test_row || !test_col || !test_val) return CDMF_ERR_INVALID;
    if (nnz_test > CDMF_NOALLOC_MAX_TEST) return CDMF_ERR_TOO_LARGE;
    const int grid = (int)std::min<int64_t>(kNoAllocBlocks, (nnz_test + cdmf::kBlock - 1) / cdmf::kBlock);
    if (grid > kNoAllocBlocks) return CDMF_ERR_TOO_LARGE;
    cudaStream_t s = (cudaStream_t)stream;
    NoAllocScratch* sc = nullptr;
    if (scratch_on_current_device(&sc) != cudaSuccess) return CDMF_ERR_CUDA;
    // the previous call left its values behind: the NaN count and the arrival
    // counter must start at zero
    if (cudaMemsetAsync(&sc->nans, 0, sizeof(sc->nans), s) != cudaSuccess ||
        cudaMemsetAsync(&sc->counter, 0, sizeof(sc->counter), s) != cudaSuccess)
        return CDMF_ERR_CUDA;
    cdmf::rmse_kernel<double><<<grid, cdmf::kBlock, 0, s>>>(test_row, test_col, test_val, nnz_test, W, H, m, n, k,
                                                            sc->part, &sc->counter, &sc->out, &sc->nans);
    if (cudaGetLastError() != cudaSuccess) return CDMF_ERR_CUDA;
    unsigned long long nans = 0;
    if (cudaMemcpyAsync(rmse, &sc->out, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&nans, &sc->nans, sizeof(nans), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return CDMF_ERR_CUDA;
    if (nan_count) *nan_count = (int64_t)nans;
    return CDMF_OK;
}
