// FP64 training objective, as a convergence monitor:
//     sum over the nonzeros of r_ij^2                       (the residual)
//   + lambda * (sum_i nnz_i |w_i|^2 + sum_j nnz_j |h_j|^2)  (the regulariser)
// The first term is the `loss` that the reference's UpdateRating computes and
// discards (src/cdmf_ref.cpp:20-43); the second is the regulariser of the
// CCD++ objective whose per-coordinate minimiser is RankOneUpdate
// (src/cdmf_ref.cpp:7-17: lambda is scaled by the line's nonzero count).
//
// One launch, three grid-stride ranges: the stored CSR residual copy
// (coalesced), then rows (W feature-major, coalesced across threads), then
// columns.  Squares and sums are in FP64.  Block partials are combined by the
// last block in block order, so the result is deterministic.
#pragma once
#include <stdint.h>

namespace cdmf {

template <int RT>
__global__ void __launch_bounds__(kBlock) objective_kernel(const void* __restrict__ res, int64_t nnz,
                                                           const uint32_t* __restrict__ csr_ptr, int64_t m,
                                                           const uint32_t* __restrict__ csc_ptr, int64_t n,
                                                           const float* __restrict__ W, const float* __restrict__ H,
                                                           uint32_t k, double* part, uint32_t* counter, double* out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double s[3] = {0.0, 0.0, 0.0};
    for (int64_t q = t0; q < nnz; q += stride) {
        const double r = (double)Res<RT>::ld(res, (uint32_t)q);
        s[0] = fma(r, r, s[0]);
    }
    for (int64_t i = t0; i < m; i += stride) {
        double w2 = 0.0;
        for (uint32_t t = 0; t < k; ++t) {
            const double w = (double)__ldg(W + (size_t)t * m + i);
            w2 = fma(w, w, w2);
        }
        s[1] = fma((double)(__ldg(csr_ptr + i + 1) - __ldg(csr_ptr + i)), w2, s[1]);
    }
    for (int64_t j = t0; j < n; j += stride) {
        double h2 = 0.0;
        for (uint32_t t = 0; t < k; ++t) {
            const double h = (double)__ldg(H + (size_t)t * n + j);
            h2 = fma(h, h, h2);
        }
        s[2] = fma((double)(__ldg(csc_ptr + j + 1) - __ldg(csc_ptr + j)), h2, s[2]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s[c] = __dadd_rn(s[c], __shfl_xor_sync(0xffffffffu, s[c], o));
    __shared__ double sm[3][kWarps];
    __shared__ int last;
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; ++c) sm[c][threadIdx.x >> 5] = s[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int c = 0; c < 3; ++c) {
            double v = sm[c][0];
            for (int w = 1; w < kWarps; ++w) v = __dadd_rn(v, sm[c][w]);
            part[3 * (size_t)blockIdx.x + c] = v;
        }
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        for (int c = 0; c < 3; ++c) {
            double v = 0.0;
            for (uint32_t b = 0; b < gridDim.x; ++b) v = __dadd_rn(v, __ldcg(part + 3 * (size_t)b + c));
            out[c] = v;
        }
        *counter = 0;
    }
}

}  // namespace cdmf
