// Residual refresh for the 16-bit residual modes (BF16 / FP16 storage).
//
// CCD++ keeps the residual R - W^T H on the nonzeros and updates it
// incrementally (src/cdmf_ref.cpp:86-89,120-121).  With 16-bit storage every
// incremental update rounds, so once per outer iteration the residual is
// recomputed from the FP32 ratings and the FP32 factors:
//     r_ij = R_ij - sum_t W[t][i] * H[t][j]
// in CSR order (coalesced over the ratings), written to the CSR copy (in
// place, or through a position map when the copies are blocked) and
// scattered to the CSC copy through the CSR->CSC position map.  The
// scatter is L2-friendly: rows are visited in increasing order, so the
// writes into a column's segment advance monotonically and partial sectors
// merge in L2.  The same pass measures, in FP64, how far the stored residual
// had drifted from the exact one (the residual-drift check) and counts
// non-finite results.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace cdmf {

constexpr int kRefreshPerThread = 8;
constexpr int kRefreshChunk = kBlock * kRefreshPerThread;

// X (k x len, feature-major) -> Y (len x kp, row-major, padded with zeros).
static __global__ void __launch_bounds__(kBlock) to_row_major_kernel(const float* __restrict__ X, float* __restrict__ Y,
                                                              uint32_t k, uint32_t kp, int64_t len) {
    __shared__ float tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const uint32_t t0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        const uint32_t t = t0 + r;
        const int64_t i = i0 + tx;
        tile[r][tx] = (t < k && i < len) ? X[(size_t)t * len + i] : 0.0f;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int64_t i = i0 + r;
        const uint32_t t = t0 + tx;
        if (i < len && t < kp) Y[(size_t)i * kp + t] = tile[tx][r];
    }
}

template <int RT>
__global__ void __launch_bounds__(kBlock) refresh_kernel(
    const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ idx, const float* __restrict__ val,
    const uint32_t* __restrict__ to_csr, const uint32_t* __restrict__ to_csc, int64_t m, int64_t nnz, const float* __restrict__ Wrm,
    const float* __restrict__ Hrm, uint32_t kp, void* __restrict__ res_csr, void* __restrict__ res_csc,
    const float* __restrict__ pa, const float* __restrict__ pb_,  // pending subtract: a = H[tp] (cols), b = W[tp] (rows)
    double* part, uint32_t* counter, double* drift_out, unsigned long long* nonfinite_out) {
    __shared__ uint32_t srow[2];
    double drift = 0.0;
    unsigned bad = 0;
    const int64_t nchunks = (nnz + kRefreshChunk - 1) / kRefreshChunk;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int64_t p0 = c * kRefreshChunk;
        const int64_t p1 = (p0 + kRefreshChunk < nnz) ? p0 + kRefreshChunk : nnz;
        if (threadIdx.x < 2) {
            // row containing p0 (thread 0) and p1 - 1 (thread 1): last row with ptr[row] <= p
            const int64_t p = threadIdx.x == 0 ? p0 : p1 - 1;
            int64_t lo = 0, hi = m;   // ptr[lo] <= p < ptr[hi]
            while (hi - lo > 1) {
                const int64_t mid = (lo + hi) >> 1;
                if ((int64_t)ptr[mid] <= p) lo = mid; else hi = mid;
            }
            srow[threadIdx.x] = (uint32_t)lo;
        }
        __syncthreads();
        const uint32_t rlo = srow[0], rhi = srow[1];
        // each thread takes kRefreshPerThread consecutive nonzeros: one
        // binary search for the first, then the row advances by walking
        const int64_t pb = p0 + (int64_t)threadIdx.x * kRefreshPerThread;
        uint32_t i = rlo, bound = 0;
        if (pb < p1) {
            uint32_t lo = rlo, hi = rhi + 1;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if ((int64_t)__ldg(ptr + mid) <= pb) lo = mid; else hi = mid;
            }
            i = lo;
            bound = __ldg(ptr + i + 1);
        }
        for (int u = 0; u < kRefreshPerThread; ++u) {
            const int64_t p = pb + u;
            if (p >= p1) break;
            while ((uint32_t)p >= bound) bound = __ldg(ptr + (++i) + 1);
            const uint32_t j = __ldg(idx + p);
            const float4* wr = (const float4*)(Wrm + (size_t)i * kp);
            const float4* hr = (const float4*)(Hrm + (size_t)j * kp);
            float dot = 0.0f;
            for (uint32_t q = 0; q < kp / 4; ++q) {
                const float4 w = __ldg(wr + q), h = __ldg(hr + q);
                dot = fmaf(w.x, h.x, dot);
                dot = fmaf(w.y, h.y, dot);
                dot = fmaf(w.z, h.z, dot);
                dot = fmaf(w.w, h.w, dot);
            }
            const float rnew = __fsub_rn(__ldg(val + p), dot);
            const uint32_t pr = to_csr ? __ldg(to_csr + p) : (uint32_t)p;
            float rold = Res<RT>::ld(res_csr, pr);
            if (pa) rold = __fsub_rn(rold, __fmul_rn(__ldg(pa + j), __ldg(pb_ + i)));
            const float stored = Res<RT>::st(res_csr, pr, rnew);
            Res<RT>::st(res_csc, __ldg(to_csc + p), rnew);
            if (!isfinite(stored)) bad++;
            const double d = (double)rnew - (double)rold;
            drift = __dadd_rn(drift, __dmul_rn(d, d));
        }
        __syncthreads();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        drift = __dadd_rn(drift, __shfl_xor_sync(0xffffffffu, drift, o));
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    __shared__ double sm[kWarps];
    __shared__ unsigned smb[kWarps];
    __shared__ int last;
    if ((threadIdx.x & 31) == 0) {
        sm[threadIdx.x >> 5] = drift;
        smb[threadIdx.x >> 5] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = sm[0];
        unsigned long long b = smb[0];
        for (int q = 1; q < kWarps; ++q) { s = __dadd_rn(s, sm[q]); b += smb[q]; }
        part[blockIdx.x] = s;
        if (b) atomicAdd(nonfinite_out, b);
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double s = 0.0;
        for (uint32_t q = 0; q < gridDim.x; ++q) s = __dadd_rn(s, __ldcg(part + q));
        *drift_out = s;
        *counter = 0;
    }
}

}  // namespace cdmf
