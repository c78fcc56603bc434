// Device kernels of the CCD++ engine (sm_103a).
//
// One kernel, `sweep_kernel`, performs a whole half-step of the rank-one
// update over one compressed copy of the residual: the CSC copy to solve h_t
// (src/cdmf_ref.cpp:96-99, kcode/ccd_1.cl:60-78) or the CSR copy to solve w_t
// (src/cdmf_ref.cpp:104-107, kcode/ccd_1.cl:83-100).  For line j (a column
// of CSC or a row of CSR) with entries (i, r):
//     r <- r - a_i * b_j      pending subtract of the previous feature
//                             (src/cdmf_ref.cpp:120-121, deferred to here)
//     r <- r + c_i * d_j      add-back of this feature (src/cdmf_ref.cpp:86-89)
//     g += y_i * r ; h += y_i * y_i
//     x_j = g / (lambda * nnz_j + h), 0 for an empty line (src/cdmf_ref.cpp:7-17)
// Every product and sum is rounded separately (no FMA), as in the reference's
// x86-64 build, so a line summed by one thread in index order reproduces the
// reference bit for bit.
//
// Lines are binned by length and all bins run in the same launch:
//   blocks [0, nx)            one chunk of a split line (len > cta_max); the
//                             last chunk to finish combines the chunk partials
//                             in chunk order (deterministic, no float atomics)
//   blocks [nx, nx+nc)        one line per CTA
//   blocks [.., +nwb)         one line per warp
//   blocks [.., +ntb)         one line per thread, index order = reference order
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace cdmf {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

struct XTask {            // one chunk of a split line
    uint32_t line, beg, end, slot;
    uint32_t xl, first_slot, nchunks, pad;
};

struct SweepArgs {
    const uint32_t* __restrict__ ptr;
    const uint32_t* __restrict__ idx;
    void* __restrict__ res;
    const float* __restrict__ a;   // subtract: cross vector (previous feature, final)
    const float* b;                // subtract: line vector  (previous feature, final)
    const float* __restrict__ c;   // add-back: cross vector (this feature, old)
    const float* d;                // add-back: line vector  (this feature, old)
    const float* __restrict__ y;   // solve: cross vector
    float* out;                    // solve: line vector (written)
    float* save;                   // optional copy of out's old value
    float lambda;
    // work lists
    const XTask* xt;
    const uint32_t* cl;
    const uint32_t* wl;
    const uint32_t* tl;
    uint32_t nx, nc, nw, nt;
    uint32_t nwb;                  // blocks of the warp bin
    float2* part;                  // split-line partials
    uint32_t* xcount;              // split-line arrival counters (left at 0)
};

// ---- residual element access -------------------------------------------------
template <int RT> struct Res;
template <> struct Res<0> {
    using T = float;
    static __device__ __forceinline__ float ld(const void* p, uint32_t q) { return __ldcs((const float*)p + q); }
    static __device__ __forceinline__ float st(void* p, uint32_t q, float v) { __stcs((float*)p + q, v); return v; }
};
template <> struct Res<1> {
    using T = __nv_bfloat16;
    static __device__ __forceinline__ float ld(const void* p, uint32_t q) {
        unsigned short u = __ldcs((const unsigned short*)p + q);
        return __bfloat162float(__ushort_as_bfloat16(u));
    }
    static __device__ __forceinline__ float st(void* p, uint32_t q, float v) {
        __nv_bfloat16 h = __float2bfloat16_rn(v);
        __stcs((unsigned short*)p + q, __bfloat16_as_ushort(h));
        return __bfloat162float(h);
    }
};
template <> struct Res<2> {
    using T = __half;
    static __device__ __forceinline__ float ld(const void* p, uint32_t q) {
        unsigned short u = __ldcs((const unsigned short*)p + q);
        return __half2float(__ushort_as_half(u));
    }
    static __device__ __forceinline__ float st(void* p, uint32_t q, float v) {
        __half h = __float2half_rn(v);
        __stcs((unsigned short*)p + q, __half_as_ushort(h));
        return __half2float(h);
    }
};

// One element: fused residual update + accumulation.
template <int RT, bool SUB, bool ADD>
__device__ __forceinline__ void elem(const SweepArgs& A, uint32_t q, float r, uint32_t i, float bj, float dj,
                                     float& g, float& h) {
    if (SUB) r = __fsub_rn(r, __fmul_rn(__ldg(A.a + i), bj));
    if (ADD) r = __fadd_rn(r, __fmul_rn(__ldg(A.c + i), dj));
    if (SUB || ADD) r = Res<RT>::st(A.res, q, r);
    const float yi = __ldg(A.y + i);
    g = __fadd_rn(g, __fmul_rn(yi, r));
    h = __fadd_rn(h, __fmul_rn(yi, yi));
}

// Strided pass over [beg, end): this thread takes beg+lane, beg+lane+S, ...
// in increasing order, four loads in flight per step.
template <int RT, bool SUB, bool ADD, int S>
__device__ __forceinline__ void strided(const SweepArgs& A, uint32_t beg, uint32_t end, uint32_t lane, float bj,
                                        float dj, float& g, float& h) {
    uint32_t q = beg + lane;
    for (; q + 3 * S < end; q += 4 * S) {
        uint32_t i0 = __ldcs(A.idx + q), i1 = __ldcs(A.idx + q + S), i2 = __ldcs(A.idx + q + 2 * S),
                 i3 = __ldcs(A.idx + q + 3 * S);
        float r0 = Res<RT>::ld(A.res, q), r1 = Res<RT>::ld(A.res, q + S), r2 = Res<RT>::ld(A.res, q + 2 * S),
              r3 = Res<RT>::ld(A.res, q + 3 * S);
        elem<RT, SUB, ADD>(A, q, r0, i0, bj, dj, g, h);
        elem<RT, SUB, ADD>(A, q + S, r1, i1, bj, dj, g, h);
        elem<RT, SUB, ADD>(A, q + 2 * S, r2, i2, bj, dj, g, h);
        elem<RT, SUB, ADD>(A, q + 3 * S, r3, i3, bj, dj, g, h);
    }
    for (; q < end; q += S) elem<RT, SUB, ADD>(A, q, Res<RT>::ld(A.res, q), __ldcs(A.idx + q), bj, dj, g, h);
}

__device__ __forceinline__ void warp_sum2(float& g, float& h) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        g = __fadd_rn(g, __shfl_xor_sync(0xffffffffu, g, o));
        h = __fadd_rn(h, __shfl_xor_sync(0xffffffffu, h, o));
    }
}

// CTA-wide sum; the result is valid in thread 0.  Fixed shape: per-warp xor
// tree, then warps 0..7 in order.
__device__ __forceinline__ void cta_sum2(float& g, float& h) {
    __shared__ float2 sm[kWarps];
    warp_sum2(g, h);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) sm[w] = make_float2(g, h);
    __syncthreads();
    if (threadIdx.x == 0) {
        float G = sm[0].x, Hs = sm[0].y;
        for (int q = 1; q < kWarps; ++q) { G = __fadd_rn(G, sm[q].x); Hs = __fadd_rn(Hs, sm[q].y); }
        g = G;
        h = Hs;
    }
}

// x_j from the accumulated sums; h excludes lambda * nnz_j.
__device__ __forceinline__ void finish_line(const SweepArgs& A, uint32_t j, uint32_t len, float g, float h) {
    const float lam = __fmul_rn(A.lambda, __uint2float_rn(len));
    const float x = len == 0 ? 0.0f : __fdiv_rn(g, __fadd_rn(lam, h));
    if (A.save) A.save[j] = A.out[j];
    A.out[j] = x;
}

template <int RT, bool SUB, bool ADD>
__global__ void __launch_bounds__(kBlock) sweep_kernel(const SweepArgs A) {
    uint32_t b = blockIdx.x;
    if (b < A.nx) {                                        // split-line chunk
        const XTask T = A.xt[b];
        const float bj = SUB ? A.b[T.line] : 0.0f, dj = ADD ? A.d[T.line] : 0.0f;
        float g = 0.0f, h = 0.0f;
        strided<RT, SUB, ADD, kBlock>(A, T.beg, T.end, threadIdx.x, bj, dj, g, h);
        cta_sum2(g, h);
        __shared__ int last;
        if (threadIdx.x == 0) {
            A.part[T.slot] = make_float2(g, h);
            __threadfence();
            const uint32_t prev = atomicAdd(A.xcount + T.xl, 1u);
            last = (prev == T.nchunks - 1);
        }
        __syncthreads();
        if (last && threadIdx.x == 0) {
            __threadfence();
            float G = 0.0f, Hs = 0.0f;
            for (uint32_t q = 0; q < T.nchunks; ++q) {
                const float2 p = __ldcg(A.part + T.first_slot + q);
                G = __fadd_rn(G, p.x);
                Hs = __fadd_rn(Hs, p.y);
            }
            const uint32_t len = A.ptr[T.line + 1] - A.ptr[T.line];
            finish_line(A, T.line, len, G, Hs);
            A.xcount[T.xl] = 0;
        }
        return;
    }
    b -= A.nx;
    if (b < A.nc) {                                        // one line per CTA
        const uint32_t j = A.cl[b];
        const uint32_t beg = A.ptr[j], end = A.ptr[j + 1];
        const float bj = SUB ? A.b[j] : 0.0f, dj = ADD ? A.d[j] : 0.0f;
        float g = 0.0f, h = 0.0f;
        strided<RT, SUB, ADD, kBlock>(A, beg, end, threadIdx.x, bj, dj, g, h);
        cta_sum2(g, h);
        if (threadIdx.x == 0) finish_line(A, j, end - beg, g, h);
        return;
    }
    b -= A.nc;
    if (b < A.nwb) {                                       // one line per warp
        const uint32_t w = b * kWarps + (threadIdx.x >> 5);
        if (w >= A.nw) return;
        const uint32_t lane = threadIdx.x & 31;
        const uint32_t j = A.wl[w];
        const uint32_t beg = A.ptr[j], end = A.ptr[j + 1];
        const float bj = SUB ? A.b[j] : 0.0f, dj = ADD ? A.d[j] : 0.0f;
        float g = 0.0f, h = 0.0f;
        strided<RT, SUB, ADD, 32>(A, beg, end, lane, bj, dj, g, h);
        warp_sum2(g, h);
        if (lane == 0) finish_line(A, j, end - beg, g, h);
        return;
    }
    b -= A.nwb;
    const uint32_t t = b * kBlock + threadIdx.x;           // one line per thread
    if (t >= A.nt) return;
    const uint32_t j = A.tl[t];
    const uint32_t beg = A.ptr[j], end = A.ptr[j + 1];
    const uint32_t len = end - beg;
    if (len == 0) {
        if (A.save) A.save[j] = A.out[j];
        A.out[j] = 0.0f;
        return;
    }
    const float bj = SUB ? A.b[j] : 0.0f, dj = ADD ? A.d[j] : 0.0f;
    float g = 0.0f;
    float h = __fmul_rn(A.lambda, __uint2float_rn(len));   // h starts at lambda*nnz (src/cdmf_ref.cpp:8)
    for (uint32_t q = beg; q < end; ++q)
        elem<RT, SUB, ADD>(A, q, Res<RT>::ld(A.res, q), __ldcs(A.idx + q), bj, dj, g, h);
    if (A.save) A.save[j] = A.out[j];
    A.out[j] = __fdiv_rn(g, h);
}

// Applies a pending subtract r -= a_i * b_j to one residual copy (warp per
// line, grid-stride).  Used only when the state is read back.
template <int RT>
__global__ void __launch_bounds__(kBlock) flush_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ idx,
                                                       void* __restrict__ res, const float* __restrict__ a,
                                                       const float* __restrict__ b, uint32_t lines) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t j = blockIdx.x * kWarps + (threadIdx.x >> 5); j < lines; j += gridDim.x * kWarps) {
        const float bj = b[j];
        for (uint32_t q = ptr[j] + lane; q < ptr[j + 1]; q += 32) {
            float r = Res<RT>::ld(res, q);
            r = __fsub_rn(r, __fmul_rn(a[idx[q]], bj));
            Res<RT>::st(res, q, r);
        }
    }
}

// Test RMSE (src/tools.cpp:543-582): per entry the float products
// W[t][i]*H[t][j] are summed in double in t order, (pred - v)^2 in double, NaN
// terms skipped but counted.  Fixed grid; block partials in double; the last
// block adds them in block order and writes sqrt(sum / nnz_test).
__global__ void __launch_bounds__(kBlock) rmse_kernel(const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                                                      const float* __restrict__ val, int64_t nt,
                                                      const float* __restrict__ W, const float* __restrict__ H,
                                                      int64_t m, int64_t n, uint32_t k, double* part,
                                                      uint32_t* counter, double* out) {
    double acc = 0.0;
    for (int64_t e = (int64_t)blockIdx.x * kBlock + threadIdx.x; e < nt; e += (int64_t)gridDim.x * kBlock) {
        const uint32_t i = row[e], j = col[e];
        double pred = 0.0;
        for (uint32_t t = 0; t < k; ++t)
            pred = __dadd_rn(pred, (double)__fmul_rn(__ldg(W + (size_t)t * m + i), __ldg(H + (size_t)t * n + j)));
        const double dv = __dsub_rn(pred, (double)val[e]);
        const double tmp = __dmul_rn(dv, dv);
        if (!isnan(tmp)) acc = __dadd_rn(acc, tmp);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = __dadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    __shared__ double sm[kWarps];
    __shared__ int last;
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = sm[0];
        for (int q = 1; q < kWarps; ++q) s = __dadd_rn(s, sm[q]);
        part[blockIdx.x] = s;
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double s = 0.0;
        for (uint32_t q = 0; q < gridDim.x; ++q) s = __dadd_rn(s, __ldcg(part + q));
        *out = sqrt(s / (double)nt);
        *counter = 0;
    }
}

}  // namespace cdmf
