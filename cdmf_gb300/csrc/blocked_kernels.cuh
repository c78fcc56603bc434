// Sweeps over the cross-index-blocked layout (see blocked.h).
//
// blocked_sweep_kernel: one CTA per work unit (block b, lines [j0, j1)).  The
// CTA copies block b's slice of the packed gather table (P, Q or y) into
// shared memory, then walks its segments: the long ones with the whole CTA,
// the medium ones one per warp, the short ones one per 8-lane group.  Every
// nonzero does the same fused update as sweep_kernel (pending subtract,
// add-back, store, g += y r, h += y^2) with its gather served from shared
// memory.  Each segment leaves (g, h) in part[b * lines + j].
// blocked_combine_kernel: x_j from the partials of line j in block order.
#pragma once
#include "sweep_kernels.cuh"

namespace cdmf {

constexpr uint32_t kXbRow = 6144;   // rows per block of the CSC copy (P slice: 48 KB)
constexpr uint32_t kXbCol = 3072;   // columns per block of the CSR copy (Q slice: 48 KB)
constexpr uint32_t kUnitNnz = 16384;

struct BlockedArgs {
    const uint32_t* segptr;
    const uint16_t* idx;
    void* res;
    const void* table;     // whole-range gather table: float2 P, float4 Q or float y
    const float* b;        // per-line scalars, as in SweepArgs
    const float* d;
    float2* part;          // per segment (g, h)
    const uint32_t* units; // 5 per unit
    uint32_t xb, lines;
    uint64_t cross;
};

template <int MODE> struct Tbl { using T = float; };
template <> struct Tbl<M_CSC> { using T = float2; };
template <> struct Tbl<M_CSR> { using T = float4; };

template <int MODE>
__device__ __forceinline__ void tfetch(const typename Tbl<MODE>::T* t, uint32_t i, float& a, float& c, float& y) {
    if constexpr (MODE == M_CSC) {
        const float2 p = t[i];
        a = p.x;
        c = p.y;
        y = p.y;
    } else if constexpr (MODE == M_CSR) {
        const float4 q = t[i];
        a = q.x;
        c = q.y;
        y = q.z;
    } else {
        a = c = 0.0f;
        y = t[i];
    }
}

template <int RT, int MODE, bool SUB, bool ADD, class AccT>
__device__ __forceinline__ void belem(const BlockedArgs& A, const typename Tbl<MODE>::T* tbl, uint32_t q, float bj,
                                      float dj, AccT& g, AccT& h) {
    const uint32_t i = __ldcs((const unsigned short*)A.idx + q);
    float r = Res<RT>::ld(A.res, q);
    float a, c, y;
    tfetch<MODE>(tbl, i, a, c, y);
    if (SUB || ADD) r = Res<RT>::st(A.res, q, update<SUB, ADD>(r, a, c, bj, dj));
    accumulate(g, h, y, r);
}

// Segment [s0, s1) by S cooperating threads; 4-nonzero vector chunks after a
// scalar head, two chunks in flight per lane, scalar tail.
template <int RT, int MODE, bool SUB, bool ADD, int S, bool KAHAN>
__device__ __forceinline__ void bstrided(const BlockedArgs& A, const typename Tbl<MODE>::T* tbl, uint32_t s0,
                                         uint32_t s1, uint32_t lane, float bj, float dj, float& gs, float& hs) {
    Acc<KAHAN> g, h;
    uint32_t vbeg = (s0 + 3u) & ~3u;
    if (vbeg > s1) vbeg = s1;
    const uint32_t vend = vbeg + ((s1 - vbeg) & ~3u);
    if (lane < vbeg - s0) belem<RT, MODE, SUB, ADD>(A, tbl, s0 + lane, bj, dj, g, h);
    uint32_t q = vbeg + 4u * lane;
    for (; q + 4u * S < vend; q += 8u * S) {
        uint2 iv[2];
        float r[2][4];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            iv[u] = __ldcs((const uint2*)((const unsigned short*)A.idx + q + 4u * S * u));
            Res<RT>::ld4(A.res, q + 4u * S * u, r[u]);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const uint32_t ii[4] = {iv[u].x & 0xffffu, iv[u].x >> 16, iv[u].y & 0xffffu, iv[u].y >> 16};
            float y[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                float a, c;
                tfetch<MODE>(tbl, ii[e], a, c, y[e]);
                r[u][e] = update<SUB, ADD>(r[u][e], a, c, bj, dj);
            }
            if (SUB || ADD) Res<RT>::st4(A.res, q + 4u * S * u, r[u]);
#pragma unroll
            for (int e = 0; e < 4; ++e) accumulate(g, h, y[e], r[u][e]);
        }
    }
    if (q < vend) {
        const uint2 v = __ldcs((const uint2*)((const unsigned short*)A.idx + q));
        const uint32_t ii[4] = {v.x & 0xffffu, v.x >> 16, v.y & 0xffffu, v.y >> 16};
        float r[4], y[4];
        Res<RT>::ld4(A.res, q, r);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            float a, c;
            tfetch<MODE>(tbl, ii[e], a, c, y[e]);
            r[e] = update<SUB, ADD>(r[e], a, c, bj, dj);
        }
        if (SUB || ADD) Res<RT>::st4(A.res, q, r);
#pragma unroll
        for (int e = 0; e < 4; ++e) accumulate(g, h, y[e], r[e]);
    }
    if (lane < s1 - vend) belem<RT, MODE, SUB, ADD>(A, tbl, vend + lane, bj, dj, g, h);
    gs = g.value();
    hs = h.value();
}

template <int MODE, bool SUB, bool ADD>
__device__ __forceinline__ void bscalars(const BlockedArgs& A, uint32_t j, float& bj, float& dj) {
    bj = SUB && A.b ? A.b[j] : 0.0f;
    dj = ADD ? A.d[j] : 0.0f;
}

template <int RT, int MODE, bool SUB, bool ADD>
__global__ void __launch_bounds__(kBlock) blocked_sweep_kernel(const BlockedArgs A) {
    using T = typename Tbl<MODE>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* tbl = (T*)smem_raw;
    const uint32_t* U = A.units + 5 * (size_t)blockIdx.x;
    const uint32_t b = U[0], j0 = U[1], jc = U[2], jw = U[3], j1 = U[4];
    const uint64_t x0 = (uint64_t)b * A.xb;
    const uint32_t cnt = (uint32_t)min((uint64_t)A.xb, A.cross - x0);
    const T* src = (const T*)A.table + x0;
    for (uint32_t x = threadIdx.x; x < cnt; x += kBlock) tbl[x] = __ldg(src + x);
    __syncthreads();
    const uint64_t base = (uint64_t)b * A.lines;
    // long segments: the whole CTA
    for (uint32_t j = j0; j < jc; ++j) {
        const uint32_t s0 = A.segptr[base + j], s1 = A.segptr[base + j + 1];
        float bj, dj;
        bscalars<MODE, SUB, ADD>(A, j, bj, dj);
        float g, h;
        bstrided<RT, MODE, SUB, ADD, kBlock, RT != 0>(A, tbl, s0, s1, threadIdx.x, bj, dj, g, h);
        cta_sum2(g, h);
        if (threadIdx.x == 0) A.part[base + j] = make_float2(g, h);
        __syncthreads();
    }
    // medium segments: one warp each
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t j = jc + warp; j < jw; j += kWarps) {
        const uint32_t s0 = A.segptr[base + j], s1 = A.segptr[base + j + 1];
        float bj, dj;
        bscalars<MODE, SUB, ADD>(A, j, bj, dj);
        float g, h;
        bstrided<RT, MODE, SUB, ADD, 32, false>(A, tbl, s0, s1, lane, bj, dj, g, h);
        warp_sum2(g, h);
        if (lane == 0) A.part[base + j] = make_float2(g, h);
    }
    // short segments: one 8-lane group each (warp-uniform trip count)
    const uint32_t sub = threadIdx.x & 7, grp = (threadIdx.x >> 3) & 3;
    for (uint32_t jj = jw + warp * 4; jj < j1; jj += kBlock / 8) {
        const uint32_t j = jj + grp;
        const bool valid = j < j1;
        const uint32_t s0 = valid ? A.segptr[base + j] : 0u, s1 = valid ? A.segptr[base + j + 1] : 0u;
        float bj = 0.0f, dj = 0.0f;
        if (valid && s1 > s0) bscalars<MODE, SUB, ADD>(A, j, bj, dj);
        float g, h;
        bstrided<RT, MODE, SUB, ADD, 8, false>(A, tbl, s0, s1, sub, bj, dj, g, h);
        warp_sum2<8>(g, h);
        if (valid && sub == 0 && s1 > s0) A.part[base + j] = make_float2(g, h);
    }
}

// x_j = (sum over blocks of g) / (lambda * nnz_j + sum over blocks of h),
// partials added in block order; writes out / Q / P as the line sweeps do.
template <int MODE>
__global__ void __launch_bounds__(kBlock) blocked_combine_kernel(const SweepArgs S, const uint32_t* __restrict__ segptr,
                                                                 const float2* __restrict__ part, uint32_t nb,
                                                                 uint32_t lines) {
    const uint32_t j = blockIdx.x * kBlock + threadIdx.x;
    if (j >= lines) return;
    float G = 0.0f, H = 0.0f;
    for (uint32_t b = 0; b < nb; ++b) {
        const size_t s = (size_t)b * lines + j;
        if (segptr[s + 1] > segptr[s]) {
            const float2 p = part[s];
            G = __fadd_rn(G, p.x);
            H = __fadd_rn(H, p.y);
        }
    }
    const float bj = MODE == M_CSC && S.b ? S.b[j] : 0.0f;
    const float dj = MODE == M_CSC ? S.d[j] : 0.0f;
    const uint32_t len = S.ptr[j + 1] - S.ptr[j];
    finish_line<MODE>(S, j, len, G, H, bj, dj);
}

// Pending subtract r -= a[i] * bvec[j] over a blocked copy (state read-back).
template <int RT>
__global__ void __launch_bounds__(kBlock) blocked_flush_kernel(const uint32_t* __restrict__ segptr,
                                                               const uint16_t* __restrict__ idx, void* res,
                                                               const float* __restrict__ a,
                                                               const float* __restrict__ bvec, uint32_t nb,
                                                               uint32_t lines, uint32_t xb) {
    const uint64_t nseg = (uint64_t)nb * lines;
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t s = (uint64_t)blockIdx.x * kWarps + (threadIdx.x >> 5); s < nseg; s += (uint64_t)gridDim.x * kWarps) {
        const uint32_t b = (uint32_t)(s / lines), j = (uint32_t)(s % lines);
        const float bj = bvec[j];
        for (uint32_t q = segptr[s] + lane; q < segptr[s + 1]; q += 32) {
            float r = Res<RT>::ld(res, q);
            r = __fsub_rn(r, __fmul_rn(a[(size_t)b * xb + idx[q]], bj));
            Res<RT>::st(res, q, r);
        }
    }
}

// res[map[p]] = src[p]: the ratings (line layout, float) into a copy's layout
template <int RT>
__global__ void scatter_res_kernel(const float* __restrict__ src, const uint32_t* __restrict__ map, void* dst,
                                   int64_t count) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < count; p += (int64_t)gridDim.x * blockDim.x)
        Res<RT>::st(dst, map[p], src[p]);
}

}  // namespace cdmf
