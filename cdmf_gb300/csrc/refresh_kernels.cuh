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
// merge in L2.  The same pass measures how far the stored residual had
// drifted from the exact one (the residual-drift check: squares summed in
// FP32 over at most 8 terms per lane, then in FP64) and counts non-finite
// results.  The pass is bound by the gathers of factor rows from L2 (k * 8
// bytes per nonzero), not by DRAM.
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

// Lane-group refresh.  Each warp owns runs of 32 consecutive CSR nonzeros;
// lane l loads the index, rating and row of nonzero l (coalesced).  The dot
// products W_i . H_j then run on groups of kRefG = 4 lanes: in each of four
// rounds the eight groups take eight of the 32 nonzeros, and each lane reads
// S 16-byte slices of the W row and of the H row (64 contiguous bytes per
// group and slice: whole sectors), all independent loads in flight at once.
// Two xor steps finish each sum and one shuffle hands it to the lane that
// owns the nonzero, which then writes both residual copies.  S = float4
// slices per lane (k <= 16, 32, 64, 128 -> S = 1, 2, 4, 8); S = 0 walks any
// k.  Products are summed in a fixed order: deterministic.
constexpr int kRefG = 4;

// Block `bid` of `nblk` blocks of one refresh.  crow[c] is the row holding
// the chunk's first nonzero c * kRefreshChunk, and crow[nchunks] the row of
// the last nonzero (built at create), so a lane's row search starts inside
// the chunk's few rows.
template <int RT, int S>
__device__ __forceinline__ void refresh_body(
    const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ crow, const uint32_t* __restrict__ idx,
    const float* __restrict__ val, const uint32_t* __restrict__ to_csr, const uint32_t* __restrict__ to_csc,
    int64_t nnz, const float* __restrict__ Wrm, const float* __restrict__ Hrm, uint32_t kp, void* __restrict__ res_csr,
    void* __restrict__ res_csc, const float* __restrict__ pa, const float* __restrict__ pb_, double* part,
    uint32_t* counter, double* drift_out, unsigned long long* nonfinite_out, uint32_t bid, uint32_t nblk) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int kPer = 32 / kRefG;   // nonzeros per round
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gl = lane % kRefG, gi = lane / kRefG;
    const int my_round = lane / kPer, my_src = (lane % kPer) * kRefG;
    const uint32_t kq = kp / 4;   // float4 slices of a factor row (zero-padded past k)
    double drift = 0.0;
    unsigned bad = 0;
    const int64_t nchunks = (nnz + kRefreshChunk - 1) / kRefreshChunk;
    for (int64_t c = bid; c < nchunks; c += nblk) {
        const int64_t p0 = c * kRefreshChunk;
        const int64_t p1 = (p0 + kRefreshChunk < nnz) ? p0 + kRefreshChunk : nnz;
        const uint32_t rlo = __ldg(crow + c), rhi = __ldg(crow + c + 1);
        float dsq = 0.0f;   // this chunk's squared drift (at most kRefreshPerThread terms per lane)
        for (int s = 0; s < kRefreshPerThread; ++s) {
            const int64_t base = p0 + ((int64_t)warp * kRefreshPerThread + s) * 32;
            if (base >= p1) break;   // warp-uniform
            const int cnt = (int)((p1 - base) < 32 ? (p1 - base) : 32);
            const int64_t p = base + lane;
            // lanes past the end keep row 0 and column 0 (both exist when
            // nnz > 0): their products are computed and discarded
            uint32_t i = 0, j = 0;
            float v = 0.0f;
            if (lane < cnt) {
                uint32_t lo = rlo, hi = rhi + 1;   // ptr[lo] <= p < ptr[hi]
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if ((int64_t)__ldg(ptr + mid) <= p) lo = mid; else hi = mid;
                }
                i = lo;
                j = __ldg(idx + p);
                v = __ldg(val + p);
            }
            float dot = 0.0f;
            // two rounds' loads in flight together (measured: 2 > 1, 4 = 2)
#pragma unroll 2
            for (int r = 0; r < kRefG; ++r) {
                const int src = r * kPer + gi;
                const uint32_t ii = __shfl_sync(FULL, i, src);
                const uint32_t jj = __shfl_sync(FULL, j, src);
                const float4* wr = (const float4*)(Wrm + (size_t)ii * kp);
                const float4* hr = (const float4*)(Hrm + (size_t)jj * kp);
                float acc = 0.0f;
                if (S > 0) {
                    constexpr int SN = S > 0 ? S : 1;
                    float4 w[SN], h[SN];
#pragma unroll
                    for (int u = 0; u < SN; ++u) {
                        const uint32_t cq = gl + kRefG * u;
                        w[u] = cq < kq ? __ldg(wr + cq) : make_float4(0.f, 0.f, 0.f, 0.f);
                        h[u] = cq < kq ? __ldg(hr + cq) : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
#pragma unroll
                    for (int u = 0; u < SN; ++u) {
                        acc = fmaf(w[u].x, h[u].x, acc);
                        acc = fmaf(w[u].y, h[u].y, acc);
                        acc = fmaf(w[u].z, h[u].z, acc);
                        acc = fmaf(w[u].w, h[u].w, acc);
                    }
                } else {
                    for (uint32_t cq = gl; cq < kq; cq += kRefG) {
                        const float4 w = __ldg(wr + cq), h = __ldg(hr + cq);
                        acc = fmaf(w.x, h.x, acc);
                        acc = fmaf(w.y, h.y, acc);
                        acc = fmaf(w.z, h.z, acc);
                        acc = fmaf(w.w, h.w, acc);
                    }
                }
#pragma unroll
                for (int o = 1; o < kRefG; o <<= 1) acc = __fadd_rn(acc, __shfl_xor_sync(FULL, acc, o));
                const float got = __shfl_sync(FULL, acc, my_src);
                if (my_round == r) dot = got;
            }
            if (lane < cnt) {
                const float rnew = __fsub_rn(v, dot);
                const uint32_t pr = to_csr ? __ldg(to_csr + p) : (uint32_t)p;
                float rold = Res<RT>::ld(res_csr, pr);
                if (pa) rold = __fsub_rn(rold, __fmul_rn(__ldg(pa + j), __ldg(pb_ + i)));
                const float stored = Res<RT>::st(res_csr, pr, rnew);
                Res<RT>::st(res_csc, __ldg(to_csc + p), rnew);
                if (!isfinite(stored)) bad++;
                const float d = __fsub_rn(rnew, rold);
                dsq = __fadd_rn(dsq, __fmul_rn(d, d));
            }
        }
        drift = __dadd_rn(drift, (double)dsq);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        drift = __dadd_rn(drift, __shfl_xor_sync(FULL, drift, o));
        bad += __shfl_xor_sync(FULL, bad, o);
    }
    __shared__ double sm[kWarps];
    __shared__ unsigned smb[kWarps];
    __shared__ int last;
    if (lane == 0) {
        sm[warp] = drift;
        smb[warp] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = sm[0];
        unsigned long long b = smb[0];
        for (int q = 1; q < kWarps; ++q) { s = __dadd_rn(s, sm[q]); b += smb[q]; }
        part[bid] = s;
        if (b) atomicAdd(nonfinite_out, b);
        __threadfence();
        last = (atomicAdd(counter, 1u) == nblk - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double s = 0.0;
        for (uint32_t q = 0; q < nblk; ++q) s = __dadd_rn(s, __ldcg(part + q));
        *drift_out = s;
        *counter = 0;
    }
}

template <int RT, int S>
__global__ void __launch_bounds__(kBlock) refresh_warp_kernel(
    const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ crow, const uint32_t* __restrict__ idx,
    const float* __restrict__ val, const uint32_t* __restrict__ to_csr, const uint32_t* __restrict__ to_csc,
    int64_t nnz, const float* __restrict__ Wrm, const float* __restrict__ Hrm, uint32_t kp, void* __restrict__ res_csr,
    void* __restrict__ res_csc, const float* __restrict__ pa, const float* __restrict__ pb_, double* part,
    uint32_t* counter, double* drift_out, unsigned long long* nonfinite_out) {
    refresh_body<RT, S>(ptr, crow, idx, val, to_csr, to_csc, nnz, Wrm, Hrm, kp, res_csr, res_csc, pa, pb_, part,
                        counter, drift_out, nonfinite_out, blockIdx.x, gridDim.x);
}

// One refresh's arguments (launch_refresh_rt).
struct RefreshDesc {
    const uint32_t *ptr, *crow, *idx;
    const float* val;
    const uint32_t *to_csr, *to_csc;
    int64_t m, nnz;
    const float *Wrm, *Hrm;
    uint32_t kp, slices;   // slices: the S of refresh_warp_kernel (0 = any k)
    void *res_csr, *res_csc;
    const float *pa, *pb;
    double* part;
    uint32_t* counter;
    double* drift_out;
    unsigned long long* nonfinite;
};

}  // namespace cdmf
