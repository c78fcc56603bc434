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
// Gathers.  The per-nonzero cross-vector values (a_i, c_i, y_i) are read from
// one packed table per sweep so each nonzero costs a single gather:
//   CSC first sweep: P[i] = (W[t-1][i] new, W[t][i] old)         float2, = (a, c=y)
//   CSR first sweep: Q[j] = (H[t-1][j] new, H[t][j] old, H[t][j] new, 0)  float4
// The CSC sweep writes Q as it finishes each column; the last CSR sweep of a
// feature writes P for the next feature as it finishes each row.
//
// Streams.  Inside a line, index and residual are read with 128-bit (16-bit
// residual or 16-bit column index: 64-bit) vector loads, 4 nonzeros per lane
// per load, after a scalar head that reaches a 4-element boundary;
// cache-streaming hints keep them out of L1, which holds the gather tables.
// Matrices with at most 65,536 columns read 16-bit column indices in their
// first CSR sweeps (M_CSR16, M_CSRS16).  Narrow matrices with an FP32
// residual stage Q in shared memory for those sweeps (sweep_smemq_kernel).
//
// Lines are binned by length and all bins run in the same launch:
//   blocks [0, nx)            one chunk of a split line (len > cta_max); the
//                             last chunk to finish combines the chunk partials
//                             in chunk order (deterministic, no float atomics)
//   blocks [nx, nx+nc)        one line per CTA
//   blocks [.., +nwb)         one line per warp
//   blocks [.., +ngb)         one line per 4- or 8-lane group (8 or 4 lines per warp)
//   blocks [.., +ntb)         one line per thread, index order = reference order
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <type_traits>

namespace cdmf {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
constexpr int kTileBlocks = 6;

// sweep modes
constexpr int M_PLAIN = 0;  // inner iterations >= 2: y only, no residual writes
constexpr int M_CSC = 1;    // first CSC sweep of a feature: P gathers, emits Q
constexpr int M_CSR = 2;    // first CSR sweep of a feature: Q gathers
constexpr int M_DUAL = 3;   // dual SpMV (CSR5-style front end): y gathers, raw sums out
constexpr int M_CSRS = 4;   // M_CSR with the cross table staged in shared memory (narrow matrices)
constexpr int M_CSR16 = 5;  // M_CSR reading 16-bit column indices (at most 65,536 columns)
constexpr int M_CSRS16 = 6; // M_CSRS reading 16-bit column indices
constexpr int M_CSCP = 7;   // M_CSC, software-pipelined at 4 blocks per SM (large matrices)
constexpr int M_CSCQ = 8;   // M_CSCP reading 16-bit row offsets (rows below 2^19)
template <int MODE> constexpr bool kIdx16 = MODE == M_CSR16 || MODE == M_CSRS16 || MODE == M_CSCQ;
template <int MODE> constexpr bool kCsrFirst = MODE == M_CSR || MODE == M_CSR16;
template <int MODE> constexpr bool kCsrShared = MODE == M_CSRS || MODE == M_CSRS16;
template <int MODE> constexpr bool kCscFirst = MODE == M_CSC || MODE == M_CSCP || MODE == M_CSCQ;

// Resident blocks per SM asked of the compiler (register cap) and the
// software-pipeline depth of the vector layout, per sweep mode.  Measured on
// the 480,189 x 17,770 workload (BF16 / FP32 residual, us per launch):
//   CSC sweep: 6 blocks, no pipeline 223 / 269; M_CSCP, 4 blocks (56
//              registers), streams of the next 2 chunks loaded before the
//              gathers of the current 2: 200 / 251; 3 blocks 200; 5 blocks
//              205; 1 or 3 chunks at 4 blocks 213 / 201.
//   CSR sweeps: 6 blocks, no pipeline 216; 5 blocks 220; 4 blocks, 2 chunks
//              231; 6 blocks with a pipeline spill (40 registers): 411.  They
//              are bound by L1 data-pipe wavefronts (82-86 % of peak), not
//              by latency.
// On the 64-problem batch (short lines) M_CSCP measured 5 % slower than
// M_CSC, so the engine takes it from 16M nonzeros up.
template <int MODE> constexpr int kSweepBlocks = MODE == M_CSCP || MODE == M_CSCQ ? 4 : 6;
template <int MODE> constexpr int kPipe = MODE == M_CSCP || MODE == M_CSCQ ? 2 : 0;

struct XTask {            // one chunk of a split line
    uint32_t line, beg, end, slot;
    uint32_t xl, first_slot, nchunks, pad;
};

struct SweepArgs {
    const uint32_t* __restrict__ ptr;
    const uint32_t* __restrict__ idx;
    void* __restrict__ res;
    const float* __restrict__ y;   // M_PLAIN: cross vector
    const float2* __restrict__ P;  // M_CSC: packed cross table
    const float4* __restrict__ Q;  // M_CSR: packed cross table
    const float* b;                // subtract: line vector (previous feature, final)
    const float* d;                // add-back: line vector (this feature, old)
    float* out;                    // solve: line vector (written)
    float4* emitQ;                 // M_CSC: Q[j] = (b_j, d_j, x_j, 0)
    float2* emitP;                 // CSR sweeps that end a feature: P[i] = (x_i, next_old[i])
    const float* next_old;         // W of the next feature (old), for emitP
    float lambda;
    // work lists
    const XTask* xt;
    const uint32_t* cl;
    const uint32_t* wl;
    const uint32_t* gl;
    const uint32_t* tl;
    uint32_t nx, nc, nw, ng, nt;
    uint32_t nwb;                  // blocks of the warp bin
    uint32_t ngb;                  // blocks of the group bin (32 lines per block)
    float2* part;                  // split-line partials
    uint32_t* xcount;              // split-line arrival counters (left at 0)
    float* out2;                   // M_DUAL: sum of y^2 per line (out gets the sum of y * r)
    uint32_t ncross;               // M_CSRS: entries of the cross table (columns)
    uint32_t group_short;          // group lines up to this length: interleaved layout
    uint32_t group_lanes;          // lanes per group-bin line: 4 or 8
    const uint16_t* __restrict__ idx16;   // M_CSR16 / M_CSRS16: the column indices; M_CSCQ: the row offsets
    const uint32_t* __restrict__ cseg;    // M_CSCQ: per column, kCSeg segment ends (see RowDec)
};

// The cross table of an M_CSRS sweep, as three float planes (a | c | y) in
// dynamic shared memory.
extern __shared__ float cdmf_qsm[];

// Thread teams that run the work of one sweep block.
// CtaTeam: the whole CTA (kBlock threads).
struct CtaTeam {
    static __device__ __forceinline__ uint32_t tid() { return threadIdx.x; }
    static __device__ __forceinline__ void sync() { __syncthreads(); }
    static __device__ __forceinline__ float2* red() {
        __shared__ float2 sm[kWarps];
        return sm;
    }
    static __device__ __forceinline__ int* flag() {
        __shared__ int f;
        return &f;
    }
};
// SubTeam: one of kSubs groups of kBlock threads in a kSubs * kBlock CTA,
// synchronised by its own named barrier (ids 1..kSubs).
constexpr int kSubs = 4;
struct SubTeam {
    static __device__ __forceinline__ uint32_t sub() { return threadIdx.x / kBlock; }
    static __device__ __forceinline__ uint32_t tid() { return threadIdx.x % kBlock; }
    static __device__ __forceinline__ void sync() {
        asm volatile("bar.sync %0, %1;" ::"r"(sub() + 1), "r"(kBlock) : "memory");
    }
    static __device__ __forceinline__ float2* red() {
        __shared__ float2 sm[kSubs][kWarps];
        return sm[sub()];
    }
    static __device__ __forceinline__ int* flag() {
        __shared__ int f[kSubs];
        return &f[sub()];
    }
};

// ---- streaming loads -----------------------------------------------------------
// 128-bit and 64-bit loads of the index and residual streams, evict-first
// (read once per sweep), with the 256-byte L2 prefetch-size hint: an L2 miss
// fetches that many bytes from DRAM, so the next chunk of a lane's stream is
// on its way before the lane asks for it.  (Measured: +0.9 % FP32 updates/s,
// neutral at BF16; an L1::no_allocate hint instead of evict-first: neutral.)
__device__ __forceinline__ uint4 ld_stream4(const void* p) {
    uint4 v;
    asm("ld.global.cs.L2::256B.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ uint2 ld_stream2(const void* p) {
    uint2 v;
    asm("ld.global.cs.L2::256B.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

// ---- residual element access -------------------------------------------------
template <int RT> struct Res;
template <> struct Res<0> {
    static __device__ __forceinline__ float ld(const void* p, uint32_t q) { return __ldcs((const float*)p + q); }
    static __device__ __forceinline__ float st(void* p, uint32_t q, float v) { __stcs((float*)p + q, v); return v; }
    static __device__ __forceinline__ void ld4(const void* p, uint32_t q, float (&r)[4]) {
        const uint4 v = ld_stream4((const float*)p + q);
        r[0] = __uint_as_float(v.x); r[1] = __uint_as_float(v.y); r[2] = __uint_as_float(v.z); r[3] = __uint_as_float(v.w);
    }
    static __device__ __forceinline__ void st4(void* p, uint32_t q, float (&r)[4]) {
        __stcs((float4*)((float*)p + q), make_float4(r[0], r[1], r[2], r[3]));
    }
};
template <int KIND> struct Res16 {
    static __device__ __forceinline__ float to_f(unsigned short u) {
        if (KIND == 1) return __bfloat162float(__ushort_as_bfloat16(u));
        return __half2float(__ushort_as_half(u));
    }
    static __device__ __forceinline__ unsigned short from_f(float v, float& rounded) {
        if (KIND == 1) {
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            rounded = __bfloat162float(h);
            return __bfloat16_as_ushort(h);
        }
        const __half h = __float2half_rn(v);
        rounded = __half2float(h);
        return __half_as_ushort(h);
    }
    static __device__ __forceinline__ float ld(const void* p, uint32_t q) {
        return to_f(__ldcs((const unsigned short*)p + q));
    }
    static __device__ __forceinline__ float st(void* p, uint32_t q, float v) {
        float rv;
        __stcs((unsigned short*)p + q, from_f(v, rv));
        return rv;
    }
    static __device__ __forceinline__ void ld4(const void* p, uint32_t q, float (&r)[4]) {
        const uint2 v = ld_stream2((const unsigned short*)p + q);
        r[0] = to_f((unsigned short)(v.x & 0xffff));
        r[1] = to_f((unsigned short)(v.x >> 16));
        r[2] = to_f((unsigned short)(v.y & 0xffff));
        r[3] = to_f((unsigned short)(v.y >> 16));
    }
    // rounds r[] to storage precision in place and stores
    static __device__ __forceinline__ void st4(void* p, uint32_t q, float (&r)[4]) {
        const unsigned u0 = from_f(r[0], r[0]), u1 = from_f(r[1], r[1]), u2 = from_f(r[2], r[2]),
                       u3 = from_f(r[3], r[3]);
        __stcs((uint2*)((unsigned short*)p + q), make_uint2(u0 | (u1 << 16), u2 | (u3 << 16)));
    }
};
template <> struct Res<1> : Res16<1> {};
template <> struct Res<2> : Res16<2> {};

// Running sum; with KAHAN the lost low-order part is carried in `c`
// (compensated summation).  With a 16-bit residual every line longer than
// kKahanMin nonzeros sums with it: CTA and split lines always, warp lines
// above kKahanMin.
constexpr uint32_t kKahanMin = 4096;
template <bool KAHAN> struct Acc {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        if (KAHAN) {
            const float y = __fsub_rn(x, c);
            const float t = __fadd_rn(s, y);
            c = __fsub_rn(__fsub_rn(t, s), y);
            s = t;
        } else {
            s = __fadd_rn(s, x);
        }
    }
    __device__ __forceinline__ float value() const { return KAHAN ? __fsub_rn(s, c) : s; }
};

// Cross-vector values of one nonzero with cross index i.
template <int MODE>
__device__ __forceinline__ void fetch(const SweepArgs& A, uint32_t i, float& a, float& c, float& y) {
    if (kCscFirst<MODE>) {
        const float2 p = __ldg(A.P + i);
        a = p.x;
        c = p.y;
        y = p.y;
    } else if (kCsrFirst<MODE>) {
        const float4 q = __ldg(A.Q + i);
        a = q.x;
        c = q.y;
        y = q.z;
    } else if (kCsrShared<MODE>) {
        a = cdmf_qsm[i];
        c = cdmf_qsm[A.ncross + i];
        y = cdmf_qsm[2 * A.ncross + i];
    } else {
        a = c = 0.0f;
        y = __ldg(A.y + i);
    }
}

template <bool SUB, bool ADD>
__device__ __forceinline__ float update(float r, float a, float c, float bj, float dj) {
    if (SUB) r = __fsub_rn(r, __fmul_rn(a, bj));
    if (ADD) r = __fadd_rn(r, __fmul_rn(c, dj));
    return r;
}

template <class AccT>
__device__ __forceinline__ void accumulate(AccT& g, AccT& h, float y, float r) {
    g.add(__fmul_rn(y, r));
    h.add(__fmul_rn(y, y));
}

// Index stream loads: one index, or the 4 indices at a 4-aligned position.
template <int MODE>
__device__ __forceinline__ uint32_t ld_idx1(const SweepArgs& A, uint32_t q) {
    if (kIdx16<MODE>) return __ldcs(A.idx16 + q);
    return __ldcs(A.idx + q);
}
template <int MODE>
__device__ __forceinline__ void ld_idx4(const SweepArgs& A, uint32_t q, uint32_t (&iv)[4]) {
    if (kIdx16<MODE>) {
        const uint2 v = ld_stream2(A.idx16 + q);
        iv[0] = v.x & 0xffffu; iv[1] = v.x >> 16; iv[2] = v.y & 0xffffu; iv[3] = v.y >> 16;
    } else {
        const uint4 v = ld_stream4(A.idx + q);
        iv[0] = v.x; iv[1] = v.y; iv[2] = v.z; iv[3] = v.w;
    }
}

// Index decoding.  M_CSCQ stores each row as its 16-bit offset inside a
// segment of 65,536 rows; rows are sorted inside a column, so a column is cut
// into at most kCSeg runs of one segment each, and cseg[kCSeg * j + h] holds
// where run h of column j ends (the column's end from the last non-empty run
// on).  A lane keeps the segment of its current position and moves forward as
// its positions grow (they only grow inside one strided pass).  Other modes
// read indices as stored.
constexpr uint32_t kCSeg = 8;
template <int MODE, bool ON = (MODE == M_CSCQ)>
struct RowDec {
    __device__ __forceinline__ void init(const SweepArgs&, uint32_t, uint32_t) {}
    __device__ __forceinline__ uint32_t row(uint32_t, uint32_t raw) { return raw; }
};
template <int MODE>
struct RowDec<MODE, true> {
    const uint32_t* seg;
    uint32_t hi, nxt;
    __device__ __forceinline__ void init(const SweepArgs& A, uint32_t line, uint32_t q) {
        seg = A.cseg + (size_t)line * kCSeg;
        hi = 0;
        nxt = __ldg(seg);
        (void)row(q, 0);
    }
    __device__ __forceinline__ uint32_t row(uint32_t q, uint32_t raw) {
        while (q >= nxt && hi < kCSeg - 1) nxt = __ldg(seg + ++hi);
        return (hi << 16) | raw;
    }
};

// One scalar element: update, store, accumulate.
template <int RT, int MODE, bool SUB, bool ADD, class AccT>
__device__ __forceinline__ void elem1(const SweepArgs& A, uint32_t q, float bj, float dj, AccT& g, AccT& h,
                                      RowDec<MODE>& dec) {
    const uint32_t i = dec.row(q, ld_idx1<MODE>(A, q));
    float r = Res<RT>::ld(A.res, q);
    float a, c, y;
    fetch<MODE>(A, i, a, c, y);
    if (SUB || ADD) r = Res<RT>::st(A.res, q, update<SUB, ADD>(r, a, c, bj, dj));
    accumulate(g, h, y, r);
}

// Pass over [beg, end) by S cooperating threads (this one is `lane`): a scalar
// head up to the first 4-aligned position (lanes 0..2), then 4-element vector
// chunks (chunk c to lane c mod S, kChunks chunks in flight per lane), then a
// scalar tail.  Each lane visits its elements in increasing order.
constexpr int kChunks = 2;   // vector layout: 4-element chunks in flight per lane
constexpr int kIlp = 4;      // interleaved layout: elements in flight per lane

// Packed stream values of one 4-element chunk, index (4 x 32-bit or 4 x
// 16-bit) and residual (4 x FP32 or 4 x 16-bit), held packed while in flight.
template <int RT, int MODE>
struct Chunk4 {
    using IT = typename std::conditional<kIdx16<MODE>, uint2, uint4>::type;
    using VT = typename std::conditional<RT == 0, uint4, uint2>::type;
    IT i;
    VT r;
    __device__ __forceinline__ void load(const SweepArgs& A, uint32_t q) {
        if constexpr (kIdx16<MODE>) i = ld_stream2(A.idx16 + q);
        else i = ld_stream4(A.idx + q);
        if constexpr (RT == 0) r = ld_stream4((const float*)A.res + q);
        else r = ld_stream2((const unsigned short*)A.res + q);
    }
    __device__ __forceinline__ uint32_t idx(int e) const {
        if constexpr (kIdx16<MODE>) {
            const uint32_t w = e < 2 ? i.x : i.y;
            return (e & 1) ? (w >> 16) : (w & 0xffffu);
        } else {
            return e == 0 ? i.x : e == 1 ? i.y : e == 2 ? i.z : i.w;
        }
    }
    __device__ __forceinline__ float res(int e) const {
        if constexpr (RT == 0) {
            return __uint_as_float(e == 0 ? r.x : e == 1 ? r.y : e == 2 ? r.z : r.w);
        } else {
            const uint32_t w = e < 2 ? r.x : r.y;
            return Res16<RT>::to_f((unsigned short)((e & 1) ? (w >> 16) : (w & 0xffffu)));
        }
    }
};

// Update, store and accumulate the 4 elements of a loaded chunk at q.
template <int RT, int MODE, bool SUB, bool ADD, class AccT>
__device__ __forceinline__ void chunk4(const SweepArgs& A, uint32_t q, const Chunk4<RT, MODE>& C, float bj, float dj,
                                       AccT& g, AccT& h, RowDec<MODE>& dec) {
    float r[4], y[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float a, c;
        fetch<MODE>(A, dec.row(q + e, C.idx(e)), a, c, y[e]);
        r[e] = update<SUB, ADD>(C.res(e), a, c, bj, dj);
    }
    if (SUB || ADD) Res<RT>::st4(A.res, q, r);
#pragma unroll
    for (int e = 0; e < 4; ++e) accumulate(g, h, y[e], r[e]);
}

// Vector layout (default; measured faster for 16-bit residuals): lane takes
// 4 consecutive nonzeros per 128-bit load, after a scalar head that reaches a
// 4-aligned position, then a scalar tail.  PIPE = 0: kChunks chunks loaded,
// then their gathers; PIPE > 0: software-pipelined, the streams of the next
// PIPE chunks are loaded before the gathers of the current PIPE chunks.  Both
// visit a lane's elements in increasing order, so their sums are identical.
template <int RT, int MODE, bool SUB, bool ADD, int S, bool KAHAN, int PIPE>
__device__ __forceinline__ void strided_vec(const SweepArgs& A, uint32_t beg, uint32_t end, uint32_t lane, float bj,
                                            float dj, float& gs, float& hs, RowDec<MODE>& dec) {
    Acc<KAHAN> g, h;
    uint32_t vbeg = (beg + 3u) & ~3u;
    if (vbeg > end) vbeg = end;
    const uint32_t vend = vbeg + ((end - vbeg) & ~3u);
    if (lane < vbeg - beg) elem1<RT, MODE, SUB, ADD>(A, beg + lane, bj, dj, g, h, dec);
    uint32_t q = vbeg + 4u * lane;
    if constexpr (PIPE > 0) {
        constexpr uint32_t STEP = 4u * S;
        if (q < vend) {
            Chunk4<RT, MODE> cur[PIPE];
#pragma unroll
            for (int u = 0; u < PIPE; ++u)
                if (q + u * STEP < vend) cur[u].load(A, q + u * STEP);
            for (;;) {
                const uint32_t qn = q + PIPE * STEP;
                Chunk4<RT, MODE> nxt[PIPE];
#pragma unroll
                for (int u = 0; u < PIPE; ++u)
                    if (qn + u * STEP < vend) nxt[u].load(A, qn + u * STEP);
#pragma unroll
                for (int u = 0; u < PIPE; ++u)
                    if (q + u * STEP < vend) chunk4<RT, MODE, SUB, ADD>(A, q + u * STEP, cur[u], bj, dj, g, h, dec);
                if (qn >= vend) break;
                q = qn;
#pragma unroll
                for (int u = 0; u < PIPE; ++u) cur[u] = nxt[u];
            }
        }
        q = vend;
    }
    for (; q + 4u * S * (kChunks - 1) < vend; q += 4u * S * kChunks) {
        uint32_t iv[kChunks][4];
        float r[kChunks][4];
#pragma unroll
        for (int u = 0; u < kChunks; ++u) {
            ld_idx4<MODE>(A, q + 4u * S * u, iv[u]);
            Res<RT>::ld4(A.res, q + 4u * S * u, r[u]);
        }
#pragma unroll
        for (int u = 0; u < kChunks; ++u) {
            float y[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                float a, c;
                fetch<MODE>(A, dec.row(q + 4u * S * u + e, iv[u][e]), a, c, y[e]);
                r[u][e] = update<SUB, ADD>(r[u][e], a, c, bj, dj);
            }
            if (SUB || ADD) Res<RT>::st4(A.res, q + 4u * S * u, r[u]);
#pragma unroll
            for (int e = 0; e < 4; ++e) accumulate(g, h, y[e], r[u][e]);
        }
    }
    for (; q < vend; q += 4u * S) {
        uint32_t iv[4];
        ld_idx4<MODE>(A, q, iv);
        float r[4], y[4];
        Res<RT>::ld4(A.res, q, r);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            float a, c;
            fetch<MODE>(A, dec.row(q + e, iv[e]), a, c, y[e]);
            r[e] = update<SUB, ADD>(r[e], a, c, bj, dj);
        }
        if (SUB || ADD) Res<RT>::st4(A.res, q, r);
#pragma unroll
        for (int e = 0; e < 4; ++e) accumulate(g, h, y[e], r[e]);
    }
    if (lane < end - vend) elem1<RT, MODE, SUB, ADD>(A, vend + lane, bj, dj, g, h, dec);
    gs = g.value();
    hs = h.value();
}
// Interleaved layout: lane takes nonzeros beg+lane, beg+lane+S, ... so that
// the S lanes of one load, and of the gather that follows it, touch S
// consecutive nonzeros -- neighbouring cross indices, few cache lines per
// gather.  ILP nonzeros per lane are in flight per step.
template <int RT, int MODE, bool SUB, bool ADD, int S, bool KAHAN>
__device__ __forceinline__ void strided_il(const SweepArgs& A, uint32_t beg, uint32_t end, uint32_t lane, float bj,
                                           float dj, float& gs, float& hs, RowDec<MODE>& dec) {
    Acc<KAHAN> g, h;
    uint32_t q = beg + lane;
    for (; q + (uint32_t)S * (kIlp - 1) < end; q += (uint32_t)S * kIlp) {
        uint32_t iv[kIlp];
        float r[kIlp], a[kIlp], c[kIlp], y[kIlp];
#pragma unroll
        for (int u = 0; u < kIlp; ++u) {
            iv[u] = ld_idx1<MODE>(A, q + S * u);
            r[u] = Res<RT>::ld(A.res, q + S * u);
        }
#pragma unroll
        for (int u = 0; u < kIlp; ++u) fetch<MODE>(A, dec.row(q + S * u, iv[u]), a[u], c[u], y[u]);
#pragma unroll
        for (int u = 0; u < kIlp; ++u) {
            if (SUB || ADD) r[u] = Res<RT>::st(A.res, q + S * u, update<SUB, ADD>(r[u], a[u], c[u], bj, dj));
            accumulate(g, h, y[u], r[u]);
        }
    }
    for (; q < end; q += S) elem1<RT, MODE, SUB, ADD>(A, q, bj, dj, g, h, dec);
    gs = g.value();
    hs = h.value();
}

// Thread-bin lines: loads of this many nonzeros in flight per thread
// (measured: 4 takes the 64-problem batch from 178 to 172 ms, neutral on the
// Netflix-shaped matrix).
constexpr int kThreadUnroll = 4;
// Lane-group lines of at most SweepArgs::group_short nonzeros take the
// interleaved layout with the whole line in flight at once; everything else
// the vector layout.  (Measured slower: the interleaved layout for all
// lines, -8 % on the Netflix-shaped matrix with 8-lane groups at 4 in
// flight; 8-nonzero chunks; staging the streams through shared memory with
// cp.async, which takes L1 capacity from the gather tables.)
template <int RT, int MODE, bool SUB, bool ADD, int S, bool KAHAN>
__device__ __forceinline__ void strided(const SweepArgs& A, uint32_t line, uint32_t beg, uint32_t end, uint32_t lane,
                                        float bj, float dj, float& gs, float& hs) {
    RowDec<MODE> dec;
    dec.init(A, line, beg);
    if (S <= 8 && end - beg <= A.group_short)
        strided_il<RT, MODE, SUB, ADD, S, KAHAN>(A, beg, end, lane, bj, dj, gs, hs, dec);
    else
        strided_vec<RT, MODE, SUB, ADD, S, KAHAN, kPipe<MODE>>(A, beg, end, lane, bj, dj, gs, hs, dec);
}

template <int WIDTH = 32>
__device__ __forceinline__ void warp_sum2(float& g, float& h) {
#pragma unroll
    for (int o = WIDTH / 2; o > 0; o >>= 1) {
        g = __fadd_rn(g, __shfl_xor_sync(0xffffffffu, g, o));
        h = __fadd_rn(h, __shfl_xor_sync(0xffffffffu, h, o));
    }
}

// CTA-wide sum; the result is valid in thread 0.  Fixed shape: per-warp xor
// tree, then warps 0..7 in order.
template <class Team = CtaTeam>
__device__ __forceinline__ void cta_sum2(float& g, float& h) {
    float2* sm = Team::red();
    warp_sum2(g, h);
    const uint32_t w = Team::tid() >> 5;
    if ((Team::tid() & 31) == 0) sm[w] = make_float2(g, h);
    Team::sync();
    if (Team::tid() == 0) {
        float G = sm[0].x, Hs = sm[0].y;
        for (int q = 1; q < kWarps; ++q) { G = __fadd_rn(G, sm[q].x); Hs = __fadd_rn(Hs, sm[q].y); }
        g = G;
        h = Hs;
    }
}

// Writes x_j and the packed table entries derived from it.
template <int MODE>
__device__ __forceinline__ void write_line(const SweepArgs& A, uint32_t j, float x, float bj, float dj) {
    A.out[j] = x;
    if (kCscFirst<MODE>) A.emitQ[j] = make_float4(bj, dj, x, 0.0f);
    if (A.emitP) A.emitP[j] = make_float2(x, A.next_old == A.out ? x : A.next_old[j]);
}

// x_j from tree sums; h excludes lambda * nnz_j.
template <int MODE>
__device__ __forceinline__ void finish_line(const SweepArgs& A, uint32_t j, uint32_t len, float g, float h, float bj,
                                            float dj) {
    if (MODE == M_DUAL) {
        A.out[j] = g;
        A.out2[j] = h;
        return;
    }
    const float lam = __fmul_rn(A.lambda, __uint2float_rn(len));
    write_line<MODE>(A, j, len == 0 ? 0.0f : __fdiv_rn(g, __fadd_rn(lam, h)), bj, dj);
}

// Per-line scalars: b_j (previous feature's final value) and d_j (this
// feature's old value).  The CSC sweep also forwards them into Q.
template <int MODE, bool SUB, bool ADD>
__device__ __forceinline__ void line_scalars(const SweepArgs& A, uint32_t j, float& bj, float& dj) {
    bj = (SUB || kCscFirst<MODE>) && A.b ? A.b[j] : 0.0f;
    dj = (ADD || kCscFirst<MODE>) ? A.d[j] : 0.0f;
}

// Block b of the group bin: one line per L-lane group, kBlock / L lines.
template <int RT, int MODE, bool SUB, bool ADD, int L>
__device__ __forceinline__ void group_line(const SweepArgs& A, uint32_t b, uint32_t tid) {
    const uint32_t slot = b * (kBlock / L) + tid / L;
    const uint32_t sub = tid % L;
    const bool valid = slot < A.ng;
    const uint32_t j = valid ? A.gl[slot] : 0u;
    const uint32_t beg = valid ? A.ptr[j] : 0u, end = valid ? A.ptr[j + 1] : 0u;
    float bj = 0.0f, dj = 0.0f;
    if (valid) line_scalars<MODE, SUB, ADD>(A, j, bj, dj);
    float g = 0.0f, h = 0.0f;
    strided<RT, MODE, SUB, ADD, L, false>(A, j, beg, end, sub, bj, dj, g, h);
    warp_sum2<L>(g, h);
    if (valid && sub == 0) finish_line<MODE>(A, j, end - beg, g, h, bj, dj);
}

// Work of block b of one sweep (b in [0, nx + nc + nwb + ngb + ntb)).
template <int RT, int MODE, bool SUB, bool ADD, class Team = CtaTeam>
__device__ __forceinline__ void sweep_block(const SweepArgs& A, uint32_t b) {
    const uint32_t tid = Team::tid();
    if (b < A.nx) {                                        // split-line chunk
        const XTask T = A.xt[b];
        float bj, dj;
        line_scalars<MODE, SUB, ADD>(A, T.line, bj, dj);
        float g = 0.0f, h = 0.0f;
        strided<RT, MODE, SUB, ADD, kBlock, RT != 0>(A, T.line, T.beg, T.end, tid, bj, dj, g, h);
        cta_sum2<Team>(g, h);
        int& last = *Team::flag();
        if (tid == 0) {
            A.part[T.slot] = make_float2(g, h);
            __threadfence();
            const uint32_t prev = atomicAdd(A.xcount + T.xl, 1u);
            last = (prev == T.nchunks - 1);
        }
        Team::sync();
        if (last && tid == 0) {
            __threadfence();
            float G = 0.0f, Hs = 0.0f;
            for (uint32_t q = 0; q < T.nchunks; ++q) {
                const float2 p = __ldcg(A.part + T.first_slot + q);
                G = __fadd_rn(G, p.x);
                Hs = __fadd_rn(Hs, p.y);
            }
            const uint32_t len = A.ptr[T.line + 1] - A.ptr[T.line];
            finish_line<MODE>(A, T.line, len, G, Hs, bj, dj);
            A.xcount[T.xl] = 0;
        }
        return;
    }
    b -= A.nx;
    if (b < A.nc) {                                        // one line per CTA
        const uint32_t j = A.cl[b];
        const uint32_t beg = A.ptr[j], end = A.ptr[j + 1];
        float bj, dj;
        line_scalars<MODE, SUB, ADD>(A, j, bj, dj);
        float g = 0.0f, h = 0.0f;
        strided<RT, MODE, SUB, ADD, kBlock, RT != 0>(A, j, beg, end, tid, bj, dj, g, h);
        cta_sum2<Team>(g, h);
        if (tid == 0) finish_line<MODE>(A, j, end - beg, g, h, bj, dj);
        return;
    }
    b -= A.nc;
    if (b < A.nwb) {                                       // one line per warp
        const uint32_t w = b * kWarps + (tid >> 5);
        if (w >= A.nw) return;
        const uint32_t lane = tid & 31;
        const uint32_t j = A.wl[w];
        const uint32_t beg = A.ptr[j], end = A.ptr[j + 1];
        float bj, dj;
        line_scalars<MODE, SUB, ADD>(A, j, bj, dj);
        float g = 0.0f, h = 0.0f;
        if (RT != 0 && end - beg > kKahanMin)
            strided<RT, MODE, SUB, ADD, 32, true>(A, j, beg, end, lane, bj, dj, g, h);
        else
            strided<RT, MODE, SUB, ADD, 32, false>(A, j, beg, end, lane, bj, dj, g, h);
        warp_sum2(g, h);
        if (lane == 0) finish_line<MODE>(A, j, end - beg, g, h, bj, dj);
        return;
    }
    b -= A.nwb;
    if (b < A.ngb) {                                       // one line per lane group
        if (A.group_lanes == 4) group_line<RT, MODE, SUB, ADD, 4>(A, b, tid);
        else group_line<RT, MODE, SUB, ADD, 8>(A, b, tid);
        return;
    }
    b -= A.ngb;
    const uint32_t t = b * kBlock + tid;           // one line per thread
    if (t >= A.nt) return;
    const uint32_t j = A.tl[t];
    const uint32_t beg = A.ptr[j], end = A.ptr[j + 1];
    const uint32_t len = end - beg;
    float bj, dj;
    line_scalars<MODE, SUB, ADD>(A, j, bj, dj);
    RowDec<MODE> dec;
    dec.init(A, j, beg);
    if (MODE == M_DUAL) {
        Acc<false> g, h;
        for (uint32_t q = beg; q < end; ++q) elem1<RT, MODE, SUB, ADD>(A, q, bj, dj, g, h, dec);
        A.out[j] = g.s;
        A.out2[j] = h.s;
        return;
    }
    if (len == 0) {
        write_line<MODE>(A, j, 0.0f, bj, dj);
        return;
    }
    Acc<false> g, h;
    h.s = __fmul_rn(A.lambda, __uint2float_rn(len));         // h starts at lambda*nnz (src/cdmf_ref.cpp:8)
    uint32_t q = beg;
    // loads of kThreadUnroll nonzeros in flight; sums still in index order
    for (; q + kThreadUnroll <= end; q += kThreadUnroll) {
        uint32_t iv[kThreadUnroll];
        float r[kThreadUnroll];
#pragma unroll
        for (int e = 0; e < kThreadUnroll; ++e) {
            iv[e] = ld_idx1<MODE>(A, q + e);
            r[e] = Res<RT>::ld(A.res, q + e);
        }
#pragma unroll
        for (int e = 0; e < kThreadUnroll; ++e) {
            float a, c, y;
            fetch<MODE>(A, dec.row(q + e, iv[e]), a, c, y);
            if (SUB || ADD) r[e] = Res<RT>::st(A.res, q + e, update<SUB, ADD>(r[e], a, c, bj, dj));
            accumulate(g, h, y, r[e]);
        }
    }
    for (; q < end; ++q) elem1<RT, MODE, SUB, ADD>(A, q, bj, dj, g, h, dec);
    write_line<MODE>(A, j, __fdiv_rn(g.s, h.s), bj, dj);
}

template <int RT, int MODE, bool SUB, bool ADD>
__global__ void __launch_bounds__(kBlock, kSweepBlocks<MODE>) sweep_kernel(const SweepArgs A) {
    sweep_block<RT, MODE, SUB, ADD>(A, blockIdx.x);
}

// CSR sweep of a narrow matrix (the cross table fits in shared memory): one
// CTA of kSubs * kBlock threads per SM copies Q into shared memory as three
// float planes, then its kSubs teams pull sweep blocks from a device work
// queue and run them with every gather served from shared memory.  The
// arithmetic is M_CSR's, element for element.
template <int RT, bool SUB, bool ADD, int MS = M_CSRS>
__global__ void __launch_bounds__(kBlock * kSubs, 1) sweep_smemq_kernel(const SweepArgs A, uint32_t nblocks,
                                                                      uint32_t* queue) {
    const uint32_t n = A.ncross;
    for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
        const float4 v = __ldg(A.Q + j);
        cdmf_qsm[j] = v.x;
        cdmf_qsm[n + j] = v.y;
        cdmf_qsm[2 * n + j] = v.z;
    }
    __syncthreads();
    __shared__ uint32_t blk[kSubs];
    const uint32_t sub = SubTeam::sub();
    for (;;) {
        if (SubTeam::tid() == 0) blk[sub] = atomicAdd(queue, 1u);
        SubTeam::sync();
        const uint32_t b = blk[sub];
        SubTeam::sync();
        if (b >= nblocks) return;
        sweep_block<RT, MS, SUB, ADD, SubTeam>(A, b);
    }
}

// P[i] = (prev[i] or 0, cur[i]): the packed CSC table when no sweep has
// written it (start of a run, after a state change).
static __global__ void pack_p_kernel(float2* __restrict__ P, const float* __restrict__ prev, const float* __restrict__ cur,
                              int64_t len) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x)
        P[i] = make_float2(prev ? prev[i] : 0.0f, cur[i]);
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

// Test RMSE (src/tools.cpp:543-582, and :489-541 for the text test file):
// per entry the float products W[t][i]*H[t][j] are summed in double in t
// order, (pred - v)^2 in double, NaN terms skipped but counted.  Fixed grid;
// block partials in double; the last block adds them in block order and
// writes sqrt(sum / nnz_test) and the NaN count.
// float -> double, exactly, without the FP64 pipe for normal values: the
// exponent is rebiased and the mantissa shifted with integer operations (the
// GB300's FP64 units are few, and the test RMSE widens k products per test
// entry).  Zero keeps its sign; subnormals, infinities and NaN take the
// conversion instruction.  Same value as (double)x for every float.
__device__ __forceinline__ double widen(float x) {
    const uint32_t u = __float_as_uint(x);
    const uint32_t e = (u >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) {
        if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
        return (double)x;
    }
    const uint32_t hi = (u & 0x80000000u) | ((e + (1023u - 127u)) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)((u & 7u) << 29));
}

// Block `bid` of `nblk` blocks of one test-RMSE reduction.
template <class VT>
__device__ __forceinline__ void rmse_body(const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                                          const VT* __restrict__ val, int64_t nt, const float* __restrict__ W,
                                          const float* __restrict__ H, int64_t m, int64_t n, uint32_t k, double* part,
                                          uint32_t* counter, double* out, unsigned long long* nan_out, uint32_t bid,
                                          uint32_t nblk) {
    double acc = 0.0;
    unsigned nans = 0;
    for (int64_t e = (int64_t)bid * kBlock + threadIdx.x; e < nt; e += (int64_t)nblk * kBlock) {
        const uint32_t i = row[e], j = col[e];
        double pred = 0.0;
        for (uint32_t t = 0; t < k; ++t)
            pred = __dadd_rn(pred, widen(__fmul_rn(__ldg(W + (size_t)t * m + i), __ldg(H + (size_t)t * n + j))));
        const double dv = __dsub_rn(pred, (double)val[e]);
        const double tmp = __dmul_rn(dv, dv);
        if (!isnan(tmp)) acc = __dadd_rn(acc, tmp);
        else nans++;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc = __dadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
        nans += __shfl_xor_sync(0xffffffffu, nans, o);
    }
    __shared__ double sm[kWarps];
    __shared__ unsigned smn[kWarps];
    __shared__ int last;
    if ((threadIdx.x & 31) == 0) {
        sm[threadIdx.x >> 5] = acc;
        smn[threadIdx.x >> 5] = nans;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = sm[0];
        unsigned long long c = smn[0];
        for (int q = 1; q < kWarps; ++q) { s = __dadd_rn(s, sm[q]); c += smn[q]; }
        part[bid] = s;
        if (nan_out && c) atomicAdd(nan_out, c);
        __threadfence();
        last = (atomicAdd(counter, 1u) == nblk - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double s = 0.0;
        for (uint32_t q = 0; q < nblk; ++q) s = __dadd_rn(s, __ldcg(part + q));
        *out = sqrt(s / (double)nt);
        *counter = 0;
    }
}

template <class VT>
__global__ void __launch_bounds__(kBlock) rmse_kernel(const uint32_t* __restrict__ row, const uint32_t* __restrict__ col,
                                                      const VT* __restrict__ val, int64_t nt,
                                                      const float* __restrict__ W, const float* __restrict__ H,
                                                      int64_t m, int64_t n, uint32_t k, double* part,
                                                      uint32_t* counter, double* out,
                                                      unsigned long long* nan_out) {
    rmse_body<VT>(row, col, val, nt, W, H, m, n, k, part, counter, out, nan_out, blockIdx.x, gridDim.x);
}

}  // namespace cdmf
