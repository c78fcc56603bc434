// Definitions of the launchers declared in launch.h, for one residual type
// (-DCDMF_LAUNCH_RT=0|1|2) and one kernel family (-DCDMF_LAUNCH_PART=0|1).
// The build compiles this file once per pair, so each object holds one slice
// of the kernel instantiations and the slices compile in parallel.  Without
// the macros the file instantiates everything (one slow translation unit).
#include "launch.h"

#if !defined(CDMF_LAUNCH_PART)
#define CDMF_PART0 1
#define CDMF_PART1 1
#elif CDMF_LAUNCH_PART == 0
#define CDMF_PART0 1
#define CDMF_PART1 0
#elif CDMF_LAUNCH_PART == 1
#define CDMF_PART0 0
#define CDMF_PART1 1
#else
#error "CDMF_LAUNCH_PART is 0 or 1"
#endif

#if !defined(CDMF_LAUNCH_RT)
#define CDMF_FOR_RT(X) X(0) X(1) X(2)
#define CDMF_FOR_RT16(X) X(1) X(2)
#define CDMF_HAS_RT0 1
#elif CDMF_LAUNCH_RT == 0
#define CDMF_FOR_RT(X) X(0)
#define CDMF_FOR_RT16(X)
#define CDMF_HAS_RT0 1
#elif CDMF_LAUNCH_RT == 1 || CDMF_LAUNCH_RT == 2
#define CDMF_FOR_RT(X) X(CDMF_LAUNCH_RT)
#define CDMF_FOR_RT16(X) X(CDMF_LAUNCH_RT)
#define CDMF_HAS_RT0 0
#else
#error "CDMF_LAUNCH_RT is 0, 1 or 2"
#endif

namespace cdmf {

#if CDMF_PART0

namespace {

template <int RT, int MODE>
void launch_mode(const SweepArgs& A, bool sub, bool add, unsigned grid, cudaStream_t s) {
    prefer_l1(sweep_kernel<RT, MODE, true, true>);
    prefer_l1(sweep_kernel<RT, MODE, true, false>);
    prefer_l1(sweep_kernel<RT, MODE, false, true>);
    prefer_l1(sweep_kernel<RT, MODE, false, false>);
    if (MODE == M_PLAIN) sweep_kernel<RT, M_PLAIN, false, false><<<grid, kBlock, 0, s>>>(A);
    else if (sub && add) sweep_kernel<RT, MODE, true, true><<<grid, kBlock, 0, s>>>(A);
    else if (sub) sweep_kernel<RT, MODE, true, false><<<grid, kBlock, 0, s>>>(A);
    else if (add) sweep_kernel<RT, MODE, false, true><<<grid, kBlock, 0, s>>>(A);
    else sweep_kernel<RT, MODE, false, false><<<grid, kBlock, 0, s>>>(A);
}

template <int RT, int MS>
void smemq_attrs_ms(int bytes) {
    cudaFuncSetAttribute(sweep_smemq_kernel<RT, true, true, MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(sweep_smemq_kernel<RT, true, false, MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(sweep_smemq_kernel<RT, false, true, MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(sweep_smemq_kernel<RT, false, false, MS>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int RT, int MS>
void smemq_ms(const SweepArgs& A, bool sub, bool add, unsigned grid, size_t smem, uint32_t nb, uint32_t* queue,
              cudaStream_t s) {
    if (sub && add) sweep_smemq_kernel<RT, true, true, MS><<<grid, kBlock * kSubs, smem, s>>>(A, nb, queue);
    else if (sub) sweep_smemq_kernel<RT, true, false, MS><<<grid, kBlock * kSubs, smem, s>>>(A, nb, queue);
    else if (add) sweep_smemq_kernel<RT, false, true, MS><<<grid, kBlock * kSubs, smem, s>>>(A, nb, queue);
    else sweep_smemq_kernel<RT, false, false, MS><<<grid, kBlock * kSubs, smem, s>>>(A, nb, queue);
}

}  // namespace

template <int RT>
void launch_rt(const SweepArgs& A, int mode, bool sub, bool add, unsigned grid, cudaStream_t s) {
    if (mode == M_CSC) launch_mode<RT, M_CSC>(A, sub, add, grid, s);
    else if (mode == M_CSCP) launch_mode<RT, M_CSCP>(A, sub, add, grid, s);
    else if (mode == M_CSCQ) launch_mode<RT, M_CSCQ>(A, sub, add, grid, s);
    else if (mode == M_CSR) launch_mode<RT, M_CSR>(A, sub, add, grid, s);
    else if (mode == M_CSR16) launch_mode<RT, M_CSR16>(A, sub, add, grid, s);
    else launch_mode<RT, M_PLAIN>(A, false, false, grid, s);
}

template <int RT>
void smemq_attrs(int bytes) {
    smemq_attrs_ms<RT, M_CSRS>(bytes);
    smemq_attrs_ms<RT, M_CSRS16>(bytes);
}

template <int RT>
void smemq_rt(const SweepArgs& A, bool i16, bool sub, bool add, unsigned grid, size_t smem, uint32_t nb,
              uint32_t* queue, cudaStream_t s) {
    if (i16) smemq_ms<RT, M_CSRS16>(A, sub, add, grid, smem, nb, queue, s);
    else smemq_ms<RT, M_CSRS>(A, sub, add, grid, smem, nb, queue, s);
}

#define CDMF_INST(RT)                                                                                  \
    template void launch_rt<RT>(const SweepArgs&, int, bool, bool, unsigned, cudaStream_t);             \
    template void smemq_attrs<RT>(int);                                                                 \
    template void smemq_rt<RT>(const SweepArgs&, bool, bool, bool, unsigned, size_t, uint32_t, uint32_t*, \
                               cudaStream_t);
CDMF_FOR_RT(CDMF_INST)
#undef CDMF_INST

#if CDMF_HAS_RT0
void launch_dual(const SweepArgs& A, unsigned grid, cudaStream_t s) {
    prefer_l1(sweep_kernel<0, M_DUAL, false, false>);
    sweep_kernel<0, M_DUAL, false, false><<<grid, kBlock, 0, s>>>(A);
}
#endif

#endif  // CDMF_PART0

#if CDMF_PART1

namespace {

template <int RT, int MODE>
void tile_mode(const TileArgs& T, bool sub, bool add, unsigned grid, cudaStream_t s) {
    prefer_l1(tile_sweep_kernel<RT, MODE, true, true>);
    prefer_l1(tile_sweep_kernel<RT, MODE, true, false>);
    prefer_l1(tile_sweep_kernel<RT, MODE, false, true>);
    prefer_l1(tile_sweep_kernel<RT, MODE, false, false>);
    if (MODE == M_PLAIN) tile_sweep_kernel<RT, M_PLAIN, false, false><<<grid, kBlock, 0, s>>>(T);
    else if (sub && add) tile_sweep_kernel<RT, MODE, true, true><<<grid, kBlock, 0, s>>>(T);
    else if (sub) tile_sweep_kernel<RT, MODE, true, false><<<grid, kBlock, 0, s>>>(T);
    else if (add) tile_sweep_kernel<RT, MODE, false, true><<<grid, kBlock, 0, s>>>(T);
    else tile_sweep_kernel<RT, MODE, false, false><<<grid, kBlock, 0, s>>>(T);
}

template <int RT, int MODE, bool SUB, bool ADD>
void blocked_launch(const BlockedArgs& B, unsigned grid, cudaStream_t s) {
    using T = typename Tbl<MODE>::T;
    allow_smem(blocked_sweep_kernel<RT, MODE, SUB, ADD>, (size_t)kXbRow * sizeof(float4));
    blocked_sweep_kernel<RT, MODE, SUB, ADD><<<grid, kBlock, B.xb * sizeof(T), s>>>(B);
}

template <int RT, int MODE>
void blocked_mode(const BlockedArgs& B, bool sub, bool add, unsigned grid, cudaStream_t s) {
    if (MODE == M_PLAIN) blocked_launch<RT, M_PLAIN, false, false>(B, grid, s);
    else if (sub && add) blocked_launch<RT, MODE, true, true>(B, grid, s);
    else if (sub) blocked_launch<RT, MODE, true, false>(B, grid, s);
    else if (add) blocked_launch<RT, MODE, false, true>(B, grid, s);
    else blocked_launch<RT, MODE, false, false>(B, grid, s);
}

template <int RT, int NU>
void refresh_t(const RefreshDesc& D, unsigned grid, cudaStream_t s) {
    refresh_warp_kernel<RT, NU><<<grid, kBlock, 0, s>>>(D.ptr, D.crow, D.idx, D.val, D.to_csr, D.to_csc, D.nnz,
                                                        D.Wrm, D.Hrm, D.kp, D.res_csr, D.res_csc, D.pa, D.pb, D.part,
                                                        D.counter, D.drift_out, D.nonfinite);
}

}  // namespace

template <int RT>
void tile_rt(const TileArgs& T, int mode, bool sub, bool add, unsigned grid, cudaStream_t s) {
    if (mode == M_CSC) tile_mode<RT, M_CSC>(T, sub, add, grid, s);
    else if (mode == M_CSR) tile_mode<RT, M_CSR>(T, sub, add, grid, s);
    else tile_mode<RT, M_PLAIN>(T, false, false, grid, s);
}

template <int RT>
void blocked_rt(const BlockedArgs& B, int mode, bool sub, bool add, unsigned grid, cudaStream_t s) {
    if (mode == M_CSC) blocked_mode<RT, M_CSC>(B, sub, add, grid, s);
    else if (mode == M_CSR) blocked_mode<RT, M_CSR>(B, sub, add, grid, s);
    else blocked_mode<RT, M_PLAIN>(B, false, false, grid, s);
}

#define CDMF_INST(RT)                                                                                  \
    template void tile_rt<RT>(const TileArgs&, int, bool, bool, unsigned, cudaStream_t);                \
    template void blocked_rt<RT>(const BlockedArgs&, int, bool, bool, unsigned, cudaStream_t);
CDMF_FOR_RT(CDMF_INST)
#undef CDMF_INST


template <int RT>
void launch_refresh_rt(const RefreshDesc& D, unsigned grid, cudaStream_t s) {
    switch (D.slices) {
        case 1: refresh_t<RT, 1>(D, grid, s); break;
        case 2: refresh_t<RT, 2>(D, grid, s); break;
        case 4: refresh_t<RT, 4>(D, grid, s); break;
        case 8: refresh_t<RT, 8>(D, grid, s); break;
        default: refresh_t<RT, 0>(D, grid, s); break;
    }
}

#define CDMF_INST(RT) template void launch_refresh_rt<RT>(const RefreshDesc&, unsigned, cudaStream_t);
CDMF_FOR_RT16(CDMF_INST)
#undef CDMF_INST

#endif  // CDMF_PART1

}  // namespace cdmf
