// Nonzero-balanced ("tile") sweep -- the engine's rewrite of the reference's
// CSR5 load-balancing variant (src/cdmf_csr5.cpp, src/detail/kcode/
// csr5_spmv.cl): the same rank-one-update math as sweep_kernel, but work is
// split by nonzeros instead of by lines, so short and long lines cost the same
// per nonzero and no lane idles on a short line.
//
// Each warp owns a tile of kWarpTile consecutive nonzeros of one compressed
// copy.  In step s lane l handles nonzero p0 + 32 s + l (coalesced loads),
// tracks the line that nonzero belongs to, applies the fused residual update
// (subtract, add-back, store) and forms g = y r, h = y^2.  Sums per line:
//   - while all 32 nonzeros of a step belong to the line that is still open
//     and none is its last, each lane accumulates privately (fast path);
//   - otherwise the private sums are folded into the warp's carry and a
//     segmented inclusive scan over the lanes (keyed by line id) adds each
//     line's values; a lane holding the last nonzero of a line finishes it.
// A line that lies inside one tile is finished by its tile.  A line crossing
// tile boundaries leaves one partial per tile it touches (tail slot of the
// tiles it continues out of, head slot of the tile it ends in); the last of
// those tiles to arrive adds the partials in tile order and finishes the line.
// All orders are fixed, so results are deterministic; there are no float
// atomics.  Empty lines are finished by extra blocks at the end of the grid.
// The reference's CSR5 needs an AoSoA transpose of the matrix and back around
// every residual update (src/cdmf_csr5.cpp:246-325); here the residual stays
// in CSR/CSC order and the tile bookkeeping is one line index per tile.
#pragma once
#include "sweep_kernels.cuh"

namespace cdmf {

// Measured on the Netflix-shaped matrix (BF16): 1,024-nonzero warp tiles and
// 6 blocks per SM run 1,190 / 1,150 updates/s against 1,060 for 512 and 5.
constexpr int kTileSteps = 32;
constexpr int kWarpTile = 32 * kTileSteps;   // nonzeros per warp tile

struct TileArgs {
    SweepArgs s;                    // vectors, residual, emits (work lists unused)
    const uint32_t* tile_line;      // line containing the first nonzero of each tile
    float2* head;                   // per tile: partial of the line that ends in it
    float2* tail;                   // per tile: partial of the line that continues out of it
    uint32_t* lcount;               // per line: tiles arrived (left at 0)
    const uint32_t* empty;          // empty lines
    uint32_t nempty, ntiles, tile_blocks;
    uint32_t nnz;
};

// Per-line scalars: b (previous feature, final) and d (this feature, old).
// d is also the vector this sweep writes, but only the line's own finishing
// lane writes it, after every tile of the line has read it.
template <int MODE, bool SUB, bool ADD>
__device__ __forceinline__ void tile_line_scalars(const SweepArgs& A, uint32_t j, float& bj, float& dj) {
    bj = (SUB || MODE == M_CSC) && A.b ? A.b[j] : 0.0f;
    dj = (ADD || MODE == M_CSC) ? A.d[j] : 0.0f;
}

template <int MODE>
__device__ __forceinline__ void tile_finish(const SweepArgs& A, uint32_t j, uint32_t len, float g, float h, float bj,
                                            float dj) {
    const float lam = __fmul_rn(A.lambda, __uint2float_rn(len));
    write_line<MODE>(A, j, __fdiv_rn(g, __fadd_rn(lam, h)), bj, dj);
}

// A tile's partial for a line that spans tiles; the last arriving tile
// finishes the line.
template <int MODE, bool SUB, bool ADD>
__device__ __forceinline__ void tile_arrive(const TileArgs& T, uint32_t line, bool is_head, uint32_t tau, float g,
                                            float h) {
    const SweepArgs& A = T.s;
    (is_head ? T.head : T.tail)[tau] = make_float2(g, h);
    __threadfence();
    const uint32_t b0 = A.ptr[line], b1 = A.ptr[line + 1];
    const uint32_t t0 = b0 / kWarpTile, t1 = (b1 - 1) / kWarpTile;
    const uint32_t prev = atomicAdd(T.lcount + line, 1u);
    if (prev != t1 - t0) return;
    __threadfence();
    float G = 0.0f, Hs = 0.0f;
    for (uint32_t q = t0; q < t1; ++q) {
        const float2 p = __ldcg(T.tail + q);
        G = __fadd_rn(G, p.x);
        Hs = __fadd_rn(Hs, p.y);
    }
    const float2 p = __ldcg(T.head + t1);
    G = __fadd_rn(G, p.x);
    Hs = __fadd_rn(Hs, p.y);
    float bj, dj;
    tile_line_scalars<MODE, SUB, ADD>(A, line, bj, dj);
    tile_finish<MODE>(A, line, b1 - b0, G, Hs, bj, dj);
    T.lcount[line] = 0;
}

template <int RT, int MODE, bool SUB, bool ADD>
__global__ void __launch_bounds__(kBlock, kTileBlocks) tile_sweep_kernel(const TileArgs T) {
    const SweepArgs& A = T.s;
    const uint32_t lane = threadIdx.x & 31;
    if (blockIdx.x >= T.tile_blocks) {                      // empty lines
        const uint32_t e = (blockIdx.x - T.tile_blocks) * kBlock + threadIdx.x;
        if (e < T.nempty) {
            const uint32_t j = T.empty[e];
            float bj, dj;
            tile_line_scalars<MODE, SUB, ADD>(A, j, bj, dj);
            write_line<MODE>(A, j, 0.0f, bj, dj);
        }
        return;
    }
    const uint32_t tau = blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (tau >= T.ntiles) return;
    const uint32_t p0 = tau * kWarpTile;
    const uint32_t pend = min(T.nnz, p0 + kWarpTile);
    // this lane's current line and its end
    uint32_t line = T.tile_line[tau];
    uint32_t bound = __ldg(A.ptr + line + 1);
    float bj = 0.0f, dj = 0.0f;
    uint32_t scal_line = 0xffffffffu;
    // the warp's open line: carry (uniform) plus lane-private fast-path sums
    uint32_t cl = line;
    float cg = 0.0f, ch = 0.0f, pg = 0.0f, ph = 0.0f;
    for (int s0 = 0; s0 < kTileSteps; s0 += 4) {
        uint32_t iv[4];
        float rv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t p = p0 + 32u * (s0 + u) + lane;
            if (p < pend) {
                iv[u] = __ldcs(A.idx + p);
                rv[u] = Res<RT>::ld(A.res, p);
            } else {
                iv[u] = 0;
                rv[u] = 0.0f;
            }
        }
        float av[4], cv[4], yv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t p = p0 + 32u * (s0 + u) + lane;
            if (p < pend) fetch<MODE>(A, iv[u], av[u], cv[u], yv[u]);
            else av[u] = cv[u] = yv[u] = 0.0f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t p = p0 + 32u * (s0 + u) + lane;
            const bool active = p < pend;
            if (active) {
                while (p >= bound) {
                    ++line;
                    bound = __ldg(A.ptr + line + 1);
                }
                if ((SUB || ADD || MODE == M_CSC) && line != scal_line) {
                    tile_line_scalars<MODE, SUB, ADD>(A, line, bj, dj);
                    scal_line = line;
                }
            }
            float r = rv[u];
            if (active && (SUB || ADD)) r = Res<RT>::st(A.res, p, update<SUB, ADD>(r, av[u], cv[u], bj, dj));
            float gv = active ? __fmul_rn(yv[u], r) : 0.0f;
            float hv = active ? __fmul_rn(yv[u], yv[u]) : 0.0f;
            const bool last_of_line = active && p + 1 == bound;
            const uint32_t key = active ? line : 0xffffffffu;
            if (__all_sync(0xffffffffu, active && line == cl && !last_of_line)) {
                pg = __fadd_rn(pg, gv);                      // fast path: one open line
                ph = __fadd_rn(ph, hv);
                continue;
            }
            // fold the private sums of the open line into the carry
            float fg = pg, fh = ph;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                fg = __fadd_rn(fg, __shfl_xor_sync(0xffffffffu, fg, o));
                fh = __fadd_rn(fh, __shfl_xor_sync(0xffffffffu, fh, o));
            }
            cg = __fadd_rn(cg, fg);
            ch = __fadd_rn(ch, fh);
            pg = ph = 0.0f;
            // segmented inclusive scan keyed by line
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float og = __shfl_up_sync(0xffffffffu, gv, o);
                const float oh = __shfl_up_sync(0xffffffffu, hv, o);
                const uint32_t ok = __shfl_up_sync(0xffffffffu, key, o);
                if (lane >= (uint32_t)o && ok == key) {
                    gv = __fadd_rn(og, gv);
                    hv = __fadd_rn(oh, hv);
                }
            }
            if (active && line == cl) {
                gv = __fadd_rn(cg, gv);
                hv = __fadd_rn(ch, hv);
            }
            if (last_of_line) {
                const uint32_t lb = __ldg(A.ptr + line);
                if (lb >= p0) tile_finish<MODE>(A, line, bound - lb, gv, hv, bj, dj);
                else tile_arrive<MODE, SUB, ADD>(T, line, true, tau, gv, hv);
            }
            // new carry: the segment of lane 31 if its line goes on
            const uint32_t l31 = __shfl_sync(0xffffffffu, key, 31);
            const int open31 = __shfl_sync(0xffffffffu, (int)(active && !last_of_line), 31);
            const float g31 = __shfl_sync(0xffffffffu, gv, 31);
            const float h31 = __shfl_sync(0xffffffffu, hv, 31);
            if (open31) {
                cl = l31;
                cg = g31;
                ch = h31;
            } else {
                cl = 0xfffffffeu;
                cg = ch = 0.0f;
            }
        }
    }
    // end of tile: the open line continues into the next tile
    float fg = pg, fh = ph;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fg = __fadd_rn(fg, __shfl_xor_sync(0xffffffffu, fg, o));
        fh = __fadd_rn(fh, __shfl_xor_sync(0xffffffffu, fh, o));
    }
    if (cl < 0xfffffffeu && lane == 0)
        tile_arrive<MODE, SUB, ADD>(T, cl, false, tau, __fadd_rn(cg, fg), __fadd_rn(ch, fh));
}

}  // namespace cdmf
