// CCD++ engine on one GB300: the C ABI of include/cdmf_cuda.h.
//
// Schedule of one outer iteration (src/cdmf_ref.cpp:69-137), per feature t:
//   inner 1:  CSC sweep  -> H[t]   (+ pending subtract of feature t-1, + add-back of t)
//             CSR sweep  -> W[t]   (+ pending subtract of feature t-1, + add-back of t)
//   inner 2..T: the same two sweeps without residual writes
// The subtract of feature t (src/cdmf_ref.cpp:120-121) is carried into the
// first sweeps of feature t+1 (or of the next outer iteration), so every
// residual element is read and written once per feature per copy.  The
// operations on an element happen in the reference's order (subtract t, then
// add back t+1), so the arithmetic is unchanged; only the number of passes
// over HBM drops from 6 to 2.
//
// The reference reads W[t], H[t] into u, v and writes them back after the
// inner loop (src/cdmf_ref.cpp:80-83,115-118).  Here the CSC sweep overwrites
// H[t] in place and forwards the old H[t] (which the CSR add-back needs) in
// the packed table Q; the CSR sweep overwrites W[t] in place (each row reads
// only its own old w_i before writing it) and writes the packed table P the
// next feature's CSC sweep gathers from.
#include <cdmf_cuda.h>
#include "sweep_kernels.cuh"
#include "refresh_kernels.cuh"
#include "objective_kernels.cuh"
#include "gpu_build.h"
#include "tile_kernels.cuh"
#include "blocked_kernels.cuh"
#include "launch.h"
#include "relabel.h"
#include "blocked.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <set>
#include <mutex>
#include <tuple>
#include <cstdio>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace cdmf;

namespace {

// bins: 0 thread, 1 8-lane group, 2 warp, 3 CTA, 4 split
struct Bins {
    std::vector<XTask> x;
    std::vector<uint32_t> c, w, g, t;
    uint32_t nslots = 0, nxl = 0;
    int64_t count[5] = {0, 0, 0, 0, 0}, nnz[5] = {0, 0, 0, 0, 0};
};

// nonzero-balanced tiles of one compressed copy (version 3)
struct DevTiles {
    uint32_t* tile_line = nullptr;
    float2 *head = nullptr, *tail = nullptr;
    uint32_t* lcount = nullptr;
    uint32_t* empty = nullptr;
    uint32_t ntiles = 0, nempty = 0, tile_blocks = 0, empty_blocks = 0;
};

// cross-index-blocked copy (layout 1)
struct DevBlocked {
    uint32_t* segptr = nullptr;
    uint16_t* idx = nullptr;
    uint32_t* units = nullptr;
    float2* part = nullptr;
    uint32_t* map = nullptr;     // line-layout position -> blocked position
    uint32_t nunits = 0, nb = 0, lines = 0, xb = 0;
    uint64_t cross = 0;
};

struct DevBins {
    XTask* x = nullptr;
    uint32_t *c = nullptr, *w = nullptr, *g = nullptr, *t = nullptr;
    float2* part = nullptr;
    uint32_t* xcount = nullptr;
    uint32_t nx = 0, nc = 0, nw = 0, ng = 0, nt = 0, nwb = 0, ngb = 0, ntb = 0;
    Bins host;
};

// Bin thresholds (line length in nonzeros).
// Bin thresholds when the caller sets none.  Large matrices (the line
// counts fill the GPU with warps) keep long lines on one warp: on the
// Netflix-shaped matrix (99M nonzeros, BF16) warp lines up to 16384, CTA
// lines up to 65536 and split chunks of 16384 measured +11 % over 2048 /
// 16384 / 8192.  Small matrices keep
// 2048 / 16384: on the 64-problem batch (50k-5M nonzeros each) the larger
// thresholds measured -2 % batched and -21 % one problem after another, as
// their few long lines then fill too few warps.  cdmf_cuda_autotune picks per
// matrix.
constexpr int64_t kLargeNnz = 16 << 20;
// Large matrices with a 16-bit residual give group-bin lines 4 lanes (8 lines
// per warp): +2 % on the Netflix-shaped matrix at BF16, but -2 % at FP32 and
// on the 64-problem batch, which keep 8.
// Small matrices also run 8-lane group lines of up to 32 nonzeros on the
// interleaved layout (the whole line in flight): the 64-problem batch
// measured 169 -> 161 ms; the Netflix-shaped matrix -1 %, so not there.
constexpr uint32_t kGroupShort = 32;
// 16-bit modes: features between refreshes in the first outer iteration.
constexpr uint32_t kEarlyRefresh = 32;
struct BinCfg {
    uint32_t thread_max = 12;     // <= : one thread per line
    uint32_t group_max = 256;     // <= : one lane group per line
    uint32_t warp_max = 2048;     // <= : one warp per line
    uint32_t cta_max = 16384;     // <= : one CTA per line; above: split
    uint32_t chunk = 8192;        // nonzeros per chunk of a split line
};

BinCfg default_bins(int64_t nnz) {
    BinCfg c;
    if (nnz >= kLargeNnz) {
        c.warp_max = 16384;
        c.cta_max = 65536;
        c.chunk = 16384;
    }
    return c;
}

Bins plan_bins(const uint32_t* ptr, int64_t lines, bool sequential, const BinCfg& cfg) {
    Bins B;
    for (int64_t j = 0; j < lines; ++j) {
        const uint32_t len = ptr[j + 1] - ptr[j];
        int bin;
        if (sequential || len <= cfg.thread_max) bin = 0;
        else if (len <= cfg.group_max) bin = 1;
        else if (len <= cfg.warp_max) bin = 2;
        else if (len <= cfg.cta_max) bin = 3;
        else bin = 4;
        B.count[bin]++;
        B.nnz[bin] += len;
        switch (bin) {
            case 0: B.t.push_back((uint32_t)j); break;
            case 1: B.g.push_back((uint32_t)j); break;
            case 2: B.w.push_back((uint32_t)j); break;
            case 3: B.c.push_back((uint32_t)j); break;
            default: {
                const uint32_t nch = (len + cfg.chunk - 1) / cfg.chunk;
                const uint32_t first = B.nslots;
                for (uint32_t q = 0; q < nch; ++q) {
                    XTask T;
                    T.line = (uint32_t)j;
                    T.beg = ptr[j] + q * cfg.chunk;
                    T.end = std::min<uint32_t>(ptr[j + 1], T.beg + cfg.chunk);
                    T.slot = first + q;
                    T.xl = B.nxl;
                    T.first_slot = first;
                    T.nchunks = nch;
                    T.pad = 0;
                    B.x.push_back(T);
                }
                B.nslots += nch;
                B.nxl++;
            }
        }
    }
    // longest lines first inside the CTA bin so the tail of the launch is short
    std::stable_sort(B.c.begin(), B.c.end(), [&](uint32_t a, uint32_t b) {
        return (ptr[a + 1] - ptr[a]) > (ptr[b + 1] - ptr[b]);
    });
    return B;
}

const char* kErrStr[] = {"ok",          "invalid argument or sparse structure", "allocation failed",
                         "CUDA error",  "no CUDA device",                        "empty test set",
                         "numeric check failed", "unsupported option",           "size beyond limit"};

}  // namespace

struct cdmf_handle {
    cdmf_opts o{};
    int64_t m = 0, n = 0, nnz = 0, nt = 0;
    int rt = 0;                      // residual type 0/1/2
    size_t rbytes = 4;
    cudaStream_t s = nullptr;
    // device arrays
    uint32_t *csr_ptr = nullptr, *csr_idx = nullptr, *csc_ptr = nullptr, *csc_idx = nullptr;
    float *csr_val = nullptr, *csc_val = nullptr;  // pristine ratings
    void *res_csr = nullptr, *res_csc = nullptr;   // residual copies
    float *W = nullptr, *H = nullptr;
    float2* P = nullptr;             // packed CSC gather table (m)
    float4* Q = nullptr;             // packed CSR gather table (n)
    int p_for = -1;                  // feature whose CSC sweep P is valid for
    uint32_t *te_row = nullptr, *te_col = nullptr;
    float* te_val = nullptr;
    double *rmse_part = nullptr, *rmse_out = nullptr;
    uint32_t* rmse_count = nullptr;
    int rmse_grid = 0;
    DevBins csr, csc;
    DevTiles tcsr, tcsc;
    bool tiles = false;              // version 3: nonzero-balanced tile sweeps
    DevBlocked bcsr, bcsc;
    bool blocked = false;            // layout 1: cross-index-blocked copies
    uvec<uint32_t> hmap_r, hmap_c;   // host copies of the blocked maps
    uint32_t* ref_to_csr = nullptr;  // refresh: CSR line position -> CSR copy position (blocked)
    // degree relabelling: new id -> caller id, new position -> caller position
    bool relabeled = false;
    uvec<uint32_t> row_old, col_old, csr_pos, csc_pos, csc_from_csr;
    uvec<uint32_t> ucsr_ptr, ucsr_idx;   // caller's CSR structure, for csc_pos on demand
    // relabelling built on the device: the position maps and the caller's CSR
    // structure stay there until a state move needs them on the host
    uint32_t *d_csr_pos = nullptr, *d_csc_from_csr = nullptr, *d_ucsr_ptr = nullptr, *d_ucsr_idx = nullptr;
    // relabelled factors cross the boundary through a device permutation
    uint32_t *d_row_old = nullptr, *d_col_old = nullptr;
    float* ftmp = nullptr;           // k * max(m, n) staging for the caller's factor order
    // narrow matrices: CSR sweeps gather from a shared-memory copy of Q
    uint32_t group_lanes = 8;        // lanes per group-bin line (4 on large matrices)
    uint16_t* csr_idx16 = nullptr;   // narrow matrices: the CSR column indices in 16 bits
    bool idx16 = false;
    // large matrices with fewer than 2^19 rows: the CSC row indices as 16-bit
    // offsets inside segments of 65,536 rows, and each column's run ends
    uint16_t* csc_idx16 = nullptr;
    uint32_t* csc_seg = nullptr;
    bool cidx16 = false;
    bool smemq = false;
    int sms = 0;
    uint32_t* smemq_queue = nullptr;
    // host copies of the line pointers (engine numbering) and the bin plan
    std::vector<uint32_t> hptr_r, hptr_c;
    BinCfg cfg;                      // bin limits of the CSR copy (and of the CSC copy unless tuned apart)
    BinCfg cfg_c;                    // bin limits of the CSC copy
    bool seq = false;
    // 16-bit residual modes: CSR->CSC position map, row-major factor copies
    uint32_t* to_csc = nullptr;
    float *Wrm = nullptr, *Hrm = nullptr;
    uint32_t kp = 0;
    int ref_grid = 0;
    uint32_t* ref_crow = nullptr;    // refresh: row of each chunk's first nonzero, then of the last one
    double *ref_part = nullptr, *drift_out = nullptr;
    uint32_t* ref_count = nullptr;
    unsigned long long* nonfinite = nullptr;
    bool refreshed = false;
    // FP64 objective monitor (allocated on first use)
    double *obj_part = nullptr, *obj_out = nullptr;
    uint32_t* obj_count = nullptr;
    // CUDA graphs of whole outer iterations, keyed by the schedule's signature
    struct Graph {
        int sig[5];
        cudaGraphExec_t exec;
        int end_pending, end_p_for;
        int64_t launches, csc, csr, rmse, refresh;
    };
    std::vector<Graph> graphs;
    double* rmse_graph_slot = nullptr;
    // state
    int next_oiter = 1;
    int pending = -1;                // feature whose subtract is still owed, -1 = none
    // timing
    bool profiling = false;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    struct Mark { int kind; cudaEvent_t a, b; };
    std::vector<Mark> marks;
    std::vector<cudaEvent_t> pool;
    size_t pool_used = 0;
    cdmf_stats st{};
    std::string err;
    std::vector<void*> allocs;
};

namespace {

int fail(cdmf_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

#define CU(h, call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(h, CDMF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(cdmf_handle* h, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(h, CDMF_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    h->allocs.push_back((void*)*p);
    return CDMF_OK;
}

// (branch-free reductions, so the compiler vectorises the scans)
int check_compressed(const uint32_t* ptr, const uint32_t* idx, int64_t lines, int64_t cross, int64_t nnz) {
    if (!ptr || (nnz > 0 && !idx)) return CDMF_ERR_INVALID;
    if (ptr[0] != 0 || (int64_t)ptr[lines] != nnz) return CDMF_ERR_INVALID;
    int64_t down = 0;   // decreasing pointer pairs
#pragma omp parallel for schedule(static) reduction(+ : down)
    for (int64_t j = 0; j < lines; ++j) down += ptr[j] > ptr[j + 1];
    if (down) return CDMF_ERR_INVALID;
    uint32_t hi = 0;
#pragma omp parallel for schedule(static) reduction(max : hi)
    for (int64_t q = 0; q < nnz; ++q) hi = std::max(hi, idx[q]);
    return nnz > 0 && (int64_t)hi >= cross ? CDMF_ERR_INVALID : CDMF_OK;
}

int upload_bins(cdmf_handle* h, DevBins& D, Bins&& B) {
    D.nx = (uint32_t)B.x.size();
    D.nc = (uint32_t)B.c.size();
    D.nw = (uint32_t)B.w.size();
    D.ng = (uint32_t)B.g.size();
    D.nt = (uint32_t)B.t.size();
    D.nwb = (D.nw + kWarps - 1) / kWarps;
    const uint32_t per = kBlock / h->group_lanes;   // group lines per block
    D.ngb = (D.ng + per - 1) / per;
    D.ntb = (D.nt + kBlock - 1) / kBlock;
    int r;
    if ((r = dalloc(h, &D.x, B.x.size())) || (r = dalloc(h, &D.c, B.c.size())) || (r = dalloc(h, &D.w, B.w.size())) ||
        (r = dalloc(h, &D.g, B.g.size())) || (r = dalloc(h, &D.t, B.t.size())) || (r = dalloc(h, &D.part, B.nslots)) ||
        (r = dalloc(h, &D.xcount, B.nxl)))
        return r;
    if (D.nx) CU(h, cudaMemcpyAsync(D.x, B.x.data(), sizeof(XTask) * D.nx, cudaMemcpyHostToDevice, h->s));
    if (D.nc) CU(h, cudaMemcpyAsync(D.c, B.c.data(), 4 * D.nc, cudaMemcpyHostToDevice, h->s));
    if (D.nw) CU(h, cudaMemcpyAsync(D.w, B.w.data(), 4 * D.nw, cudaMemcpyHostToDevice, h->s));
    if (D.ng) CU(h, cudaMemcpyAsync(D.g, B.g.data(), 4 * D.ng, cudaMemcpyHostToDevice, h->s));
    if (D.nt) CU(h, cudaMemcpyAsync(D.t, B.t.data(), 4 * D.nt, cudaMemcpyHostToDevice, h->s));
    CU(h, cudaMemsetAsync(D.xcount, 0, 4 * std::max<uint32_t>(1, B.nxl), h->s));
    CU(h, cudaStreamSynchronize(h->s));  // host vectors are released below
    D.host = std::move(B);
    D.host.x.clear(); D.host.x.shrink_to_fit();
    D.host.c.clear(); D.host.c.shrink_to_fit();
    D.host.w.clear(); D.host.w.shrink_to_fit();
    D.host.g.clear(); D.host.g.shrink_to_fit();
    D.host.t.clear(); D.host.t.shrink_to_fit();
    return CDMF_OK;
}

void free_bins(cdmf_handle* h, DevBins& D) {
    void* ps[] = {D.x, D.c, D.w, D.g, D.t, D.part, D.xcount};
    for (void* p : ps) {
        if (!p) continue;
        cudaFree(p);
        auto it = std::find(h->allocs.begin(), h->allocs.end(), p);
        if (it != h->allocs.end()) h->allocs.erase(it);
    }
    D = DevBins();
}

int upload_tiles(cdmf_handle* h, DevTiles& D, const uint32_t* ptr, int64_t lines, int64_t nnz) {
    std::vector<uint32_t> tl, empty;
    const int64_t ntiles = (nnz + kWarpTile - 1) / kWarpTile;
    tl.reserve(ntiles + 1);
    int64_t L = 0;
    for (int64_t t = 0; t < ntiles; ++t) {
        const int64_t p = t * (int64_t)kWarpTile;
        while (L < lines && (int64_t)ptr[L + 1] <= p) ++L;
        tl.push_back((uint32_t)L);
    }
    tl.push_back((uint32_t)lines);
    for (int64_t j = 0; j < lines; ++j)
        if (ptr[j + 1] == ptr[j]) empty.push_back((uint32_t)j);
    D.ntiles = (uint32_t)ntiles;
    D.nempty = (uint32_t)empty.size();
    D.tile_blocks = (D.ntiles + kWarps - 1) / kWarps;
    D.empty_blocks = (D.nempty + kBlock - 1) / kBlock;
    int r;
    if ((r = dalloc(h, &D.tile_line, tl.size())) || (r = dalloc(h, &D.head, ntiles)) ||
        (r = dalloc(h, &D.tail, ntiles)) || (r = dalloc(h, &D.lcount, lines)) || (r = dalloc(h, &D.empty, empty.size())))
        return r;
    CU(h, cudaMemcpyAsync(D.tile_line, tl.data(), 4 * tl.size(), cudaMemcpyHostToDevice, h->s));
    if (!empty.empty()) CU(h, cudaMemcpyAsync(D.empty, empty.data(), 4 * empty.size(), cudaMemcpyHostToDevice, h->s));
    CU(h, cudaMemsetAsync(D.lcount, 0, 4 * std::max<int64_t>(1, lines), h->s));
    CU(h, cudaStreamSynchronize(h->s));
    return CDMF_OK;
}

int upload_blocked(cdmf_handle* h, DevBlocked& D, BlockedHost&& B, uvec<uint32_t>& hmap) {
    D.nb = B.nb;
    D.lines = B.lines;
    D.xb = B.xb;
    D.cross = B.cross;
    D.nunits = (uint32_t)(B.units.size() / 5);
    int r;
    if ((r = dalloc(h, &D.segptr, B.segptr.size())) || (r = dalloc(h, &D.idx, B.idx16.size())) ||
        (r = dalloc(h, &D.units, B.units.size())) || (r = dalloc(h, &D.part, (size_t)B.nb * B.lines)) ||
        (r = dalloc(h, &D.map, B.pos.size())))
        return r;
    CU(h, cudaMemcpyAsync(D.segptr, B.segptr.data(), 4 * B.segptr.size(), cudaMemcpyHostToDevice, h->s));
    if (!B.idx16.empty()) CU(h, cudaMemcpyAsync(D.idx, B.idx16.data(), 2 * B.idx16.size(), cudaMemcpyHostToDevice, h->s));
    CU(h, cudaMemcpyAsync(D.units, B.units.data(), 4 * B.units.size(), cudaMemcpyHostToDevice, h->s));
    if (!B.pos.empty()) CU(h, cudaMemcpyAsync(D.map, B.pos.data(), 4 * B.pos.size(), cudaMemcpyHostToDevice, h->s));
    CU(h, cudaStreamSynchronize(h->s));
    hmap = std::move(B.pos);
    return CDMF_OK;
}

cudaEvent_t pool_event(cdmf_handle* h) {
    if (h->pool_used == h->pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        h->pool.push_back(e);
    }
    return h->pool[h->pool_used++];
}

enum { K_CSC = 0, K_CSR = 1, K_RMSE = 2, K_REFRESH = 3 };

struct Timed {
    cdmf_handle* h;
    int kind;
    cudaEvent_t b = nullptr;
    Timed(cdmf_handle* h_, int kind_) : h(h_), kind(kind_) {
        if (h->profiling) {
            cudaEvent_t a = pool_event(h);
            b = pool_event(h);
            if (a && b) {
                cudaEventRecord(a, h->s);
                h->marks.push_back({kind, a, b});
            } else {
                b = nullptr;
            }
        }
    }
    ~Timed() {
        if (b) cudaEventRecord(b, h->s);
    }
};

SweepArgs base_args(cdmf_handle* h, const DevBins& D, const uint32_t* ptr, const uint32_t* idx, void* res) {
    SweepArgs A;
    std::memset(&A, 0, sizeof(A));
    A.ptr = ptr;
    A.idx = idx;
    A.res = res;
    A.lambda = h->o.lambda;
    A.xt = D.x;
    A.cl = D.c;
    A.wl = D.w;
    A.gl = D.g;
    A.tl = D.t;
    A.nx = D.nx;
    A.nc = D.nc;
    A.nw = D.nw;
    A.ng = D.ng;
    A.nt = D.nt;
    A.nwb = D.nwb;
    A.ngb = D.ngb;
    A.part = D.part;
    A.xcount = D.xcount;
    A.group_short = h->nnz < kLargeNnz ? kGroupShort : 0;
    A.group_lanes = h->group_lanes;
    return A;
}

int launch_blocked(cdmf_handle* h, int kind, const SweepArgs& A, int mode, bool sub, bool add) {
    const DevBlocked& D = kind == K_CSC ? h->bcsc : h->bcsr;
    BlockedArgs B;
    B.segptr = D.segptr;
    B.idx = D.idx;
    B.res = A.res;
    B.table = mode == M_CSC ? (const void*)A.P : mode == M_CSR ? (const void*)A.Q : (const void*)A.y;
    B.b = A.b;
    B.d = A.d;
    B.part = D.part;
    B.units = D.units;
    B.xb = D.xb;
    B.lines = D.lines;
    B.cross = D.cross;
    {
        Timed tm(h, kind);
        if (D.nunits) {
            switch (h->rt) {
                case 0: blocked_rt<0>(B, mode, sub, add, D.nunits, h->s); break;
                case 1: blocked_rt<1>(B, mode, sub, add, D.nunits, h->s); break;
                default: blocked_rt<2>(B, mode, sub, add, D.nunits, h->s); break;
            }
        }
        const unsigned cg = (D.lines + kBlock - 1) / kBlock;
        if (cg) {
            if (mode == M_CSC) blocked_combine_kernel<M_CSC><<<cg, kBlock, 0, h->s>>>(A, D.segptr, D.part, D.nb, D.lines);
            else if (mode == M_CSR) blocked_combine_kernel<M_CSR><<<cg, kBlock, 0, h->s>>>(A, D.segptr, D.part, D.nb, D.lines);
            else blocked_combine_kernel<M_PLAIN><<<cg, kBlock, 0, h->s>>>(A, D.segptr, D.part, D.nb, D.lines);
        }
    }
    CU(h, cudaGetLastError());
    h->st.launches += 2;
    if (kind == K_CSC) h->st.sweep_csc_launches++;
    else h->st.sweep_csr_launches++;
    return CDMF_OK;
}

// Whether the CSR sweeps of this matrix can stage Q in shared memory; sets
// the kernels' dynamic shared memory limit once per process and device.
bool smemq_possible(int device, int64_t n, int* sms) {
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess ||
        cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return false;
    const int64_t need = 12 * n + 1024;   // three float planes + the static shared memory of the teams
    if (n <= 0 || need > optin) return false;
    static std::mutex mu;
    static std::set<int> done;
    std::lock_guard<std::mutex> lk(mu);
    if (done.insert(device).second) {
        smemq_attrs<0>(optin - 1024);
        smemq_attrs<1>(optin - 1024);
        smemq_attrs<2>(optin - 1024);
    }
    return true;
}

int launch_sweep(cdmf_handle* h, int kind, const DevBins& D, const SweepArgs& A, int mode, bool sub, bool add) {
    if (mode == M_CSR && h->smemq && !h->blocked && !h->tiles) {
        const uint32_t nb = D.nx + D.nc + D.nwb + D.ngb + D.ntb;
        if (nb == 0) return CDMF_OK;
        const size_t smem = 12 * (size_t)A.ncross;
        {
            Timed tm(h, kind);
            CU(h, cudaMemsetAsync(h->smemq_queue, 0, 4, h->s));
            switch (h->rt) {
                case 0: smemq_rt<0>(A, h->idx16, sub, add, (unsigned)h->sms, smem, nb, h->smemq_queue, h->s); break;
                case 1: smemq_rt<1>(A, h->idx16, sub, add, (unsigned)h->sms, smem, nb, h->smemq_queue, h->s); break;
                default: smemq_rt<2>(A, h->idx16, sub, add, (unsigned)h->sms, smem, nb, h->smemq_queue, h->s); break;
            }
        }
        CU(h, cudaGetLastError());
        h->st.launches++;
        h->st.sweep_csr_launches++;
        return CDMF_OK;
    }
    if (h->blocked) return launch_blocked(h, kind, A, mode, sub, add);
    if (h->tiles) {
        const DevTiles& D3 = kind == K_CSC ? h->tcsc : h->tcsr;
        TileArgs T;
        T.s = A;
        T.tile_line = D3.tile_line;
        T.head = D3.head;
        T.tail = D3.tail;
        T.lcount = D3.lcount;
        T.empty = D3.empty;
        T.nempty = D3.nempty;
        T.ntiles = D3.ntiles;
        T.tile_blocks = D3.tile_blocks;
        T.nnz = (uint32_t)h->nnz;
        const unsigned grid = D3.tile_blocks + D3.empty_blocks;
        if (grid == 0) return CDMF_OK;
        {
            Timed tm(h, kind);
            switch (h->rt) {
                case 0: tile_rt<0>(T, mode, sub, add, grid, h->s); break;
                case 1: tile_rt<1>(T, mode, sub, add, grid, h->s); break;
                default: tile_rt<2>(T, mode, sub, add, grid, h->s); break;
            }
        }
        CU(h, cudaGetLastError());
        h->st.launches++;
        if (kind == K_CSC) h->st.sweep_csc_launches++;
        else h->st.sweep_csr_launches++;
        return CDMF_OK;
    }
    const unsigned grid = D.nx + D.nc + D.nwb + D.ngb + D.ntb;
    if (grid == 0) return CDMF_OK;
    if (mode == M_CSR && h->idx16) mode = M_CSR16;
    if (mode == M_CSC && h->nnz >= kLargeNnz) mode = h->cidx16 ? M_CSCQ : M_CSCP;
    {
        Timed tm(h, kind);
        switch (h->rt) {
            case 0: launch_rt<0>(A, mode, sub, add, grid, h->s); break;
            case 1: launch_rt<1>(A, mode, sub, add, grid, h->s); break;
            default: launch_rt<2>(A, mode, sub, add, grid, h->s); break;
        }
    }
    CU(h, cudaGetLastError());
    h->st.launches++;
    if (kind == K_CSC) h->st.sweep_csc_launches++;
    else h->st.sweep_csr_launches++;
    return CDMF_OK;
}

// The two sweeps of inner iteration `it` of feature t: A over CSC (solves
// H[t]), B over CSR (solves W[t]).
void feature_args(cdmf_handle* h, uint32_t t, int it, SweepArgs& A, SweepArgs& B) {
    const int64_t m = h->m, n = h->n;
    const uint32_t k = h->o.k;
    float* Wt = h->W + (size_t)t * m;
    float* Ht = h->H + (size_t)t * n;
    const int tp = h->pending;
    const float* Wp = tp >= 0 ? h->W + (size_t)tp * m : nullptr;
    const float* Hp = tp >= 0 ? h->H + (size_t)tp * n : nullptr;
    const bool first = it == 1, last = it == h->o.maxinneriter;
    // h_t over CSC: cross vectors are rows (length m)
    A = base_args(h, h->csc, h->csc_ptr, h->csc_idx, h->res_csc);
    A.out = Ht;
    if (first) {
        A.P = h->P;
        A.b = Hp;
        A.d = Ht;
        A.emitQ = h->Q;
        A.idx16 = h->csc_idx16;
        A.cseg = h->csc_seg;
    } else {
        A.y = Wt;
    }
    // w_t over CSR: cross vectors are columns (length n)
    B = base_args(h, h->csr, h->csr_ptr, h->csr_idx, h->res_csr);
    B.out = Wt;
    if (first) {
        B.Q = h->Q;
        B.ncross = (uint32_t)n;
        B.idx16 = h->csr_idx16;
        B.b = Wp;
        B.d = Wt;
    } else {
        B.y = Ht;
    }
    if (last) {
        B.emitP = h->P;
        B.next_old = h->W + (size_t)((t + 1) % k) * m;
    }
}

// Makes P valid for feature t (it is, in steady state: the previous feature's
// last CSR sweep wrote it).
int feature_prepare(cdmf_handle* h, uint32_t t) {
    if (h->p_for == (int)t) return CDMF_OK;
    const int64_t m = h->m;
    const int tp = h->pending;
    if (m) {
        pack_p_kernel<<<(unsigned)std::min<int64_t>(4096, (m + 255) / 256), 256, 0, h->s>>>(
            h->P, tp >= 0 ? h->W + (size_t)tp * m : nullptr, h->W + (size_t)t * m, m);
        CU(h, cudaGetLastError());
        h->st.launches++;
    }
    h->p_for = (int)t;
    return CDMF_OK;
}

void feature_finish(cdmf_handle* h, uint32_t t) {
    h->p_for = (int)((t + 1) % h->o.k);
    h->pending = (int)t;
}

// One feature t of outer iteration `oiter`.
int feature_step(cdmf_handle* h, uint32_t t, int oiter) {
    const int T = h->o.maxinneriter;
    if (T <= 0) return CDMF_OK;
    const bool sub = h->pending >= 0, add = oiter > 1;
    int r;
    if ((r = feature_prepare(h, t))) return r;
    for (int it = 1; it <= T; ++it) {
        SweepArgs A, B;
        feature_args(h, t, it, A, B);
        if ((r = launch_sweep(h, K_CSC, h->csc, A, it == 1 ? M_CSC : M_PLAIN, sub, add))) return r;
        if ((r = launch_sweep(h, K_CSR, h->csr, B, it == 1 ? M_CSR : M_PLAIN, sub, add))) return r;
    }
    feature_finish(h, t);
    return CDMF_OK;
}

int launch_rmse(cdmf_handle* h, double* dst) {
    Timed tm(h, K_RMSE);
    rmse_kernel<float><<<h->rmse_grid, kBlock, 0, h->s>>>(h->te_row, h->te_col, h->te_val, h->nt, h->W, h->H, h->m,
                                                         h->n, h->o.k, h->rmse_part, h->rmse_count, dst, nullptr);
    CU(h, cudaGetLastError());
    h->st.launches++;
    h->st.rmse_launches++;
    return CDMF_OK;
}

int flush_pending(cdmf_handle* h) {
    if (h->pending < 0) return CDMF_OK;
    const int tp = h->pending;
    const float* Wp = h->W + (size_t)tp * h->m;
    const float* Hp = h->H + (size_t)tp * h->n;
    if (h->blocked) {
        const DevBlocked& C = h->bcsc;
        const DevBlocked& R = h->bcsr;
        switch (h->rt) {
            case 0:
                blocked_flush_kernel<0><<<2048, kBlock, 0, h->s>>>(C.segptr, C.idx, h->res_csc, Wp, Hp, C.nb, C.lines, C.xb);
                blocked_flush_kernel<0><<<2048, kBlock, 0, h->s>>>(R.segptr, R.idx, h->res_csr, Hp, Wp, R.nb, R.lines, R.xb);
                break;
            case 1:
                blocked_flush_kernel<1><<<2048, kBlock, 0, h->s>>>(C.segptr, C.idx, h->res_csc, Wp, Hp, C.nb, C.lines, C.xb);
                blocked_flush_kernel<1><<<2048, kBlock, 0, h->s>>>(R.segptr, R.idx, h->res_csr, Hp, Wp, R.nb, R.lines, R.xb);
                break;
            default:
                blocked_flush_kernel<2><<<2048, kBlock, 0, h->s>>>(C.segptr, C.idx, h->res_csc, Wp, Hp, C.nb, C.lines, C.xb);
                blocked_flush_kernel<2><<<2048, kBlock, 0, h->s>>>(R.segptr, R.idx, h->res_csr, Hp, Wp, R.nb, R.lines, R.xb);
                break;
        }
        CU(h, cudaGetLastError());
        h->pending = -1;
        h->p_for = -1;
        return CDMF_OK;
    }
    const unsigned gc = (unsigned)std::min<int64_t>(4096, (h->n + kWarps - 1) / kWarps + 1);
    const unsigned gr = (unsigned)std::min<int64_t>(4096, (h->m + kWarps - 1) / kWarps + 1);
    switch (h->rt) {
        case 0:
            flush_kernel<0><<<gc, kBlock, 0, h->s>>>(h->csc_ptr, h->csc_idx, h->res_csc, Wp, Hp, (uint32_t)h->n);
            flush_kernel<0><<<gr, kBlock, 0, h->s>>>(h->csr_ptr, h->csr_idx, h->res_csr, Hp, Wp, (uint32_t)h->m);
            break;
        case 1:
            flush_kernel<1><<<gc, kBlock, 0, h->s>>>(h->csc_ptr, h->csc_idx, h->res_csc, Wp, Hp, (uint32_t)h->n);
            flush_kernel<1><<<gr, kBlock, 0, h->s>>>(h->csr_ptr, h->csr_idx, h->res_csr, Hp, Wp, (uint32_t)h->m);
            break;
        default:
            flush_kernel<2><<<gc, kBlock, 0, h->s>>>(h->csc_ptr, h->csc_idx, h->res_csc, Wp, Hp, (uint32_t)h->n);
            flush_kernel<2><<<gr, kBlock, 0, h->s>>>(h->csr_ptr, h->csr_idx, h->res_csr, Hp, Wp, (uint32_t)h->m);
            break;
    }
    CU(h, cudaGetLastError());
    h->pending = -1;
    h->p_for = -1;
    return CDMF_OK;
}

void launch_refresh(cdmf_handle* h, int rt, int nu, const float* pa, const float* pb) {
    RefreshDesc D;
    D.ptr = h->csr_ptr;
    D.crow = h->ref_crow;
    D.idx = h->csr_idx;
    D.val = h->csr_val;
    D.to_csr = h->ref_to_csr;
    D.to_csc = h->to_csc;
    D.m = h->m;
    D.nnz = h->nnz;
    D.Wrm = h->Wrm;
    D.Hrm = h->Hrm;
    D.kp = h->kp;
    D.slices = (uint32_t)nu;
    D.res_csr = h->res_csr;
    D.res_csc = h->res_csc;
    D.pa = pa;
    D.pb = pb;
    D.part = h->ref_part;
    D.counter = h->ref_count;
    D.drift_out = h->drift_out;
    D.nonfinite = h->nonfinite;
    if (rt == 1) launch_refresh_rt<1>(D, (unsigned)h->ref_grid, h->s);
    else launch_refresh_rt<2>(D, (unsigned)h->ref_grid, h->s);
}

// 16-bit modes: recompute both residual copies from the FP32 ratings and
// factors (clears the pending subtract).
int refresh_residual(cdmf_handle* h) {
    const int tp = h->pending;
    const float* pa = tp >= 0 ? h->H + (size_t)tp * h->n : nullptr;
    const float* pb = tp >= 0 ? h->W + (size_t)tp * h->m : nullptr;
    {
        Timed tm(h, K_REFRESH);
        dim3 gw((unsigned)((h->m + 31) / 32), (h->kp + 31) / 32), gh((unsigned)((h->n + 31) / 32), (h->kp + 31) / 32);
        if (h->m) to_row_major_kernel<<<gw, kBlock, 0, h->s>>>(h->W, h->Wrm, h->o.k, h->kp, h->m);
        if (h->n) to_row_major_kernel<<<gh, kBlock, 0, h->s>>>(h->H, h->Hrm, h->o.k, h->kp, h->n);
        const uint32_t kq = h->kp / 4;
        const int nu = kq <= kRefG ? 1 : kq <= 2 * kRefG ? 2 : kq <= 4 * kRefG ? 4 : kq <= 8 * kRefG ? 8 : 0;
        launch_refresh(h, h->rt, nu, pa, pb);
    }
    CU(h, cudaGetLastError());
    h->st.launches += 3;
    h->st.refresh_launches += 1;
    h->pending = -1;
    h->refreshed = true;
    return CDMF_OK;
}

// Factor rows between the caller's numbering and the engine's: gather
// (dst[t][q] = src[t][old[q]]) on the way in, scatter on the way out.
__global__ void permute_factors_kernel(const float* __restrict__ src, float* __restrict__ dst,
                                       const uint32_t* __restrict__ old_of_new, uint32_t k, int64_t len, int scatter) {
    const int64_t total = (int64_t)k * len;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = e / len, q = e - t * len;
        const int64_t o = t * len + old_of_new[q];
        if (scatter) dst[o] = src[e];
        else dst[e] = src[o];
    }
}

// Caller-order factors (host) -> engine order (device), through ftmp.
int factors_in(cdmf_handle* h, const float* user, float* dev, int64_t len, const uint32_t* old_of_new) {
    const size_t bytes = sizeof(float) * h->o.k * len;
    CU(h, cudaMemcpyAsync(h->ftmp, user, bytes, cudaMemcpyHostToDevice, h->s));
    permute_factors_kernel<<<1216, kBlock, 0, h->s>>>(h->ftmp, dev, old_of_new, h->o.k, len, 0);
    CU(h, cudaGetLastError());
    return CDMF_OK;
}

int factors_out(cdmf_handle* h, const float* dev, float* user, int64_t len, const uint32_t* old_of_new) {
    const size_t bytes = sizeof(float) * h->o.k * len;
    permute_factors_kernel<<<1216, kBlock, 0, h->s>>>(dev, h->ftmp, old_of_new, h->o.k, len, 1);
    CU(h, cudaGetLastError());
    CU(h, cudaMemcpyAsync(user, h->ftmp, bytes, cudaMemcpyDeviceToHost, h->s));
    return CDMF_OK;
}

__global__ void narrow_idx_kernel(const uint32_t* __restrict__ src, uint16_t* __restrict__ dst, int64_t count) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x)
        dst[q] = (uint16_t)src[q];
}

// cseg[kCSeg * j + h]: the end of run h of column j, i.e. the first position
// of the column whose row is at least (h + 1) * 65,536 (the column's end for
// h = kCSeg - 1).  One thread per (column, run); rows ascend in a column.
__global__ void csc_segments_kernel(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ idx, int64_t n,
                                    uint32_t* __restrict__ seg) {
    const int64_t total = n * kCSeg;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = t / kCSeg;
        const uint32_t h = (uint32_t)(t % kCSeg);
        uint32_t lo = ptr[j], hi = ptr[j + 1];
        if (h + 1 < kCSeg) {
            const uint32_t bound = (h + 1) << 16;
            while (lo < hi) {   // first position with row >= bound
                const uint32_t mid = lo + (hi - lo) / 2;
                if (idx[mid] < bound) lo = mid + 1; else hi = mid;
            }
        }
        seg[t] = lo;
    }
}

__global__ void f32_to_res_kernel(const float* __restrict__ src, void* __restrict__ dst, int64_t count, int rt) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x) {
        if (rt == 1) ((__nv_bfloat16*)dst)[q] = __float2bfloat16_rn(src[q]);
        else ((__half*)dst)[q] = __float2half_rn(src[q]);
    }
}
__global__ void res_to_f32_kernel(const void* __restrict__ src, float* __restrict__ dst, int64_t count, int rt) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x) {
        if (rt == 1) dst[q] = __bfloat162float(((const __nv_bfloat16*)src)[q]);
        else dst[q] = __half2float(((const __half*)src)[q]);
    }
}

// dst residual := src ratings (device, float)
int reset_residual(cdmf_handle* h, void* dst, const float* src) {
    if (h->nnz == 0) return CDMF_OK;
    if (h->blocked) {
        const uint32_t* map = dst == h->res_csr ? h->bcsr.map : h->bcsc.map;
        if (h->rt == 0) scatter_res_kernel<0><<<1216, 256, 0, h->s>>>(src, map, dst, h->nnz);
        else if (h->rt == 1) scatter_res_kernel<1><<<1216, 256, 0, h->s>>>(src, map, dst, h->nnz);
        else scatter_res_kernel<2><<<1216, 256, 0, h->s>>>(src, map, dst, h->nnz);
        CU(h, cudaGetLastError());
        return CDMF_OK;
    }
    if (h->rt == 0) {
        CU(h, cudaMemcpyAsync(dst, src, sizeof(float) * h->nnz, cudaMemcpyDeviceToDevice, h->s));
    } else {
        f32_to_res_kernel<<<1216, 256, 0, h->s>>>(src, dst, h->nnz, h->rt);
        CU(h, cudaGetLastError());
    }
    return CDMF_OK;
}

// Caller numbering <-> engine numbering (identity unless relabelled).
// X is k x len feature-major; `old_of_new` maps an engine id to a caller id.
void gather_ids(const float* user, float* eng, uint32_t k, int64_t len, const uvec<uint32_t>& old_of_new) {
    for (uint32_t t = 0; t < k; ++t) {
        const float* u = user + (size_t)t * len;
        float* e = eng + (size_t)t * len;
        for (int64_t q = 0; q < len; ++q) e[q] = u[old_of_new[q]];
    }
}

int need_host_maps(cdmf_handle* h) {
    if (!h->d_csr_pos || !h->csr_pos.empty()) return CDMF_OK;
    const int64_t N = h->nnz;
    h->csr_pos.resize(N);
    h->csc_from_csr.resize(N);
    h->ucsr_ptr.resize(h->m + 1);
    h->ucsr_idx.resize(N);
    CU(h, cudaMemcpyAsync(h->csr_pos.data(), h->d_csr_pos, 4 * (size_t)N, cudaMemcpyDeviceToHost, h->s));
    CU(h, cudaMemcpyAsync(h->csc_from_csr.data(), h->d_csc_from_csr, 4 * (size_t)N, cudaMemcpyDeviceToHost, h->s));
    CU(h, cudaMemcpyAsync(h->ucsr_ptr.data(), h->d_ucsr_ptr, 4 * (size_t)(h->m + 1), cudaMemcpyDeviceToHost, h->s));
    CU(h, cudaMemcpyAsync(h->ucsr_idx.data(), h->d_ucsr_idx, 4 * (size_t)N, cudaMemcpyDeviceToHost, h->s));
    CU(h, cudaStreamSynchronize(h->s));
    return CDMF_OK;
}

int need_csc_pos(cdmf_handle* h) {
    if (!h->relabeled || !h->csc_pos.empty() || h->nnz == 0) return CDMF_OK;
    if (int r = need_host_maps(h)) return r;
    if (!relabel_csc_positions(h->m, h->n, h->ucsr_ptr.data(), h->ucsr_idx.data(), h->csr_pos, h->csc_from_csr,
                               h->csc_pos))
        return fail(h, CDMF_ERR_ALLOC, "caller CSC positions");
    return CDMF_OK;
}

// Whether the 16-bit modes refresh the residual before feature t of outer
// iteration oiter: at the start of every outer iteration after the first,
// and every kEarlyRefresh features of the first, where no refresh has run
// yet and every rank-one update rounds each residual entry once more.
bool refresh_before(const cdmf_handle* h, int oiter, uint32_t t) {
    if (h->rt == 0 || h->nnz == 0) return false;
    if (oiter > 1) return t == 0;
    return t > 0 && t % kEarlyRefresh == 0;
}

// One outer iteration (src/cdmf_ref.cpp:69-137): refreshes (16-bit modes),
// k rank-one updates, test RMSE into rmse_dst.
int do_outer(cdmf_handle* h, int oiter, double* rmse_dst) {
    int r;
    for (uint32_t t = 0; t < h->o.k; ++t) {
        if (refresh_before(h, oiter, t))
            if ((r = refresh_residual(h))) return r;
        if ((r = feature_step(h, t, oiter))) return r;
    }
    if (h->o.rmse_each_outer && h->nt > 0)
        if ((r = launch_rmse(h, rmse_dst))) return r;
    return CDMF_OK;
}

// The same outer iteration replayed from a CUDA graph.  The launch sequence
// depends only on (first outer, pending feature, P validity, refresh, RMSE),
// so one graph per signature is captured on first use and replayed after.
int do_outer_graph(cdmf_handle* h, int oiter, double* rmse_dst) {
    const bool want_refresh =
        refresh_before(h, oiter, 0) || (h->o.k > kEarlyRefresh && refresh_before(h, oiter, kEarlyRefresh));
    const bool want_rmse = h->o.rmse_each_outer && h->nt > 0;
    const int sig[5] = {oiter == 1, h->pending, h->p_for, want_refresh, want_rmse};
    cdmf_handle::Graph* G = nullptr;
    for (auto& g : h->graphs)
        if (std::memcmp(g.sig, sig, sizeof(sig)) == 0) G = &g;
    if (!G) {
        const cdmf_stats before = h->st;
        CU(h, cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
        const int r = do_outer(h, oiter, h->rmse_graph_slot);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->s, &graph);
        if (r || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return r ? r : fail(h, CDMF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        }
        cdmf_handle::Graph g;
        std::memcpy(g.sig, sig, sizeof(sig));
        const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return fail(h, CDMF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
        g.end_pending = h->pending;
        g.end_p_for = h->p_for;
        g.launches = h->st.launches - before.launches;
        g.csc = h->st.sweep_csc_launches - before.sweep_csc_launches;
        g.csr = h->st.sweep_csr_launches - before.sweep_csr_launches;
        g.rmse = h->st.rmse_launches - before.rmse_launches;
        g.refresh = h->st.refresh_launches - before.refresh_launches;
        h->graphs.push_back(g);
        G = &h->graphs.back();
    } else {
        h->pending = G->end_pending;
        h->p_for = G->end_p_for;
        if (G->refresh > 0) h->refreshed = true;
        h->st.launches += G->launches;
        h->st.sweep_csc_launches += G->csc;
        h->st.sweep_csr_launches += G->csr;
        h->st.rmse_launches += G->rmse;
        h->st.refresh_launches += G->refresh;
    }
    CU(h, cudaGraphLaunch(G->exec, h->s));
    if (want_rmse) CU(h, cudaMemcpyAsync(rmse_dst, h->rmse_graph_slot, sizeof(double), cudaMemcpyDeviceToDevice, h->s));
    return CDMF_OK;
}

int replan(cdmf_handle* h, const BinCfg& cfg, const BinCfg& cfg_c) {
    // the captured outer iterations hold the old bins' arrays and counts
    CU(h, cudaStreamSynchronize(h->s));
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
    free_bins(h, h->csr);
    free_bins(h, h->csc);
    h->cfg = cfg;
    h->cfg_c = cfg_c;
    int r;
    if ((r = upload_bins(h, h->csr, plan_bins(h->hptr_r.data(), h->m, h->seq, cfg))) ||
        (r = upload_bins(h, h->csc, plan_bins(h->hptr_c.data(), h->n, h->seq, cfg_c))))
        return r;
    return CDMF_OK;
}

int replan(cdmf_handle* h, const BinCfg& cfg) { return replan(h, cfg, cfg); }

// Time of one steady-state feature (CSC + CSR sweep with subtract and
// add-back) under the current bins, in ms; the state is scratch.
int time_feature(cdmf_handle* h, int reps, double* ms) {
    h->pending = 0;
    h->p_for = 0;
    SweepArgs A, B;
    feature_args(h, 0, 1, A, B);
    int r;
    for (int w = 0; w < 1 + reps; ++w) {
        if (w == 1) CU(h, cudaEventRecord(h->ev_start, h->s));
        if ((r = launch_sweep(h, K_CSC, h->csc, A, M_CSC, true, true)) ||
            (r = launch_sweep(h, K_CSR, h->csr, B, M_CSR, true, true)))
            return r;
    }
    CU(h, cudaEventRecord(h->ev_stop, h->s));
    CU(h, cudaEventSynchronize(h->ev_stop));
    float t = 0;
    CU(h, cudaEventElapsedTime(&t, h->ev_start, h->ev_stop));
    *ms = t / reps;
    return CDMF_OK;
}

struct TuneKey {
    int64_t m, n, nnz;
    int rt, relabeled, device;
    bool operator<(const TuneKey& o) const {
        return std::tie(m, n, nnz, rt, relabeled, device) < std::tie(o.m, o.n, o.nnz, o.rt, o.relabeled, o.device);
    }
};
// the autotuner's pick for a shape: the bin limits and the lanes per
// group-bin line
struct TunePick {
    BinCfg cfg, cfg_c;
    uint32_t lanes;
};
std::map<TuneKey, TunePick>& tune_cache() {
    static std::map<TuneKey, TunePick> c;
    return c;
}
std::mutex& tune_mutex() {
    static std::mutex mu;
    return mu;
}
TuneKey tune_key(const cdmf_handle* h) {
    return TuneKey{h->m, h->n, h->nnz, h->rt, h->relabeled ? 1 : 0, h->o.device};
}
bool cached_pick(const TuneKey& key, TunePick* out) {
    std::lock_guard<std::mutex> lk(tune_mutex());
    auto it = tune_cache().find(key);
    if (it == tune_cache().end()) return false;
    *out = it->second;
    return true;
}
bool same_cfg(const BinCfg& a, const BinCfg& b) {
    return a.thread_max == b.thread_max && a.group_max == b.group_max && a.warp_max == b.warp_max &&
           a.cta_max == b.cta_max && a.chunk == b.chunk;
}

}  // namespace

namespace {

// cdmf_cuda_train's outer iterations, queued one ahead of the host: outer
// iteration it + 1 is on the stream before the host waits for the RMSE of
// outer iteration it, so the GPU does not sit idle while the host reads a
// result, calls the callback and queues the next iteration.  The launches and
// their order are those of cdmf_cuda_run(h, 1, ...) called once per outer
// iteration, so are the results.  A non-finite residual at a refresh ends the
// run with CDMF_ERR_NUMERIC after the callback of the outer iteration before
// it, as the per-iteration calls did.  cb's ms: time since the first outer
// iteration started, on the engine stream.
int run_queued(cdmf_handle* h, double* rmse_out, cdmf_outer_cb cb, void* user) {
    const int n = h->o.maxiter;
    if (n <= 0) return CDMF_OK;
    CU(h, cudaSetDevice(h->o.device));
    const bool want_rmse = h->o.rmse_each_outer && h->nt > 0;
    struct Slot {              // read back after each outer iteration
        double rmse;
        unsigned long long bad;   // non-finite refresh results so far
    };
    struct Res {
        cudaStream_t s;
        Slot* slots = nullptr;
        std::vector<cudaEvent_t> ev;
        ~Res() {
            // (an early return can leave copies into slots on the stream)
            cudaStreamSynchronize(s);
            for (cudaEvent_t e : ev) cudaEventDestroy(e);
            if (slots) cudaFreeHost(slots);
        }
    } res{h->s};
    CU(h, cudaMallocHost((void**)&res.slots, sizeof(Slot) * (size_t)n));
    res.ev.reserve(n);
    for (int it = 0; it < n; ++it) {
        cudaEvent_t e = nullptr;
        CU(h, cudaEventCreate(&e));
        res.ev.push_back(e);
    }
    h->refreshed = false;
    h->marks.clear();
    h->pool_used = 0;
    if (h->rt != 0) CU(h, cudaMemsetAsync(h->nonfinite, 0, 8, h->s));
    CU(h, cudaEventRecord(h->ev_start, h->s));
    auto finish = [&](int it) -> int {
        CU(h, cudaEventSynchronize(res.ev[it]));
        if (h->rt != 0 && res.slots[it].bad)
            return fail(h, CDMF_ERR_NUMERIC, "non-finite residual values at the refresh");
        float ms = 0;
        CU(h, cudaEventElapsedTime(&ms, h->ev_start, res.ev[it]));
        const double rm = want_rmse ? res.slots[it].rmse : -1.0;
        if (rmse_out) rmse_out[it] = rm;
        if (cb) cb(it + 1, rm, ms, user);
        return CDMF_OK;
    };
    // rmse_out on the device has maxiter + 1 slots: one per outer iteration
    for (int it = 0; it < n; ++it) {
        const int oiter = h->next_oiter;
        int r = (h->o.use_graph && !h->profiling) ? do_outer_graph(h, oiter, h->rmse_out + it)
                                                  : do_outer(h, oiter, h->rmse_out + it);
        if (r) return r;
        h->st.updates += h->o.k;
        h->next_oiter++;
        if (want_rmse)
            CU(h, cudaMemcpyAsync(&res.slots[it].rmse, h->rmse_out + it, 8, cudaMemcpyDeviceToHost, h->s));
        if (h->rt != 0) CU(h, cudaMemcpyAsync(&res.slots[it].bad, h->nonfinite, 8, cudaMemcpyDeviceToHost, h->s));
        CU(h, cudaEventRecord(res.ev[it], h->s));
        if (it > 0 && (r = finish(it - 1))) return r;
    }
    return finish(n - 1);
}

}  // namespace

extern "C" {

void cdmf_opts_default(cdmf_opts* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->k = 10;                 // src/pmf.h:17-18 defaults
    o->lambda = 0.1f;
    o->maxiter = 5;
    o->maxinneriter = 5;
    o->version = 1;
    o->residual = CDMF_RES_F32;
    o->reduce = CDMF_REDUCE_TREE;
    o->rmse_each_outer = 1;
    o->use_graph = 0;
    o->threads_per_block = 0;
    o->device = 0;
    o->verbose = 0;
    o->relabel = 1;
    o->autotune = 0;
    o->layout = CDMF_LAYOUT_LINES;
}

const char* cdmf_cuda_strerror(int status) {
    if (status > 0 || status < -8) return "unknown status";
    return kErrStr[-status];
}

int cdmf_cuda_version(void) { return 100; }

void* cdmf_cuda_host_alloc(uint64_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return p;
}

void cdmf_cuda_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

const char* cdmf_cuda_last_error(const cdmf_handle* h) { return h ? h->err.c_str() : ""; }

void cdmf_cuda_destroy(cdmf_handle* h) {
    if (!h) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(h->o.device);
    if (h->s) cudaStreamSynchronize(h->s);
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
    for (void* p : h->allocs) cudaFree(p);
    for (cudaEvent_t e : h->pool) cudaEventDestroy(e);
    if (h->ev_start) cudaEventDestroy(h->ev_start);
    if (h->ev_stop) cudaEventDestroy(h->ev_stop);
    if (h->s) cudaStreamDestroy(h->s);
    cudaSetDevice(dev);
    delete h;
}

int cdmf_cuda_create(const cdmf_problem* p, const cdmf_opts* o, cdmf_handle** out) {
    if (!out) return CDMF_ERR_INVALID;
    *out = nullptr;
    if (!p || !o) return CDMF_ERR_INVALID;
    if (p->m < 0 || p->n < 0 || p->nnz < 0 || p->nnz_test < 0 || o->k == 0 || o->maxinneriter < 0 ||
        o->maxiter < 0 || !(o->lambda >= 0.0f))
        return CDMF_ERR_INVALID;
    if (o->residual < 0 || o->residual > 2 || o->reduce < 0 || o->reduce > 1 || o->version < 1 || o->version > 3)
        return CDMF_ERR_INVALID;
    if (p->nnz > (int64_t)UINT32_MAX - 8192 || p->m >= (int64_t)UINT32_MAX || p->n >= (int64_t)UINT32_MAX ||
        p->nnz_test > (int64_t)INT32_MAX * 64)
        return CDMF_ERR_TOO_LARGE;
    int r;
    // o->verbose: phase times of the set-up on stderr
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* what) {
        if (!o->verbose) return;
        const auto t = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[cdmf] create: %-12s %8.1f ms\n", what,
                     std::chrono::duration<double, std::milli>(t - t_last).count());
        t_last = t;
    };
    if ((r = check_compressed(p->csr_row_ptr, p->csr_col_idx, p->m, p->n, p->nnz))) return r;
    if ((r = check_compressed(p->csc_col_ptr, p->csc_row_idx, p->n, p->m, p->nnz))) return r;
    if (p->nnz > 0 && (!p->csr_val || !p->csc_val)) return CDMF_ERR_INVALID;
    if (p->nnz_test > 0) {
        if (!p->test_row || !p->test_col || !p->test_val) return CDMF_ERR_INVALID;
        uint32_t hr = 0, hc = 0;
#pragma omp parallel for schedule(static) reduction(max : hr, hc)
        for (int64_t e = 0; e < p->nnz_test; ++e) {
            hr = std::max(hr, p->test_row[e]);
            hc = std::max(hc, p->test_col[e]);
        }
        if ((int64_t)hr >= p->m || (int64_t)hc >= p->n) return CDMF_ERR_INVALID;
    }
    phase("checks");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CDMF_ERR_NO_DEVICE;
    if (o->device < 0 || o->device >= ndev) return CDMF_ERR_NO_DEVICE;

    const bool seq_order = o->reduce == CDMF_REDUCE_SEQUENTIAL;
    Relabel RL;
    const cdmf_problem q0 = *p;
    cdmf_problem q = *p;
    // relabel 1 with the line layout: the renumbered structures are built on
    // the device below; otherwise (relabel 2, or the blocked layout, which
    // plans on host copies) on the host here
    const bool relabel_on_gpu = o->relabel == 1 && !seq_order && p->nnz > 0 && o->layout != CDMF_LAYOUT_BLOCKED;
    if (o->relabel && !seq_order && p->nnz > 0 && !relabel_on_gpu) {
        if (!relabel(*p, RL)) return CDMF_ERR_INVALID;
        q.csr_row_ptr = RL.csr_ptr.data();
        q.csr_col_idx = RL.csr_idx.data();
        q.csr_val = RL.csr_val.data();
        q.csc_col_ptr = RL.csc_ptr.data();
        q.csc_row_idx = RL.csc_idx.data();
        q.csc_val = RL.csc_val.data();
        q.test_row = RL.te_row.data();
        q.test_col = RL.te_col.data();
        p = &q;
        phase("relabel");
    }
    cdmf_handle* h = new cdmf_handle();
    if (p == &q) {
        h->relabeled = true;
        h->row_old = std::move(RL.row_old);
        h->col_old = std::move(RL.col_old);
        h->csr_pos = std::move(RL.csr_pos);
        h->csc_from_csr = std::move(RL.csc_from_csr);
        h->ucsr_ptr.assign(q0.csr_row_ptr, q0.csr_row_ptr + q0.m + 1);
        h->ucsr_idx.assign(q0.csr_col_idx, q0.csr_col_idx + q0.nnz);
        phase("keep maps");
    }
    h->o = *o;
    h->m = p->m;
    h->n = p->n;
    h->nnz = p->nnz;
    h->nt = p->nnz_test;
    h->rt = o->residual;
    h->rbytes = o->residual == CDMF_RES_F32 ? 4 : 2;
    auto bail = [&](int code) { cdmf_cuda_destroy(h); return code; };
    if (cudaSetDevice(o->device) != cudaSuccess) return bail(CDMF_ERR_NO_DEVICE);
    if (cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking) != cudaSuccess) return bail(CDMF_ERR_CUDA);
    if (cudaEventCreate(&h->ev_start) != cudaSuccess || cudaEventCreate(&h->ev_stop) != cudaSuccess)
        return bail(CDMF_ERR_CUDA);
    const int64_t m = p->m, n = p->n, N = p->nnz, k = o->k;
    GpuRelabel G;
    uvec<uint32_t> te_row, te_col;
    if (relabel_on_gpu) {
        if ((r = gpu_relabel(*p, h->s, G, h->allocs)))
            return bail(r == CDMF_ERR_ALLOC ? r : fail(h, r, "degree relabelling on the device"));
        h->relabeled = true;
        h->row_old = std::move(G.row_old);
        h->col_old = std::move(G.col_old);
        h->csr_ptr = G.csr_ptr;
        h->csr_idx = G.csr_idx;
        h->csr_val = G.csr_val;
        h->csc_ptr = G.csc_ptr;
        h->csc_idx = G.csc_idx;
        h->csc_val = G.csc_val;
        h->d_csr_pos = G.csr_pos;
        h->d_csc_from_csr = G.csc_from_csr;
        h->d_ucsr_ptr = G.uptr;
        h->d_ucsr_idx = G.uidx;
        h->d_row_old = G.d_row_old;
        h->d_col_old = G.d_col_old;
        // the test set in the new numbering
        uvec<uint32_t> row_new(m), col_new(n);
        for (int64_t v = 0; v < m; ++v) row_new[h->row_old[v]] = (uint32_t)v;
        for (int64_t v = 0; v < n; ++v) col_new[h->col_old[v]] = (uint32_t)v;
        te_row.resize(p->nnz_test);
        te_col.resize(p->nnz_test);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < p->nnz_test; ++e) {
            te_row[e] = row_new[p->test_row[e]];
            te_col[e] = col_new[p->test_col[e]];
        }
        q.test_row = te_row.data();
        q.test_col = te_col.data();
        p = &q;
        phase("relabel (GPU)");
    } else if ((r = dalloc(h, &h->csr_ptr, m + 1)) || (r = dalloc(h, &h->csr_idx, N)) ||
               (r = dalloc(h, &h->csc_ptr, n + 1)) || (r = dalloc(h, &h->csc_idx, N)) ||
               (r = dalloc(h, &h->csr_val, N)) || (r = dalloc(h, &h->csc_val, N))) {
        return bail(r);
    }
    if (h->relabeled) {
        if ((r = dalloc(h, &h->ftmp, (size_t)k * std::max(m, n)))) return bail(r);
        if (!relabel_on_gpu) {   // host-built numbering: its maps to the device
            if ((r = dalloc(h, &h->d_row_old, m)) || (r = dalloc(h, &h->d_col_old, n))) return bail(r);
            if (cudaMemcpyAsync(h->d_row_old, h->row_old.data(), 4 * (size_t)m, cudaMemcpyHostToDevice, h->s) !=
                    cudaSuccess ||
                cudaMemcpyAsync(h->d_col_old, h->col_old.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, h->s) !=
                    cudaSuccess)
                return bail(CDMF_ERR_CUDA);
        }
    }
    if ((r = dalloc(h, (char**)&h->res_csr, N * h->rbytes)) || (r = dalloc(h, (char**)&h->res_csc, N * h->rbytes)) ||
        (r = dalloc(h, &h->W, k * m)) || (r = dalloc(h, &h->H, k * n)) || (r = dalloc(h, &h->P, m)) ||
        (r = dalloc(h, &h->Q, n)) ||
        (r = dalloc(h, &h->te_row, h->nt)) || (r = dalloc(h, &h->te_col, h->nt)) || (r = dalloc(h, &h->te_val, h->nt)))
        return bail(r);
    h->rmse_grid = (int)std::max<int64_t>(1, std::min<int64_t>(4 * 152, (h->nt + kBlock - 1) / kBlock));
    if ((r = dalloc(h, &h->rmse_part, h->rmse_grid)) || (r = dalloc(h, &h->rmse_out, 1 + std::max(0, o->maxiter))) ||
        (r = dalloc(h, &h->rmse_graph_slot, 1)) ||
        (r = dalloc(h, &h->rmse_count, 1)))
        return bail(r);
    auto up = [&](void* dst, const void* src, size_t bytes) -> int {
        if (bytes == 0) return CDMF_OK;
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->s);
        if (e != cudaSuccess) return fail(h, CDMF_ERR_CUDA, cudaGetErrorString(e));
        return CDMF_OK;
    };
    if (!relabel_on_gpu &&
        ((r = up(h->csr_ptr, p->csr_row_ptr, 4 * (m + 1))) || (r = up(h->csr_idx, p->csr_col_idx, 4 * N)) ||
         (r = up(h->csc_ptr, p->csc_col_ptr, 4 * (n + 1))) || (r = up(h->csc_idx, p->csc_row_idx, 4 * N)) ||
         (r = up(h->csr_val, p->csr_val, 4 * N)) || (r = up(h->csc_val, p->csc_val, 4 * N))))
        return bail(r);
    if ((r = up(h->te_row, p->test_row, 4 * h->nt)) || (r = up(h->te_col, p->test_col, 4 * h->nt)) ||
        (r = up(h->te_val, p->test_val, 4 * h->nt)))
        return bail(r);
    if (cudaMemsetAsync(h->rmse_count, 0, 4, h->s) != cudaSuccess) return bail(CDMF_ERR_CUDA);
    phase("alloc+upload");
    const bool seq = o->reduce == CDMF_REDUCE_SEQUENTIAL;
    h->blocked = o->layout == 1 && !seq && N > 0;
    if (h->blocked) {
        BlockedHost br, bc;
        if (!build_blocked(p->csr_row_ptr, p->csr_col_idx, (uint32_t)m, (uint64_t)n, kXbCol, kUnitNnz, br) ||
            !build_blocked(p->csc_col_ptr, p->csc_row_idx, (uint32_t)n, (uint64_t)m, kXbRow, kUnitNnz, bc))
            return bail(CDMF_ERR_ALLOC);
        if ((r = upload_blocked(h, h->bcsr, std::move(br), h->hmap_r)) ||
            (r = upload_blocked(h, h->bcsc, std::move(bc), h->hmap_c)))
            return bail(r);
    }
    if (h->rt != 0) {
        // CSR position -> CSC position; also proves the CSC arrays are the
        // transpose of the CSR arrays, which the refresh scatter relies on
        uvec<uint32_t> to_csc(relabel_on_gpu ? 0 : N);
        if (relabel_on_gpu) {
            // built on the device with the copies
        } else if (h->relabeled) {
            // both copies were built from the CSR: invert the CSC -> CSR map
#pragma omp parallel for schedule(static)
            for (int64_t o = 0; o < N; ++o) to_csc[h->csc_from_csr[o]] = (uint32_t)o;
        } else {
            std::vector<uint32_t> next(p->csc_col_ptr, p->csc_col_ptr + n);
            for (int64_t i = 0; i < m; ++i)
                for (uint32_t q = p->csr_row_ptr[i]; q < p->csr_row_ptr[i + 1]; ++q) {
                    const uint32_t j = p->csr_col_idx[q];
                    const uint32_t pos = next[j]++;
                    if (pos >= p->csc_col_ptr[j + 1] || p->csc_row_idx[pos] != (uint32_t)i ||
                        p->csc_val[pos] != p->csr_val[q])
                        return bail(CDMF_ERR_INVALID);
                    to_csc[q] = pos;
                }
        }
        h->kp = (o->k + 3) / 4 * 4;
        const int64_t nchunks = (N + kRefreshChunk - 1) / kRefreshChunk;
        h->ref_grid = (int)std::max<int64_t>(1, std::min<int64_t>(152 * 8, nchunks));
        if (relabel_on_gpu) h->to_csc = G.to_csc;
        if ((!relabel_on_gpu && (r = dalloc(h, &h->to_csc, N))) || (r = dalloc(h, &h->Wrm, (size_t)m * h->kp)) ||
            (r = dalloc(h, &h->Hrm, (size_t)n * h->kp)) || (r = dalloc(h, &h->ref_part, h->ref_grid)) ||
            (r = dalloc(h, &h->drift_out, 1)) || (r = dalloc(h, &h->ref_count, 1)) || (r = dalloc(h, &h->nonfinite, 1)))
            return bail(r);
        if (h->blocked) {
            // the refresh writes both copies at their blocked positions
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < N; ++q) to_csc[q] = h->hmap_c[to_csc[q]];
            h->ref_to_csr = h->bcsr.map;
        }
        if (!relabel_on_gpu && (r = up(h->to_csc, to_csc.data(), 4 * N))) return bail(r);
        phase("refresh map");
        if (cudaMemsetAsync(h->ref_count, 0, 4, h->s) != cudaSuccess ||
            cudaMemsetAsync(h->nonfinite, 0, 8, h->s) != cudaSuccess ||
            cudaMemsetAsync(h->drift_out, 0, 8, h->s) != cudaSuccess ||
            cudaStreamSynchronize(h->s) != cudaSuccess)
            return bail(CDMF_ERR_CUDA);
    }
    h->seq = seq;
    h->cfg = default_bins(N);
    h->cfg_c = h->cfg;
    h->group_lanes = N >= kLargeNnz && h->rt != 0 ? 4 : 8;
    if (o->autotune && !seq && !h->tiles && !h->blocked) {   // a pick already made for this shape: plan with it
        TunePick pick;
        if (cached_pick(tune_key(h), &pick)) {
            h->cfg = pick.cfg;
            h->cfg_c = pick.cfg_c;
            h->group_lanes = pick.lanes;
        }
    }
    if (relabel_on_gpu) {
        h->hptr_r = std::move(G.hptr_r);
        h->hptr_c = std::move(G.hptr_c);
    } else {
        h->hptr_r.assign(p->csr_row_ptr, p->csr_row_ptr + m + 1);
        h->hptr_c.assign(p->csc_col_ptr, p->csc_col_ptr + n + 1);
    }
    if ((r = upload_bins(h, h->csr, plan_bins(h->hptr_r.data(), m, seq, h->cfg))) ||
        (r = upload_bins(h, h->csc, plan_bins(h->hptr_c.data(), n, seq, h->cfg_c))))
        return bail(r);
    if (h->rt != 0 && N > 0) {
        // the refresh's chunk start rows: the row holding nonzero c * kRefreshChunk, then the last row
        const int64_t nch = (N + kRefreshChunk - 1) / kRefreshChunk;
        std::vector<uint32_t> crow(nch + 1);
        for (int64_t c = 0; c <= nch; ++c) {
            const uint32_t pos = (uint32_t)std::min<int64_t>(c * kRefreshChunk, N - 1);
            crow[c] = (uint32_t)(std::upper_bound(h->hptr_r.begin(), h->hptr_r.end(), pos) - h->hptr_r.begin() - 1);
        }
        if ((r = dalloc(h, &h->ref_crow, nch + 1)) || (r = up(h->ref_crow, crow.data(), 4 * (nch + 1))))
            return bail(r);
        if (cudaStreamSynchronize(h->s) != cudaSuccess) return bail(CDMF_ERR_CUDA);
    }
    phase("bins");
    h->tiles = o->version == 3 && !seq && !h->blocked;
    if (h->tiles && ((r = upload_tiles(h, h->tcsr, h->hptr_r.data(), m, N)) ||
                     (r = upload_tiles(h, h->tcsc, h->hptr_c.data(), n, N))))
        return bail(r);
    // measured on the Netflix-shaped matrix: FP32 CSR sweeps +6 % with the
    // shared-memory table, 16-bit ones -6 % (the 1024-thread CTAs hold 32
    // warps per SM against 48 for the global path), so FP32 only
    if (h->rt == 0 && !h->blocked && !h->tiles && N > 0 && smemq_possible(o->device, n, &h->sms) &&
        !std::getenv("CDMF_NO_SMEMQ")) {
        if ((r = dalloc(h, &h->smemq_queue, 1))) return bail(r);
        h->smemq = true;
    }
    // at most 65,536 columns: the first CSR sweep of each feature streams
    // 16-bit column indices (6 bytes per nonzero instead of 8 at BF16)
    if (!seq && !h->blocked && !h->tiles && N > 0 && n <= 65536 && !std::getenv("CDMF_NO_IDX16")) {
        if ((r = dalloc(h, &h->csr_idx16, N))) return bail(r);
        narrow_idx_kernel<<<1216, kBlock, 0, h->s>>>(h->csr_idx, h->csr_idx16, N);
        if (cudaGetLastError() != cudaSuccess) return bail(CDMF_ERR_CUDA);
        h->idx16 = true;
    }
    // large matrices (the pipelined CSC sweep) with at most kCSeg * 65,536
    // rows: the first CSC sweep of each feature streams 16-bit row offsets.
    // Measured on the 480,189 x 17,770 workload: FP32 CSC sweep 251 -> 231 us;
    // BF16 199.4 -> 198.9 us (its sweep is bound by the gathers, not the
    // streams), so FP32 only
    if (h->rt == 0 && !seq && !h->blocked && !h->tiles && N >= kLargeNnz && m <= (int64_t)kCSeg << 16 &&
        !std::getenv("CDMF_NO_IDX16")) {
        if ((r = dalloc(h, &h->csc_idx16, N)) || (r = dalloc(h, &h->csc_seg, (size_t)n * kCSeg))) return bail(r);
        narrow_idx_kernel<<<1216, kBlock, 0, h->s>>>(h->csc_idx, h->csc_idx16, N);
        csc_segments_kernel<<<(unsigned)std::min<int64_t>(4096, (n * kCSeg + kBlock - 1) / kBlock), kBlock, 0, h->s>>>(
            h->csc_ptr, h->csc_idx, n, h->csc_seg);
        if (cudaGetLastError() != cudaSuccess) return bail(CDMF_ERR_CUDA);
        h->cidx16 = true;
    }
    // fresh state: W := 0 until set, H := 0, residual := ratings
    if (cudaMemsetAsync(h->W, 0, sizeof(float) * k * m, h->s) != cudaSuccess ||
        cudaMemsetAsync(h->H, 0, sizeof(float) * k * n, h->s) != cudaSuccess)
        return bail(CDMF_ERR_CUDA);
    if ((r = reset_residual(h, h->res_csr, h->csr_val)) || (r = reset_residual(h, h->res_csc, h->csc_val)))
        return bail(r);
    if (cudaStreamSynchronize(h->s) != cudaSuccess) return bail(CDMF_ERR_CUDA);
    phase("state");
    if (o->autotune && (r = cdmf_cuda_autotune(h, nullptr, nullptr))) return bail(r);
    const double T = std::max(1, o->maxinneriter);
    const double br = (double)h->rbytes;
    const double bi = h->blocked ? 2.0 : 4.0;   // index bytes as stored
    // the first CSR (CSC) sweep of a feature reads 16-bit indices when idx16
    // (cidx16) is on
    const double bi_csr1 = h->idx16 ? 2.0 : bi;
    const double bi_csc1 = h->cidx16 ? 2.0 : bi;
    h->st.bytes_per_update = N * (bi_csc1 + br) + (T - 1) * N * (bi + br) + N * (bi_csr1 + br) +
                             (T - 1) * N * (bi + br) + 2.0 * N * br + T * 4.0 * (m + n + 2) + 8.0 * (m + n);
    *out = h;
    return CDMF_OK;
}

int cdmf_cuda_set_factors(cdmf_handle* h, const float* W0, const float* H0) {
    if (!h) return CDMF_ERR_INVALID;
    CU(h, cudaSetDevice(h->o.device));
    const size_t wb = sizeof(float) * h->o.k * h->m, hb = sizeof(float) * h->o.k * h->n;
    int r;
    if (h->relabeled && W0) {
        if ((r = factors_in(h, W0, h->W, h->m, h->d_row_old))) return r;
    } else if (W0) {
        CU(h, cudaMemcpyAsync(h->W, W0, wb, cudaMemcpyHostToDevice, h->s));
    } else {
        CU(h, cudaMemsetAsync(h->W, 0, wb, h->s));
    }
    if (h->relabeled && H0) {
        if ((r = factors_in(h, H0, h->H, h->n, h->d_col_old))) return r;
    } else if (H0) {
        CU(h, cudaMemcpyAsync(h->H, H0, hb, cudaMemcpyHostToDevice, h->s));
    } else {
        CU(h, cudaMemsetAsync(h->H, 0, hb, h->s));
    }
    if ((r = reset_residual(h, h->res_csr, h->csr_val)) || (r = reset_residual(h, h->res_csc, h->csc_val))) return r;
    h->pending = -1;
    h->p_for = -1;
    h->next_oiter = 1;
    CU(h, cudaStreamSynchronize(h->s));
    return CDMF_OK;
}

int cdmf_cuda_run(cdmf_handle* h, int n_outer, double* rmse_out) {
    if (!h || n_outer < 0) return CDMF_ERR_INVALID;
    if (rmse_out && h->o.rmse_each_outer && h->nt == 0) return fail(h, CDMF_ERR_EMPTY_TEST, "empty test set");
    CU(h, cudaSetDevice(h->o.device));
    h->st.train_ms = 0;
    h->st.sweep_csc_ms = h->st.sweep_csr_ms = h->st.rmse_ms = h->st.refresh_ms = 0;
    h->st.launches = h->st.sweep_csc_launches = h->st.sweep_csr_launches = 0;
    h->st.rmse_launches = h->st.refresh_launches = 0;
    h->st.updates = 0;
    h->st.drift_rms = 0;
    h->st.nonfinite = 0;
    h->refreshed = false;
    if (h->rt != 0) CU(h, cudaMemsetAsync(h->nonfinite, 0, 8, h->s));
    h->marks.clear();
    h->pool_used = 0;
    std::vector<double> rm(std::max(1, n_outer), 0.0);
    // rmse values land in a device ring of maxiter+1 slots, copied back per chunk
    const int slots = 1 + std::max(0, h->o.maxiter);
    CU(h, cudaEventRecord(h->ev_start, h->s));
    int done = 0;
    while (done < n_outer) {
        const int chunk = std::min(n_outer - done, slots);
        for (int q = 0; q < chunk; ++q) {
            const int oiter = h->next_oiter;
            const int r = (h->o.use_graph && !h->profiling) ? do_outer_graph(h, oiter, h->rmse_out + q)
                                                            : do_outer(h, oiter, h->rmse_out + q);
            if (r) return r;
            h->st.updates += h->o.k;
            h->next_oiter++;
        }
        if (rmse_out && h->o.rmse_each_outer && h->nt > 0) {
            CU(h, cudaMemcpyAsync(rm.data() + done, h->rmse_out, sizeof(double) * chunk, cudaMemcpyDeviceToHost, h->s));
            CU(h, cudaStreamSynchronize(h->s));
        }
        done += chunk;
    }
    CU(h, cudaEventRecord(h->ev_stop, h->s));
    CU(h, cudaEventSynchronize(h->ev_stop));
    float ms = 0;
    CU(h, cudaEventElapsedTime(&ms, h->ev_start, h->ev_stop));
    h->st.train_ms = ms;
    for (const auto& mk : h->marks) {
        float t = 0;
        if (cudaEventElapsedTime(&t, mk.a, mk.b) != cudaSuccess) continue;
        if (mk.kind == K_CSC) h->st.sweep_csc_ms += t;
        else if (mk.kind == K_CSR) h->st.sweep_csr_ms += t;
        else if (mk.kind == K_RMSE) h->st.rmse_ms += t;
        else h->st.refresh_ms += t;
    }
    if (rmse_out) for (int q = 0; q < n_outer; ++q) rmse_out[q] = rm[q];
    if (h->rt != 0 && h->refreshed) {
        double drift = 0;
        unsigned long long bad = 0;
        CU(h, cudaMemcpy(&drift, h->drift_out, 8, cudaMemcpyDeviceToHost));
        CU(h, cudaMemcpy(&bad, h->nonfinite, 8, cudaMemcpyDeviceToHost));
        h->st.drift_rms = h->nnz ? std::sqrt(drift / (double)h->nnz) : 0.0;
        h->st.nonfinite = (int64_t)bad;
        if (bad) return fail(h, CDMF_ERR_NUMERIC, "non-finite residual values at the refresh");
    }
    return CDMF_OK;
}

int cdmf_cuda_get_factors(cdmf_handle* h, float* W, float* H) {
    if (!h) return CDMF_ERR_INVALID;
    CU(h, cudaSetDevice(h->o.device));
    int r;
    if (h->relabeled && W) {
        if ((r = factors_out(h, h->W, W, h->m, h->d_row_old))) return r;
    } else if (W) {
        CU(h, cudaMemcpyAsync(W, h->W, sizeof(float) * h->o.k * h->m, cudaMemcpyDeviceToHost, h->s));
    }
    if (h->relabeled && H) {
        if ((r = factors_out(h, h->H, H, h->n, h->d_col_old))) return r;
    } else if (H) {
        CU(h, cudaMemcpyAsync(H, h->H, sizeof(float) * h->o.k * h->n, cudaMemcpyDeviceToHost, h->s));
    }
    CU(h, cudaStreamSynchronize(h->s));
    return CDMF_OK;
}

int cdmf_cuda_rmse(cdmf_handle* h, double* rmse) {
    if (!h || !rmse) return CDMF_ERR_INVALID;
    if (h->nt == 0) return fail(h, CDMF_ERR_EMPTY_TEST, "empty test set");
    CU(h, cudaSetDevice(h->o.device));
    int r = launch_rmse(h, h->rmse_out);
    if (r) return r;
    CU(h, cudaMemcpyAsync(rmse, h->rmse_out, sizeof(double), cudaMemcpyDeviceToHost, h->s));
    CU(h, cudaStreamSynchronize(h->s));
    return CDMF_OK;
}

int cdmf_cuda_objective(cdmf_handle* h, double* sq_residual, double* regularizer, double* objective) {
    if (!h) return CDMF_ERR_INVALID;
    CU(h, cudaSetDevice(h->o.device));
    int r = flush_pending(h);
    if (r) return r;
    constexpr int kObjGrid = 4 * 152;
    if (!h->obj_part) {
        if ((r = dalloc(h, &h->obj_part, 3 * kObjGrid)) || (r = dalloc(h, &h->obj_out, 3)) ||
            (r = dalloc(h, &h->obj_count, 1)))
            return r;
        CU(h, cudaMemsetAsync(h->obj_count, 0, sizeof(uint32_t), h->s));
    }
    const int64_t work = std::max<int64_t>(h->nnz, std::max(h->m, h->n));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(kObjGrid, (work + kBlock - 1) / kBlock));
    switch (h->rt) {
        case 0:
            objective_kernel<0><<<grid, kBlock, 0, h->s>>>(h->res_csr, h->nnz, h->csr_ptr, h->m, h->csc_ptr, h->n, h->W,
                                                           h->H, h->o.k, h->obj_part, h->obj_count, h->obj_out);
            break;
        case 1:
            objective_kernel<1><<<grid, kBlock, 0, h->s>>>(h->res_csr, h->nnz, h->csr_ptr, h->m, h->csc_ptr, h->n, h->W,
                                                           h->H, h->o.k, h->obj_part, h->obj_count, h->obj_out);
            break;
        default:
            objective_kernel<2><<<grid, kBlock, 0, h->s>>>(h->res_csr, h->nnz, h->csr_ptr, h->m, h->csc_ptr, h->n, h->W,
                                                           h->H, h->o.k, h->obj_part, h->obj_count, h->obj_out);
            break;
    }
    CU(h, cudaGetLastError());
    h->st.launches++;
    double o[3];
    CU(h, cudaMemcpyAsync(o, h->obj_out, sizeof(o), cudaMemcpyDeviceToHost, h->s));
    CU(h, cudaStreamSynchronize(h->s));
    const double reg = (double)h->o.lambda * (o[1] + o[2]);
    if (sq_residual) *sq_residual = o[0];
    if (regularizer) *regularizer = reg;
    if (objective) *objective = o[0] + reg;
    return CDMF_OK;
}

int cdmf_cuda_get_state(cdmf_handle* h, float* W, float* H, float* res_csc, float* res_csr, int* next_oiter) {
    if (!h) return CDMF_ERR_INVALID;
    CU(h, cudaSetDevice(h->o.device));
    int r = flush_pending(h);
    if (r) return r;
    if ((r = cdmf_cuda_get_factors(h, W, H))) return r;
    auto down = [&](float* dst, void* src) -> int {
        if (!dst || h->nnz == 0) return CDMF_OK;
        if (h->rt == 0) {
            CU(h, cudaMemcpyAsync(dst, src, sizeof(float) * h->nnz, cudaMemcpyDeviceToHost, h->s));
        } else {
            float* tmp = nullptr;
            CU(h, cudaMallocAsync((void**)&tmp, sizeof(float) * h->nnz, h->s));
            res_to_f32_kernel<<<1216, 256, 0, h->s>>>(src, tmp, h->nnz, h->rt);
            CU(h, cudaGetLastError());
            CU(h, cudaMemcpyAsync(dst, tmp, sizeof(float) * h->nnz, cudaMemcpyDeviceToHost, h->s));
            CU(h, cudaFreeAsync(tmp, h->s));
        }
        return CDMF_OK;
    };
    if ((r = need_csc_pos(h))) return r;
    std::vector<float> tc, tr, bc, bq;
    float* dc = res_csc;
    float* dr = res_csr;
    if (h->relabeled && res_csc) { tc.resize(h->nnz); dc = tc.data(); }
    if (h->relabeled && res_csr) { tr.resize(h->nnz); dr = tr.data(); }
    float* gc = dc;
    float* gr = dr;
    if (h->blocked && dc) { bc.resize(h->nnz); gc = bc.data(); }
    if (h->blocked && dr) { bq.resize(h->nnz); gr = bq.data(); }
    if ((r = down(gc, h->res_csc)) || (r = down(gr, h->res_csr))) return r;
    CU(h, cudaStreamSynchronize(h->s));
    if (h->blocked) {   // blocked positions -> line-layout positions
        if (dc) for (int64_t o = 0; o < h->nnz; ++o) dc[o] = gc[h->hmap_c[o]];
        if (dr) for (int64_t o = 0; o < h->nnz; ++o) dr[o] = gr[h->hmap_r[o]];
    }
    if (h->relabeled) {
        if (res_csc) for (int64_t o = 0; o < h->nnz; ++o) res_csc[h->csc_pos[o]] = dc[o];
        if (res_csr) for (int64_t o = 0; o < h->nnz; ++o) res_csr[h->csr_pos[o]] = dr[o];
    }
    if (next_oiter) *next_oiter = h->next_oiter;
    return CDMF_OK;
}

int cdmf_cuda_set_state(cdmf_handle* h, const float* W, const float* H, const float* res_csc, const float* res_csr,
                        int next_oiter) {
    if (!h || !W || !H || next_oiter < 1) return CDMF_ERR_INVALID;
    if (h->nnz > 0 && (!res_csc || !res_csr)) return CDMF_ERR_INVALID;
    CU(h, cudaSetDevice(h->o.device));
    int r0 = need_csc_pos(h);
    if (r0) return r0;
    std::vector<float> tw, th, tc, tr;
    if (h->relabeled) {
        tw.resize((size_t)h->o.k * h->m);
        th.resize((size_t)h->o.k * h->n);
        gather_ids(W, tw.data(), h->o.k, h->m, h->row_old);
        gather_ids(H, th.data(), h->o.k, h->n, h->col_old);
        W = tw.data();
        H = th.data();
        tc.resize(h->nnz);
        tr.resize(h->nnz);
        for (int64_t o = 0; o < h->nnz; ++o) {
            tc[o] = res_csc[h->csc_pos[o]];
            tr[o] = res_csr[h->csr_pos[o]];
        }
        res_csc = tc.data();
        res_csr = tr.data();
    }
    std::vector<float> bc, bq;
    if (h->blocked && h->nnz > 0) {   // line-layout positions -> blocked positions
        bc.resize(h->nnz);
        bq.resize(h->nnz);
        for (int64_t o = 0; o < h->nnz; ++o) {
            bc[h->hmap_c[o]] = res_csc[o];
            bq[h->hmap_r[o]] = res_csr[o];
        }
        res_csc = bc.data();
        res_csr = bq.data();
    }
    CU(h, cudaMemcpyAsync(h->W, W, sizeof(float) * h->o.k * h->m, cudaMemcpyHostToDevice, h->s));
    CU(h, cudaMemcpyAsync(h->H, H, sizeof(float) * h->o.k * h->n, cudaMemcpyHostToDevice, h->s));
    auto upres = [&](void* dst, const float* src) -> int {
        if (h->nnz == 0) return CDMF_OK;
        if (h->rt == 0) {
            CU(h, cudaMemcpyAsync(dst, src, sizeof(float) * h->nnz, cudaMemcpyHostToDevice, h->s));
        } else {
            float* tmp = nullptr;
            CU(h, cudaMallocAsync((void**)&tmp, sizeof(float) * h->nnz, h->s));
            CU(h, cudaMemcpyAsync(tmp, src, sizeof(float) * h->nnz, cudaMemcpyHostToDevice, h->s));
            f32_to_res_kernel<<<1216, 256, 0, h->s>>>(tmp, dst, h->nnz, h->rt);
            CU(h, cudaGetLastError());
            CU(h, cudaFreeAsync(tmp, h->s));
        }
        return CDMF_OK;
    };
    int r;
    if ((r = upres(h->res_csc, res_csc)) || (r = upres(h->res_csr, res_csr))) return r;
    CU(h, cudaStreamSynchronize(h->s));
    h->pending = -1;
    h->p_for = -1;
    h->next_oiter = next_oiter;
    return CDMF_OK;
}

int cdmf_cuda_set_profiling(cdmf_handle* h, int on) {
    if (!h) return CDMF_ERR_INVALID;
    h->profiling = on != 0;
    return CDMF_OK;
}

int cdmf_cuda_stats(const cdmf_handle* h, cdmf_stats* s) {
    if (!h || !s) return CDMF_ERR_INVALID;
    *s = h->st;
    return CDMF_OK;
}

int cdmf_cuda_bins(const cdmf_handle* h, int which, int64_t counts[5], int64_t nnz[5]) {
    if (!h || (which != 0 && which != 1)) return CDMF_ERR_INVALID;
    const Bins& B = which == 0 ? h->csr.host : h->csc.host;
    for (int q = 0; q < 5; ++q) {
        if (counts) counts[q] = B.count[q];
        if (nnz) nnz[q] = B.nnz[q];
    }
    return CDMF_OK;
}

int cdmf_cuda_get_bincfg(const cdmf_handle* h, cdmf_bincfg* c) {
    if (!h || !c) return CDMF_ERR_INVALID;
    c->thread_max = h->cfg.thread_max;
    c->group_max = h->cfg.group_max;
    c->warp_max = h->cfg.warp_max;
    c->cta_max = h->cfg.cta_max;
    c->chunk = h->cfg.chunk;
    return CDMF_OK;
}

int cdmf_cuda_set_bincfg(cdmf_handle* h, const cdmf_bincfg* c) {
    if (!h || !c) return CDMF_ERR_INVALID;
    if (c->chunk < 256 || c->chunk % 4 || c->thread_max > c->warp_max || c->warp_max > c->cta_max ||
        c->cta_max < c->chunk || (c->group_max && (c->group_max < c->thread_max || c->group_max > c->warp_max)))
        return fail(h, CDMF_ERR_INVALID, "inconsistent bin thresholds");
    CU(h, cudaSetDevice(h->o.device));
    BinCfg cfg;
    cfg.thread_max = c->thread_max;
    cfg.group_max = c->group_max ? c->group_max : c->thread_max;
    cfg.warp_max = c->warp_max;
    cfg.cta_max = c->cta_max;
    cfg.chunk = c->chunk;
    return replan(h, cfg);
}

int cdmf_cuda_autotune(cdmf_handle* h, cdmf_bincfg* chosen, double* best_ms) {
    if (!h) return CDMF_ERR_INVALID;
    CU(h, cudaSetDevice(h->o.device));
    // nothing to pick where the sweeps do not run on the length bins: one
    // thread per line (reference order), the tile kernel, the blocked layout
    if (h->seq || h->tiles || h->blocked || h->nnz == 0 || h->o.maxinneriter <= 0) {
        if (chosen) cdmf_cuda_get_bincfg(h, chosen);
        if (best_ms) *best_ms = 0;
        return CDMF_OK;
    }
    const TuneKey key = tune_key(h);
    int r;
    BinCfg best = h->cfg, best_c = h->cfg_c;
    uint32_t best_lanes = h->group_lanes;
    double best_t = 0;
    TunePick pick;
    const bool cached = cached_pick(key, &pick);
    if (cached) {
        best = pick.cfg;
        best_c = pick.cfg_c;
        best_lanes = pick.lanes;
    } else {
        const bool prof = h->profiling;
        h->profiling = false;
        // coordinate search over group_max, warp_max, cta_max and the split
        // chunk, from the defaults (0 = no lane-group bin): first one plan
        // for both copies, then the CSC copy's plan alone; last the lanes per
        // group-bin line.  On the 480,189 x 17,770 workload (BF16, k = 64) it
        // moves the lines of 257-1,024 nonzeros from warps to lane groups:
        // 29.34 -> 28.72 ms per outer iteration.
        if ((r = time_feature(h, 3, &best_t))) return r;
        // (group lines sum without compensation, so the group limit stays at
        // or below kKahanMin)
        const uint32_t gvals[] = {0, 64, 128, 256, 512, 1024, 2048, 4096};
        const uint32_t wvals[] = {1024, 2048, 4096, 16384};
        const uint32_t cvals[] = {8192, 16384, 65536};
        const uint32_t kvals[] = {8192, 16384, 32768};
        static_assert(4096 <= kKahanMin, "group lines must not need compensated sums");
        for (int pass = 0; pass < 2; ++pass) {   // 0: both copies, 1: the CSC copy alone
            if (pass == 1) best_c = best;
            for (int dim = 0; dim < 4; ++dim) {
                const uint32_t* vals = dim == 0 ? gvals : dim == 1 ? wvals : dim == 2 ? cvals : kvals;
                const int nv = dim == 0 ? 8 : dim == 1 ? 4 : 3;
                const BinCfg base = pass == 0 ? best : best_c;
                for (int v = 0; v < nv; ++v) {
                    BinCfg c = base;
                    if (dim == 0) c.group_max = vals[v] ? vals[v] : c.thread_max;
                    if (dim == 1) c.warp_max = vals[v];
                    if (dim == 2) c.cta_max = vals[v];
                    if (dim == 3) c.chunk = vals[v];
                    if (c.group_max > c.warp_max || c.warp_max > c.cta_max || c.chunk > c.cta_max) continue;
                    const BinCfg& cur = pass == 0 ? best : best_c;
                    if (c.group_max == cur.group_max && c.warp_max == cur.warp_max && c.cta_max == cur.cta_max &&
                        c.chunk == cur.chunk)
                        continue;
                    if ((r = pass == 0 ? replan(h, c) : replan(h, best, c))) return r;
                    double t = 0;
                    if ((r = time_feature(h, 3, &t))) return r;
                    if (t < best_t) {
                        best_t = t;
                        (pass == 0 ? best : best_c) = c;
                    }
                }
            }
        }
        {   // the other lane count for the group bin
            const uint32_t lanes = best_lanes == 4 ? 8 : 4;
            h->group_lanes = lanes;
            if ((r = replan(h, best, best_c))) return r;
            double t = 0;
            if ((r = time_feature(h, 3, &t))) return r;
            if (t < best_t) { best_t = t; best_lanes = lanes; }
        }
        h->profiling = prof;
        std::lock_guard<std::mutex> lk(tune_mutex());
        tune_cache()[key] = TunePick{best, best_c, best_lanes};
    }
    // (a handle created with the cached pick already has these bins)
    if (!(cached && best_lanes == h->group_lanes && same_cfg(best, h->cfg) && same_cfg(best_c, h->cfg_c))) {
        h->group_lanes = best_lanes;
        if ((r = replan(h, best, best_c))) return r;
    }
    // the timing sweeps used the factors and residual as scratch
    if ((r = cdmf_cuda_set_factors(h, nullptr, nullptr))) return r;
    CU(h, cudaMemsetAsync(h->P, 0, sizeof(float2) * std::max<int64_t>(1, h->m), h->s));
    CU(h, cudaMemsetAsync(h->Q, 0, sizeof(float4) * std::max<int64_t>(1, h->n), h->s));
    CU(h, cudaStreamSynchronize(h->s));
    if (chosen) cdmf_cuda_get_bincfg(h, chosen);
    if (best_ms) *best_ms = best_t;
    return CDMF_OK;
}

int cdmf_cuda_rmse_coo(uint32_t k, int64_t m, int64_t n, const float* W, const float* H, int64_t nnz_test,
                       const uint32_t* test_row, const uint32_t* test_col, const double* test_val, int device,
                       double* rmse, int64_t* nan_count) {
    if (k == 0 || m < 0 || n < 0 || nnz_test < 0 || !W || !H || !rmse) return CDMF_ERR_INVALID;
    if (nnz_test == 0) return CDMF_ERR_EMPTY_TEST;
    if (!test_row || !test_col || !test_val) return CDMF_ERR_INVALID;
    for (int64_t e = 0; e < nnz_test; ++e)
        if ((int64_t)test_row[e] >= m || (int64_t)test_col[e] >= n) return CDMF_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return CDMF_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return CDMF_ERR_NO_DEVICE;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(4 * 152, (nnz_test + kBlock - 1) / kBlock));
    const size_t wb = sizeof(float) * k * m, hb = sizeof(float) * k * n;
    char* buf = nullptr;
    // one block: W | H | rows | cols | vals | partials | out | nan count | counter
    size_t off[9], tot = 0;
    const size_t sz[9] = {wb, hb, 4 * (size_t)nnz_test, 4 * (size_t)nnz_test, 8 * (size_t)nnz_test,
                          8 * (size_t)grid, 8, 8, 4};
    for (int q = 0; q < 9; ++q) { off[q] = tot; tot += (sz[q] + 255) / 256 * 256; }
    if (cudaMalloc((void**)&buf, tot) != cudaSuccess) return CDMF_ERR_ALLOC;
    int st = CDMF_OK;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { cudaFree(buf); return CDMF_ERR_CUDA; }
    unsigned long long nans = 0;
    bool ok = cudaMemcpyAsync(buf + off[0], W, wb, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(buf + off[1], H, hb, cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(buf + off[2], test_row, sz[2], cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(buf + off[3], test_col, sz[3], cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemcpyAsync(buf + off[4], test_val, sz[4], cudaMemcpyHostToDevice, s) == cudaSuccess &&
              cudaMemsetAsync(buf + off[7], 0, 8, s) == cudaSuccess && cudaMemsetAsync(buf + off[8], 0, 4, s) == cudaSuccess;
    if (ok) {
        rmse_kernel<double><<<grid, kBlock, 0, s>>>((const uint32_t*)(buf + off[2]), (const uint32_t*)(buf + off[3]),
                                                    (const double*)(buf + off[4]), nnz_test, (const float*)(buf + off[0]),
                                                    (const float*)(buf + off[1]), m, n, k, (double*)(buf + off[5]),
                                                    (uint32_t*)(buf + off[8]), (double*)(buf + off[6]),
                                                    (unsigned long long*)(buf + off[7]));
        ok = cudaGetLastError() == cudaSuccess &&
             cudaMemcpyAsync(rmse, buf + off[6], 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
             cudaMemcpyAsync(&nans, buf + off[7], 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
             cudaStreamSynchronize(s) == cudaSuccess;
    }
    if (!ok) st = CDMF_ERR_CUDA;
    if (nan_count) *nan_count = (int64_t)nans;
    cudaStreamDestroy(s);
    cudaFree(buf);
    return st;
}

int cdmf_cuda_train(const cdmf_problem* p, const cdmf_opts* o, float* W, float* H, double* rmse_out, cdmf_outer_cb cb,
                    void* user) {
    if (!p || !o || !W || !H) return CDMF_ERR_INVALID;
    // o->verbose: phase times on stderr
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* what) {
        if (!o->verbose) return;
        const auto t = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[cdmf] train: %-12s %8.1f ms\n", what,
                     std::chrono::duration<double, std::milli>(t - t_last).count());
        t_last = t;
    };
    cdmf_handle* h = nullptr;
    int r = cdmf_cuda_create(p, o, &h);
    if (r) return r;
    phase("create");
    if ((r = cdmf_cuda_set_factors(h, W, nullptr))) { cdmf_cuda_destroy(h); return r; }
    phase("set_factors");
    if ((r = run_queued(h, rmse_out, cb, user))) { cdmf_cuda_destroy(h); return r; }
    phase("outer loop");
    r = cdmf_cuda_get_factors(h, W, H);
    phase("get_factors");
    cdmf_cuda_destroy(h);
    phase("destroy");
    return r;
}

}  // extern "C"

// ============================================================================
// Batches of independent factorisations (uneven sizes, own k and lambda).
//
// Every problem keeps its own engine handle and its own CUDA stream, and runs
// exactly its single-problem schedule (refreshes, sweeps, test RMSE) on that
// stream.  A batched run forks all the streams from the batch stream, issues
// the problems' outer iterations interleaved (outer iteration by outer
// iteration, problem by problem), and joins them back; with use_graph the
// whole run is captured once as one CUDA graph of independent branches and
// replayed after.  The GPU's scheduler then overlaps the problems' kernels:
// while one problem's launch drains, the next launches of the other problems
// fill the SMs, and each problem's data stays in L2 between its own launches.
// Results are bit-identical to running each problem alone.  (Measured on the
// 64-problem workload, FP16, 10 x 1: 108 ms against 159 ms for all problems
// in lockstep, one grouped launch per half step, and 223 ms for one persistent
// launch per outer iteration with per-problem dependencies; 370 ms one after
// another.)
// ============================================================================

struct cdmf_batch {
    std::vector<cdmf_handle*> hs;
    cudaStream_t s = nullptr;        // the batch stream: fork, join, timing
    int device = 0, use_graph = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr, fork = nullptr;
    std::vector<cudaEvent_t> joins;  // one per problem stream
    cudaGraphExec_t gexec = nullptr;
    int g_outer = -1;
    std::vector<int> g_start;        // per problem: next_oiter, pending, p_for at capture
    std::vector<int> g_end;
    cdmf_stats g_single{};           // the problems' launches recorded while capturing
    cdmf_stats st{};
    std::string err;
};

namespace {

int bfail(cdmf_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

#define BCU(b, call)                                                                            \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return bfail(b, CDMF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Issues n_outer outer iterations of every problem, each on its own stream
// after the fork event of the batch stream, then joins the streams back into
// the batch stream.
int issue_streams(cdmf_batch* B, int n_outer) {
    const int P = (int)B->hs.size();
    BCU(B, cudaEventRecord(B->fork, B->s));
    for (cdmf_handle* h : B->hs) BCU(B, cudaStreamWaitEvent(h->s, B->fork, 0));
    for (int o = 0; o < n_outer; ++o)
        for (int q = 0; q < P; ++q) {
            cdmf_handle* h = B->hs[q];
            const int r = do_outer(h, h->next_oiter + o, h->rmse_out + o);
            if (r) return bfail(B, r, h->err);
        }
    for (int q = 0; q < P; ++q) {
        BCU(B, cudaEventRecord(B->joins[q], B->hs[q]->s));
        BCU(B, cudaStreamWaitEvent(B->s, B->joins[q], 0));
    }
    return CDMF_OK;
}

void add_launches(cdmf_stats& to, const cdmf_stats& from) {
    to.launches += from.launches;
    to.sweep_csc_launches += from.sweep_csc_launches;
    to.sweep_csr_launches += from.sweep_csr_launches;
    to.rmse_launches += from.rmse_launches;
    to.refresh_launches += from.refresh_launches;
}

}  // namespace

extern "C" {

void cdmf_cuda_batch_destroy(cdmf_batch* B) {
    if (!B) return;
    cudaSetDevice(B->device);
    if (B->s) cudaStreamSynchronize(B->s);
    for (cdmf_handle* h : B->hs)
        if (h) cdmf_cuda_destroy(h);
    if (B->gexec) cudaGraphExecDestroy(B->gexec);
    for (cudaEvent_t e : {B->e0, B->e1, B->fork})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : B->joins)
        if (e) cudaEventDestroy(e);
    if (B->s) cudaStreamDestroy(B->s);
    delete B;
}

const char* cdmf_cuda_batch_last_error(const cdmf_batch* B) { return B ? B->err.c_str() : ""; }

int cdmf_cuda_batch_create(const cdmf_problem* probs, const cdmf_opts* opts, int nprob, cdmf_batch** out) {
    if (!out) return CDMF_ERR_INVALID;
    *out = nullptr;
    if (!probs || !opts || nprob <= 0) return CDMF_ERR_INVALID;
    for (int q = 1; q < nprob; ++q)
        if (opts[q].residual != opts[0].residual || opts[q].maxinneriter != opts[0].maxinneriter ||
            opts[q].device != opts[0].device || opts[q].reduce != opts[0].reduce)
            return CDMF_ERR_UNSUPPORTED;
    cdmf_batch* B = new cdmf_batch();
    B->device = opts[0].device;
    B->use_graph = opts[0].use_graph;
    auto bail = [&](int code) { cdmf_cuda_batch_destroy(B); return code; };
    if (cudaSetDevice(B->device) != cudaSuccess) return bail(CDMF_ERR_NO_DEVICE);
    if (cudaStreamCreateWithFlags(&B->s, cudaStreamNonBlocking) != cudaSuccess) return bail(CDMF_ERR_CUDA);
    if (cudaEventCreate(&B->e0) != cudaSuccess || cudaEventCreate(&B->e1) != cudaSuccess ||
        cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming) != cudaSuccess)
        return bail(CDMF_ERR_CUDA);
    B->joins.assign(nprob, nullptr);
    for (int q = 0; q < nprob; ++q)
        if (cudaEventCreateWithFlags(&B->joins[q], cudaEventDisableTiming) != cudaSuccess) return bail(CDMF_ERR_CUDA);
    for (int q = 0; q < nprob; ++q) {
        cdmf_opts o = opts[q];
        o.use_graph = 0;   // the batch captures the problems' launches itself
        cdmf_handle* h = nullptr;
        const int r = cdmf_cuda_create(probs + q, &o, &h);
        if (r) return bail(r);
        B->hs.push_back(h);
    }
    *out = B;
    return CDMF_OK;
}

int cdmf_cuda_batch_set_factors(cdmf_batch* B, const float* const* W0) {
    if (!B) return CDMF_ERR_INVALID;
    for (size_t q = 0; q < B->hs.size(); ++q) {
        const int r = cdmf_cuda_set_factors(B->hs[q], W0 ? W0[q] : nullptr, nullptr);
        if (r) return bfail(B, r, B->hs[q]->err);
    }
    return CDMF_OK;
}

int cdmf_cuda_batch_run(cdmf_batch* B, int n_outer, double* rmse_out) {
    if (!B || n_outer < 0) return CDMF_ERR_INVALID;
    const int P = (int)B->hs.size();
    for (cdmf_handle* h : B->hs)
        if (n_outer > h->o.maxiter + 1) return bfail(B, CDMF_ERR_INVALID, "n_outer beyond the RMSE slots");
    BCU(B, cudaSetDevice(B->device));
    B->st = cdmf_stats{};
    std::vector<int> start(3 * P);
    for (int q = 0; q < P; ++q) {
        cdmf_handle* h = B->hs[q];
        h->st = cdmf_stats{};
        h->refreshed = false;
        if (h->rt != 0) BCU(B, cudaMemsetAsync(h->nonfinite, 0, 8, h->s));
        start[3 * q] = h->next_oiter;
        start[3 * q + 1] = h->pending;
        start[3 * q + 2] = h->p_for;
    }
    int r;
    BCU(B, cudaEventRecord(B->e0, B->s));
    if (B->use_graph && B->gexec && B->g_outer == n_outer && B->g_start == start) {
        BCU(B, cudaGraphLaunch(B->gexec, B->s));
        for (int q = 0; q < P; ++q) {
            B->hs[q]->pending = B->g_end[3 * q + 1];
            B->hs[q]->p_for = B->g_end[3 * q + 2];
        }
        add_launches(B->st, B->g_single);
    } else if (B->use_graph) {
        if (B->gexec) {
            cudaGraphExecDestroy(B->gexec);
            B->gexec = nullptr;
        }
        BCU(B, cudaStreamBeginCapture(B->s, cudaStreamCaptureModeThreadLocal));
        r = issue_streams(B, n_outer);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(B->s, &g);
        if (r || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return r ? r : bfail(B, CDMF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        }
        const cudaError_t ei = cudaGraphInstantiate(&B->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) return bfail(B, CDMF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
        B->g_outer = n_outer;
        B->g_start = start;
        B->g_single = cdmf_stats{};
        for (cdmf_handle* h : B->hs) add_launches(B->g_single, h->st);
        B->g_end.assign(3 * P, 0);
        for (int q = 0; q < P; ++q) {
            B->g_end[3 * q] = B->hs[q]->next_oiter + n_outer;
            B->g_end[3 * q + 1] = B->hs[q]->pending;
            B->g_end[3 * q + 2] = B->hs[q]->p_for;
        }
        add_launches(B->st, B->g_single);
        BCU(B, cudaGraphLaunch(B->gexec, B->s));
    } else {
        if ((r = issue_streams(B, n_outer))) return r;
        for (cdmf_handle* h : B->hs) add_launches(B->st, h->st);
    }
    for (cdmf_handle* h : B->hs) h->next_oiter += n_outer;
    BCU(B, cudaEventRecord(B->e1, B->s));
    BCU(B, cudaEventSynchronize(B->e1));
    float ms = 0;
    BCU(B, cudaEventElapsedTime(&ms, B->e0, B->e1));
    B->st.train_ms = ms;
    for (cdmf_handle* h : B->hs) B->st.updates += (int64_t)h->o.k * n_outer;
    for (int q = 0; q < P; ++q) {
        cdmf_handle* h = B->hs[q];
        if (h->rt == 0) continue;
        unsigned long long bad = 0;
        BCU(B, cudaMemcpy(&bad, h->nonfinite, 8, cudaMemcpyDeviceToHost));
        B->st.nonfinite += (int64_t)bad;
    }
    if (rmse_out)
        for (int q = 0; q < P; ++q) {
            cdmf_handle* h = B->hs[q];
            if (h->o.rmse_each_outer && h->nt > 0) {
                BCU(B, cudaMemcpy(rmse_out + (size_t)q * n_outer, h->rmse_out, sizeof(double) * n_outer,
                                  cudaMemcpyDeviceToHost));
            } else {
                for (int o = 0; o < n_outer; ++o) rmse_out[(size_t)q * n_outer + o] = -1.0;
            }
        }
    if (B->st.nonfinite) return bfail(B, CDMF_ERR_NUMERIC, "non-finite residual values at a refresh");
    return CDMF_OK;
}

int cdmf_cuda_batch_run_sequential(cdmf_batch* B, int n_outer, double* rmse_out, double* ms_out) {
    if (!B || n_outer < 0) return CDMF_ERR_INVALID;
    BCU(B, cudaSetDevice(B->device));
    BCU(B, cudaEventRecord(B->e0, B->s));
    std::vector<std::vector<double>> rm(B->hs.size());
    for (size_t q = 0; q < B->hs.size(); ++q) {
        cdmf_handle* h = B->hs[q];
        const bool want = h->o.rmse_each_outer && h->nt > 0;
        rm[q].assign(std::max(1, n_outer), -1.0);
        const int r = cdmf_cuda_run(h, n_outer, want ? rm[q].data() : nullptr);
        if (r) return bfail(B, r, h->err);
    }
    BCU(B, cudaEventRecord(B->e1, B->s));
    BCU(B, cudaEventSynchronize(B->e1));
    float ms = 0;
    BCU(B, cudaEventElapsedTime(&ms, B->e0, B->e1));
    if (ms_out) *ms_out = ms;
    if (rmse_out)
        for (size_t q = 0; q < B->hs.size(); ++q)
            for (int o = 0; o < n_outer; ++o) rmse_out[q * n_outer + o] = rm[q][o];
    return CDMF_OK;
}

int cdmf_cuda_batch_get_factors(cdmf_batch* B, float* const* W, float* const* H) {
    if (!B) return CDMF_ERR_INVALID;
    for (size_t q = 0; q < B->hs.size(); ++q) {
        const int r = cdmf_cuda_get_factors(B->hs[q], W ? W[q] : nullptr, H ? H[q] : nullptr);
        if (r) return bfail(B, r, B->hs[q]->err);
    }
    return CDMF_OK;
}

int cdmf_cuda_batch_stats(const cdmf_batch* B, cdmf_stats* s) {
    if (!B || !s) return CDMF_ERR_INVALID;
    *s = B->st;
    return CDMF_OK;
}

}  // extern "C"

// ============================================================================
// Dual SpMV front end: the anonymouslibHandle life cycle the reference's -V 3
// engine drives (src/anonymouslib_opencl.h:11-26; src/cdmf_csr5.cpp:205-286):
// create(m, n), inputCSR(nnz, ptr, idx, val), asCSR5(), setX(x), then
// spmv(alpha, y_t, y_b) computing, for every row i,
//     y_t[i] = sum_j val_ij * x[col_j]      y_b[i] = sum_j x[col_j]^2
// (csr5_spmv.cl:135-147: the per-nonzero pair; alpha is accepted and, as in
// that kernel, not applied).  The CSR5 tiles become the engine's line-length
// bins over the same CSR arrays: split chunks, CTA, warp, 8-lane group and
// thread lines, each summed in a fixed tree order (deterministic).  Arrays
// are the caller's device memory, as cl_mem buffers are in the reference.
// ============================================================================

namespace {

__global__ void check_cols_kernel(const uint32_t* __restrict__ idx, int64_t nnz, uint32_t n, uint32_t* bad) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
        if (idx[q] >= n) atomicOr(bad, 1u);
}

}  // namespace

struct cdmf_spmv {
    cdmf_handle* h = nullptr;        // stream, bins, allocations, error text
    const uint32_t* row_ptr = nullptr;
    const uint32_t* col_idx = nullptr;
    const float* val = nullptr;
    const float* x = nullptr;
    bool have_csr = false, csr5 = false;
};

extern "C" {

int cdmf_spmv_create(int64_t m, int64_t n, int device, cdmf_spmv** out) {
    if (!out) return CDMF_ERR_INVALID;
    *out = nullptr;
    if (m < 0 || n < 0) return CDMF_ERR_INVALID;
    if (m >= (int64_t)UINT32_MAX || n >= (int64_t)UINT32_MAX) return CDMF_ERR_TOO_LARGE;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CDMF_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return CDMF_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return CDMF_ERR_CUDA;
    cdmf_spmv* S = new cdmf_spmv();
    S->h = new cdmf_handle();
    cdmf_opts_default(&S->h->o);
    S->h->o.device = device;
    S->h->m = m;
    S->h->n = n;
    if (cudaStreamCreateWithFlags(&S->h->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&S->h->ev_start) != cudaSuccess || cudaEventCreate(&S->h->ev_stop) != cudaSuccess) {
        cdmf_cuda_destroy(S->h);
        delete S;
        return CDMF_ERR_CUDA;
    }
    *out = S;
    return CDMF_OK;
}

void cdmf_spmv_destroy(cdmf_spmv* S) {
    if (!S) return;
    cdmf_cuda_destroy(S->h);
    delete S;
}

const char* cdmf_spmv_last_error(const cdmf_spmv* S) { return S ? S->h->err.c_str() : ""; }

int cdmf_spmv_input_csr(cdmf_spmv* S, int64_t nnz, const uint32_t* row_ptr, const uint32_t* col_idx,
                        const float* val) {
    if (!S || nnz < 0 || !row_ptr || (nnz > 0 && (!col_idx || !val))) return CDMF_ERR_INVALID;
    if (nnz > (int64_t)UINT32_MAX - 8192) return CDMF_ERR_TOO_LARGE;
    cdmf_handle* h = S->h;
    CU(h, cudaSetDevice(h->o.device));
    if (S->csr5) free_bins(h, h->csr);
    S->csr5 = false;
    // the row pointers are read back to plan the work and checked here: a
    // malformed structure is refused before any kernel reads through it
    h->hptr_r.resize(h->m + 1);
    CU(h, cudaMemcpyAsync(h->hptr_r.data(), row_ptr, 4 * (size_t)(h->m + 1), cudaMemcpyDeviceToHost, h->s));
    CU(h, cudaStreamSynchronize(h->s));
    if (h->hptr_r[0] != 0 || (int64_t)h->hptr_r[h->m] != nnz) return fail(h, CDMF_ERR_INVALID, "row_ptr ends");
    for (int64_t i = 0; i < h->m; ++i)
        if (h->hptr_r[i + 1] < h->hptr_r[i]) return fail(h, CDMF_ERR_INVALID, "row_ptr not monotone");
    h->nnz = nnz;
    S->row_ptr = row_ptr;
    S->col_idx = col_idx;
    S->val = val;
    S->have_csr = true;
    return CDMF_OK;
}

int cdmf_spmv_as_csr5(cdmf_spmv* S) {
    if (!S) return CDMF_ERR_INVALID;
    cdmf_handle* h = S->h;
    if (!S->have_csr) return fail(h, CDMF_ERR_INVALID, "no matrix: call cdmf_spmv_input_csr first");
    if (S->csr5) return CDMF_OK;
    CU(h, cudaSetDevice(h->o.device));
    if (h->nnz > 0) {   // every column index must address x
        uint32_t* bad = nullptr;
        int r;
        if ((r = dalloc(h, &bad, 1))) return r;
        CU(h, cudaMemsetAsync(bad, 0, 4, h->s));
        check_cols_kernel<<<1216, kBlock, 0, h->s>>>(S->col_idx, h->nnz, (uint32_t)h->n, bad);
        CU(h, cudaGetLastError());
        uint32_t hb = 0;
        CU(h, cudaMemcpyAsync(&hb, bad, 4, cudaMemcpyDeviceToHost, h->s));
        CU(h, cudaStreamSynchronize(h->s));
        if (hb) return fail(h, CDMF_ERR_INVALID, "column index out of range");
    }
    h->cfg = default_bins(h->nnz);
    const int r = upload_bins(h, h->csr, plan_bins(h->hptr_r.data(), h->m, false, h->cfg));
    if (r) return r;
    S->csr5 = true;
    return CDMF_OK;
}

int cdmf_spmv_as_csr(cdmf_spmv* S) {
    if (!S) return CDMF_ERR_INVALID;
    if (S->csr5) {
        CU(S->h, cudaSetDevice(S->h->o.device));
        CU(S->h, cudaStreamSynchronize(S->h->s));
        free_bins(S->h, S->h->csr);
    }
    S->csr5 = false;
    return CDMF_OK;
}

int cdmf_spmv_set_x(cdmf_spmv* S, const float* x) {
    if (!S || (!x && S->h->n > 0)) return CDMF_ERR_INVALID;
    S->x = x;
    return CDMF_OK;
}

int cdmf_spmv_run(cdmf_spmv* S, float alpha, float* y_t, float* y_b, double* ms) {
    (void)alpha;
    if (!S) return CDMF_ERR_INVALID;
    cdmf_handle* h = S->h;
    if (!S->csr5) return fail(h, CDMF_ERR_UNSUPPORTED, "the matrix is in CSR form: call cdmf_spmv_as_csr5");
    if ((h->m > 0 && (!y_t || !y_b)) || (h->nnz > 0 && !S->x)) return CDMF_ERR_INVALID;
    CU(h, cudaSetDevice(h->o.device));
    SweepArgs A = base_args(h, h->csr, S->row_ptr, S->col_idx, (void*)S->val);
    A.y = S->x;
    A.out = y_t;
    A.out2 = y_b;
    const unsigned grid = h->csr.nx + h->csr.nc + h->csr.nwb + h->csr.ngb + h->csr.ntb;
    CU(h, cudaEventRecord(h->ev_start, h->s));
    if (grid) {
        launch_dual(A, grid, h->s);
        CU(h, cudaGetLastError());
    }
    CU(h, cudaEventRecord(h->ev_stop, h->s));
    CU(h, cudaEventSynchronize(h->ev_stop));
    float t = 0.0f;
    CU(h, cudaEventElapsedTime(&t, h->ev_start, h->ev_stop));
    if (ms) *ms = t;
    return CDMF_OK;
}

}  // extern "C"
