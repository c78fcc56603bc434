// COO -> canonical CSR and CSC on the GPU (cdmf_cuda_compress).
//
// The reference builds its binary CSR/CSC files offline with scipy
// (data/a/a_compress.py:130-155: coo_matrix(...).tocsr() / .tocsc()) and the
// engine loads them (src/tools.cpp:271-347).  This entry point produces the
// same arrays from a COO rating list on the device:
//   1. key = row * n + col (64-bit), checked against m and n;
//   2. stable radix sort of (key, input position): entries in (row, col)
//      order, equal keys in input order;
//   3. one thread per distinct key sums its duplicates in FP64 in input order
//      and stores the float value (scipy sums duplicates; the reference then
//      writes float32);
//   4. row pointers from the sorted keys;
//   5. stable radix sort of the distinct entries by column gives the CSC
//      order with rows ascending inside each column (scipy's canonical CSC)
//      and the CSR -> CSC permutation.
// The sorts are CUB's DeviceRadixSort (shipped with the CUDA toolkit); the
// other steps are the kernels below.  Inputs and outputs are host arrays; the
// device scratch is allocated per call and freed before it returns.
#include <cdmf_cuda.h>

#include "gpu_build.h"

#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

namespace {

constexpr int kThreads = 256;

unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + kThreads - 1) / kThreads, 1 << 20)); }

__global__ void make_keys(const uint32_t* __restrict__ rows, const uint32_t* __restrict__ cols, int64_t nnz, uint64_t m,
                          uint64_t n, uint64_t* __restrict__ keys, uint32_t* __restrict__ pos, uint32_t* bad) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t r = rows[e], c = cols[e];
        if (r >= m || c >= n) {
            atomicOr(bad, 1u);
            keys[e] = 0;
        } else {
            keys[e] = r * n + c;
        }
        pos[e] = (uint32_t)e;
    }
}

// head[i] = 1 where a run of equal keys starts
__global__ void run_heads(const uint64_t* __restrict__ keys, int64_t nnz, uint32_t* __restrict__ head) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
        head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// start[uid[i]] = i at every run head; start[U] = nnz
__global__ void run_starts(const uint32_t* __restrict__ head, const uint32_t* __restrict__ uid, int64_t nnz,
                           uint32_t* __restrict__ start) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        if (head[i]) start[uid[i]] = (uint32_t)i;
        if (i == nnz - 1) start[uid[i] + head[i]] = (uint32_t)nnz;
    }
}

// One distinct (row, col): duplicates summed in FP64 in input order.
__global__ void reduce_runs(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ pos,
                            const double* __restrict__ vals, const uint32_t* __restrict__ start, int64_t U, uint64_t n,
                            uint32_t* __restrict__ row, uint32_t* __restrict__ col, float* __restrict__ val) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < U; u += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t b = start[u], e = start[u + 1];
        double s = 0.0;
        for (uint32_t i = b; i < e; ++i) s = __dadd_rn(s, vals[pos[i]]);
        const uint64_t key = keys[b];
        row[u] = (uint32_t)(key / n);
        col[u] = (uint32_t)(key % n);
        val[u] = __double2float_rn(s);
    }
}

// ptr[l] = first position of line l in a line-sorted list of U entries
// (lines with no entries point at the next line's first entry).
__global__ void line_pointers(const uint32_t* __restrict__ line, int64_t U, int64_t lines, uint32_t* __restrict__ ptr) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < U; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = line[u];
        const int64_t prev = u == 0 ? -1 : (int64_t)line[u - 1];
        for (int64_t q = prev + 1; q <= l; ++q) ptr[q] = (uint32_t)u;
        if (u == U - 1)
            for (int64_t q = l + 1; q <= lines; ++q) ptr[q] = (uint32_t)U;
    }
}

__global__ void gather_csc(const uint32_t* __restrict__ perm, const uint32_t* __restrict__ row,
                           const float* __restrict__ val, int64_t U, uint32_t* __restrict__ cidx, float* __restrict__ cval) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < U; v += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t u = perm[v];
        cidx[v] = row[u];
        cval[v] = val[u];
    }
}

int bits_for(uint64_t maxval) {
    int b = 1;
    while (b < 64 && (maxval >> b) != 0) ++b;
    return b;
}

// Device buffers of one call, freed on every return path.
struct Scratch {
    std::vector<void*> ptrs;
    template <class T>
    bool get(T** p, size_t count) {
        *p = nullptr;
        if (cudaMalloc((void**)p, std::max<size_t>(1, count) * sizeof(T)) != cudaSuccess) return false;
        ptrs.push_back(*p);
        return true;
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
};

}  // namespace

#define CC(x)                                  \
    do {                                       \
        if ((x) != cudaSuccess) {              \
            cudaStreamSynchronize(s);          \
            cudaStreamDestroy(s);              \
            return CDMF_ERR_CUDA;              \
        }                                      \
    } while (0)
#define CA(x)                                  \
    do {                                       \
        if (!(x)) {                            \
            cudaStreamDestroy(s);              \
            return CDMF_ERR_ALLOC;             \
        }                                      \
    } while (0)

extern "C" int cdmf_cuda_compress(int64_t m, int64_t n, int64_t nnz, const uint32_t* rows, const uint32_t* cols,
                                  const double* vals, int device, uint32_t* csr_ptr, uint32_t* csr_idx, float* csr_val,
                                  uint32_t* csc_ptr, uint32_t* csc_idx, float* csc_val, int64_t* nnz_out) {
    if (m < 0 || n < 0 || nnz < 0 || !csr_ptr || !csc_ptr || !nnz_out) return CDMF_ERR_INVALID;
    if (nnz > 0 && (!rows || !cols || !vals || !csr_idx || !csr_val || !csc_idx || !csc_val || m == 0 || n == 0))
        return CDMF_ERR_INVALID;
    if (nnz > (int64_t)UINT32_MAX - 8192 || m >= (int64_t)UINT32_MAX || n >= (int64_t)UINT32_MAX)
        return CDMF_ERR_TOO_LARGE;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CDMF_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return CDMF_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return CDMF_ERR_CUDA;
    *nnz_out = 0;
    if (nnz == 0) {
        std::fill(csr_ptr, csr_ptr + m + 1, 0u);
        std::fill(csc_ptr, csc_ptr + n + 1, 0u);
        return CDMF_OK;
    }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return CDMF_ERR_CUDA;
    const size_t N = (size_t)nnz;
    int64_t U = 0;
    {
        Scratch S;
        uint32_t *d_rows, *d_cols, *pos_a, *pos_b, *head, *uid, *start, *row, *col, *cidx, *perm, *ccol,
            *d_rptr, *d_cptr, *bad;
        uint64_t *key_a, *key_b;
        double* d_vals;
        float *val, *cval;
        CA(S.get(&d_rows, N) && S.get(&d_cols, N) && S.get(&d_vals, N) && S.get(&key_a, N) && S.get(&key_b, N) &&
           S.get(&pos_a, N) && S.get(&pos_b, N) && S.get(&head, N) && S.get(&uid, N) && S.get(&start, N + 1) &&
           S.get(&bad, 1));
        CC(cudaMemcpyAsync(d_rows, rows, 4 * N, cudaMemcpyHostToDevice, s));
        CC(cudaMemcpyAsync(d_cols, cols, 4 * N, cudaMemcpyHostToDevice, s));
        CC(cudaMemcpyAsync(d_vals, vals, 8 * N, cudaMemcpyHostToDevice, s));
        CC(cudaMemsetAsync(bad, 0, 4, s));
        make_keys<<<grid_for(nnz), kThreads, 0, s>>>(d_rows, d_cols, nnz, (uint64_t)m, (uint64_t)n, key_a, pos_a, bad);
        CC(cudaGetLastError());
        uint32_t h_bad = 0;
        CC(cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, s));
        CC(cudaStreamSynchronize(s));
        if (h_bad) {
            cudaStreamDestroy(s);
            return CDMF_ERR_INVALID;
        }
        // 1. stable sort by (row, col)
        const int kbits = bits_for((uint64_t)m * (uint64_t)n - 1);
        size_t tmp_bytes = 0, t2 = 0, t3 = 0;
        CC(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key_a, key_b, pos_a, pos_b, nnz, 0, kbits, s));
        CC(cub::DeviceScan::ExclusiveSum(nullptr, t2, head, uid, nnz, s));
        const int cbits = bits_for((uint64_t)n - 1);
        CC(cub::DeviceRadixSort::SortPairs(nullptr, t3, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                           (const uint32_t*)nullptr, (uint32_t*)nullptr, nnz, 0, cbits, s));
        tmp_bytes = std::max(tmp_bytes, std::max(t2, t3));
        char* tmp = nullptr;
        CA(S.get(&tmp, tmp_bytes));
        CC(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key_a, key_b, pos_a, pos_b, nnz, 0, kbits, s));
        // 2. runs of equal keys
        run_heads<<<grid_for(nnz), kThreads, 0, s>>>(key_b, nnz, head);
        CC(cudaGetLastError());
        CC(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, head, uid, nnz, s));
        run_starts<<<grid_for(nnz), kThreads, 0, s>>>(head, uid, nnz, start);
        CC(cudaGetLastError());
        uint32_t last_uid = 0, last_head = 0;
        CC(cudaMemcpyAsync(&last_uid, uid + N - 1, 4, cudaMemcpyDeviceToHost, s));
        CC(cudaMemcpyAsync(&last_head, head + N - 1, 4, cudaMemcpyDeviceToHost, s));
        CC(cudaStreamSynchronize(s));
        U = (int64_t)last_uid + last_head;
        // 3. distinct entries in CSR order
        CA(S.get(&row, U) && S.get(&col, U) && S.get(&val, U) && S.get(&d_rptr, m + 1) && S.get(&d_cptr, n + 1) &&
           S.get(&perm, U) && S.get(&ccol, U) && S.get(&cidx, U) && S.get(&cval, U));
        reduce_runs<<<grid_for(U), kThreads, 0, s>>>(key_b, pos_b, d_vals, start, U, (uint64_t)n, row, col, val);
        CC(cudaGetLastError());
        line_pointers<<<grid_for(U), kThreads, 0, s>>>(row, U, m, d_rptr);
        CC(cudaGetLastError());
        // 4. CSC: stable sort of the distinct entries by column; the values are
        // their CSR positions (pos_a still holds 0..nnz-1: the first sort wrote
        // its output to pos_b and left its input alone)
        CC(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, col, ccol, pos_a, perm, U, 0, cbits, s));
        gather_csc<<<grid_for(U), kThreads, 0, s>>>(perm, row, val, U, cidx, cval);
        CC(cudaGetLastError());
        line_pointers<<<grid_for(U), kThreads, 0, s>>>(ccol, U, n, d_cptr);
        CC(cudaGetLastError());
        // 5. results to the host
        CC(cudaMemcpyAsync(csr_ptr, d_rptr, 4 * (size_t)(m + 1), cudaMemcpyDeviceToHost, s));
        CC(cudaMemcpyAsync(csr_idx, col, 4 * (size_t)U, cudaMemcpyDeviceToHost, s));
        CC(cudaMemcpyAsync(csr_val, val, 4 * (size_t)U, cudaMemcpyDeviceToHost, s));
        CC(cudaMemcpyAsync(csc_ptr, d_cptr, 4 * (size_t)(n + 1), cudaMemcpyDeviceToHost, s));
        CC(cudaMemcpyAsync(csc_idx, cidx, 4 * (size_t)U, cudaMemcpyDeviceToHost, s));
        CC(cudaMemcpyAsync(csc_val, cval, 4 * (size_t)U, cudaMemcpyDeviceToHost, s));
        CC(cudaStreamSynchronize(s));
    }
    cudaStreamDestroy(s);
    *nnz_out = U;
    return CDMF_OK;
}

// ============================================================================
// Degree relabelling on the GPU (the engine's create step for the line
// layout).  Same result as relabel() in relabel.cpp, bit for bit:
//   rows / columns ordered by decreasing degree, ties by id (stable radix
//   sort of the complemented degree over ids in order);
//   new CSR: entries keyed (new row, new column), stable-sorted;
//   new CSC: stable sort of the new CSR entries by column.
// ============================================================================

namespace {

__global__ void row_degrees(const uint32_t* __restrict__ ptr, int64_t m, uint32_t* __restrict__ key,
                            uint32_t* __restrict__ id) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        key[i] = ~(ptr[i + 1] - ptr[i]);   // ascending key = descending degree
        id[i] = (uint32_t)i;
    }
}

__global__ void count_cols(const uint32_t* __restrict__ idx, int64_t nnz, uint32_t* __restrict__ cnt) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(cnt + idx[q], 1u);
}

__global__ void col_keys(const uint32_t* __restrict__ cnt, int64_t n, uint32_t* __restrict__ key,
                         uint32_t* __restrict__ id) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        key[j] = ~cnt[j];
        id[j] = (uint32_t)j;
    }
}

__global__ void invert(const uint32_t* __restrict__ old_of_new, int64_t len, uint32_t* __restrict__ new_of_old) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < len; q += (int64_t)gridDim.x * blockDim.x)
        new_of_old[old_of_new[q]] = (uint32_t)q;
}

// new row q: its length, for the scan that gives the new row pointers
__global__ void new_lengths(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ row_old, int64_t m,
                            uint32_t* __restrict__ len) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t i = row_old[q];
        len[q] = ptr[i + 1] - ptr[i];
    }
}

// one warp per caller row: key (new row, new column) and the caller position
__global__ void entry_keys(const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ idx,
                           const uint32_t* __restrict__ row_new, const uint32_t* __restrict__ col_new, int64_t m,
                           uint64_t n, uint64_t* __restrict__ key, uint32_t* __restrict__ pos) {
    const int64_t warps = (int64_t)gridDim.x * blockDim.x / 32;
    const int lane = threadIdx.x & 31;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; i < m; i += warps) {
        const uint64_t q = row_new[i];
        for (uint32_t s = ptr[i] + lane; s < ptr[i + 1]; s += 32) {
            key[s] = q * n + col_new[idx[s]];
            pos[s] = s;
        }
    }
}

__global__ void csr_fill(const uint64_t* __restrict__ key, const uint32_t* __restrict__ pos,
                         const float* __restrict__ uval, int64_t nnz, uint64_t n, uint32_t* __restrict__ idx,
                         float* __restrict__ val, uint32_t* __restrict__ iota) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < nnz; o += (int64_t)gridDim.x * blockDim.x) {
        idx[o] = (uint32_t)(key[o] % n);
        val[o] = uval[pos[o]];
        iota[o] = (uint32_t)o;
    }
}

__global__ void csc_fill(const uint32_t* __restrict__ from_csr, const uint64_t* __restrict__ key,
                         const float* __restrict__ val, int64_t nnz, uint64_t n, uint32_t* __restrict__ cidx,
                         float* __restrict__ cval, uint32_t* __restrict__ to_csc) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nnz; v += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t o = from_csr[v];
        cidx[v] = (uint32_t)(key[o] / n);
        cval[v] = val[o];
        if (to_csc) to_csc[o] = (uint32_t)v;
    }
}

}  // namespace

namespace cdmf {

int gpu_relabel(const cdmf_problem& p, cudaStream_t s, GpuRelabel& out, std::vector<void*>& allocs) {
    const int64_t m = p.m, n = p.n, N = p.nnz;
    auto keep = [&](auto** ptr, size_t count) -> bool {
        using T = std::remove_pointer_t<std::remove_reference_t<decltype(*ptr)>>;
        if (cudaMalloc((void**)ptr, std::max<size_t>(1, count) * sizeof(T)) != cudaSuccess) return false;
        allocs.push_back((void*)*ptr);
        return true;
    };
    if (!keep(&out.d_row_old, m) || !keep(&out.d_col_old, n) || !keep(&out.uptr, m + 1) || !keep(&out.uidx, N) || !keep(&out.csr_ptr, m + 1) || !keep(&out.csr_idx, N) || !keep(&out.csr_val, N) || !keep(&out.csc_ptr, n + 1) ||
        !keep(&out.csc_idx, N) || !keep(&out.csc_val, N) || !keep(&out.csr_pos, N) || !keep(&out.csc_from_csr, N) ||
        !keep(&out.to_csc, N))
        return CDMF_ERR_ALLOC;
    Scratch S;
    uint32_t *uptr = out.uptr, *uidx = out.uidx, *row_old = out.d_row_old, *col_old = out.d_col_old;
    uint32_t *rkey, *rkey2, *rid, *ccnt, *ckey, *ckey2, *cid, *row_new, *col_new, *nlen, *pos_a, *iota, *col_sorted;
    uint64_t *key_a, *key_b;
    float* uval;
    if (!S.get(&uval, N) || !S.get(&rkey, m) || !S.get(&rkey2, m) ||
        !S.get(&rid, m) || !S.get(&ccnt, n) || !S.get(&ckey, n) || !S.get(&ckey2, n) || !S.get(&cid, n) ||
        !S.get(&row_new, m) || !S.get(&col_new, n) ||
        !S.get(&nlen, m + 1) || !S.get(&pos_a, N) || !S.get(&iota, N) || !S.get(&col_sorted, N) || !S.get(&key_a, N) ||
        !S.get(&key_b, N))
        return CDMF_ERR_ALLOC;
#define RC(x) do { if ((x) != cudaSuccess) return CDMF_ERR_CUDA; } while (0)
    // the ratings are first read by csr_fill, after the sorts: they are
    // uploaded on a side stream while the sorts run (queued below, after the
    // sorts, so that a synchronous copy from pageable memory overlaps them too)
    struct Side {
        cudaStream_t s = nullptr;
        cudaEvent_t done = nullptr;
        ~Side() {
            if (s) {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
            if (done) cudaEventDestroy(done);
        }
    } side;
    RC(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
    RC(cudaEventCreateWithFlags(&side.done, cudaEventDisableTiming));
    RC(cudaMemcpyAsync(uptr, p.csr_row_ptr, 4 * (size_t)(m + 1), cudaMemcpyHostToDevice, s));
    RC(cudaMemcpyAsync(uidx, p.csr_col_idx, 4 * (size_t)N, cudaMemcpyHostToDevice, s));
    RC(cudaMemsetAsync(ccnt, 0, 4 * (size_t)n, s));
    // degree orders
    row_degrees<<<grid_for(m), kThreads, 0, s>>>(uptr, m, rkey, rid);
    count_cols<<<grid_for(N), kThreads, 0, s>>>(uidx, N, ccnt);
    col_keys<<<grid_for(n), kThreads, 0, s>>>(ccnt, n, ckey, cid);
    RC(cudaGetLastError());
    const int kbits = bits_for((uint64_t)m * (uint64_t)n - 1), cbits = bits_for((uint64_t)n - 1);
    size_t t0 = 0, t1 = 0, t2 = 0, t3 = 0, t4 = 0;
    RC(cub::DeviceRadixSort::SortPairs(nullptr, t0, rkey, rkey2, rid, row_old, m, 0, 32, s));
    RC(cub::DeviceRadixSort::SortPairs(nullptr, t1, ckey, ckey2, cid, col_old, n, 0, 32, s));
    RC(cub::DeviceScan::ExclusiveSum(nullptr, t2, nlen, out.csr_ptr, m + 1, s));
    RC(cub::DeviceRadixSort::SortPairs(nullptr, t3, key_a, key_b, pos_a, out.csr_pos, N, 0, kbits, s));
    RC(cub::DeviceRadixSort::SortPairs(nullptr, t4, out.csr_idx, col_sorted, iota, out.csc_from_csr, N, 0, cbits, s));
    const size_t tb = std::max({t0, t1, t2, t3, t4});
    char* tmp = nullptr;
    if (!S.get(&tmp, tb)) return CDMF_ERR_ALLOC;
    size_t tbv = tb;
    RC(cub::DeviceRadixSort::SortPairs(tmp, tbv, rkey, rkey2, rid, row_old, m, 0, 32, s));
    tbv = tb;
    RC(cub::DeviceRadixSort::SortPairs(tmp, tbv, ckey, ckey2, cid, col_old, n, 0, 32, s));
    invert<<<grid_for(m), kThreads, 0, s>>>(row_old, m, row_new);
    invert<<<grid_for(n), kThreads, 0, s>>>(col_old, n, col_new);
    // new row pointers: lengths in the new order, scanned (the extra last
    // element of nlen is 0, so ptr[m] = nnz)
    RC(cudaMemsetAsync(nlen + m, 0, 4, s));
    new_lengths<<<grid_for(m), kThreads, 0, s>>>(uptr, row_old, m, nlen);
    RC(cudaGetLastError());
    tbv = tb;
    RC(cub::DeviceScan::ExclusiveSum(tmp, tbv, nlen, out.csr_ptr, m + 1, s));
    // entries in (new row, new column) order
    entry_keys<<<grid_for(32 * m), kThreads, 0, s>>>(uptr, uidx, row_new, col_new, m, (uint64_t)n, key_a, pos_a);
    RC(cudaGetLastError());
    tbv = tb;
    RC(cub::DeviceRadixSort::SortPairs(tmp, tbv, key_a, key_b, pos_a, out.csr_pos, N, 0, kbits, s));
    RC(cudaMemcpyAsync(uval, p.csr_val, 4 * (size_t)N, cudaMemcpyHostToDevice, side.s));
    RC(cudaEventRecord(side.done, side.s));
    RC(cudaStreamWaitEvent(s, side.done, 0));
    csr_fill<<<grid_for(N), kThreads, 0, s>>>(key_b, out.csr_pos, uval, N, (uint64_t)n, out.csr_idx, out.csr_val, iota);
    RC(cudaGetLastError());
    // CSC: stable transposition
    tbv = tb;
    RC(cub::DeviceRadixSort::SortPairs(tmp, tbv, out.csr_idx, col_sorted, iota, out.csc_from_csr, N, 0, cbits, s));
    csc_fill<<<grid_for(N), kThreads, 0, s>>>(out.csc_from_csr, key_b, out.csr_val, N, (uint64_t)n, out.csc_idx,
                                              out.csc_val, out.to_csc);
    line_pointers<<<grid_for(N), kThreads, 0, s>>>(col_sorted, N, n, out.csc_ptr);
    RC(cudaGetLastError());
    // host copies of what the set-up plans with
    out.row_old.resize(m);
    out.col_old.resize(n);
    out.hptr_r.resize(m + 1);
    out.hptr_c.resize(n + 1);
    RC(cudaMemcpyAsync(out.row_old.data(), row_old, 4 * (size_t)m, cudaMemcpyDeviceToHost, s));
    RC(cudaMemcpyAsync(out.col_old.data(), col_old, 4 * (size_t)n, cudaMemcpyDeviceToHost, s));
    RC(cudaMemcpyAsync(out.hptr_r.data(), out.csr_ptr, 4 * (size_t)(m + 1), cudaMemcpyDeviceToHost, s));
    RC(cudaMemcpyAsync(out.hptr_c.data(), out.csc_ptr, 4 * (size_t)(n + 1), cudaMemcpyDeviceToHost, s));
    RC(cudaStreamSynchronize(s));
#undef RC
    return CDMF_OK;
}

}  // namespace cdmf
