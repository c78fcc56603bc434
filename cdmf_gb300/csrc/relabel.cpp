// Degree relabelling of rows and columns (host side of cdmf_cuda_create).
//
// Rows and columns are renumbered by decreasing number of nonzeros (ties by
// the original id).  The engine's sweeps then gather the cross vectors of
// the heavy lines from a small, dense prefix of each table, so neighbouring
// nonzeros of a long column hit the same cache sectors, and the row-length
// bins become contiguous id ranges.  Only the numbering changes: every line
// keeps its entries, and the results are mapped back to the caller's
// numbering on the way out.  The summation order inside a column follows
// the new row numbering, which is why the reference-order mode does not
// relabel.
//
// All passes run on the host threads (OpenMP).  Transpositions use a stable
// counting sort with per-thread histograms over contiguous line ranges, so
// the result does not depend on the thread count.
#include "relabel.h"

#include <algorithm>
#include <numeric>
#include <omp.h>

namespace cdmf {

static uvec<uint32_t> degree_order(const uint32_t* ptr, int64_t lines) {
    uvec<uint32_t> order(lines);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return (ptr[a + 1] - ptr[a]) > (ptr[b + 1] - ptr[b]);
    });
    return order;
}

static bool transpose(int64_t lines, int64_t cross, const uint32_t* ptr, const uint32_t* idx, std::vector<uint32_t>& tptr,
               uint32_t* tidx, uint32_t* src_pos) {
    const int64_t N = ptr[lines];
    const int T = std::max(1, std::min(omp_get_max_threads(), 64));
    // contiguous line ranges of about equal nonzeros per thread
    std::vector<int64_t> lb(T + 1, lines);
    lb[0] = 0;
    {
        int64_t t = 1;
        for (int64_t j = 0; j < lines && t < T; ++j)
            while (t < T && (int64_t)ptr[j] >= N * t / T) lb[t++] = j;
    }
    std::vector<std::vector<uint32_t>> hist(T, std::vector<uint32_t>(cross, 0));
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t)
        for (int64_t j = lb[t]; j < lb[t + 1]; ++j)
            for (uint32_t p = ptr[j]; p < ptr[j + 1]; ++p) hist[t][idx[p]]++;
    tptr.assign(cross + 1, 0);
    // offsets: column-major over threads, so each thread's entries of a column
    // follow those of earlier (lower) line ranges -- stable
    uint64_t run = 0;
    for (int64_t c = 0; c < cross; ++c) {
        tptr[c] = (uint32_t)run;
        for (int t = 0; t < T; ++t) {
            const uint32_t h = hist[t][c];
            hist[t][c] = (uint32_t)run;
            run += h;
        }
    }
    tptr[cross] = (uint32_t)run;
    if ((int64_t)run != N) return false;
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
        std::vector<uint32_t>& next = hist[t];
        for (int64_t j = lb[t]; j < lb[t + 1]; ++j)
            for (uint32_t p = ptr[j]; p < ptr[j + 1]; ++p) {
                const uint32_t o = next[idx[p]]++;
                tidx[o] = (uint32_t)j;
                if (src_pos) src_pos[o] = p;
            }
    }
    return true;
}

bool relabel_csc_positions(int64_t m, int64_t n, const uint32_t* ucsr_ptr, const uint32_t* ucsr_idx,
                           const uvec<uint32_t>& csr_pos, const uvec<uint32_t>& csc_from_csr, uvec<uint32_t>& csc_pos) {
    // caller's CSC position of each new CSC position: the caller's CSC is the
    // stable transposition of its CSR (scipy's canonical order)
    const int64_t N = ucsr_ptr[m];
    try {
        std::vector<uint32_t> uptr;
        uvec<uint32_t> urow(N), usrc(N), user_csr_to_csc(N);
        if (!transpose(m, n, ucsr_ptr, ucsr_idx, uptr, urow.data(), usrc.data())) return false;
#pragma omp parallel for schedule(static)
        for (int64_t o = 0; o < N; ++o) user_csr_to_csc[usrc[o]] = (uint32_t)o;
        csc_pos.resize(N);
#pragma omp parallel for schedule(static)
        for (int64_t o = 0; o < N; ++o) csc_pos[o] = user_csr_to_csc[csr_pos[csc_from_csr[o]]];
    } catch (...) {
        return false;
    }
    return true;
}

bool relabel(const cdmf_problem& p, Relabel& R) {
    const int64_t m = p.m, n = p.n, N = p.nnz;
    try {
        R.row_old = degree_order(p.csr_row_ptr, m);
        R.col_old = degree_order(p.csc_col_ptr, n);
        R.row_new.assign(m, 0);
        R.col_new.assign(n, 0);
        for (int64_t q = 0; q < m; ++q) R.row_new[R.row_old[q]] = (uint32_t)q;
        for (int64_t q = 0; q < n; ++q) R.col_new[R.col_old[q]] = (uint32_t)q;
        // CSR in the new numbering: rows in new order, entries sorted by new column
        R.csr_ptr.assign(m + 1, 0);
        for (int64_t q = 0; q < m; ++q) {
            const uint32_t i = R.row_old[q];
            R.csr_ptr[q + 1] = R.csr_ptr[q] + (p.csr_row_ptr[i + 1] - p.csr_row_ptr[i]);
        }
        R.csr_idx.resize(N);
        R.csr_val.resize(N);
        R.csr_pos.resize(N);   // new CSR position -> caller's CSR position
#pragma omp parallel
        {
            std::vector<std::pair<uint32_t, uint32_t>> tmp;
#pragma omp for schedule(dynamic, 256)
            for (int64_t q = 0; q < m; ++q) {
                const uint32_t i = R.row_old[q];
                const uint32_t b = p.csr_row_ptr[i], e = p.csr_row_ptr[i + 1];
                tmp.clear();
                for (uint32_t s = b; s < e; ++s) tmp.emplace_back(R.col_new[p.csr_col_idx[s]], s);
                std::sort(tmp.begin(), tmp.end());
                uint32_t o = R.csr_ptr[q];
                for (const auto& pr : tmp) {
                    R.csr_idx[o] = pr.first;
                    R.csr_val[o] = p.csr_val[pr.second];
                    R.csr_pos[o] = pr.second;
                    ++o;
                }
            }
        }
        // CSC of the new CSR (rows ascending in a column)
        R.csc_idx.resize(N);
        R.csc_val.resize(N);
        R.csc_from_csr.resize(N);   // new CSC position -> new CSR position
        if (!transpose(m, n, R.csr_ptr.data(), R.csr_idx.data(), R.csc_ptr, R.csc_idx.data(), R.csc_from_csr.data()))
            return false;
#pragma omp parallel for schedule(static)
        for (int64_t o = 0; o < N; ++o) R.csc_val[o] = R.csr_val[R.csc_from_csr[o]];
        R.te_row.resize(p.nnz_test);
        R.te_col.resize(p.nnz_test);
        for (int64_t e = 0; e < p.nnz_test; ++e) {
            R.te_row[e] = R.row_new[p.test_row[e]];
            R.te_col[e] = R.col_new[p.test_col[e]];
        }
    } catch (...) {
        return false;
    }
    return true;
}

}  // namespace cdmf
