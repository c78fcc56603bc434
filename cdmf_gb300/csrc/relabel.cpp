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
#include "relabel.h"

#include <algorithm>
#include <numeric>
#include <omp.h>

namespace cdmf {

static std::vector<uint32_t> degree_order(const uint32_t* ptr, int64_t lines) {
    std::vector<uint32_t> order(lines);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return (ptr[a + 1] - ptr[a]) > (ptr[b + 1] - ptr[b]);
    });
    return order;
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
        // CSC by a stable counting sort of the new CSR (rows ascending in a column)
        R.csc_ptr.assign(n + 1, 0);
        for (int64_t q = 0; q < N; ++q) R.csc_ptr[R.csr_idx[q] + 1]++;
        for (int64_t j = 0; j < n; ++j) R.csc_ptr[j + 1] += R.csc_ptr[j];
        R.csc_idx.resize(N);
        R.csc_val.resize(N);
        R.csc_from_csr.resize(N);   // new CSC position -> new CSR position
        std::vector<uint32_t> next(R.csc_ptr.begin(), R.csc_ptr.end() - 1);
        for (int64_t q = 0; q < m; ++q)
            for (uint32_t s = R.csr_ptr[q]; s < R.csr_ptr[q + 1]; ++s) {
                const uint32_t o = next[R.csr_idx[s]]++;
                R.csc_idx[o] = (uint32_t)q;
                R.csc_val[o] = R.csr_val[s];
                R.csc_from_csr[o] = s;
            }
        // caller's CSC position of each new CSC position: through the caller's
        // CSR position and the caller's own CSR->CSC map
        std::vector<uint32_t> user_csr_to_csc(N), unext(p.csc_col_ptr, p.csc_col_ptr + n);
        for (int64_t i = 0; i < m; ++i)
            for (uint32_t s = p.csr_row_ptr[i]; s < p.csr_row_ptr[i + 1]; ++s) {
                const uint32_t j = p.csr_col_idx[s];
                const uint32_t o = unext[j]++;
                if (o >= p.csc_col_ptr[j + 1] || p.csc_row_idx[o] != (uint32_t)i) return false;
                user_csr_to_csc[s] = o;
            }
        R.csc_pos.resize(N);
        for (int64_t o = 0; o < N; ++o) R.csc_pos[o] = user_csr_to_csc[R.csr_pos[R.csc_from_csr[o]]];
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
