// Cross-index-blocked layout builder (see blocked.h).  The counting and the
// fill run in parallel over lines: segment (b, j) belongs to line j alone,
// so threads never share a counter.
#include "blocked.h"

#include <algorithm>
#include <omp.h>

namespace cdmf {

bool build_blocked(const uint32_t* ptr, const uint32_t* idx, uint32_t lines, uint64_t cross, uint32_t xb,
                   uint32_t unit_nnz, BlockedHost& B) {
    if (xb == 0 || xb > 65536) return false;
    try {
        const uint64_t nnz = ptr[lines];
        B.xb = xb;
        B.lines = lines;
        B.cross = cross;
        B.nb = (uint32_t)((cross + xb - 1) / xb);
        if (B.nb == 0) B.nb = 1;
        const uint64_t nseg = (uint64_t)B.nb * lines;
        B.segptr.assign(nseg + 1, 0);
        // count per segment: a line's entries are sorted, so its segments are
        // consecutive runs of its range
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t j = 0; j < (int64_t)lines; ++j)
            for (uint32_t p = ptr[j]; p < ptr[j + 1]; ++p) B.segptr[(uint64_t)(idx[p] / xb) * lines + j + 1]++;
        for (uint64_t s = 0; s < nseg; ++s) B.segptr[s + 1] += B.segptr[s];
        if (B.segptr[nseg] != nnz) return false;
        B.idx16.resize(nnz);
        B.pos.resize(nnz);
#pragma omp parallel for schedule(dynamic, 1024)
        for (int64_t j = 0; j < (int64_t)lines; ++j) {
            uint32_t p = ptr[j];
            while (p < ptr[j + 1]) {
                const uint32_t b = idx[p] / xb;
                uint32_t q = B.segptr[(uint64_t)b * lines + j];
                for (; p < ptr[j + 1] && idx[p] / xb == b; ++p, ++q) {
                    B.idx16[q] = (uint16_t)(idx[p] - b * xb);
                    B.pos[p] = q;
                }
            }
        }
        // work units: consecutive lines of one block up to ~unit_nnz nonzeros,
        // with the line ranges handled by the whole CTA (segments >= cta_len),
        // by single warps (>= warp_len) and by 8-lane groups (the rest);
        // lines are degree-sorted, so segment lengths mostly fall along a unit
        const uint32_t cta_len = 2048, warp_len = 48;
        B.units.clear();
        for (uint32_t b = 0; b < B.nb; ++b) {
            const uint64_t base = (uint64_t)b * lines;
            uint32_t j0 = 0;
            while (j0 < lines) {
                uint32_t j1 = j0;
                const uint32_t start = B.segptr[base + j0];
                while (j1 < lines && (j1 == j0 || B.segptr[base + j1 + 1] - start <= unit_nnz)) ++j1;
                uint32_t jc = j0, jw;
                while (jc < j1 && B.segptr[base + jc + 1] - B.segptr[base + jc] >= cta_len) ++jc;
                jw = jc;
                while (jw < j1 && B.segptr[base + jw + 1] - B.segptr[base + jw] >= warp_len) ++jw;
                const uint32_t u[5] = {b, j0, jc, jw, j1};
                B.units.insert(B.units.end(), u, u + 5);
                j0 = j1;
            }
        }
    } catch (...) {
        return false;
    }
    return true;
}

}  // namespace cdmf
