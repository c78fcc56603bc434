// Cross-index-blocked layout of one compressed copy (host side).
//
// A copy with L lines (columns of CSC, rows of CSR) and cross indices in
// [0, cross) is cut into NB = ceil(cross / XB) blocks of XB cross indices.
// Storage is block-major: for block b, for line j, the entries of line j
// whose cross index lies in block b, in their original order.  A "segment"
// is one (b, j) pair; segptr[b * L + j] is its first position.  Inside a
// block the cross index is stored as a 16-bit offset from b * XB.
//
// The sweep over such a copy stages block b's slice of the gather table in
// shared memory once per work unit, so every per-nonzero gather is a
// shared-memory read; each segment leaves a partial sum, and a second
// kernel adds a line's partials in block order.
#pragma once
#include "relabel.h"

#include <cstdint>
#include <vector>

namespace cdmf {

struct BlockedHost {
    uint32_t xb = 0, nb = 0, lines = 0;
    uint64_t cross = 0;
    std::vector<uint32_t> segptr;       // nb * lines + 1
    uvec<uint16_t> idx16;               // nnz: cross index - b * xb
    uvec<uint32_t> pos;                 // position in the line layout -> blocked position
    std::vector<uint32_t> units;        // 5 per unit: b, first line, end of CTA lines, end of warp lines, end line
};

// ptr/idx: the copy in line layout (lines ascending, cross indices ascending
// inside a line).  unit_nnz: target nonzeros per work unit.
bool build_blocked(const uint32_t* ptr, const uint32_t* idx, uint32_t lines, uint64_t cross, uint32_t xb,
                   uint32_t unit_nnz, BlockedHost& out);

}  // namespace cdmf
