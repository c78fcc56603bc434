// Host-side harness for the sanitizer tests (tests/test_host_sanitizers.py).
//
// Links the engine's host code -- the synthetic generator and CSR->CSC
// transposition (synth.cpp), the degree relabelling (relabel.cpp), the
// blocked-layout builder (blocked.cpp) and the `cdmf` driver's loader, flag
// parser and checks (cli/loader.cpp) -- without the CUDA library, so it can
// be built with AddressSanitizer and UndefinedBehaviorSanitizer on a machine
// without a GPU.  The two library entry points the loader calls are stubbed
// below: cdmf_cuda_rmse_coo computes the RMSE on the host, after the same
// argument checks as the library.
//
//   host_harness host                 generator, transposition, relabelling and
//                                     blocked layouts on several shapes, with
//                                     their invariants checked
//   host_harness load DIR             the driver's loader on DIR
//   host_harness rmse DIR K           loader + initial_col + calculate_rmse (-p 1)
//   host_harness args FLAGS... DIR    the driver's flag parser
// Exit status 0 when every check holds (or the load succeeds), 1 otherwise.
#include "../../cdmf_gb300/csrc/blocked.h"
#include "../../cdmf_gb300/csrc/cli/cdmf_host.h"
#include "../../cdmf_gb300/csrc/relabel.h"

#include <cdmf_cuda.h>
#include <cdmf_synth.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

extern "C" const char* cdmf_cuda_strerror(int status) { return status == CDMF_OK ? "ok" : "error (host stub)"; }

extern "C" int cdmf_cuda_rmse_coo(uint32_t k, int64_t m, int64_t n, const float* W, const float* H, int64_t nnz_test,
                                  const uint32_t* test_row, const uint32_t* test_col, const double* test_val,
                                  int device, double* rmse, int64_t* nan_count) {
    (void)device;
    if (k == 0 || m < 0 || n < 0 || nnz_test < 0 || !W || !H || !rmse) return CDMF_ERR_INVALID;
    if (nnz_test == 0) return CDMF_ERR_EMPTY_TEST;
    if (!test_row || !test_col || !test_val) return CDMF_ERR_INVALID;
    double sum = 0.0;
    int64_t nans = 0;
    for (int64_t e = 0; e < nnz_test; ++e) {
        if ((int64_t)test_row[e] >= m || (int64_t)test_col[e] >= n) return CDMF_ERR_INVALID;
        double pred = 0.0;
        for (uint32_t t = 0; t < k; ++t) pred += (double)W[t * m + test_row[e]] * H[t * n + test_col[e]];
        const double d = pred - test_val[e];
        if (std::isnan(d)) ++nans;
        else sum += d * d;
    }
    *rmse = std::sqrt(sum / (double)nnz_test);
    if (nan_count) *nan_count = nans;
    return CDMF_OK;
}

namespace {

int failures = 0;

void expect(bool ok, const char* what, const std::string& where) {
    if (!ok) {
        fprintf(stderr, "FAILED: %s (%s)\n", what, where.c_str());
        ++failures;
    }
}

bool is_permutation(const uint32_t* a, size_t n) {
    std::vector<char> seen(n, 0);
    for (size_t i = 0; i < n; ++i) {
        if (a[i] >= n || seen[a[i]]) return false;
        seen[a[i]] = 1;
    }
    return true;
}

bool sorted_lines(const uint32_t* ptr, const uint32_t* idx, int64_t lines) {
    for (int64_t j = 0; j < lines; ++j)
        for (uint32_t p = ptr[j] + 1; p < ptr[j + 1]; ++p)
            if (idx[p - 1] >= idx[p]) return false;
    return true;
}

void check_blocked(const uint32_t* ptr, const uint32_t* idx, uint32_t lines, uint64_t cross, uint32_t xb,
                   const std::string& where) {
    cdmf::BlockedHost B;
    expect(cdmf::build_blocked(ptr, idx, lines, cross, xb, 4096, B), "build_blocked", where);
    const size_t nnz = ptr[lines];
    expect(B.segptr.size() == (size_t)B.nb * lines + 1 && B.segptr.back() == nnz, "segment table", where);
    for (size_t s = 1; s < B.segptr.size(); ++s)
        if (B.segptr[s] < B.segptr[s - 1]) { expect(false, "segment table monotone", where); break; }
    expect(is_permutation(B.pos.data(), nnz), "blocked positions form a permutation", where);
    bool idx_ok = true;
    for (uint32_t j = 0; j < lines && idx_ok; ++j)
        for (uint32_t p = ptr[j]; p < ptr[j + 1]; ++p) {
            const uint32_t b = idx[p] / xb, q = B.pos[p];
            if (B.idx16[q] != idx[p] - b * xb || q < B.segptr[(size_t)b * lines + j] ||
                q >= B.segptr[(size_t)b * lines + j + 1]) { idx_ok = false; break; }
        }
    expect(idx_ok, "blocked offsets and segments", where);
    expect(B.units.size() % 5 == 0, "work units", where);
}

void check_shape(const cdmf_synth_spec& sp, const std::string& where) {
    cdmf_synth* s = nullptr;
    if (cdmf_synth_create(&sp, 4, &s) != 0) { expect(false, "cdmf_synth_create", where); return; }
    int64_t m, n, N, nt;
    cdmf_synth_info(s, &m, &n, &N, &nt);
    std::vector<uint32_t> rp(m + 1), ci(N), cp(n + 1), ri(N), tr(nt), tc(nt);
    std::vector<float> rv(N), cv(N), tv(nt);
    expect(cdmf_synth_copy(s, rp.data(), ci.data(), rv.data(), cp.data(), ri.data(), cv.data(), tr.data(), tc.data(),
                           tv.data()) == 0, "cdmf_synth_copy", where);
    cdmf_synth_destroy(s);
    expect(rp[m] == N && cp[n] == N, "pointer ends", where);
    expect(sorted_lines(rp.data(), ci.data(), m) && sorted_lines(cp.data(), ri.data(), n), "canonical order", where);
    // transposition: the generator's own CSC again, and a position map
    std::vector<uint32_t> cp2(n + 1), ri2(N), perm(N);
    std::vector<float> cv2(N);
    expect(cdmf_csr_to_csc(m, n, N, rp.data(), ci.data(), rv.data(), cp2.data(), ri2.data(), cv2.data(),
                           perm.data()) == 0, "cdmf_csr_to_csc", where);
    expect(cp2 == cp && ri2 == ri && cv2 == cv, "transposition equals the generated CSC", where);
    expect(is_permutation(perm.data(), N), "CSR->CSC map is a permutation", where);
    // relabelling
    cdmf_problem p{};
    p.m = m; p.n = n; p.nnz = N;
    p.csr_row_ptr = rp.data(); p.csr_col_idx = ci.data(); p.csr_val = rv.data();
    p.csc_col_ptr = cp.data(); p.csc_row_idx = ri.data(); p.csc_val = cv.data();
    p.nnz_test = nt; p.test_row = tr.data(); p.test_col = tc.data(); p.test_val = tv.data();
    cdmf::Relabel R;
    if (!cdmf::relabel(p, R)) { expect(false, "relabel", where); return; }
    expect(is_permutation(R.row_old.data(), m) && is_permutation(R.col_old.data(), n), "new numbering", where);
    bool inv = true, deg = true;
    for (int64_t q = 0; q < m; ++q) {
        inv = inv && R.row_new[R.row_old[q]] == (uint32_t)q;
        const uint32_t i = R.row_old[q];
        deg = deg && R.csr_ptr[q + 1] - R.csr_ptr[q] == rp[i + 1] - rp[i];
        if (q) deg = deg && R.csr_ptr[q + 1] - R.csr_ptr[q] <= R.csr_ptr[q] - R.csr_ptr[q - 1];
    }
    for (int64_t q = 0; q < n; ++q) inv = inv && R.col_new[R.col_old[q]] == (uint32_t)q;
    expect(inv, "numbering maps are inverse", where);
    expect(deg, "rows in decreasing degree, lengths kept", where);
    bool entries = true;
    for (int64_t o = 0; o < N && entries; ++o)
        entries = R.csr_val[o] == rv[R.csr_pos[o]] && R.csr_idx[o] == R.col_new[ci[R.csr_pos[o]]];
    expect(entries, "relabelled CSR entries", where);
    expect(sorted_lines(R.csr_ptr.data(), R.csr_idx.data(), m) &&
           sorted_lines(R.csc_ptr.data(), R.csc_idx.data(), n), "relabelled canonical order", where);
    bool cross = true;
    for (int64_t o = 0; o < N && cross; ++o) cross = R.csc_val[o] == R.csr_val[R.csc_from_csr[o]];
    expect(cross, "relabelled CSC from CSR", where);
    cdmf::uvec<uint32_t> csc_pos;
    expect(cdmf::relabel_csc_positions(m, n, rp.data(), ci.data(), R.csr_pos, R.csc_from_csr, csc_pos),
           "relabel_csc_positions", where);
    bool cpos = csc_pos.size() == (size_t)N;
    for (int64_t o = 0; o < N && cpos; ++o) cpos = cv[csc_pos[o]] == R.csc_val[o];
    expect(cpos, "CSC positions in the caller's order", where);
    bool test_ok = true;
    for (int64_t e = 0; e < nt && test_ok; ++e)
        test_ok = R.te_row[e] == R.row_new[tr[e]] && R.te_col[e] == R.col_new[tc[e]];
    expect(test_ok, "test set renumbered", where);
    check_blocked(R.csr_ptr.data(), R.csr_idx.data(), (uint32_t)m, (uint64_t)n, 64, where + " CSR blocks");
    check_blocked(R.csc_ptr.data(), R.csc_idx.data(), (uint32_t)n, (uint64_t)m, 128, where + " CSC blocks");
}

cdmf_synth_spec base_spec() {
    cdmf_synth_spec s{};
    s.m = 3000; s.n = 700; s.nnz_total = 60000; s.nnz_test = -1; s.test_fraction = 0.02;
    s.row_alpha = 0.9; s.row_min = 1; s.row_max = 350; s.col_alpha = 0.9; s.col_cap = 1500;
    s.rank = 6; s.factor_std = 0.5; s.offset = 3.0; s.noise_std = 0.5; s.quantum = 1.0; s.vmin = 1.0; s.vmax = 5.0;
    s.seed = 3;
    return s;
}

int run_host() {
    cdmf_synth_spec a = base_spec();
    check_shape(a, "zipf 3000x700");
    cdmf_synth_spec b = base_spec();
    b.m = 500; b.n = 40; b.nnz_total = 9000; b.row_min = 0; b.row_max = 40; b.col_alpha = 0.3; b.seed = 5;
    check_shape(b, "narrow with empty rows");
    cdmf_synth_spec c = base_spec();
    c.m = 2000; c.n = 30; c.nnz_total = 0; c.row_mode = 1; c.row_min = 3; c.row_max = 30; c.col_mode = 1;
    c.col_beta_a = 2.0; c.col_beta_b = 1.5; c.quantum = 0.0; c.vmin = -10.0; c.vmax = 10.0; c.seed = 7;
    check_shape(c, "uniform rows, beta columns");
    cdmf_synth_spec d = base_spec();
    d.m = 1; d.n = 1; d.nnz_total = 1; d.row_max = 1; d.col_cap = 1; d.test_fraction = 0.0; d.seed = 1;
    check_shape(d, "1x1");
    std::vector<float> X(3 * 1000);
    cdmf_initial_col(X.data(), 3, 1000);
    bool range = true;
    for (float x : X) range = range && x >= 0.001f && x <= 0.1011f;   // 0.1 U(0,1) + 0.001
    expect(range, "initial_col range", "3x1000");
    if (failures == 0) printf("host ok\n");
    return failures ? 1 : 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string mode = argv[1];
    if (mode == "host") return run_host();
    if (mode == "load" && argc == 3) {
        SparseMatrix R;
        TestData T;
        if (!load(argv[2], R, T)) return 1;
        printf("loaded %ld %ld %lu %lu %lu %lu\n", R.rows, R.cols, R.nnz, T.nnz, R.max_row_nnz, R.max_col_nnz);
        return 0;
    }
    if (mode == "rmse" && argc == 4) {
        SparseMatrix R;
        TestData T;
        if (!load(argv[2], R, T)) return 1;
        const unsigned k = (unsigned)atoi(argv[3]);
        MatData W, H;
        initial_col(W, k, (unsigned)R.rows);
        initial_col(H, k, (unsigned)R.cols);
        return calculate_rmse(W, H, argv[2], k, 0) ? 0 : 1;
    }
    if (mode == "args") {
        parameter p = parse_command_line(argc - 1, argv + 1);
        printf("k=%u lambda=%g maxiter=%d inner=%d version=%d residual=%d reduce=%d graph=%d predict=%d ref=%d "
               "dir=%s\n", p.k, p.lambda, p.maxiter, p.maxinneriter, p.version, p.residual, p.reduce, p.graph,
               p.do_predict, p.do_ref, p.scr_dir);
        return 0;
    }
    return 2;
}
