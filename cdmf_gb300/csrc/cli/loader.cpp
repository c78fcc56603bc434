// Loader, flag parser, initialisation and checks of the `cdmf` driver
// (the reference's src/tools.cpp:271-541 surface, OpenCL parts left out).
#include "cdmf_host.h"

#include <cdmf_cuda.h>
#include <cdmf_synth.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <new>
#include <system_error>

// Whether `path` holds at least `bytes` bytes (the reference's fread needs no
// more); checked for every binary before any array is sized from the meta.
static bool file_holds(const std::string& path, unsigned long long bytes) {
    std::error_code ec;
    const auto have = std::filesystem::file_size(path, ec);
    if (ec) {
        fprintf(stderr, "Can't open %s\n", path.c_str());
        return false;
    }
    if (have < bytes) {
        fprintf(stderr, "FREAD: %s holds %llu bytes, needs %llu\n", path.c_str(), (unsigned long long)have, bytes);
        return false;
    }
    return true;
}

static bool read_exact(const std::string& path, void* dst, size_t bytes) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) {
        fprintf(stderr, "Can't open %s\n", path.c_str());
        return false;
    }
    size_t got = bytes ? fread(dst, bytes, 1, f) : 1;
    fclose(f);
    if (got != 1) {
        fprintf(stderr, "FREAD read %zu, needed %d, in file %s\n", got, 1, path.c_str());
        return false;
    }
    return true;
}

static unsigned long max_gap(const std::vector<uint32_t>& ptr) {
    unsigned long mx = 0;
    for (size_t i = 1; i < ptr.size(); ++i) mx = std::max<unsigned long>(mx, ptr[i] - ptr[i - 1]);
    return mx;
}

bool load(const char* srcdir, SparseMatrix& R, TestData& T) {
    std::string dir(srcdir);
    FILE* fp = fopen((dir + "/meta_modified_all").c_str(), "r");
    if (!fp) {
        printf("Can't open meta input file.\n");
        return false;
    }
    long m, n;
    unsigned long nnz, nnz_test;
    char buf[9][1024], tbuf[3][1024];
    bool ok = fscanf(fp, "%ld %ld %lu", &m, &n, &nnz) == 3;
    for (int q = 0; ok && q < 9; ++q) ok = fscanf(fp, "%1023s", buf[q]) == 1;
    ok = ok && fscanf(fp, "%lu", &nnz_test) == 1;
    for (int q = 0; ok && q < 3; ++q) ok = fscanf(fp, "%1023s", tbuf[q]) == 1;
    fclose(fp);
    // the arrays hold 32-bit unsigned indices and pointers (src/pmf_util.h:110-113)
    const unsigned long kMax = 0xFFFFFFFFul;
    if (!ok || m < 0 || n < 0 || (unsigned long)m >= kMax || (unsigned long)n >= kMax || nnz > kMax ||
        nnz_test > kMax) {
        fprintf(stderr, "malformed meta_modified_all\n");
        return false;
    }
    const unsigned long long b_m = 4ull * (m + 1), b_n = 4ull * (n + 1), b_nnz = 4ull * nnz, b_t = 4ull * nnz_test;
    if (!file_holds(dir + "/" + buf[3], b_m) || !file_holds(dir + "/" + buf[4], b_nnz) ||
        !file_holds(dir + "/" + buf[5], b_nnz) || !file_holds(dir + "/" + buf[6], b_n) ||
        !file_holds(dir + "/" + buf[7], b_nnz) || !file_holds(dir + "/" + buf[8], b_nnz) ||
        !file_holds(dir + "/" + tbuf[0], b_t) || !file_holds(dir + "/" + tbuf[1], b_t) ||
        !file_holds(dir + "/" + tbuf[2], b_t))
        return false;
    auto t2 = std::chrono::high_resolution_clock::now();
    R.rows = m;
    R.cols = n;
    R.nnz = nnz;
    try {
        R.csr_row_ptr.resize(m + 1);
        R.csr_col_indx.resize(nnz);
        R.csr_val.resize(nnz);
        R.csc_col_ptr.resize(n + 1);
        R.csc_row_indx.resize(nnz);
        R.csc_val.resize(nnz);
        T.test_row.resize(nnz_test);
        T.test_col.resize(nnz_test);
        T.test_val.resize(nnz_test);
    } catch (const std::bad_alloc&) {
        fprintf(stderr, "out of host memory for a %ld x %ld matrix with %lu + %lu entries\n", m, n, nnz, nnz_test);
        return false;
    }
    // names 3..8: csr indptr/indices/data, csc indptr/indices/data (src/tools.cpp:318-320)
    if (!read_exact(dir + "/" + buf[3], R.csr_row_ptr.data(), 4 * (m + 1)) ||
        !read_exact(dir + "/" + buf[4], R.csr_col_indx.data(), 4 * nnz) ||
        !read_exact(dir + "/" + buf[5], R.csr_val.data(), 4 * nnz) ||
        !read_exact(dir + "/" + buf[6], R.csc_col_ptr.data(), 4 * (n + 1)) ||
        !read_exact(dir + "/" + buf[7], R.csc_row_indx.data(), 4 * nnz) ||
        !read_exact(dir + "/" + buf[8], R.csc_val.data(), 4 * nnz))
        return false;
    R.max_row_nnz = max_gap(R.csr_row_ptr);
    R.max_col_nnz = max_gap(R.csc_col_ptr);
    auto t3 = std::chrono::high_resolution_clock::now();
    std::chrono::duration<double> dT = t3 - t2;
    std::cout << "[info] Train TIMER: " << dT.count() << "s.\n";
    T.rows = m;
    T.cols = n;
    T.nnz = nnz_test;
    if (!read_exact(dir + "/" + tbuf[0], T.test_val.data(), 4 * nnz_test) ||
        !read_exact(dir + "/" + tbuf[1], T.test_row.data(), 4 * nnz_test) ||
        !read_exact(dir + "/" + tbuf[2], T.test_col.data(), 4 * nnz_test))
        return false;
    auto t5 = std::chrono::high_resolution_clock::now();
    dT = t5 - t3;
    std::cout << "[info] Tests TIMER: " << dT.count() << "s.\n";
    return true;
}

void initial_col(MatData& X, unsigned k, unsigned n) {
    std::vector<float> flat((size_t)k * n);
    cdmf_initial_col(flat.data(), k, n);
    X.assign(k, VecData(n));
    for (unsigned t = 0; t < k; ++t) std::copy(flat.begin() + (size_t)t * n, flat.begin() + (size_t)(t + 1) * n, X[t].begin());
}

static void exit_with_help() {
    printf("Usage: cdmf [options] data_dir\n"
           "options:\n"
           "    -c: path to the kernel code (accepted, unused: kernels are compiled in)\n"
           "    -k rank: set the rank (default 10)\n"
           "    -n threads: set the number of host threads (default 16)\n"
           "    -l lambda: set the regularization parameter lambda (default 0.1)\n"
           "    -t max_outer_iter: set the number of outer iterations (default 5)\n"
           "    -T max_inner_iter: set the number of inner iterations used in CCD (default 5)\n"
           "    -d device_type: select a device (0=gpu) (default 0)\n"
           "    -P platform_id: CUDA device ordinal (default 0)\n"
           "    -q verbose: show information or not (default 0)\n"
           "    -p predict: test RMSE from the meta/test.txt files after training (default 0)\n"
           "    -r compare: re-run in reference summation order and compare (default 0)\n"
           "    -V version: 1 row-length-binned sweeps; 2 the same engine (an alias kept for\n"
           "       the reference's scripts: the bins already give short lines lane groups and\n"
           "       long lines warps or CTAs); 3 nnz-balanced tiles (default 1)\n"
           "    -nBlocks: accepted, unused (grids are sized by the engine)\n"
           "    -nThreadsPerBlock: accepted, unused (default 32)\n"
           "    -residual f32|bf16|f16: residual storage precision (default f32)\n"
           "    -reduce tree|sequential: summation order (default tree)\n"
           "    -graph 0|1: replay outer iterations as CUDA graphs (default 0)\n");
    exit(EXIT_FAILURE);
}

parameter parse_command_line(int argc, char** argv) {
    parameter param{};
    int device_id = 0;
    int i;
    for (i = 1; i < argc; i++) {
        if (argv[i][0] != '-') break;
        if (++i >= argc) exit_with_help();
        const char* flag = argv[i - 1];
        const char* val = argv[i];
        // long flags first: the single-letter switch below looks at flag[1] only
        if (strcmp(flag, "-nBlocks") == 0) {
            param.nBlocks = atoi(val);
        } else if (strcmp(flag, "-nThreadsPerBlock") == 0) {
            param.nThreadsPerBlock = atoi(val);
        } else if (strcmp(flag, "-residual") == 0) {
            if (strcmp(val, "f32") == 0) param.residual = CDMF_RES_F32;
            else if (strcmp(val, "bf16") == 0) param.residual = CDMF_RES_BF16;
            else if (strcmp(val, "f16") == 0) param.residual = CDMF_RES_F16;
            else exit_with_help();
        } else if (strcmp(flag, "-reduce") == 0) {
            if (strcmp(val, "tree") == 0) param.reduce = CDMF_REDUCE_TREE;
            else if (strcmp(val, "sequential") == 0) param.reduce = CDMF_REDUCE_SEQUENTIAL;
            else exit_with_help();
        } else if (strcmp(flag, "-graph") == 0) {
            param.graph = atoi(val);
        } else {
            switch (flag[1]) {
                case 'c': snprintf(param.kcode_path, 1024, "%s", val); break;
                case 'k': param.k = (unsigned)atoi(val); break;
                case 'n': param.threads = atoi(val); break;
                case 'l': param.lambda = (float)atof(val); break;
                case 't': param.maxiter = atoi(val); break;
                case 'T': param.maxinneriter = atoi(val); break;
                case 'P': param.platform_id = (unsigned)atoi(val); break;
                case 'd': device_id = atoi(val); break;
                case 'p': param.do_predict = atoi(val); break;
                case 'r': param.do_ref = atoi(val); break;
                case 'q': param.verbose = atoi(val); break;
                case 'V': param.version = atoi(val); break;
                default:
                    fprintf(stderr, "unknown option: -%c\n", flag[1]);
                    exit_with_help();
            }
        }
    }
    if (device_id != 0) {
        fprintf(stderr, "unknown device type!\n");
        exit_with_help();
    }
    printf("[info] - selected device type: %s, on platform with index: %u | Will be using %d threads | "
           "Value type is %s\n", param.device_type, param.platform_id, param.threads, "float");
    if (i >= argc) exit_with_help();
    snprintf(param.scr_dir, 1024, "%s", argv[i]);
    return param;
}

void golden_compare(const MatData& W, const MatData& W_ref, unsigned k, unsigned m) {
    unsigned error_count = 0;
    for (unsigned i = 0; i < k; i++)
        for (unsigned j = 0; j < m; j++) {
            double delta = fabs(W[i][j] - W_ref[i][j]);
            if (delta > 0.1 * fabs(W_ref[i][j])) error_count++;
        }
    if (error_count == 0) {
        std::cout << "Check... PASS!" << std::endl;
    } else {
        unsigned entries = k * m;
        double pct = 100 * (double)error_count / entries;
        printf("Check... NO PASS! [%f%%] #Error = %u out of %u entries.\n", pct, error_count, entries);
    }
}

bool calculate_rmse(const MatData& W, const MatData& H, const char* srcdir, unsigned k, int device) {
    std::string dir(srcdir);
    FILE* fp = fopen((dir + "/meta").c_str(), "r");
    if (!fp) {
        printf("Can't open meta input file.\n");
        return false;
    }
    char buf_train[1024], buf_test[1024];
    unsigned m, n, nnz, nnz_test;
    bool ok = fscanf(fp, "%u %u", &m, &n) == 2 && fscanf(fp, "%u %1023s", &nnz, buf_train) == 2 &&
              fscanf(fp, "%u %1023s", &nnz_test, buf_test) == 2;
    fclose(fp);
    if (!ok || k > W.size() || k > H.size()) return false;
    for (unsigned t = 0; t < k; ++t)
        if (W[t].size() < m || H[t].size() < n) {
            fprintf(stderr, "meta: %u x %u, but the factors cover %zu x %zu\n", m, n, W[t].size(), H[t].size());
            return false;
        }
    FILE* tf = fopen((dir + "/" + buf_test).c_str(), "r");
    if (!tf) {
        printf("Can't open test file.\n");
        return false;
    }
    std::vector<uint32_t> rows, cols;
    std::vector<double> vals;
    unsigned i, j;
    double v;
    while (fscanf(tf, "%u %u %lf", &i, &j, &v) == 3) {
        rows.push_back(i - 1);   // 1-based in the text file (src/tools.cpp:522)
        cols.push_back(j - 1);
        vals.push_back(v);
    }
    fclose(tf);
    if (rows.empty()) return false;
    std::vector<float> Wf((size_t)k * m), Hf((size_t)k * n);
    for (unsigned t = 0; t < k; ++t) {
        std::copy(W[t].begin(), W[t].begin() + m, Wf.begin() + (size_t)t * m);
        std::copy(H[t].begin(), H[t].begin() + n, Hf.begin() + (size_t)t * n);
    }
    double rmse = 0;
    int64_t nans = 0;
    int st = cdmf_cuda_rmse_coo(k, m, n, Wf.data(), Hf.data(), (int64_t)rows.size(), rows.data(), cols.data(),
                                vals.data(), device, &rmse, &nans);
    if (st != CDMF_OK) {
        fprintf(stderr, "cdmf_cuda_rmse_coo: %s\n", cdmf_cuda_strerror(st));
        return false;
    }
    const int num = (int)rows.size();
    printf("[INFO] NaNs: [%lf%%], NaNs Count: %d out of %d entries.\n", (double)nans / num, (int)nans, num);
    printf("[INFO] Test RMSE = %lf\n", rmse);
    return true;
}
