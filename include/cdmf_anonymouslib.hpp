// C++ face of the dual SpMV handle for code written against the reference's
// CSR5 library: the member names and call order of anonymouslibHandle
// (src/anonymouslib_opencl.h:11-26), over device pointers instead of cl_mem
// buffers.  Header only; every call forwards to the C ABI in cdmf_cuda.h.
//
//   cdmf::anonymouslibHandle<int, unsigned int, float> A(m, n);
//   A.setCUDAENV(device);              // in place of setOCLENV(context, queue, device)
//   A.inputCSR(nnz, d_row_ptr, d_col_idx, d_val);
//   A.asCSR5();
//   A.setX(d_x);
//   A.spmv(1.0f, d_y_t, d_y_b, &ms);   // y_t = A x, y_b = row sums of x^2
//   A.destroy();
#pragma once

#include <cdmf_cuda.h>

#include <chrono>
#include <type_traits>

namespace cdmf {

template <class IT, class UIT, class VT>
class anonymouslibHandle {
    static_assert(std::is_same<VT, float>::value, "the GPU dual SpMV computes in float");
    static_assert(sizeof(UIT) == 4 && sizeof(IT) == 4, "32-bit row pointers and column indices");

public:
    anonymouslibHandle(IT m, IT n) : m_(m), n_(n) {}
    ~anonymouslibHandle() { cdmf_spmv_destroy(h_); }
    anonymouslibHandle(const anonymouslibHandle&) = delete;
    anonymouslibHandle& operator=(const anonymouslibHandle&) = delete;

    int setCUDAENV(int device) {
        cdmf_spmv_destroy(h_);
        h_ = nullptr;
        return cdmf_spmv_create(m_, n_, device, &h_);
    }
    int warmup() { return h_ ? CDMF_OK : ensure(); }
    int inputCSR(IT nnz, const UIT* row_ptr, const UIT* col_idx, const VT* val) {
        const int r = ensure();
        return r ? r : cdmf_spmv_input_csr(h_, nnz, (const uint32_t*)row_ptr, (const uint32_t*)col_idx, val);
    }
    int asCSR() { return h_ ? cdmf_spmv_as_csr(h_) : CDMF_ERR_INVALID; }
    int asCSR5() { return h_ ? cdmf_spmv_as_csr5(h_) : CDMF_ERR_INVALID; }
    int asCSR_(double* time) { return timed(time, [&] { return asCSR(); }); }
    int asCSR5_(double* time) { return timed(time, [&] { return asCSR5(); }); }
    int setX(const VT* x) { return h_ ? cdmf_spmv_set_x(h_, x) : CDMF_ERR_INVALID; }
    // time: milliseconds of the kernel, as the reference reports through its argument
    int spmv(const VT alpha, VT* y_t, VT* y_b, double* time) {
        return h_ ? cdmf_spmv_run(h_, alpha, y_t, y_b, time) : CDMF_ERR_INVALID;
    }
    int destroy() { return asCSR(); }
    // the reference tunes its tile height sigma; the bins here need no such knob
    int setSigma(int) { return CDMF_OK; }
    const char* lastError() const { return h_ ? cdmf_spmv_last_error(h_) : ""; }

private:
    int ensure() { return h_ ? CDMF_OK : cdmf_spmv_create(m_, n_, 0, &h_); }
    template <class F>
    int timed(double* time, F f) {   // wall milliseconds of a format change
        const auto t0 = std::chrono::steady_clock::now();
        const int r = f();
        if (time) *time = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return r;
    }
    IT m_, n_;
    cdmf_spmv* h_ = nullptr;
};

}  // namespace cdmf
