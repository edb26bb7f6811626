// Header-only C++ shims: fdm::LaplRect and fdm::LaplRectFFT2 on top of
// libfdmgpu.so (reference: src/lapl_rect.h:11-105).  Host pointers; errors
// abort like the reference's verify().
#pragma once

#include "lapl_cube.h"

namespace fdm {

template <typename T, bool check, typename F = tensor_flags<>>
class LaplRect {
public:
    LaplRect(double dx, double dy, double lx, double ly, int nx, int ny) { create(FDMGPU_RECT_TRIDIAG, dx, dy, lx, ly, nx, ny); }
    ~LaplRect() { fdmgpu_lapl_rect_destroy(h_); }
    LaplRect(const LaplRect&) = delete;
    LaplRect& operator=(const LaplRect&) = delete;
    void solve(T* ans, T* rhs) { fdmgpu_verify(fdmgpu_lapl_rect_solve(h_, ans, rhs), "solve"); }

protected:
    LaplRect() = default;
    void create(int method, double dx, double dy, double lx, double ly, int nx, int ny) {
        if (tensor_flags_mask<F>::value) {
            fprintf(stderr, "verify(periodic LaplRect) failed: not implemented on the GPU\n");
            abort();
        }
        fdmgpu_verify(fdmgpu_lapl_rect_create(&h_, fdmgpu_dtype<T>::value, method, dx, dy, lx, ly, nx, ny),
                      "fdmgpu_lapl_rect_create");
    }
    fdmgpu_lapl_rect* h_ = nullptr;
};

template <typename T, bool check, typename F = tensor_flags<>>
class LaplRectFFT2 : public LaplRect<T, check, F> {
public:
    LaplRectFFT2(double dx, double dy, double lx, double ly, int nx, int ny) {
        this->create(FDMGPU_RECT_FFT2, dx, dy, lx, ly, nx, ny);
    }
};

}  // namespace fdm
