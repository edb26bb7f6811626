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
        // the reference lists the flags y, x (src/lapl_rect.h:47-49, 81-83)
        const int flags = (F::head == tensor_flag::periodic ? 2 : 0) | (F::tail::head == tensor_flag::periodic ? 1 : 0);
        fdmgpu_verify(fdmgpu_lapl_rect_create_flags(&h_, fdmgpu_dtype<T>::value, method, flags, dx, dy, lx, ly, nx, ny),
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
