// Header-only C++ shim: fdm::LaplCube<T,check,F> on top of libfdmgpu.so.
//
// Same template parameters, constructor and solve(T* ans, T* rhs) as the
// reference (src/lapl_cube.h:9-106).  Host pointers; the solve runs on the
// GPU.  Errors abort with a verify()-style message, as the reference does
// (src/verify.h:10-36).  `check` only switches bounds checks on the
// reference's tensor accessors and has no effect here.
#pragma once

#include <cstdio>
#include <cstdlib>

#include "../fdmgpu.h"
#include "tensor_flags.h"

namespace fdm {

inline void fdmgpu_verify(int status, const char* what) {
    if (status != FDMGPU_OK) {
        fprintf(stderr, "verify(%s) failed: %s\n", what, fdmgpu_last_error());
        abort();
    }
}

template <typename T> struct fdmgpu_dtype;
template <> struct fdmgpu_dtype<double> { static constexpr int value = FDMGPU_F64; };
template <> struct fdmgpu_dtype<float> { static constexpr int value = FDMGPU_F32; };

template <typename T, bool check, typename F = tensor_flags<>>
class LaplCube {
public:
    const double dx, dy, dz;
    const double lx, ly, lz;
    const int nx, ny, nz;

    LaplCube(double dx, double dy, double dz, double lx, double ly, double lz, int nx, int ny, int nz)
        : dx(dx), dy(dy), dz(dz), lx(lx), ly(ly), lz(lz), nx(nx), ny(ny), nz(nz) {
        const int flags = tensor_flags_mask<F>::value;
        fdmgpu_verify(fdmgpu_lapl_cube_create(&h_, fdmgpu_dtype<T>::value, flags, dx, dy, dz, lx, ly, lz,
                                              nx, ny, nz),
                      "fdmgpu_lapl_cube_create");
    }
    ~LaplCube() { fdmgpu_lapl_cube_destroy(h_); }
    LaplCube(const LaplCube&) = delete;
    LaplCube& operator=(const LaplCube&) = delete;

    // GB300 extension: FP32 inner solves with refinement (T = double only).
    void set_mixed(double tol = 1e-10, int max_sweeps = 3) {
        fdmgpu_verify(fdmgpu_lapl_cube_set_precision(h_, FDMGPU_MIXED, tol, max_sweeps), "set_precision");
    }

    void solve(T* ans, T* rhs) { fdmgpu_verify(fdmgpu_lapl_cube_solve(h_, ans, rhs), "solve"); }

private:
    fdmgpu_lapl_cube* h_ = nullptr;
};

}  // namespace fdm
