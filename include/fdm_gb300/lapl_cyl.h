// Header-only C++ shim: fdm::LaplCyl3FFT2<T,check,zflag,use_cyclic_reduction>
// on top of libfdmgpu.so (reference: src/lapl_cyl.h:172-249).  Same template
// parameters, constructor (dr, dz, r0, lr, lz, nr, nz, nphi) and
// solve(T* ans, T* rhs) over nphi x nz x nr host arrays (r fastest, the
// reference's {0..nphi-1, z1..zn, 1..nr} range).  The radial systems are
// solved on the GPU whichever of the reference's two radial solvers
// use_cyclic_reduction picks.
#pragma once

#include "lapl_cube.h"

namespace fdm {

template <typename T, bool check, tensor_flag zflag = tensor_flag::none, bool use_cyclic_reduction = false>
class LaplCyl3FFT2 {
public:
    const double dr, dz, r0, lr, lz;
    const int nr, nz, nphi;

    LaplCyl3FFT2(double dr, double dz, double r0, double lr, double lz, int nr, int nz, int nphi)
        : dr(dr), dz(dz), r0(r0), lr(lr), lz(lz), nr(nr), nz(nz), nphi(nphi) {
        fdmgpu_verify(fdmgpu_lapl_cyl_create(&h_, fdmgpu_dtype<T>::value, zflag == tensor_flag::periodic ? 1 : 0,
                                             dr, dz, r0, lr, lz, nr, nz, nphi),
                      "fdmgpu_lapl_cyl_create");
    }
    ~LaplCyl3FFT2() { fdmgpu_lapl_cyl_destroy(h_); }
    LaplCyl3FFT2(const LaplCyl3FFT2&) = delete;
    LaplCyl3FFT2& operator=(const LaplCyl3FFT2&) = delete;

    void solve(T* ans, T* rhs) { fdmgpu_verify(fdmgpu_lapl_cyl_solve(h_, ans, rhs), "solve"); }

private:
    fdmgpu_lapl_cyl* h_ = nullptr;
};

}  // namespace fdm
