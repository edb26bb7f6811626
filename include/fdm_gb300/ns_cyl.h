// Header-only C++ shim: fdm::NSCyl<T,check,zflag> on top of libfdmgpu.so
// (reference: src/ns_cyl.h:18-134).  Constructed from the same Config keys
// ns:{R, r, h1, h2, u0, Re, dt, nr, nz, nphi, vrandom} with the reference's
// defaults (any object with the reference Config's get(section, name,
// default) overloads works); step() and L_step() run on the GPU.  Fields are
// copied to and from host memory in the reference tensor layouts (phi, z, r;
// ghosts included) with field() / set_field(): FDMGPU_NS_U ... FDMGPU_NS_RHS,
// and u0, v0, w0 (the state L_step linearises about) as 9, 10, 11.
#pragma once

#include <cmath>
#include <vector>

#include "lapl_cube.h"

namespace fdm {

template <typename T, bool check, tensor_flag zflag = tensor_flag::none>
class NSCyl {
public:
    template <typename Config>
    explicit NSCyl(const Config& c)
        : R(c.get("ns", "R", M_PI)), r0(c.get("ns", "r", M_PI / 2)), h1(c.get("ns", "h1", 0.0)),
          h2(c.get("ns", "h2", 10.0)), U0(c.get("ns", "u0", 1.0)), Re(c.get("ns", "Re", 1.0)),
          dt(c.get("ns", "dt", 0.001)), nr(c.get("ns", "nr", 32)), nz(c.get("ns", "nz", 31)),
          nphi(c.get("ns", "nphi", 32)) {
        fdmgpu_verify(fdmgpu_nscyl_create(&h_, fdmgpu_dtype<T>::value, zflag == tensor_flag::periodic ? 1 : 0, R, r0,
                                          h1, h2, U0, Re, dt, nr, nz, nphi),
                      "fdmgpu_nscyl_create");
        if (c.get("ns", "vrandom", 0) == 1) fdmgpu_verify(fdmgpu_nscyl_vrandom(h_), "vrandom");
    }
    ~NSCyl() { fdmgpu_nscyl_destroy(h_); }
    NSCyl(const NSCyl&) = delete;
    NSCyl& operator=(const NSCyl&) = delete;

    void step() { fdmgpu_verify(fdmgpu_nscyl_step(h_, 1), "step"); }
    void L_step() { fdmgpu_verify(fdmgpu_nscyl_l_step(h_, 1), "L_step"); }

    std::vector<T> field(int which) const {
        size_t n = 0;
        fdmgpu_verify(fdmgpu_nscyl_field_info(h_, which, &n, nullptr), "field_info");
        std::vector<T> out(n);
        fdmgpu_verify(fdmgpu_nscyl_get_field(h_, which, out.data(), n), "get_field");
        return out;
    }
    void set_field(int which, const std::vector<T>& v) {
        fdmgpu_verify(fdmgpu_nscyl_set_field(h_, which, v.data(), v.size()), "set_field");
    }
    int time_index() const {
        int t = 0;
        fdmgpu_verify(fdmgpu_nscyl_time_index(h_, &t), "time_index");
        return t;
    }

    const double R, r0, h1, h2, U0, Re, dt;
    const int nr, nz, nphi;

private:
    fdmgpu_nscyl* h_ = nullptr;
};

}  // namespace fdm
