// Header-only C++ shim: fdm::NSCube<T,check> on top of libfdmgpu.so
// (reference: src/ns_cube.h:14-92).  Constructed from the same Config keys
// through a small key/value reader (any object with the reference Config's
// get(section, name, default) overloads works); step() runs on the GPU.
// Fields are copied to host in the reference tensor layout with field().
// T = double is NSCube<double>, T = float NSCube<float>.
#pragma once

#include <cmath>
#include <vector>

#include "lapl_cube.h"

namespace fdm {

template <typename T, bool check>
class NSCube {
public:
    template <typename Config>
    explicit NSCube(const Config& c)
        : x1(c.get("ns", "x1", -M_PI)), y1(c.get("ns", "y1", -M_PI)), z1(c.get("ns", "z1", -M_PI)),
          x2(c.get("ns", "x2", M_PI)), y2(c.get("ns", "y2", M_PI)), z2(c.get("ns", "z2", M_PI)),
          U0(c.get("ns", "u0", 1.0)), Re(c.get("ns", "Re", 1.0)), dt(c.get("ns", "dt", 0.001)),
          nx(c.get("ns", "nx", 32)), ny(c.get("ns", "nx", 32)), nz(c.get("ns", "nz", 32)) {
        fdmgpu_verify(fdmgpu_nscube_create(&h_, fdmgpu_dtype<T>::value, nx, nz, x1, y1, z1, x2, y2, z2, U0, Re, dt),
                      "fdmgpu_nscube_create");
    }
    ~NSCube() { fdmgpu_nscube_destroy(h_); }
    NSCube(const NSCube&) = delete;
    NSCube& operator=(const NSCube&) = delete;

    void step() { fdmgpu_verify(fdmgpu_nscube_step(h_, 1), "step"); }

    // field: FDMGPU_NS_U ... FDMGPU_NS_RHS; whole storage incl. ghost layers
    std::vector<T> field(int which) const {
        size_t n = 0;
        fdmgpu_verify(fdmgpu_nscube_field_info(h_, which, &n, nullptr), "field_info");
        std::vector<T> out(n);
        fdmgpu_verify(fdmgpu_nscube_get_field(h_, which, out.data(), n), "get_field");
        return out;
    }

    const double x1, y1, z1, x2, y2, z2, U0, Re, dt;
    const int nx, ny, nz;

private:
    fdmgpu_nscube* h_ = nullptr;
};

}  // namespace fdm
