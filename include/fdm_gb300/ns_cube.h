// Header-only C++ shim: fdm::NSCube<T,check> on top of libfdmgpu.so
// (reference: src/ns_cube.h:14-92, src/ns_cube.cpp:14-62).
//
// Same constructor (any object with the reference Config's
// get(section, name, default) overloads), the same public members (box,
// run constants, dx..dz2, verbose, the tensors u, v, w, p, x, F, G, H, RHS,
// lapl_solver, time_index and the phase-time vectors) and step().  The
// state lives on the GPU; after every step() the nine tensors are copied
// back, so a caller that reads ns.u.vec or ns.u[i][k][j] (as the reference's
// cavity driver does, test/test_ns_cube.cpp:21-69) sees the current fields.
// A caller that changes the host tensors pushes them to the device with
// push() before the next step() (the reference reads its tensors in place).
// T = double is NSCube<double>, T = float NSCube<float>; `check` only
// switches bounds checks in the reference and has no effect here.
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <vector>

#include "lapl_cube.h"

namespace fdm {

// Host copy of one NSCube field in the reference tensor layout
// (src/tensor.h:208-288): inclusive index ranges {z1,z2,y1,y2,x1,x2}, x
// fastest, storage in `storage`, `vec` pointing at its first element,
// t[i][k][j] indexing by the reference's (possibly negative) indices.
template <typename T>
class ns_tensor {
public:
    const std::array<int, 6> offsets;
    const int nxs, nys;  // extents along x and y
    const int size;
    std::vector<T> storage;
    T* vec;

    explicit ns_tensor(const std::array<int, 6>& o)
        : offsets(o), nxs(o[5] - o[4] + 1), nys(o[3] - o[2] + 1), size((o[1] - o[0] + 1) * nys * nxs),
          storage(size), vec(storage.data()) {}
    ns_tensor(const ns_tensor&) = delete;
    ns_tensor& operator=(const ns_tensor&) = delete;

    struct plane {
        T* base;  // element (i, offsets[2], offsets[4])
        const ns_tensor* t;
        T* operator[](int k) const { return base + (k - t->offsets[2]) * t->nxs - t->offsets[4]; }
    };
    plane operator[](int i) { return plane{vec + (i - offsets[0]) * nys * nxs, this}; }
    // flat position of (z, y, x)
    int index(const std::array<int, 3>& zyx) const {
        return ((zyx[0] - offsets[0]) * nys + (zyx[1] - offsets[2])) * nxs + (zyx[2] - offsets[4]);
    }
    T maxabs() const {
        T m = T(0);
        for (int e = 0; e < size; e++) m = std::max(m, (T)std::abs(vec[e]));
        return m;
    }
};

template <typename T, bool check>
class NSCube {
public:
    using tensor = ns_tensor<T>;

    const double x1, y1, z1;
    const double x2, y2, z2;
    const double U0;  // lid velocity
    const double Re;
    const double dt;
    const int nx, ny, nz;
    int verbose;
    const double dx, dy, dz;
    const double dx2, dy2, dz2;

    tensor u, v, w;
    tensor p, x;
    tensor F, G, H, RHS;

    // the pressure solver with the reference's arguments (src/ns_cube.h:77);
    // the device step uses its own plan of the same solver
    LaplCube<T, check> lapl_solver;

    int time_index = 0;

    // The reference times its four phases per step (src/ns_cube.cpp:27-62).
    // On the GPU a step is one graph launch, so step_times holds the time of
    // each step() call (launch, completion and the host copies) and the
    // phase vectors stay empty.
    std::vector<double> init_bound_times;
    std::vector<double> fgh_times;
    std::vector<double> poisson_times;
    std::vector<double> update_times;
    std::vector<double> step_times;

    template <typename Config>
    explicit NSCube(const Config& c)
        : x1(c.get("ns", "x1", -M_PI)), y1(c.get("ns", "y1", -M_PI)), z1(c.get("ns", "z1", -M_PI)),
          x2(c.get("ns", "x2", M_PI)), y2(c.get("ns", "y2", M_PI)), z2(c.get("ns", "z2", M_PI)),
          U0(c.get("ns", "u0", 1.0)), Re(c.get("ns", "Re", 1.0)), dt(c.get("ns", "dt", 0.001)),
          nx(c.get("ns", "nx", 32)), ny(c.get("ns", "nx", 32)), nz(c.get("ns", "nz", 32)),
          verbose(c.get("ns", "verbose", 0)),
          dx((x2 - x1) / nx), dy((y2 - y1) / ny), dz((z2 - z1) / nz),
          dx2(dx * dx), dy2(dy * dy), dz2(dz * dz),
          u({0, nz + 1, 0, ny + 1, -1, nx + 1}), v({0, nz + 1, -1, ny + 1, 0, nx + 1}),
          w({-1, nz + 1, 0, ny + 1, 0, nx + 1}), p({0, nz + 1, 0, ny + 1, 0, nx + 1}),
          x({1, nz, 1, ny, 1, nx}), F({1, nz, 1, ny, 0, nx}), G({1, nz, 0, ny, 1, nx}),
          H({0, nz, 1, ny, 1, nx}), RHS({1, nz, 1, ny, 1, nx}),
          lapl_solver(dx, dy, dz, x2 - x1 + dx, y2 - y1 + dy, z2 - z1 + dz, nx, ny, nz) {
        fdmgpu_verify(fdmgpu_nscube_create(&h_, fdmgpu_dtype<T>::value, nx, nz, x1, y1, z1, x2, y2, z2, U0, Re, dt),
                      "fdmgpu_nscube_create");
        pull();
    }

    ~NSCube() {
        if (verbose) {
            // the reference's summary of repeated timings (src/unixbench_score.cpp:9-20)
            std::vector<double> d = step_times;
            std::sort(d.begin(), d.end());
            const size_t keep = 2 * d.size() / 3;
            double s = 0.0;
            for (size_t i = 0; i < keep; i++) s += std::log(d[i]);
            printf("Step times (ms): step=%.2f (init_bound, FGH, poisson and update_uvwp in one GPU graph)\n",
                   keep ? std::exp(s / keep) : 0.0);
        }
        fdmgpu_nscube_destroy(h_);
    }
    NSCube(const NSCube&) = delete;
    NSCube& operator=(const NSCube&) = delete;

    void step() {
        const auto t0 = std::chrono::high_resolution_clock::now();
        fdmgpu_verify(fdmgpu_nscube_step(h_, 1), "step");
        fdmgpu_verify(fdmgpu_nscube_time_index(h_, &time_index), "time_index");
        pull();
        const auto t1 = std::chrono::high_resolution_clock::now();
        step_times.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }

    // GB300 extensions.  pull(): copy the nine device fields into the host
    // tensors (step() does it).  push(): copy the host tensors to the device
    // (after changing them, e.g. for an initial condition).
    void pull() {
        tensor* t[9] = {&u, &v, &w, &p, &x, &F, &G, &H, &RHS};
        for (int f = 0; f < 9; f++)
            fdmgpu_verify(fdmgpu_nscube_get_field(h_, f, t[f]->vec, (size_t)t[f]->size), "get_field");
    }
    void push() {
        tensor* t[9] = {&u, &v, &w, &p, &x, &F, &G, &H, &RHS};
        for (int f = 0; f < 9; f++)
            fdmgpu_verify(fdmgpu_nscube_set_field(h_, f, t[f]->vec, (size_t)t[f]->size), "set_field");
    }

    // field: FDMGPU_NS_U ... FDMGPU_NS_RHS; whole storage incl. ghost layers
    std::vector<T> field(int which) const {
        size_t n = 0;
        fdmgpu_verify(fdmgpu_nscube_field_info(h_, which, &n, nullptr), "field_info");
        std::vector<T> out(n);
        fdmgpu_verify(fdmgpu_nscube_get_field(h_, which, out.data(), n), "get_field");
        return out;
    }

private:
    fdmgpu_nscube* h_ = nullptr;
};

}  // namespace fdm
