// A reference-style caller of the C++ shims (include/fdm_gb300/*.h): the
// code a user of fdm::LaplCube / fdm::NSCube keeps, with the include and
// link line changed.  Reads right-hand sides from binary files, writes the
// answers next to them.
//
//   shim_solve dirichlet <nx> <ny> <nz> <dx> <dy> <dz> <lx> <ly> <lz> <rhs> <ans>
//   shim_solve periodic  <nx> <ny> <nz> <dx> <dy> <dz> <lx> <ly> <lz> <rhs> <ans>
//   shim_solve nscube    <n> <steps> <out_u>
//   shim_solve nsdriver  <double|float> <n> <steps> <out>   (the cavity driver)
//   shim_solve cyl       <periodic_z> <nr> <nz> <nphi> <dr> <dz> <r0> <lr> <lz> <rhs> <ans>
//   shim_solve nscyl     <periodic_z> <nr> <nz> <nphi> <steps> <out_u>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fdm_gb300/lapl_cube.h"
#include "fdm_gb300/lapl_cyl.h"
#include "fdm_gb300/ns_cube.h"
#include "fdm_gb300/ns_cyl.h"

namespace {

std::vector<double> read_all(const char* path, size_t n) {
    std::vector<double> v(n);
    FILE* f = fopen(path, "rb");
    if (!f || fread(v.data(), sizeof(double), n, f) != n) {
        fprintf(stderr, "cannot read %s\n", path);
        exit(2);
    }
    fclose(f);
    return v;
}

void write_all(const char* path, const std::vector<double>& v) {
    FILE* f = fopen(path, "wb");
    if (!f || fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(2);
    }
    fclose(f);
}

// the reference's Config::get(section, key, default) shape
struct Cfg {
    int n;
    double Re = 250.0;
    int nr = 0, nz = 0, nphi = 0;
    int steps = 1;
    double get(const char*, const char* key, double def) const {
        if (!strcmp(key, "Re")) return Re;
        if (!strcmp(key, "dt")) return 0.01;
        return def;
    }
    int get(const char*, const char* key, int def) const {
        if (!strcmp(key, "steps")) return steps;
        if (nr) {
            if (!strcmp(key, "nr")) return nr;
            if (!strcmp(key, "nz")) return nz;
            if (!strcmp(key, "nphi")) return nphi;
            return def;
        }
        if (!strcmp(key, "nx") || !strcmp(key, "nz")) return n;
        return def;
    }
};

// The reference's cavity driver (test/test_ns_cube.cpp:21-69) without its
// plotter (plplot): construct from the config, hand the velocity arrays to a
// consumer, step, time.  Writes time_index, dx, dy, dz, the step count and
// ns.u.vec (as doubles) to `out`.
template <typename T, bool check>
void calc(const Cfg& c, const char* out) {
    using namespace std::chrono;
    fdm::NSCube<T, true> ns(c);
    const int steps = c.get("ns", "steps", 1);
    const T* uvec = ns.u.vec;  // what the driver gives plot.use(ns.u.vec, ...)
    auto t1 = steady_clock::now();
    for (int i = 0; i < steps; i++) ns.step();
    auto t2 = steady_clock::now();
    printf("It took me '%f' seconds\n", duration_cast<duration<double>>(t2 - t1).count());
    std::vector<double> o = {(double)ns.time_index, ns.dx, ns.dy, ns.dz, (double)steps,
                             (double)ns.u[ns.nz + 1][3][3]};
    for (int e = 0; e < ns.u.size; e++) o.push_back((double)uvec[e]);
    write_all(out, o);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 1;
    const std::string mode = argv[1];
    if (mode == "nsdriver" && argc == 6) {
        Cfg c{atoi(argv[3])};
        c.steps = atoi(argv[4]);
        if (!strcmp(argv[2], "float")) calc<float, false>(c, argv[5]);
        else calc<double, false>(c, argv[5]);
        return 0;
    }
    if (mode == "nscube" && argc == 5) {
        Cfg c{atoi(argv[2])};
        fdm::NSCube<double, false> ns(c);
        for (int i = 0; i < atoi(argv[3]); i++) ns.step();
        write_all(argv[4], ns.field(FDMGPU_NS_U));
        return 0;
    }
    if (mode == "nscyl" && argc == 8) {
        Cfg c{0};
        c.Re = 100.0;
        c.nr = atoi(argv[3]);
        c.nz = atoi(argv[4]);
        c.nphi = atoi(argv[5]);
        std::vector<double> u;
        if (atoi(argv[2])) {
            fdm::NSCyl<double, false, fdm::tensor_flag::periodic> ns(c);  // src/ns_cyl.h:56
            for (int i = 0; i < atoi(argv[6]); i++) ns.step();
            u = ns.field(FDMGPU_NS_U);
        } else {
            fdm::NSCyl<double, false> ns(c);
            for (int i = 0; i < atoi(argv[6]); i++) ns.step();
            u = ns.field(FDMGPU_NS_U);
        }
        write_all(argv[7], u);
        return 0;
    }
    if (mode == "cyl" && argc == 13) {
        const int pz = atoi(argv[2]), nr = atoi(argv[3]), nz = atoi(argv[4]), nphi = atoi(argv[5]);
        const double dr = atof(argv[6]), dz = atof(argv[7]), r0 = atof(argv[8]), lr = atof(argv[9]),
                     lz = atof(argv[10]);
        std::vector<double> rhs = read_all(argv[11], (size_t)nr * nz * nphi), ans(rhs.size());
        if (pz) {
            fdm::LaplCyl3FFT2<double, false, fdm::tensor_flag::periodic> lapl(dr, dz, r0, lr, lz, nr, nz, nphi);
            lapl.solve(&ans[0], &rhs[0]);
        } else {
            fdm::LaplCyl3FFT2<double, false> lapl(dr, dz, r0, lr, lz, nr, nz, nphi);  // src/lapl_cyl.h:212
            lapl.solve(&ans[0], &rhs[0]);
        }
        write_all(argv[12], ans);
        return 0;
    }
    if (argc != 13) return 1;
    const int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]);
    const double dx = atof(argv[5]), dy = atof(argv[6]), dz = atof(argv[7]);
    const double lx = atof(argv[8]), ly = atof(argv[9]), lz = atof(argv[10]);
    std::vector<double> rhs = read_all(argv[11], (size_t)nx * ny * nz), ans(rhs.size());
    if (mode == "dirichlet") {
        fdm::LaplCube<double, true> lapl(dx, dy, dz, lx, ly, lz, nx, ny, nz);  // src/lapl_cube.h:58
        lapl.solve(&ans[0], &rhs[0]);
    } else if (mode == "periodic") {
        using P = fdm::tensor_flags<fdm::tensor_flag::periodic, fdm::tensor_flag::periodic,
                                    fdm::tensor_flag::periodic>;
        fdm::LaplCube<double, false, P> lapl(dx, dy, dz, lx, ly, lz, nx, ny, nz);
        lapl.solve(&ans[0], &rhs[0]);
    } else {
        return 1;
    }
    write_all(argv[12], ans);
    return 0;
}
