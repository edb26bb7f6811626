// NSCyl: incompressible flow between two coaxial cylinders (inner one
// rotating), the projection step of fdm::NSCyl<T,check,zflag>
// (src/ns_cyl.h:18-134, src/ns_cyl.cpp:22-485), on the GPU.
//
// Fields keep the reference layouts: (phi, z, r) with r fastest, phi
// periodic, z Dirichlet (ghost layers) or periodic (zflag), inclusive index
// ranges of src/ns_cyl.h:79-91.  A step is init_bound (three phases: radial
// ghosts; axial ghosts; pressure ghosts, each phase reading only what an
// earlier one wrote), FGH, the divergence right-hand side, the cylindrical
// Poisson solve (LaplCyl3FFT2, poisson.cu) and the update, captured into a
// CUDA graph after the first eager step.  Every expression is written in
// the reference's order of operations; divisions by run constants and by
// the per-column radii go through precomputed correctly rounded reciprocals
// with two remainder corrections (bit-identical to IEEE division).
#include <cmath>
#include <cstdio>
#include <memory>
#include <random>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "poisson.h"

namespace fdmgpu {

namespace cyl {

__device__ __forceinline__ double sq(double x) { return x * x; }  // asp::sq, src/asp_misc.h:295

template <typename T>
struct Field {
    T* p;
    int z1, z2, x1, x2;  // inclusive z and r ranges; phi is 0..nphi-1
    int nphi;
    int zper;
    long long sy, sz, size;
    // periodic wrap of phi (and of z when periodic), one period away at most
    __host__ __device__ T& operator()(int i, int k, int j) const {
        i = i < 0 ? i + nphi : (i >= nphi ? i - nphi : i);
        if (zper) {
            const int n = z2 - z1 + 1;
            k = k < z1 ? k + n : (k > z2 ? k - n : k);
        }
        return p[(long long)i * sz + (long long)(k - z1) * sy + (j - x1)];
    }
};

template <typename T>
static Field<T> make(int nphi, int zper, int z1, int z2, int x1, int x2) {
    Field<T> f;
    f.p = nullptr;
    f.z1 = z1; f.z2 = z2; f.x1 = x1; f.x2 = x2; f.nphi = nphi; f.zper = zper;
    f.sy = x2 - x1 + 1;
    f.sz = f.sy * (z2 - z1 + 1);
    f.size = f.sz * nphi;
    return f;
}

constexpr int kMaxR = 4096;

struct Params {
    int nr, nz, nphi, zper;
    int z_, z0, z1, zn, znn;
    double r0, dr, dz, dphi, dr2, dz2, dphi2, Re, dt, U0;
    CDiv dRe, ddr, ddz, ddphi, ddr2, ddz2, ddphi2, ddt;
    double dt_dr, dt_dz;
};

// per radial index j: face radius (F) and centre radius (G, H, RHS, w)
struct Radii {
    double rf, rf2, rf1, rfr, rc, rc2, rc1, rcr, dtdphi_r;
    CDiv drf, drfr, drc, drcr;
};

// ---- init_bound (src/ns_cyl.cpp:80-171) ------------------------------------
// phase A: radial ghosts of w, v (inner wall moves with U0) and u
template <typename T>
__global__ void k_bound_a(Field<T> u, Field<T> v, Field<T> w, Params P) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nk = P.znn - P.z_ + 1;
    if (e >= (long long)P.nphi * nk) return;
    const int i = (int)(e / nk), k = (int)(e % nk) + P.z_;
    const int nr = P.nr;
    if (k >= P.z0) {
        w(i, k, 0) = 2 * P.U0 - w(i, k, 1);  // inner
        w(i, k, nr + 1) = -w(i, k, nr);      // outer
        u(i, k, -1) = u(i, k, 1);
        u(i, k, nr + 1) = u(i, k, nr - 1);
    }
    v(i, k, 0) = -v(i, k, 1);
    v(i, k, nr + 1) = -v(i, k, nr);
}

// phase B (Dirichlet z): axial ghosts.  The reference runs the r index of
// the v loop over the z bounds z0..znn (src/ns_cyl.cpp:106-111); kept, with
// nz <= nr required so that it stays inside the row.
template <typename T>
__global__ void k_bound_b(Field<T> u, Field<T> v, Field<T> w, Params P) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nj = P.nr + 3;  // j = -1..nr+1
    if (e >= (long long)P.nphi * nj) return;
    const int i = (int)(e / nj), j = (int)(e % nj) - 1;
    const int nz = P.nz, nr = P.nr;
    if (j >= P.z0 && j <= P.znn) {
        v(i, -1, j) = v(i, 1, j);
        v(i, nz + 1, j) = v(i, nz - 1, j);
    }
    u(i, 0, j) = -u(i, 1, j);
    u(i, nz + 1, j) = -u(i, nz, j);
    if (j >= 0) {
        w(i, 0, j) = -w(i, 1, j);
        w(i, nz + 1, j) = -w(i, nz, j);
    }
    (void)nr;
}

// phase C: pressure ghosts
template <typename T>
__global__ void k_bound_c(Field<T> u, Field<T> v, Field<T> p, Params P) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nk = P.zn - P.z1 + 1;
    const int nr = P.nr, nz = P.nz;
    const long long n1 = (long long)P.nphi * nk;
    const long long n2 = P.zper ? 0 : (long long)P.nphi * nr;
    if (e < n1) {
        const int i = (int)(e / nk), k = (int)(e % nk) + P.z1;
        int j = 0;
        double r = P.r0 + j * P.dr - P.dr / 2;
        p(i, k, 0) = p(i, k, 1) - cdiv(cdiv((r + 0.5 * P.dr) * u(i, k, 1) / r - 2 * u(i, k, 0) +
                                                 (r - 0.5 * P.dr) * u(i, k, -1) / r,
                                             P.dRe),
                                        P.ddr);
        j = nr;
        r = P.r0 + j * P.dr - P.dr / 2;
        p(i, k, nr + 1) = p(i, k, nr) + cdiv(cdiv((r + 0.5 * P.dr) * u(i, k, nr + 1) / r - 2 * u(i, k, nr) +
                                                      (r - 0.5 * P.dr) * u(i, k, nr - 1) / r,
                                                  P.dRe),
                                             P.ddr);
    } else if (e < n1 + n2) {
        const long long f = e - n1;
        const int i = (int)(f / nr), j = (int)(f % nr) + 1;
        p(i, 0, j) = p(i, 1, j) - cdiv(cdiv(v(i, 1, j) - 2 * v(i, 0, j) + v(i, -1, j), P.dRe), P.ddz);
        p(i, nz + 1, j) = p(i, nz, j) + cdiv(cdiv(v(i, nz + 1, j) - 2 * v(i, nz, j) + v(i, nz - 1, j), P.dRe), P.ddz);
    }
}

// ---- FGH (src/ns_cyl.cpp:174-277) ------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_fgh(Field<T> u, Field<T> v, Field<T> w, Field<T> F, Field<T> G,
                                             Field<T> H, Params P, const Radii* __restrict__ R) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nj = P.nr + 1, nk = P.zn - P.z0 + 1;
    if (e >= (long long)P.nphi * nk * nj) return;
    const int j = (int)(e % nj);
    const int k = (int)((e / nj) % nk) + P.z0;
    const int i = (int)(e / ((long long)nj * nk));
    const double dt = P.dt;
    auto dif = [&](double x, CDiv d2) { return cdiv(cdiv(x, P.dRe), d2); };
    if (k >= P.z1) {
        // F (r), faces j = 0..nr: r = r0 + dr j
        const Radii& q = R[j];
        const double r = q.rf, r2 = q.rf2, r1 = q.rf1;
        F(i, k, j) = u(i, k, j) + dt * (
            dif(r2 * u(i, k, j + 1) - 2 * u(i, k, j) + r1 * u(i, k, j - 1), P.ddr2) +
            dif(u(i, k + 1, j) - 2 * u(i, k, j) + u(i, k - 1, j), P.ddz2) +
            cdiv(dif(u(i + 1, k, j) - 2 * u(i, k, j) + u(i - 1, k, j), P.ddphi2), q.drfr) -
            cdiv(r2 * sq(0.5 * (u(i, k, j) + u(i, k, j + 1))) - r1 * sq(0.5 * (u(i, k, j - 1) + u(i, k, j))), P.ddr) -
            cdiv(0.25 * ((u(i, k, j) + u(i, k + 1, j)) * (v(i, k, j + 1) + v(i, k, j)) -
                         (u(i, k - 1, j) + u(i, k, j)) * (v(i, k - 1, j + 1) + v(i, k - 1, j))),
                 P.ddz) -
            cdiv(cdiv(0.25 * ((u(i, k, j) + u(i + 1, k, j)) * (w(i, k, j + 1) + w(i, k, j)) -
                              (u(i - 1, k, j) + u(i, k, j)) * (w(i - 1, k, j + 1) + w(i - 1, k, j))),
                      P.ddphi),
                 q.drf)
            + cdiv(sq(0.5 * (w(i, k, j + 1) + w(i, k, j))), q.drf) - cdiv(cdiv(u(i, k, j), q.drfr), P.dRe)
            - cdiv(cdiv(cdiv(2 * (0.5 * (w(i, k, j + 1) + w(i, k, j)) - 0.5 * (w(i - 1, k, j + 1) + w(i - 1, k, j))),
                             q.drfr),
                        P.ddphi),
                   P.dRe));
    }
    if (j >= 1) {
        const Radii& q = R[j];
        const double r2 = q.rc2, r1 = q.rc1;
        // G (z), k = z0..zn
        G(i, k, j) = v(i, k, j) + dt * (
            dif(r2 * v(i, k, j + 1) - 2 * v(i, k, j) + r1 * v(i, k, j - 1), P.ddr2) +
            dif(v(i, k + 1, j) - 2 * v(i, k, j) + v(i, k - 1, j), P.ddz2) +
            cdiv(dif(v(i + 1, k, j) - 2 * v(i, k, j) + v(i - 1, k, j), P.ddphi2), q.drcr) -
            cdiv(sq(0.5 * (v(i, k, j) + v(i, k + 1, j))) - sq(0.5 * (v(i, k - 1, j) + v(i, k, j))), P.ddz) -
            cdiv(0.25 * (r2 * (u(i, k, j) + u(i, k + 1, j)) * (v(i, k, j + 1) + v(i, k, j)) -
                         r1 * (u(i, k, j - 1) + u(i, k + 1, j - 1)) * (v(i, k, j) + v(i, k, j - 1))),
                 P.ddr) -
            cdiv(cdiv(0.25 * ((w(i, k, j) + w(i, k + 1, j)) * (v(i, k, j) + v(i + 1, k, j)) -
                              (w(i - 1, k, j) + w(i - 1, k + 1, j)) * (v(i - 1, k, j) + v(i, k, j))),
                      P.ddphi),
                 q.drc));
        if (k >= P.z1) {
            // H (phi)
            H(i, k, j) = w(i, k, j) + dt * (
                dif(r2 * w(i, k, j + 1) - 2 * w(i, k, j) + r1 * w(i, k, j - 1), P.ddr2) +
                dif(w(i, k + 1, j) - 2 * w(i, k, j) + w(i, k - 1, j), P.ddz2) +
                cdiv(dif(w(i + 1, k, j) - 2 * w(i, k, j) + w(i - 1, k, j), P.ddphi2), q.drcr) -
                cdiv(cdiv(sq(0.5 * (w(i + 1, k, j) + w(i, k, j))) - sq(0.5 * (w(i - 1, k, j) + w(i, k, j))), P.ddphi),
                     q.drc) -
                cdiv(0.25 * (r2 * (u(i + 1, k, j) + u(i, k, j)) * (w(i, k, j + 1) + w(i, k, j)) -
                             r1 * (u(i + 1, k, j - 1) + u(i, k, j - 1)) * (w(i, k, j) + w(i, k, j - 1))),
                     P.ddr) -
                cdiv(0.25 * ((w(i, k, j) + w(i, k + 1, j)) * (v(i, k, j) + v(i + 1, k, j)) -
                             (w(i, k - 1, j) + w(i, k, j)) * (v(i, k - 1, j) + v(i + 1, k - 1, j))),
                     P.ddz)
                - cdiv(w(i, k, j) * 0.5 * (u(i + 1, k, j) + u(i, k, j)), q.drc) - cdiv(cdiv(w(i, k, j), q.drcr), P.dRe)
                + cdiv(cdiv(cdiv(2 * (0.5 * (u(i + 1, k, j) + u(i, k, j)) - 0.5 * (u(i, k, j) + u(i - 1, k, j))),
                                 q.drcr),
                            P.ddphi),
                       P.dRe));
        }
    }
}

// ---- L_FGH (src/ns_cyl.cpp:279-404): FGH linearised about (u0, v0, w0) ----
// The reference's expressions term for term (including its
// (0.5*u[j] + u[j+1]) factor in the radial advection of F), with the same
// correctly rounded constant and radius divisions as k_fgh.
template <typename T>
__global__ void __launch_bounds__(256) k_lfgh(Field<T> u, Field<T> v, Field<T> w, Field<T> u0, Field<T> v0,
                                              Field<T> w0, Field<T> F, Field<T> G, Field<T> H, Params P,
                                              const Radii* __restrict__ R) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nj = P.nr + 1, nk = P.zn - P.z0 + 1;
    if (e >= (long long)P.nphi * nk * nj) return;
    const int j = (int)(e % nj);
    const int k = (int)((e / nj) % nk) + P.z0;
    const int i = (int)(e / ((long long)nj * nk));
    const double dt = P.dt;
    auto dif = [&](double x, CDiv d2) { return cdiv(cdiv(x, P.dRe), d2); };
    if (k >= P.z1) {
        const Radii& q = R[j];
        const double r2 = q.rf2, r1 = q.rf1;
        F(i, k, j) = u(i, k, j) + dt * (
            dif(r2 * u(i, k, j + 1) - 2 * u(i, k, j) + r1 * u(i, k, j - 1), P.ddr2) +
            dif(u(i, k + 1, j) - 2 * u(i, k, j) + u(i, k - 1, j), P.ddz2) +
            cdiv(dif(u(i + 1, k, j) - 2 * u(i, k, j) + u(i - 1, k, j), P.ddphi2), q.drfr) -
            cdiv(r2 * (0.5 * u(i, k, j) + u(i, k, j + 1)) * (u0(i, k, j) + u0(i, k, j + 1)) -
                     r1 * (0.5 * u(i, k, j - 1) + u(i, k, j)) * (u0(i, k, j - 1) + u0(i, k, j)),
                 P.ddr) -
            cdiv(0.25 * ((u(i, k, j) + u(i, k + 1, j)) * (v0(i, k, j + 1) + v0(i, k, j)) -
                         (u(i, k - 1, j) + u(i, k, j)) * (v0(i, k - 1, j + 1) + v0(i, k - 1, j))),
                 P.ddz) -
            cdiv(0.25 * ((u0(i, k, j) + u0(i, k + 1, j)) * (v(i, k, j + 1) + v(i, k, j)) -
                         (u0(i, k - 1, j) + u0(i, k, j)) * (v(i, k - 1, j + 1) + v(i, k - 1, j))),
                 P.ddz) -
            cdiv(cdiv(0.25 * ((u(i, k, j) + u(i + 1, k, j)) * (w0(i, k, j + 1) + w0(i, k, j)) -
                              (u(i - 1, k, j) + u(i, k, j)) * (w0(i - 1, k, j + 1) + w0(i - 1, k, j))),
                      P.ddphi),
                 q.drf) -
            cdiv(cdiv(0.25 * ((u0(i, k, j) + u0(i + 1, k, j)) * (w(i, k, j + 1) + w(i, k, j)) -
                              (u0(i - 1, k, j) + u0(i, k, j)) * (w(i - 1, k, j + 1) + w(i - 1, k, j))),
                      P.ddphi),
                 q.drf)
            + cdiv(0.5 * (w(i, k, j + 1) + w(i, k, j)) * (w0(i, k, j + 1) + w0(i, k, j)), q.drf)
            - cdiv(cdiv(u(i, k, j), q.drfr), P.dRe)
            - cdiv(cdiv(cdiv(2 * (0.5 * (w(i, k, j + 1) + w(i, k, j)) - 0.5 * (w(i - 1, k, j + 1) + w(i - 1, k, j))),
                             q.drfr),
                        P.ddphi),
                   P.dRe));
    }
    if (j >= 1) {
        const Radii& q = R[j];
        const double r2 = q.rc2, r1 = q.rc1;
        G(i, k, j) = v(i, k, j) + dt * (
            dif(r2 * v(i, k, j + 1) - 2 * v(i, k, j) + r1 * v(i, k, j - 1), P.ddr2) +
            dif(v(i, k + 1, j) - 2 * v(i, k, j) + v(i, k - 1, j), P.ddz2) +
            cdiv(dif(v(i + 1, k, j) - 2 * v(i, k, j) + v(i - 1, k, j), P.ddphi2), q.drcr) -
            cdiv(0.5 * (v(i, k, j) + v(i, k + 1, j)) * (v0(i, k, j) + v0(i, k + 1, j)) -
                     0.5 * (v(i, k - 1, j) + v(i, k, j)) * (v0(i, k - 1, j) + v0(i, k, j)),
                 P.ddz) -
            cdiv(0.25 * (r2 * (u(i, k, j) + u(i, k + 1, j)) * (v0(i, k, j + 1) + v0(i, k, j)) -
                         r1 * (u(i, k, j - 1) + u(i, k + 1, j - 1)) * (v0(i, k, j) + v0(i, k, j - 1))),
                 P.ddr) -
            cdiv(0.25 * (r2 * (u0(i, k, j) + u0(i, k + 1, j)) * (v(i, k, j + 1) + v(i, k, j)) -
                         r1 * (u0(i, k, j - 1) + u0(i, k + 1, j - 1)) * (v(i, k, j) + v(i, k, j - 1))),
                 P.ddr) -
            cdiv(cdiv(0.25 * ((w(i, k, j) + w(i, k + 1, j)) * (v0(i, k, j) + v0(i + 1, k, j)) -
                              (w(i - 1, k, j) + w(i - 1, k + 1, j)) * (v0(i - 1, k, j) + v0(i, k, j))),
                      P.ddphi),
                 q.drc) -
            cdiv(cdiv(0.25 * ((w0(i, k, j) + w0(i, k + 1, j)) * (v(i, k, j) + v(i + 1, k, j)) -
                              (w0(i - 1, k, j) + w0(i - 1, k + 1, j)) * (v(i - 1, k, j) + v(i, k, j))),
                      P.ddphi),
                 q.drc));
        if (k >= P.z1) {
            H(i, k, j) = w(i, k, j) + dt * (
                dif(r2 * w(i, k, j + 1) - 2 * w(i, k, j) + r1 * w(i, k, j - 1), P.ddr2) +
                dif(w(i, k + 1, j) - 2 * w(i, k, j) + w(i, k - 1, j), P.ddz2) +
                cdiv(dif(w(i + 1, k, j) - 2 * w(i, k, j) + w(i - 1, k, j), P.ddphi2), q.drcr) -
                cdiv(cdiv(0.5 * (w(i + 1, k, j) + w(i, k, j)) * (w0(i + 1, k, j) + w0(i, k, j)) -
                              0.5 * (w(i - 1, k, j) + w(i, k, j)) * (w0(i - 1, k, j) + w0(i, k, j)),
                          P.ddphi),
                     q.drc) -
                cdiv(0.25 * (r2 * (u(i + 1, k, j) + u(i, k, j)) * (w0(i, k, j + 1) + w0(i, k, j)) -
                             r1 * (u(i + 1, k, j - 1) + u(i, k, j - 1)) * (w0(i, k, j) + w0(i, k, j - 1))),
                     P.ddr) -
                cdiv(0.25 * (r2 * (u0(i + 1, k, j) + u0(i, k, j)) * (w(i, k, j + 1) + w(i, k, j)) -
                             r1 * (u0(i + 1, k, j - 1) + u0(i, k, j - 1)) * (w(i, k, j) + w(i, k, j - 1))),
                     P.ddr) -
                cdiv(0.25 * ((w(i, k, j) + w(i, k + 1, j)) * (v0(i, k, j) + v0(i + 1, k, j)) -
                             (w(i, k - 1, j) + w(i, k, j)) * (v0(i, k - 1, j) + v0(i + 1, k - 1, j))),
                     P.ddz) -
                cdiv(0.25 * ((w0(i, k, j) + w0(i, k + 1, j)) * (v(i, k, j) + v(i + 1, k, j)) -
                             (w0(i, k - 1, j) + w0(i, k, j)) * (v(i, k - 1, j) + v(i + 1, k - 1, j))),
                     P.ddz)
                - cdiv(w0(i, k, j) * 0.5 * (u(i + 1, k, j) + u(i, k, j)), q.drc)
                - cdiv(w(i, k, j) * 0.5 * (u0(i + 1, k, j) + u0(i, k, j)), q.drc)
                - cdiv(cdiv(w(i, k, j), q.drcr), P.dRe)
                + cdiv(cdiv(cdiv(2 * (0.5 * (u(i + 1, k, j) + u(i, k, j)) - 0.5 * (u(i, k, j) + u(i - 1, k, j))),
                                 q.drcr),
                            P.ddphi),
                       P.dRe));
        }
    }
}

// ---- poisson right-hand side (src/ns_cyl.cpp:407-441) ----------------------
template <typename T>
__global__ void k_rhs(Field<T> F, Field<T> G, Field<T> H, Field<T> p, Field<T> RHS, Params P,
                      const Radii* __restrict__ R) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = P.nr, nk = P.zn - P.z1 + 1;
    if (e >= (long long)P.nphi * nk * nr) return;
    const int j = (int)(e % nr) + 1;
    const int k = (int)((e / nr) % nk) + P.z1;
    const int i = (int)(e / ((long long)nr * nk));
    const Radii& q = R[j];
    const double r = q.rc;
    // T-typed like the reference element: rounded after each update
    T x = cdiv(cdiv(cdiv((r + 0.5 * P.dr) * F(i, k, j) - (r - 0.5 * P.dr) * F(i, k, j - 1), q.drc), P.ddr) +
                   cdiv(G(i, k, j) - G(i, k - 1, j), P.ddz) + cdiv(cdiv(H(i, k, j) - H(i - 1, k, j), P.ddphi), q.drc),
               P.ddt);
    if (!P.zper && k <= 1) x -= cdiv(p(i, k - 1, j), P.ddz2);
    if (j <= 1) x -= cdiv(cdiv((r - P.dr / 2), q.drc) * p(i, k, j - 1), P.ddr2);
    if (j >= nr) x -= cdiv(cdiv((r + P.dr / 2), q.drc) * p(i, k, j + 1), P.ddr2);
    if (!P.zper && k >= P.nz) x -= cdiv(p(i, k + 1, j), P.ddz2);
    RHS(i, k, j) = x;
}

// ---- update_uvwp (src/ns_cyl.cpp:444-483) ----------------------------------
template <typename T>
__global__ void k_update(Field<T> u, Field<T> v, Field<T> w, Field<T> p, Field<T> x, Field<T> F, Field<T> G,
                         Field<T> H, Params P, const Radii* __restrict__ R) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nr = P.nr, nk = P.zn - P.z1 + 1;
    if (e >= (long long)P.nphi * nk * nr) return;
    const int j = (int)(e % nr) + 1;
    const int k = (int)((e / nr) % nk) + P.z1;
    const int i = (int)(e / ((long long)nr * nk));
    const T xc = x(i, k, j);
    if (j < nr) u(i, k, j) = F(i, k, j) - P.dt_dr * (x(i, k, j + 1) - xc);
    if (k < P.nz) v(i, k, j) = G(i, k, j) - P.dt_dz * (x(i, k + 1, j) - xc);
    w(i, k, j) = H(i, k, j) - R[j].dtdphi_r * (x(i + 1, k, j) - xc);
    p(i, k, j) = xc;
}

}  // namespace cyl

template <typename T>
struct NSCylPlan {
    cyl::Params P;
    // u v w p x F G H RHS, then the linearisation point u0 v0 w0 of L_step
    // (src/ns_cyl.h:40-41, the layouts of u, v, w)
    cyl::Field<T> f[12];
    void* mem = nullptr;
    DevBuf radii;
    fdmgpu_lapl_cyl* lapl = nullptr;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr, lgraph = nullptr;
    cudaGraphExec_t gexec = nullptr, lgexec = nullptr;
    int time_index = 0;
    int steps_run = 0, lsteps_run = 0;

    ~NSCylPlan() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        if (lgexec) cudaGraphExecDestroy(lgexec);
        if (lgraph) cudaGraphDestroy(lgraph);
        if (lapl) fdmgpu_lapl_cyl_destroy(lapl);
        if (mem) cudaFree(mem);
        if (st) cudaStreamDestroy(st);
    }

    void init(double R, double r0, double h1, double h2) {
        const int nr = P.nr, nz = P.nz, nphi = P.nphi, zp = P.zper;
        // index ranges of src/ns_cyl.h:79-91
        f[0] = cyl::make<T>(nphi, zp, P.z0, P.znn, -1, nr + 1);
        f[1] = cyl::make<T>(nphi, zp, P.z_, P.znn, 0, nr + 1);
        f[2] = cyl::make<T>(nphi, zp, P.z0, P.znn, 0, nr + 1);
        f[3] = cyl::make<T>(nphi, zp, P.z0, P.znn, 0, nr + 1);
        f[4] = cyl::make<T>(nphi, zp, P.z1, P.zn, 1, nr);
        f[5] = cyl::make<T>(nphi, zp, P.z1, P.zn, 0, nr);
        f[6] = cyl::make<T>(nphi, zp, P.z0, P.zn, 1, nr);
        f[7] = cyl::make<T>(nphi, zp, P.z1, P.zn, 1, nr);
        f[8] = cyl::make<T>(nphi, zp, P.z1, P.zn, 1, nr);
        f[9] = f[0];
        f[10] = f[1];
        f[11] = f[2];
        size_t total = 0;
        for (auto& fi : f) total += (size_t)((fi.size + 31) / 32 * 32);
        FDM_CUDA(cudaMalloc(&mem, total * sizeof(T)));
        FDM_CUDA(cudaMemset(mem, 0, total * sizeof(T)));
        size_t off = 0;
        for (auto& fi : f) {
            fi.p = (T*)mem + off;
            off += (size_t)((fi.size + 31) / 32 * 32);
        }
        std::vector<cyl::Radii> rv(nr + 2);
        for (int j = 0; j <= nr + 1; j++) {
            cyl::Radii& q = rv[j];
            q.rf = P.r0 + P.dr * j;  // F: r = r0 + dr j (src/ns_cyl.cpp:182)
            q.rf2 = (q.rf + 0.5 * P.dr) / q.rf;
            q.rf1 = (q.rf - 0.5 * P.dr) / q.rf;
            q.rfr = q.rf * q.rf;
            q.rc = P.r0 + P.dr * j - P.dr / 2;  // G, H, RHS: r = r0 + dr j - dr/2
            q.rc2 = (q.rc + 0.5 * P.dr) / q.rc;
            q.rc1 = (q.rc - 0.5 * P.dr) / q.rc;
            q.rcr = q.rc * q.rc;
            q.dtdphi_r = P.dt / P.dphi / q.rc;
            q.drf = cdiv_of(q.rf);
            q.drfr = cdiv_of(q.rfr);
            q.drc = cdiv_of(q.rc);
            q.drcr = cdiv_of(q.rcr);
        }
        FDM_CUDA(cudaMemcpy(radii.get(rv.size() * sizeof(cyl::Radii)), rv.data(), rv.size() * sizeof(cyl::Radii),
                            cudaMemcpyHostToDevice));
        FDM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        // LaplCyl3FFT2(dr, dz, r0-dr/2, R-r0+dr, lz, nr, nz, nphi), src/ns_cyl.h:93-96
        const double lz = zp ? h2 - h1 : h2 - h1 + P.dz;
        int rc = fdmgpu_lapl_cyl_create(&lapl, sizeof(T) == 8 ? FDMGPU_F64 : FDMGPU_F32, zp, P.dr, P.dz,
                                        r0 - P.dr / 2, R - r0 + P.dr, lz, nr, nz, nphi);
        if (rc) throw Error{rc};
    }

    void enqueue_step(bool linear = false) {
        const int B = 256;
        auto blocks = [&](long long n) { return (unsigned)((n + B - 1) / B); };
        const int nr = P.nr, nphi = P.nphi;
        const cyl::Radii* R = (const cyl::Radii*)radii.p;
        {
            FDM_TIMED("cyl_bound", st);
            cyl::k_bound_a<T><<<blocks((long long)nphi * (P.znn - P.z_ + 1)), B, 0, st>>>(f[0], f[1], f[2], P);
            FDM_LAUNCH_CHECK();
            if (!P.zper) {
                cyl::k_bound_b<T><<<blocks((long long)nphi * (nr + 3)), B, 0, st>>>(f[0], f[1], f[2], P);
                FDM_LAUNCH_CHECK();
            }
            const long long nc = (long long)nphi * (P.zn - P.z1 + 1) + (P.zper ? 0 : (long long)nphi * nr);
            cyl::k_bound_c<T><<<blocks(nc), B, 0, st>>>(f[0], f[1], f[3], P);
            FDM_LAUNCH_CHECK();
        }
        if (!linear) {
            FDM_TIMED("cyl_fgh", st);
            cyl::k_fgh<T><<<blocks((long long)nphi * (P.zn - P.z0 + 1) * (nr + 1)), B, 0, st>>>(
                f[0], f[1], f[2], f[5], f[6], f[7], P, R);
            FDM_LAUNCH_CHECK();
        } else {
            FDM_TIMED("cyl_lfgh", st);
            cyl::k_lfgh<T><<<blocks((long long)nphi * (P.zn - P.z0 + 1) * (nr + 1)), B, 0, st>>>(
                f[0], f[1], f[2], f[9], f[10], f[11], f[5], f[6], f[7], P, R);
            FDM_LAUNCH_CHECK();
        }
        const long long cells = (long long)nphi * (P.zn - P.z1 + 1) * nr;
        {
            FDM_TIMED("cyl_rhs", st);
            cyl::k_rhs<T><<<blocks(cells), B, 0, st>>>(f[5], f[6], f[7], f[3], f[8], P, R);
            FDM_LAUNCH_CHECK();
        }
        cyl_solve_device(lapl, f[4].p, f[8].p, 1, st);
        {
            FDM_TIMED("cyl_update", st);
            cyl::k_update<T><<<blocks(cells), B, 0, st>>>(f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], P, R);
            FDM_LAUNCH_CHECK();
        }
    }

    // step() (linear = false) or L_step() (linear = true): the first of each
    // kind runs eagerly, later ones replay its captured graph
    void step(int k, bool linear = false) {
        int& run = linear ? lsteps_run : steps_run;
        cudaGraph_t& g_ = linear ? lgraph : graph;
        cudaGraphExec_t& ge = linear ? lgexec : gexec;
        for (int s = 0; s < k; s++) {
            if (run == 0) {
                enqueue_step(linear);
            } else {
                if (!ge) {
                    FDM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                    try {
                        enqueue_step(linear);
                    } catch (...) {
                        cudaGraph_t g = nullptr;
                        cudaStreamEndCapture(st, &g);
                        if (g) cudaGraphDestroy(g);
                        throw;
                    }
                    FDM_CUDA(cudaStreamEndCapture(st, &g_));
                    FDM_CUDA(cudaGraphInstantiate(&ge, g_, 0));
                }
                FDM_CUDA(cudaGraphLaunch(ge, st));
            }
            run++;
            time_index++;
        }
    }

    // the constructor's ns:vrandom=1 perturbation (src/ns_cyl.h:99-109): v
    // over phi, z1..zn, r 1..nr drawn in that order from the standard
    // library's default engine, uniform in [-1e-3, 1e-3) in T
    void vrandom() {
        const auto& v = f[1];
        std::vector<T> host((size_t)v.size);
        FDM_CUDA(cudaStreamSynchronize(st));
        FDM_CUDA(cudaMemcpy(host.data(), v.p, host.size() * sizeof(T), cudaMemcpyDeviceToHost));
        std::default_random_engine gen;
        std::uniform_real_distribution<T> dist(-1e-3, 1e-3);
        for (int i = 0; i < P.nphi; i++)
            for (int k = P.z1; k <= P.zn; k++)
                for (int j = 1; j <= P.nr; j++)
                    host[(size_t)i * v.sz + (size_t)(k - v.z1) * v.sy + (size_t)(j - v.x1)] = dist(gen);
        FDM_CUDA(cudaMemcpy(v.p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
};

}  // namespace fdmgpu

using namespace fdmgpu;

struct fdmgpu_nscyl {
    int dtype = FDMGPU_F64;
    std::unique_ptr<NSCylPlan<double>> d;
    std::unique_ptr<NSCylPlan<float>> f;
};

namespace {
template <typename Fn>
void with_cyl(fdmgpu_nscyl* h, Fn&& fn) {
    if (h->d) fn(*h->d);
    else fn(*h->f);
}

template <typename T>
void setup_cyl(NSCylPlan<T>& s, int zper, double R, double r0, double h1, double h2, double u0, double Re,
               double dt, int nr, int nz, int nphi) {
    cyl::Params& P = s.P;
    P.nr = nr; P.nz = nz; P.nphi = nphi; P.zper = zper;
    // z bounds, src/ns_cyl.h:66-70
    P.z_ = zper ? 0 : -1;
    P.z0 = 0;
    P.z1 = zper ? 0 : 1;
    P.zn = zper ? nz - 1 : nz;
    P.znn = zper ? nz - 1 : nz + 1;
    P.r0 = r0;
    P.dr = (R - r0) / nr; P.dz = (h2 - h1) / nz; P.dphi = 2 * M_PI / nphi;
    P.dr2 = P.dr * P.dr; P.dz2 = P.dz * P.dz; P.dphi2 = P.dphi * P.dphi;
    P.Re = Re; P.dt = dt; P.U0 = u0;
    P.dRe = cdiv_of(Re);
    P.ddr = cdiv_of(P.dr); P.ddz = cdiv_of(P.dz); P.ddphi = cdiv_of(P.dphi);
    P.ddr2 = cdiv_of(P.dr2); P.ddz2 = cdiv_of(P.dz2); P.ddphi2 = cdiv_of(P.dphi2);
    P.ddt = cdiv_of(dt);
    P.dt_dr = dt / P.dr; P.dt_dz = dt / P.dz;
    s.init(R, r0, h1, h2);
}
}  // namespace

extern "C" {

int fdmgpu_nscyl_create(fdmgpu_nscyl** h, int dtype, int periodic_z, double R, double r0, double h1, double h2,
                        double u0, double Re, double dt, int nr, int nz, int nphi) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle pointer");
    *h = nullptr;
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    if (nphi < 2 || nphi > 512 || ilog2_exact(nphi) < 0) FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N): nphi=%d", nphi);
    if (periodic_z ? (nz < 2 || nz > 512 || ilog2_exact(nz) < 0) : (nz < 2 || nz > FDMGPU_MAX_N || ilog2_exact(nz + 1) < 0))
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N): nz=%d", nz);
    if (nr < 2 || nr > cyl::kMaxR) FDM_FAIL(FDMGPU_ESIZE, "nr must be in [2, %d], got %d", cyl::kMaxR, nr);
    if (!periodic_z && nz > nr)
        FDM_FAIL(FDMGPU_ENOTSUP, "Dirichlet z needs nz <= nr (the reference's axial ghost loop runs r over the "
                                 "z bounds, src/ns_cyl.cpp:106-111)");
    if (!(R > r0 && r0 > 0 && h2 > h1 && Re > 0 && dt > 0)) FDM_FAIL(FDMGPU_EINVAL, "bad geometry or parameters");
    std::unique_ptr<fdmgpu_nscyl> p(new fdmgpu_nscyl());
    p->dtype = dtype;
    if (dtype == FDMGPU_F64) {
        p->d.reset(new NSCylPlan<double>());
        setup_cyl(*p->d, periodic_z != 0, R, r0, h1, h2, u0, Re, dt, nr, nz, nphi);
    } else {
        p->f.reset(new NSCylPlan<float>());
        setup_cyl(*p->f, periodic_z != 0, R, r0, h1, h2, u0, Re, dt, nr, nz, nphi);
    }
    *h = p.release();
    FDM_API_END
}

int fdmgpu_nscyl_step(fdmgpu_nscyl* h, int k) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (k < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
    with_cyl(h, [&](auto& s) { s.step(k); });
    FDM_API_END
}

int fdmgpu_nscyl_field_info(fdmgpu_nscyl* h, int field, size_t* count, int* r) {
    FDM_API_BEGIN
    if (!h || field < 0 || field > 11) FDM_FAIL(FDMGPU_EINVAL, "bad handle or field %d", field);
    with_cyl(h, [&](auto& s) {
        const auto& f = s.f[field];
        if (count) *count = (size_t)f.size;
        if (r) {
            r[0] = 0; r[1] = f.nphi - 1; r[2] = f.z1; r[3] = f.z2; r[4] = f.x1; r[5] = f.x2;
        }
    });
    FDM_API_END
}

int fdmgpu_nscyl_set_field(fdmgpu_nscyl* h, int field, const void* host, size_t count) {
    FDM_API_BEGIN
    if (!h || !host || field < 0 || field > 11) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    with_cyl(h, [&](auto& s) {
        const auto& f = s.f[field];
        if (count != (size_t)f.size) FDM_FAIL(FDMGPU_EINVAL, "field has %lld elements, got %zu", f.size, count);
        FDM_CUDA(cudaStreamSynchronize(s.st));
        FDM_CUDA(cudaMemcpy(f.p, host, count * sizeof(*f.p), cudaMemcpyHostToDevice));
    });
    FDM_API_END
}

int fdmgpu_nscyl_l_step(fdmgpu_nscyl* h, int k) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (k < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
    with_cyl(h, [&](auto& s) { s.step(k, true); });
    FDM_API_END
}

int fdmgpu_nscyl_vrandom(fdmgpu_nscyl* h) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    with_cyl(h, [&](auto& s) {
        if (!s.P.zper)
            FDM_FAIL(FDMGPU_ENOTSUP, "vrandom perturbs v on the z walls, which the reference's Dirichlet-z "
                                     "step rejects: verify(std::abs(v[i][nz][j]) < 1e-15), src/ns_cyl.cpp:160");
        s.vrandom();
    });
    FDM_API_END
}

int fdmgpu_nscyl_get_field(fdmgpu_nscyl* h, int field, void* host, size_t count) {
    FDM_API_BEGIN
    if (!h || !host || field < 0 || field > 11) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    with_cyl(h, [&](auto& s) {
        const auto& f = s.f[field];
        if (count != (size_t)f.size) FDM_FAIL(FDMGPU_EINVAL, "field has %lld elements, got %zu", f.size, count);
        FDM_CUDA(cudaStreamSynchronize(s.st));
        FDM_CUDA(cudaMemcpy(host, f.p, count * sizeof(*f.p), cudaMemcpyDeviceToHost));
    });
    FDM_API_END
}

int fdmgpu_nscyl_time_index(fdmgpu_nscyl* h, int* t) {
    FDM_API_BEGIN
    if (!h || !t) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    with_cyl(h, [&](auto& s) { *t = s.time_index; });
    FDM_API_END
}

int fdmgpu_nscyl_destroy(fdmgpu_nscyl* h) {
    FDM_API_BEGIN
    delete h;
    FDM_API_END
}

}  // extern "C"
