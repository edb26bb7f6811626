// NSCube lid-driven cavity projection step on the GPU, FP64, and its C ABI.
//
// Restates fdm::NSCube<T,check>::step (src/ns_cube.cpp:27-62): boundary
// ghosts (init_bound, :65-122), the F,G,H predictor (FGH, :126-200), the
// divergence RHS plus the pressure Poisson solve (poisson, :204-238) and the
// velocity correction with p = x (update_uvwp, :241-277).  Fields keep the
// reference tensor layouts (src/ns_cube.h:64-75): inclusive index ranges, x
// fastest, ghost layers included.  The arithmetic of every stencil is written
// in the reference's order of operations.
//
// A step is 9 launches on the handle's stream (two boundary phases, FGH,
// RHS, the five passes of the plain FP64 Poisson solve, update).  After the
// first eager step the sequence is captured once into a CUDA graph and
// replayed, which removes the host launch cost that dominates at 63^3.
// Quotients by the run constants (Re, h, h^2, dt) are, by default, products
// with reciprocals computed on the host; the exact form (set_exact) rounds
// each one as the reference's division does.  Every kernel is bound by the
// FP64 pipe, which GB300 runs at a small fraction of its FP32 rate.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "poisson.h"

namespace fdmgpu {

template <typename T>
struct FieldT {
    T* p;
    int z1, z2, y1, y2, x1, x2;
    long long sy, sz, size;
    __host__ __device__ T& operator()(int i, int k, int j) const {
        return p[(long long)(i - z1) * sz + (long long)(k - y1) * sy + (j - x1)];
    }
};

template <typename T>
static FieldT<T> make_field(int z1, int z2, int y1, int y2, int x1, int x2) {
    FieldT<T> f;
    f.z1 = z1; f.z2 = z2; f.y1 = y1; f.y2 = y2; f.x1 = x1; f.x2 = x2;
    f.sy = x2 - x1 + 1;
    f.sz = f.sy * (y2 - y1 + 1);
    f.size = f.sz * (z2 - z1 + 1);
    f.p = nullptr;
    return f;
}

struct NSParams {
    int nx, ny, nz;
    double U0, Re, dt, dx, dy, dz, dx2, dy2, dz2;
    CDiv dRe, ddx, ddy, ddz, ddx2, ddy2, ddz2, ddt;
    double dt_dx, dt_dy, dt_dz;  // dt/dx etc., correctly rounded on the host
    // reciprocals of the run constants for the fast form (FAST = true): a
    // quotient x / a / b becomes x * (1 / (a b)), one FP64 multiply instead
    // of two correctly rounded divisions (five operations each)
    double rRe_dx2, rRe_dy2, rRe_dz2, rRe_dx, rRe_dy, rRe_dz;
    double rdx, rdy, rdz, rdx2, rdy2, rdz2, rdt;
    // the fast FGH's constants with dt folded in: dt / (Re h^2) for the
    // diffusion terms, dt / (4 h) for the convection terms (whose 0.5 and
    // 0.25 factors they absorb); the fast divergence's 1 / (h dt)
    double kCx, kCy, kCz, kAx, kAy, kAz, kRx, kRy, kRz;
    double kC0;  // 1 - 2 (kCx + kCy + kCz): the centre's weight in u + dt diffusion
};

// x / d (FAST: x * r, r = 1 / d computed on the host; otherwise the
// correctly rounded quotient of cdiv)
template <bool FAST>
__device__ __forceinline__ double qdiv(double x, CDiv d, double r) {
    if constexpr (FAST) return x * r;
    else return cdiv(x, d);
}

// (x / Re) / h^2, or x * (1 / (Re h^2)) in the fast form
template <bool FAST>
__device__ __forceinline__ double qdiv2(double x, CDiv dRe, CDiv d2, double r) {
    if constexpr (FAST) return x * r;
    else return cdiv(cdiv(x, dRe), d2);
}

// Point e of the surface of a W x H x D box (x fastest): the two z faces,
// the two y faces without their z edges, the two x faces without either.
// Returns false past the surface's 2(WH + W(D-2) + (H-2)(D-2)) points.
__device__ __forceinline__ bool surface_point(long long e, int W, int H, int D, int& i, int& k, int& j) {
    const long long zf = (long long)W * H;
    if (e < 2 * zf) {
        i = e < zf ? 0 : D - 1;
        const long long r = e < zf ? e : e - zf;
        k = (int)(r / W);
        j = (int)(r - (long long)k * W);
        return true;
    }
    e -= 2 * zf;
    const long long yf = (long long)W * (D - 2);
    if (e < 2 * yf) {
        k = e < yf ? 0 : H - 1;
        const long long r = e < yf ? e : e - yf;
        i = 1 + (int)(r / W);
        j = (int)(r % W);
        return true;
    }
    e -= 2 * yf;
    const long long xf = (long long)(H - 2) * (D - 2);
    if (e < 2 * xf) {
        j = e < xf ? 0 : W - 1;
        const long long r = e < xf ? e : e - xf;
        i = 1 + (int)(r / (H - 2));
        k = 1 + (int)(r % (H - 2));
        return true;
    }
    return false;
}

__host__ __device__ inline long long surface_points(int W, int H, int D) {
    return 2 * ((long long)W * H + (long long)W * (D - 2) + (long long)(H - 2) * (D - 2));
}

__device__ __forceinline__ double sq(double x) { return x * x; }  // asp::sq, src/asp_misc.h:295

// init_bound, first phase: the lid (without the two x-ghost columns that the
// mirror below overwrites anyway), the x-mirror of u below the lid, and the
// y-/z-mirrors of v and w.  None of these reads what another writes.  Every
// point written lies on the surface of the (z,y,x) box [-1, nz+1] x
// [-1, ny+1] x [-1, nx+1]; one thread per surface point.
template <typename T>
__device__ __forceinline__ void ns_bound1_body(FieldT<T> u, FieldT<T> v, FieldT<T> w, const NSParams& P) {
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int i, k, j;
    if (!surface_point(e, nx + 3, ny + 3, nz + 3, i, k, j)) return;
    i -= 1;
    k -= 1;
    j -= 1;
    // lid (src/ns_cube.cpp:67-72): u[nz+1][k][j] = 2U0 - u[nz][k][j], j in [-1, nz+1]
    if (i == nz + 1 && k >= 0 && k <= ny + 1 && j >= 0 && j <= min(nz + 1, nx)) u(nz + 1, k, j) = 2 * P.U0 - u(nz, k, j);
    // u x-mirror for i <= nz (:76-81)
    if (i >= 0 && i <= nz && k >= 0 && k <= ny + 1) {
        if (j == -1) u(i, k, -1) = u(i, k, 1);
        if (j == nx + 1) u(i, k, nx + 1) = u(i, k, nx - 1);
    }
    // v y-mirror (:83-88)
    if (i >= 0 && i <= nz + 1 && j >= 0 && j <= nx + 1) {
        if (k == -1) v(i, -1, j) = v(i, 1, j);
        if (k == ny + 1) v(i, ny + 1, j) = v(i, ny - 1, j);
    }
    // w z-mirror (:90-95)
    if (k >= 0 && k <= ny + 1 && j >= 0 && j <= nx + 1) {
        if (i == -1) w(-1, k, j) = w(1, k, j);
        if (i == nz + 1) w(nz + 1, k, j) = w(nz - 1, k, j);
    }
}

// init_bound, second phase: u x-mirror of the lid row (reads the lid values
// written by phase one) and the Neumann pressure ghosts (:98-121).  Every
// point written lies on the surface of the box [0, nz+1] x [0, ny+1] x
// [0, nx+1]; one thread per surface point.
template <typename T, bool FAST>
__device__ __forceinline__ void ns_bound2_body(FieldT<T> u, FieldT<T> v, FieldT<T> w, FieldT<T> p, const NSParams& P) {
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int i, k, j;
    if (!surface_point(e, nx + 2, ny + 2, nz + 2, i, k, j)) return;
    auto g = [&](double x, CDiv d, double r) { return qdiv2<FAST>(x, P.dRe, d, r); };
    if (i == nz + 1 && k <= ny + 1) {
        if (j == 0) u(nz + 1, k, -1) = u(nz + 1, k, 1);
        if (j == nx + 1) u(nz + 1, k, nx + 1) = u(nz + 1, k, nx - 1);
    }
    if (i >= 1 && i <= nz && k >= 1 && k <= ny) {
        if (j == 0) p(i, k, 0) = p(i, k, 1) - g(u(i, k, 1) - 2 * u(i, k, 0) + u(i, k, -1), P.ddx, P.rRe_dx);
        if (j == nx + 1)
            p(i, k, nx + 1) = p(i, k, nx) - g(u(i, k, nx + 1) - 2 * u(i, k, nx) + u(i, k, nx - 1), P.ddx, P.rRe_dx);
    }
    if (i >= 1 && i <= nz && j >= 1 && j <= nx) {
        if (k == 0) p(i, 0, j) = p(i, 1, j) - g(v(i, 1, j) - 2 * v(i, 0, j) + v(i, -1, j), P.ddy, P.rRe_dy);
        if (k == ny + 1)
            p(i, ny + 1, j) = p(i, ny, j) - g(v(i, ny + 1, j) - 2 * v(i, ny, j) + v(i, ny - 1, j), P.ddy, P.rRe_dy);
    }
    if (k >= 1 && k <= ny && j >= 1 && j <= nx) {
        if (i == 0) p(0, k, j) = p(1, k, j) - g(w(1, k, j) - 2 * w(0, k, j) + w(-1, k, j), P.ddz, P.rRe_dz);
        if (i == nz + 1)
            p(nz + 1, k, j) = p(nz, k, j) - g(w(nz + 1, k, j) - 2 * w(nz, k, j) + w(nz - 1, k, j), P.ddz, P.rRe_dz);
    }
}

// FGH (src/ns_cube.cpp:126-200), one thread per (i,k,j) of the box
// [0,nz] x [0,ny] x [0,nx]; each thread writes whichever of F, G, H has that
// point in its range.  FAST: quotients by the run constants as products with
// their reciprocals, and for FP64 fields dt and the convection terms' 0.5 /
// 0.25 folded into per-axis constants so that each component is one chain of
// fused multiply-adds (about a quarter of the exact form's FP64 operations;
// results within a few units in the last place of the exact form's).  The
// float cavity keeps the reference's expressions and promotions.
template <typename T, bool FAST>
__device__ __forceinline__ void ns_fgh_body(FieldT<T> u, FieldT<T> v, FieldT<T> w, FieldT<T> F, FieldT<T> G,
                                            FieldT<T> H, const NSParams& P) {
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int W = nx + 1, Hh = ny + 1, D = nz + 1;
    if (e >= (long long)W * Hh * D) return;
    const int j = (int)(e % W);
    const int k = (int)((e / W) % Hh);
    const int i = (int)(e / ((long long)W * Hh));
    const double dt = P.dt;
    // x / Re / h^2 and x / h (exact form: each quotient rounded as the
    // reference's)
    auto dif = [&](double x, CDiv d2, double r) { return qdiv2<FAST>(x, P.dRe, d2, r); };
    auto qd = [&](double x, CDiv d, double r) { return qdiv<FAST>(x, d, r); };
    // the three components are formed before any is stored, so that the
    // compiler may share the loads and the cross products they have in
    // common (the stores could alias the velocity fields)
    double fv = 0.0, gv = 0.0, hv = 0.0;
    const bool doF = i >= 1 && k >= 1, doG = i >= 1 && j >= 1, doH = k >= 1 && j >= 1;
    if constexpr (FAST && sizeof(T) == 8) {
        // FP64 fields: u + dt (diffusion - convection) as one chain of fused
        // multiply-adds.  Per component: the diffusion is kC0 c + sum over
        // the axes of kC (m + p), the centre's three -2c terms gathered in
        // kC0 = 1 - 2 (kCx + kCy + kCz); along the component's own axis
        // sq(a/2) - sq(b/2) = (a - b)(a + b) / 4 = (p - m)(m + p + 2c) / 4
        // with a = c + p, b = m + c, so the neighbour sum m + p serves both
        // terms; the cross terms' 0.25 go into dt / (4 h); the three cross
        // products that two components share (F's y term and G's x term, F's
        // z term and H's x term, G's z term and H's y term) are formed once.
        // Every read below is inside its field's range for any point of the
        // box.
        const double uc = u(i, k, j), vc = v(i, k, j), wc = w(i, k, j);
        const double puv = (uc + u(i, k + 1, j)) * (v(i, k, j + 1) + vc);
        const double puw = (uc + u(i + 1, k, j)) * (w(i, k, j + 1) + wc);
        const double pwv = (wc + w(i, k + 1, j)) * (vc + v(i + 1, k, j));
        if (doF) {
            const double m = u(i, k, j - 1), pl = u(i, k, j + 1), sx = m + pl;
            double acc = P.kC0 * uc;
            acc += P.kCx * sx;
            acc += P.kCy * (u(i, k - 1, j) + u(i, k + 1, j));
            acc += P.kCz * (u(i - 1, k, j) + u(i + 1, k, j));
            acc -= P.kAx * ((pl - m) * (sx + 2.0 * uc));
            acc -= P.kAy * (puv - (u(i, k - 1, j) + uc) * (v(i, k - 1, j + 1) + v(i, k - 1, j)));
            acc -= P.kAz * (puw - (u(i - 1, k, j) + uc) * (w(i - 1, k, j + 1) + w(i - 1, k, j)));
            fv = acc;
        }
        if (doG) {
            const double m = v(i, k - 1, j), pl = v(i, k + 1, j), sy = m + pl;
            double acc = P.kC0 * vc;
            acc += P.kCx * (v(i, k, j - 1) + v(i, k, j + 1));
            acc += P.kCy * sy;
            acc += P.kCz * (v(i - 1, k, j) + v(i + 1, k, j));
            acc -= P.kAy * ((pl - m) * (sy + 2.0 * vc));
            acc -= P.kAx * (puv - (u(i, k, j - 1) + u(i, k + 1, j - 1)) * (vc + v(i, k, j - 1)));
            acc -= P.kAz * (pwv - (w(i - 1, k, j) + w(i - 1, k + 1, j)) * (v(i - 1, k, j) + vc));
            gv = acc;
        }
        if (doH) {
            const double m = w(i - 1, k, j), pl = w(i + 1, k, j), sz = m + pl;
            double acc = P.kC0 * wc;
            acc += P.kCx * (w(i, k, j - 1) + w(i, k, j + 1));
            acc += P.kCy * (w(i, k - 1, j) + w(i, k + 1, j));
            acc += P.kCz * sz;
            acc -= P.kAz * ((pl - m) * (sz + 2.0 * wc));
            acc -= P.kAx * (puw - (u(i + 1, k, j - 1) + u(i, k, j - 1)) * (wc + w(i, k, j - 1)));
            acc -= P.kAy * (pwv - (w(i, k - 1, j) + wc) * (v(i, k - 1, j) + v(i + 1, k - 1, j)));
            hv = acc;
        }
    } else {
    if (doF) {
        fv = u(i, k, j) + dt * (
            dif(u(i, k, j + 1) - 2 * u(i, k, j) + u(i, k, j - 1), P.ddx2, P.rRe_dx2) +
            dif(u(i, k + 1, j) - 2 * u(i, k, j) + u(i, k - 1, j), P.ddy2, P.rRe_dy2) +
            dif(u(i + 1, k, j) - 2 * u(i, k, j) + u(i - 1, k, j), P.ddz2, P.rRe_dz2) -
            qd(sq(0.5 * (u(i, k, j) + u(i, k, j + 1))) - sq(0.5 * (u(i, k, j - 1) + u(i, k, j))), P.ddx, P.rdx) -
            qd(0.25 * ((u(i, k, j) + u(i, k + 1, j)) * (v(i, k, j + 1) + v(i, k, j)) -
                         (u(i, k - 1, j) + u(i, k, j)) * (v(i, k - 1, j + 1) + v(i, k - 1, j))), P.ddy, P.rdy) -
            qd(0.25 * ((u(i, k, j) + u(i + 1, k, j)) * (w(i, k, j + 1) + w(i, k, j)) -
                         (u(i - 1, k, j) + u(i, k, j)) * (w(i - 1, k, j + 1) + w(i - 1, k, j))), P.ddz, P.rdz));
    }
    if (doG) {
        gv = v(i, k, j) + dt * (
            dif(v(i, k, j + 1) - 2 * v(i, k, j) + v(i, k, j - 1), P.ddx2, P.rRe_dx2) +
            dif(v(i, k + 1, j) - 2 * v(i, k, j) + v(i, k - 1, j), P.ddy2, P.rRe_dy2) +
            dif(v(i + 1, k, j) - 2 * v(i, k, j) + v(i - 1, k, j), P.ddz2, P.rRe_dz2) -
            qd(sq(0.5 * (v(i, k, j) + v(i, k + 1, j))) - sq(0.5 * (v(i, k - 1, j) + v(i, k, j))), P.ddy, P.rdy) -
            qd(0.25 * ((u(i, k, j) + u(i, k + 1, j)) * (v(i, k, j + 1) + v(i, k, j)) -
                         (u(i, k, j - 1) + u(i, k + 1, j - 1)) * (v(i, k, j) + v(i, k, j - 1))), P.ddx, P.rdx) -
            qd(0.25 * ((w(i, k, j) + w(i, k + 1, j)) * (v(i, k, j) + v(i + 1, k, j)) -
                         (w(i - 1, k, j) + w(i - 1, k + 1, j)) * (v(i - 1, k, j) + v(i, k, j))), P.ddz, P.rdz));
    }
    if (doH) {
        hv = w(i, k, j) + dt * (
            dif(w(i, k, j + 1) - 2 * w(i, k, j) + w(i, k, j - 1), P.ddx2, P.rRe_dx2) +
            dif(w(i, k + 1, j) - 2 * w(i, k, j) + w(i, k - 1, j), P.ddy2, P.rRe_dy2) +
            dif(w(i + 1, k, j) - 2 * w(i, k, j) + w(i - 1, k, j), P.ddz2, P.rRe_dz2) -
            qd(sq(0.5 * (w(i + 1, k, j) + w(i, k, j))) - sq(0.5 * (w(i - 1, k, j) + w(i, k, j))), P.ddz, P.rdz) -
            qd(0.25 * ((u(i + 1, k, j) + u(i, k, j)) * (w(i, k, j + 1) + w(i, k, j)) -
                         (u(i + 1, k, j - 1) + u(i, k, j - 1)) * (w(i, k, j) + w(i, k, j - 1))), P.ddx, P.rdx) -
            qd(0.25 * ((w(i, k, j) + w(i, k + 1, j)) * (v(i, k, j) + v(i + 1, k, j)) -
                         (w(i, k - 1, j) + w(i, k, j)) * (v(i, k - 1, j) + v(i + 1, k - 1, j))), P.ddy, P.rdy));
    }
    }
    if (doF) F(i, k, j) = fv;
    if (doG) G(i, k, j) = gv;
    if (doH) H(i, k, j) = hv;
}

// Divergence RHS with the Dirichlet pressure ghosts folded in
// (src/ns_cube.cpp:206-235).
template <typename T, bool FAST>
__device__ __forceinline__ void ns_rhs_body(FieldT<T> F, FieldT<T> G, FieldT<T> H, FieldT<T> p, FieldT<T> RHS,
                                            const NSParams& P) {
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nx * ny * nz) return;
    const int j = (int)(e % nx) + 1;
    const int k = (int)((e / nx) % ny) + 1;
    const int i = (int)(e / ((long long)nx * ny)) + 1;
    // T-typed like the reference RHS element: rounded after each update
    auto qd = [&](double x, CDiv d, double rc) { return qdiv<FAST>(x, d, rc); };
    T r;
    if constexpr (FAST)  // 1 / (h dt) per axis
        r = (F(i, k, j) - F(i, k, j - 1)) * P.kRx + (G(i, k, j) - G(i, k - 1, j)) * P.kRy +
            (H(i, k, j) - H(i - 1, k, j)) * P.kRz;
    else
        r = qd(qd(F(i, k, j) - F(i, k, j - 1), P.ddx, P.rdx) + qd(G(i, k, j) - G(i, k - 1, j), P.ddy, P.rdy) +
                   qd(H(i, k, j) - H(i - 1, k, j), P.ddz, P.rdz), P.ddt, P.rdt);
    if (i <= 1) r -= qd(p(i - 1, k, j), P.ddz2, P.rdz2);
    if (k <= 1) r -= qd(p(i, k - 1, j), P.ddy2, P.rdy2);
    if (j <= 1) r -= qd(p(i, k, j - 1), P.ddx2, P.rdx2);
    if (j >= nx) r -= qd(p(i, k, j + 1), P.ddx2, P.rdx2);
    if (k >= ny) r -= qd(p(i, k + 1, j), P.ddy2, P.rdy2);
    if (i >= nz) r -= qd(p(i + 1, k, j), P.ddz2, P.rdz2);
    RHS(i, k, j) = r;
}

// update_uvwp (src/ns_cube.cpp:241-277): pressure-gradient correction of the
// interior faces, then p = x on the interior (src/tensor.h:280-283).
template <typename T>
__device__ __forceinline__ void ns_update_body(FieldT<T> u, FieldT<T> v, FieldT<T> w, FieldT<T> p, FieldT<T> x, FieldT<T> F, FieldT<T> G,
                            FieldT<T> H, const NSParams& P) {
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nx * ny * nz) return;
    const int j = (int)(e % nx) + 1;
    const int k = (int)((e / nx) % ny) + 1;
    const int i = (int)(e / ((long long)nx * ny)) + 1;
    const T xc = x(i, k, j);
    if (j < nx) u(i, k, j) = F(i, k, j) - P.dt_dx * (x(i, k, j + 1) - xc);
    if (k < ny) v(i, k, j) = G(i, k, j) - P.dt_dy * (x(i, k + 1, j) - xc);
    if (i < nz) w(i, k, j) = H(i, k, j) - P.dt_dz * (x(i + 1, k, j) - xc);
    p(i, k, j) = xc;
}

// Per-session state of a step: the nine fields' storage and the run
// constants.  One step kernel serves one session or several of the same
// geometry: blockIdx.y picks the session from a device table of these, the
// ranges and strides of the fields (the same for all) come as an argument.
template <typename T>
struct NSSessionT {
    T* f[9];  // u v w p x F G H RHS
    NSParams P;
};
template <typename T>
struct NSGeomT {
    FieldT<T> f[9];  // ranges and strides (p not used)
};
template <typename T>
__device__ __forceinline__ FieldT<T> ns_field(const NSGeomT<T>& g, const NSSessionT<T>& s, int i) {
    FieldT<T> r = g.f[i];
    r.p = s.f[i];
    return r;
}

template <typename T>
__global__ void k_ns_bound1(NSGeomT<T> g, const NSSessionT<T>* __restrict__ ss) {
    const NSSessionT<T>& S = ss[blockIdx.y];
    const NSParams P = S.P;
    ns_bound1_body<T>(ns_field(g, S, 0), ns_field(g, S, 1), ns_field(g, S, 2), P);
}
template <typename T, bool FAST>
__global__ void k_ns_bound2(NSGeomT<T> g, const NSSessionT<T>* __restrict__ ss) {
    const NSSessionT<T>& S = ss[blockIdx.y];
    const NSParams P = S.P;
    ns_bound2_body<T, FAST>(ns_field(g, S, 0), ns_field(g, S, 1), ns_field(g, S, 2), ns_field(g, S, 3), P);
}
template <typename T, bool FAST>
__global__ void __launch_bounds__(256) k_ns_fgh(NSGeomT<T> g, const NSSessionT<T>* __restrict__ ss) {
    const NSSessionT<T>& S = ss[blockIdx.y];
    const NSParams P = S.P;
    ns_fgh_body<T, FAST>(ns_field(g, S, 0), ns_field(g, S, 1), ns_field(g, S, 2), ns_field(g, S, 5),
                         ns_field(g, S, 6), ns_field(g, S, 7), P);
}
template <typename T, bool FAST>
__global__ void k_ns_rhs(NSGeomT<T> g, const NSSessionT<T>* __restrict__ ss) {
    const NSSessionT<T>& S = ss[blockIdx.y];
    const NSParams P = S.P;
    ns_rhs_body<T, FAST>(ns_field(g, S, 5), ns_field(g, S, 6), ns_field(g, S, 7), ns_field(g, S, 3),
                         ns_field(g, S, 8), P);
}
template <typename T>
__global__ void k_ns_update(NSGeomT<T> g, const NSSessionT<T>* __restrict__ ss) {
    const NSSessionT<T>& S = ss[blockIdx.y];
    const NSParams P = S.P;
    ns_update_body<T>(ns_field(g, S, 0), ns_field(g, S, 1), ns_field(g, S, 2), ns_field(g, S, 3), ns_field(g, S, 4),
                      ns_field(g, S, 5), ns_field(g, S, 6), ns_field(g, S, 7), P);
}

// Cell-centred velocity of the interior cells for the VTK snapshot
// (velocity_plotter::vtk_out, src/velocity_plot.cpp:200-217): out[cell*3+c]
// with cell = ((i-1)*ny + (k-1))*nx + (j-1).
template <typename T>
__global__ void k_ns_cell_velocity(FieldT<T> u, FieldT<T> v, FieldT<T> w, NSParams P, double* out) {
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nx * ny * nz) return;
    const int j = (int)(e % nx) + 1;
    const int k = (int)((e / nx) % ny) + 1;
    const int i = (int)(e / ((long long)nx * ny)) + 1;
    out[3 * e] = 0.5 * (u(i, k, j) + u(i, k, j - 1));
    out[3 * e + 1] = 0.5 * (v(i, k, j) + v(i, k - 1, j));
    out[3 * e + 2] = 0.5 * (w(i, k, j) + w(i - 1, k, j));
}

// Diagnostic: IEEE a/b and the constant-divisor quotient side by side.
__global__ void k_cdiv_check(const double* a, const double* b, double* q_ieee, double* q_c, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double bi = b[i];
    q_ieee[i] = a[i] / bi;
    q_c[i] = cdiv(a[i], CDiv{bi, 1.0 / bi});
}

template <typename T>
struct NSPlanT {
    NSParams P;
    double x1, y1, z1, x2, y2, z2;
    FieldT<T> f[9];  // u v w p x F G H RHS
    void* mem = nullptr;
    fdmgpu_lapl_cube* lapl = nullptr;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int time_index = 0;
    // a step of its own ran eagerly: kernel attributes are set and the
    // pressure solve's scratch exists, so later steps can be captured (steps
    // shared with other cavities use neither)
    bool warm = false;
    bool exact = false;  // quotients correctly rounded as the reference's (slower)
    // the step kernels' view of this session: field geometry, and on the
    // device the session table of one entry and, for the FP64 pressure
    // solve through pointer tables, {&RHS, &x}
    NSGeomT<T> geo;
    DevBuf sess_dev, io_dev;
    const void* io_host[2] = {nullptr, nullptr};  // {RHS, x}: the FP32 pressure solve's arguments

    NSSessionT<T> session() const {
        NSSessionT<T> s;
        for (int i = 0; i < 9; i++) s.f[i] = f[i].p;
        s.P = P;
        return s;
    }

    ~NSPlanT() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        if (lapl) fdmgpu_lapl_cube_destroy(lapl);
        if (mem) cudaFree(mem);
        if (own_stream && st) cudaStreamDestroy(st);
    }

    void init() {
        const int nx = P.nx, ny = P.ny, nz = P.nz;
        f[0] = make_field<T>(0, nz + 1, 0, ny + 1, -1, nx + 1);
        f[1] = make_field<T>(0, nz + 1, -1, ny + 1, 0, nx + 1);
        f[2] = make_field<T>(-1, nz + 1, 0, ny + 1, 0, nx + 1);
        f[3] = make_field<T>(0, nz + 1, 0, ny + 1, 0, nx + 1);
        f[4] = make_field<T>(1, nz, 1, ny, 1, nx);
        f[5] = make_field<T>(1, nz, 1, ny, 0, nx);
        f[6] = make_field<T>(1, nz, 0, ny, 1, nx);
        f[7] = make_field<T>(0, nz, 1, ny, 1, nx);
        f[8] = make_field<T>(1, nz, 1, ny, 1, nx);
        size_t total = 0;
        for (auto& fi : f) total += (size_t)((fi.size + 31) / 32 * 32);
        FDM_CUDA(cudaMalloc(&mem, total * sizeof(T)));
        FDM_CUDA(cudaMemset(mem, 0, total * sizeof(T)));
        size_t off = 0;
        for (auto& fi : f) {
            fi.p = (T*)mem + off;
            off += (size_t)((fi.size + 31) / 32 * 32);
        }
        FDM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        own_stream = true;
        // LaplCube(dx, dy, dz, x2-x1+dx, y2-y1+dy, z2-z1+dz, nx, ny, nz), src/ns_cube.h:77
        int rc = fdmgpu_lapl_cube_create(&lapl, sizeof(T) == 8 ? FDMGPU_F64 : FDMGPU_F32, FDMGPU_DIRICHLET, P.dx, P.dy, P.dz, x2 - x1 + P.dx,
                                         y2 - y1 + P.dy, z2 - z1 + P.dz, nx, ny, nz);
        if (rc) throw Error{rc};
        // the transforms' CTA size as for one volume however many sessions
        // a step serves, so that a session's fields come out the same alone
        // and stepped together with others
        cube_set_rule_volumes(lapl, 1);
        for (int i = 0; i < 9; i++) geo.f[i] = f[i];
        const NSSessionT<T> h = session();
        FDM_CUDA(cudaMemcpy(sess_dev.get(sizeof(h)), &h, sizeof(h), cudaMemcpyHostToDevice));
        io_host[0] = f[8].p;
        io_host[1] = f[4].p;
        FDM_CUDA(cudaMemcpy(io_dev.get(sizeof(io_host)), io_host, sizeof(io_host), cudaMemcpyHostToDevice));
    }

    void enqueue_step() {
        if (exact) enqueue_step_t<false>();
        else enqueue_step_t<true>();
    }

    template <bool FAST>
    void enqueue_step_t() {
        enqueue_steps<FAST>(geo, (const NSSessionT<T>*)sess_dev.p,
                            sizeof(T) == 8 ? (const void* const*)io_dev.p : io_host, 1, 1, lapl, nullptr, st);
    }

    // One step of nsess sessions of this geometry: the session table ss
    // and, for FP64 fields, io = {&RHS of every session, then &x of every
    // session} (nsess pointers each, on the device; for FP32 fields, one
    // session, the host pair {RHS, x}); scratch: FP64 work volumes for the
    // pressure solve (null: the plan's own).
    template <bool FAST>
    static void enqueue_steps(const NSGeomT<T>& g, const NSSessionT<T>* ss, const void* const* io, int nsess,
                              int io_stride, fdmgpu_lapl_cube* lapl, double* scratch, cudaStream_t st) {
        const int nx = g.f[4].x2, ny = g.f[4].y2, nz = g.f[4].z2;  // x: {1..nz, 1..ny, 1..nx}
        const int B = 256;
        auto grid = [&](long long n) { return dim3((unsigned)((n + B - 1) / B), (unsigned)nsess); };
        const long long vol = (long long)nx * ny * nz;
        {
            FDM_TIMED("ns_bound1", st);
            k_ns_bound1<T><<<grid(surface_points(nx + 3, ny + 3, nz + 3)), B, 0, st>>>(g, ss);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("ns_bound2", st);
            k_ns_bound2<T, FAST><<<grid(surface_points(nx + 2, ny + 2, nz + 2)), B, 0, st>>>(g, ss);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("ns_fgh", st);
            k_ns_fgh<T, FAST><<<grid((long long)(nx + 1) * (ny + 1) * (nz + 1)), B, 0, st>>>(g, ss);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("ns_rhs", st);
            k_ns_rhs<T, FAST><<<grid(vol), B, 0, st>>>(g, ss);
            FDM_LAUNCH_CHECK();
        }
        if constexpr (sizeof(T) == 8) {
            cube_solve_ptrs(lapl, io, (void* const*)(io + io_stride), nsess, scratch, st);
        } else {
            // NSCube<float>: one session per step (the FP32 plan solves
            // contiguous volumes); io = {RHS, x} are the data pointers
            cube_solve_device(lapl, (void*)io[1], io[0], 1, st);
        }
        {
            FDM_TIMED("ns_update", st);
            k_ns_update<T><<<grid(vol), B, 0, st>>>(g, ss);
            FDM_LAUNCH_CHECK();
        }
    }

    void step(int k) {
        for (int s = 0; s < k; s++) {
            if (!warm) {
                enqueue_step();  // eager first step
                warm = true;
            } else {
                if (!gexec) {
                    FDM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                    try {
                        enqueue_step();
                    } catch (...) {
                        cudaGraph_t g;
                        cudaStreamEndCapture(st, &g);
                        if (g) cudaGraphDestroy(g);
                        throw;
                    }
                    FDM_CUDA(cudaStreamEndCapture(st, &graph));
                    FDM_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
                }
                FDM_CUDA(cudaGraphLaunch(gexec, st));
            }
            time_index++;
        }
    }
};

}  // namespace fdmgpu

using namespace fdmgpu;

struct fdmgpu_nscube {
    int dtype = FDMGPU_F64;
    std::unique_ptr<NSPlanT<double>> d;
    std::unique_ptr<NSPlanT<float>> f;
};

namespace fdmgpu {

bool nscube_mergeable(const fdmgpu_nscube* a, const fdmgpu_nscube* b) {
    if (!a || !b || !a->d || !b->d) return false;
    const NSPlanT<double>& p = *a->d;
    const NSPlanT<double>& q = *b->d;
    return p.P.nx == q.P.nx && p.P.ny == q.P.ny && p.P.nz == q.P.nz && p.P.dx == q.P.dx && p.P.dy == q.P.dy &&
           p.P.dz == q.P.dz && p.x2 - p.x1 == q.x2 - q.x1 && p.y2 - p.y1 == q.y2 - q.y1 &&
           p.z2 - p.z1 == q.z2 - q.z1 && p.exact == q.exact;
}

void nscube_step_many(fdmgpu_nscube* const* hs, const int* steps, int n, cudaStream_t st, cudaMemPool_t pool) {
    if (n < 1) return;
    for (int i = 0; i < n; i++) {
        if (!hs[i] || !hs[i]->d) FDM_FAIL(FDMGPU_ENOTSUP, "shared steps are for FP64 cavities");
        if (steps[i] < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
        if (i > 0 && !nscube_mergeable(hs[0], hs[i])) FDM_FAIL(FDMGPU_EINVAL, "cavities of different geometry");
    }
    // most steps first: round r steps the prefix of cavities with steps > r
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return steps[a] > steps[b]; });
    const int rounds = steps[idx[0]];
    NSPlanT<double>& p0 = *hs[idx[0]]->d;
    std::vector<NSSessionT<double>> ss(n);
    std::vector<const void*> io((size_t)2 * n);
    for (int k = 0; k < n; k++) {
        const NSPlanT<double>& pk = *hs[idx[k]]->d;
        ss[k] = pk.session();
        io[k] = pk.io_host[0];      // RHS
        io[n + k] = pk.io_host[1];  // x
    }
    if (rounds > 0) {
        // the tables and the pressure solve's work volumes, stream-ordered
        // (the cavities' own plans and captured steps keep their buffers)
        const size_t bs = (ss.size() * sizeof(NSSessionT<double>) + 255) / 256 * 256;
        const size_t bio = (io.size() * sizeof(void*) + 255) / 256 * 256;
        const size_t bw = (size_t)n * p0.P.nx * p0.P.ny * p0.P.nz * sizeof(double);
        char* d = nullptr;
        if (pool) FDM_CUDA(cudaMallocFromPoolAsync((void**)&d, bs + bio + bw, pool, st));
        else FDM_CUDA(cudaMallocAsync((void**)&d, bs + bio + bw, st));
        try {
            FDM_CUDA(cudaMemcpyAsync(d, ss.data(), ss.size() * sizeof(NSSessionT<double>), cudaMemcpyHostToDevice, st));
            FDM_CUDA(cudaMemcpyAsync(d + bs, io.data(), io.size() * sizeof(void*), cudaMemcpyHostToDevice, st));
            const auto* dss = (const NSSessionT<double>*)d;
            const auto* dio = (const void* const*)(d + bs);
            double* W = (double*)(d + bs + bio);
            for (int r = 0; r < rounds; r++) {
                int count = 0;
                while (count < n && steps[idx[count]] > r) count++;
                if (p0.exact) NSPlanT<double>::enqueue_steps<false>(p0.geo, dss, dio, count, n, p0.lapl, W, st);
                else NSPlanT<double>::enqueue_steps<true>(p0.geo, dss, dio, count, n, p0.lapl, W, st);
            }
        } catch (...) {
            cudaFreeAsync(d, st);
            throw;
        }
        FDM_CUDA(cudaFreeAsync(d, st));
    }
    for (int i = 0; i < n; i++) {
        hs[i]->d->time_index += steps[i];
    }
}

}  // namespace fdmgpu

namespace {
// runs fn on the handle's plan, whichever element type it has
template <typename Fn>
void with_plan(fdmgpu_nscube* h, Fn&& fn) {
    if (h->d) fn(*h->d);
    else fn(*h->f);
}

template <typename T>
void setup_plan(NSPlanT<T>& s, int nx, int nz, double x1, double y1, double z1, double x2, double y2, double z2,
                double u0, double Re, double dt) {
    s.x1 = x1; s.y1 = y1; s.z1 = z1; s.x2 = x2; s.y2 = y2; s.z2 = z2;
    s.P.nx = nx; s.P.ny = nx; s.P.nz = nz;  // ny from key "nx", src/ns_cube.h:57-59
    s.P.U0 = u0; s.P.Re = Re; s.P.dt = dt;
    s.P.dx = (x2 - x1) / nx; s.P.dy = (y2 - y1) / s.P.ny; s.P.dz = (z2 - z1) / nz;
    s.P.dx2 = s.P.dx * s.P.dx; s.P.dy2 = s.P.dy * s.P.dy; s.P.dz2 = s.P.dz * s.P.dz;
    s.P.dRe = cdiv_of(Re);
    s.P.ddx = cdiv_of(s.P.dx); s.P.ddy = cdiv_of(s.P.dy); s.P.ddz = cdiv_of(s.P.dz);
    s.P.ddx2 = cdiv_of(s.P.dx2); s.P.ddy2 = cdiv_of(s.P.dy2); s.P.ddz2 = cdiv_of(s.P.dz2);
    s.P.ddt = cdiv_of(dt);
    s.P.dt_dx = dt / s.P.dx; s.P.dt_dy = dt / s.P.dy; s.P.dt_dz = dt / s.P.dz;
    s.P.rRe_dx2 = 1.0 / (Re * s.P.dx2); s.P.rRe_dy2 = 1.0 / (Re * s.P.dy2); s.P.rRe_dz2 = 1.0 / (Re * s.P.dz2);
    s.P.rRe_dx = 1.0 / (Re * s.P.dx); s.P.rRe_dy = 1.0 / (Re * s.P.dy); s.P.rRe_dz = 1.0 / (Re * s.P.dz);
    s.P.rdx = 1.0 / s.P.dx; s.P.rdy = 1.0 / s.P.dy; s.P.rdz = 1.0 / s.P.dz;
    s.P.rdx2 = 1.0 / s.P.dx2; s.P.rdy2 = 1.0 / s.P.dy2; s.P.rdz2 = 1.0 / s.P.dz2;
    s.P.rdt = 1.0 / dt;
    s.P.kCx = dt / (Re * s.P.dx2); s.P.kCy = dt / (Re * s.P.dy2); s.P.kCz = dt / (Re * s.P.dz2);
    s.P.kAx = dt / (4.0 * s.P.dx); s.P.kAy = dt / (4.0 * s.P.dy); s.P.kAz = dt / (4.0 * s.P.dz);
    s.P.kRx = 1.0 / (s.P.dx * dt); s.P.kRy = 1.0 / (s.P.dy * dt); s.P.kRz = 1.0 / (s.P.dz * dt);
    s.P.kC0 = 1.0 - 2.0 * (s.P.kCx + s.P.kCy + s.P.kCz);
    s.init();
}
}  // namespace

extern "C" {

int fdmgpu_nscube_create(fdmgpu_nscube** h, int dtype, int nx, int nz, double x1, double y1, double z1, double x2,
                         double y2, double z2, double u0, double Re, double dt) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle pointer");
    *h = nullptr;
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    if (nx < 2 || nz < 2 || nx > FDMGPU_MAX_N || nz > FDMGPU_MAX_N || ilog2_exact(nx + 1) < 0 ||
        ilog2_exact(nz + 1) < 0)
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: nx+1 and nz+1 must be powers of two (nx=%d nz=%d)", nx,
                 nz);
    if (!(x2 > x1 && y2 > y1 && z2 > z1 && Re > 0 && dt > 0)) FDM_FAIL(FDMGPU_EINVAL, "bad domain or parameters");
    std::unique_ptr<fdmgpu_nscube> p(new fdmgpu_nscube());
    p->dtype = dtype;
    if (dtype == FDMGPU_F64) {
        p->d.reset(new NSPlanT<double>());
        setup_plan(*p->d, nx, nz, x1, y1, z1, x2, y2, z2, u0, Re, dt);
    } else {
        p->f.reset(new NSPlanT<float>());
        setup_plan(*p->f, nx, nz, x1, y1, z1, x2, y2, z2, u0, Re, dt);
    }
    *h = p.release();
    FDM_API_END
}

int fdmgpu_nscube_step_many(fdmgpu_nscube* const* hs, const int* steps, int n) {
    FDM_API_BEGIN
    if (!hs || !steps || n < 1) FDM_FAIL(FDMGPU_EINVAL, "null argument or no cavity");
    for (int i = 0; i < n; i++) {
        if (!hs[i]) FDM_FAIL(FDMGPU_EINVAL, "null handle");
        for (int j = 0; j < i; j++)
            if (hs[j] == hs[i]) FDM_FAIL(FDMGPU_EINVAL, "cavity %d appears twice", i);
    }
    // nscube_step_many checks the element type, the step counts and the
    // geometry before anything is enqueued
    for (int i = 0; i < n; i++) {
        if (!hs[i]->d) FDM_FAIL(FDMGPU_ENOTSUP, "shared steps are for FP64 cavities");
        if (steps[i] < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
        if (!nscube_mergeable(hs[0], hs[i])) FDM_FAIL(FDMGPU_EINVAL, "cavities of different geometry");
    }
    // the steps run on the first cavity's stream, after the work queued on
    // every cavity's stream and before what is queued there later
    const cudaStream_t st = hs[0]->d->st;
    cudaEvent_t ev = nullptr;
    FDM_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    try {
        for (int i = 1; i < n; i++) {
            FDM_CUDA(cudaEventRecord(ev, hs[i]->d->st));
            FDM_CUDA(cudaStreamWaitEvent(st, ev, 0));
        }
        nscube_step_many(hs, steps, n, st);
        FDM_CUDA(cudaEventRecord(ev, st));
        for (int i = 1; i < n; i++) FDM_CUDA(cudaStreamWaitEvent(hs[i]->d->st, ev, 0));
    } catch (...) {
        cudaEventDestroy(ev);
        throw;
    }
    FDM_CUDA(cudaEventDestroy(ev));
    FDM_API_END
}

int fdmgpu_nscube_step(fdmgpu_nscube* h, int k) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (k < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
    with_plan(h, [&](auto& s) { s.step(k); });
    FDM_API_END
}

int fdmgpu_nscube_set_exact(fdmgpu_nscube* h, int exact) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (exact != 0 && exact != 1) FDM_FAIL(FDMGPU_EINVAL, "exact must be 0 or 1");
    with_plan(h, [&](auto& s) {
        if (s.exact == (exact == 1)) return;
        FDM_CUDA(cudaStreamSynchronize(s.st));
        s.exact = exact == 1;
        // the captured step holds the other form's kernels
        if (s.gexec) cudaGraphExecDestroy(s.gexec);
        if (s.graph) cudaGraphDestroy(s.graph);
        s.gexec = nullptr;
        s.graph = nullptr;
    });
    FDM_API_END
}

int fdmgpu_check_const_division(long long n, const double* d_a, const double* d_b, double* d_q_ieee,
                                double* d_q_const, void* stream) {
    FDM_API_BEGIN
    if (n < 0 || (n > 0 && (!d_a || !d_b || !d_q_ieee || !d_q_const))) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    if (n == 0) return FDMGPU_OK;
    k_cdiv_check<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_a, d_b, d_q_ieee, d_q_const, n);
    FDM_LAUNCH_CHECK();
    FDM_API_END
}

int fdmgpu_nscube_set_stream(fdmgpu_nscube* h, void* stream) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    with_plan(h, [&](auto& s) {
        FDM_CUDA(cudaStreamSynchronize(s.st));
        if (s.own_stream) FDM_CUDA(cudaStreamDestroy(s.st));
        s.own_stream = false;
        s.st = (cudaStream_t)stream;
    });
    FDM_API_END
}

int fdmgpu_nscube_field_info(fdmgpu_nscube* h, int field, size_t* count, int* r) {
    FDM_API_BEGIN
    if (!h || field < 0 || field > 8) FDM_FAIL(FDMGPU_EINVAL, "bad handle or field %d", field);
    with_plan(h, [&](auto& s) {
        const auto& f = s.f[field];
        if (count) *count = (size_t)f.size;
        if (r) {
            r[0] = f.z1; r[1] = f.z2; r[2] = f.y1; r[3] = f.y2; r[4] = f.x1; r[5] = f.x2;
        }
    });
    FDM_API_END
}

/* host buffers hold the handle's element type (double or float) */
int fdmgpu_nscube_get_field(fdmgpu_nscube* h, int field, void* host, size_t count) {
    FDM_API_BEGIN
    if (!h || !host || field < 0 || field > 8) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    with_plan(h, [&](auto& s) {
        const auto& f = s.f[field];
        if (count != (size_t)f.size) FDM_FAIL(FDMGPU_EINVAL, "field has %lld elements, got %zu", f.size, count);
        FDM_CUDA(cudaStreamSynchronize(s.st));
        FDM_CUDA(cudaMemcpy(host, f.p, count * sizeof(*f.p), cudaMemcpyDeviceToHost));
    });
    FDM_API_END
}

int fdmgpu_nscube_set_field(fdmgpu_nscube* h, int field, const void* host, size_t count) {
    FDM_API_BEGIN
    if (!h || !host || field < 0 || field > 8) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    with_plan(h, [&](auto& s) {
        const auto& f = s.f[field];
        if (count != (size_t)f.size) FDM_FAIL(FDMGPU_EINVAL, "field has %lld elements, got %zu", f.size, count);
        FDM_CUDA(cudaStreamSynchronize(s.st));
        FDM_CUDA(cudaMemcpy(f.p, host, count * sizeof(*f.p), cudaMemcpyHostToDevice));
    });
    FDM_API_END
}

int fdmgpu_nscube_field_device(fdmgpu_nscube* h, int field, void** dptr) {
    FDM_API_BEGIN
    if (!h || !dptr || field < 0 || field > 8) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    with_plan(h, [&](auto& s) { *dptr = (void*)s.f[field].p; });
    FDM_API_END
}

int fdmgpu_nscube_dtype(fdmgpu_nscube* h, int* dtype) {
    FDM_API_BEGIN
    if (!h || !dtype) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    *dtype = h->dtype;
    FDM_API_END
}

int fdmgpu_nscube_vtk_out(fdmgpu_nscube* h, const char* path) {
    FDM_API_BEGIN
    if (!h || !path) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    with_plan(h, [&](auto& s) {
        using T = std::remove_reference_t<decltype(*s.f[0].p)>;
        const int nx = s.P.nx, ny = s.P.ny, nz = s.P.nz;
        const long long cells = (long long)nx * ny * nz;
        DevBuf d;
        d.get((size_t)cells * 3 * sizeof(double));
        k_ns_cell_velocity<T><<<(unsigned)((cells + 255) / 256), 256, 0, s.st>>>(s.f[0], s.f[1], s.f[2], s.P,
                                                                                 (double*)d.p);
        FDM_LAUNCH_CHECK();
        std::vector<double> c((size_t)cells * 3);
        FDM_CUDA(cudaStreamSynchronize(s.st));
        FDM_CUDA(cudaMemcpy(c.data(), d.p, c.size() * sizeof(double), cudaMemcpyDeviceToHost));
        FILE* f = fopen(path, "wb");
        if (!f) FDM_FAIL(FDMGPU_EINVAL, "cannot open %s for writing", path);
        // header and number format of velocity_plotter::vtk_out for a cube
        // (src/velocity_plot.cpp:113-119, 200-217)
        fprintf(f, "# vtk DataFile Version 3.0\n");
        fprintf(f, "step %d\n", s.time_index);
        fprintf(f, "ASCII\n");
        fprintf(f, "DATASET STRUCTURED_POINTS\n");
        fprintf(f, "DIMENSIONS %d %d %d\n", nx, ny, nz);
        fprintf(f, "ASPECT_RATIO 1 1 1\n");
        fprintf(f, "ORIGIN %f %f %f\n", s.x1, s.y1, s.z1);
        fprintf(f, "SPACING %f %f %f\n", s.P.dx, s.P.dy, s.P.dz);
        fprintf(f, "POINT_DATA %lld\n", cells);
        fprintf(f, "VECTORS u double\n");
        for (long long e = 0; e < cells; e++) fprintf(f, "%f %f %f\n", c[3 * e], c[3 * e + 1], c[3 * e + 2]);
        const bool ok = ferror(f) == 0;
        fclose(f);
        if (!ok) FDM_FAIL(FDMGPU_EINVAL, "write to %s failed", path);
    });
    FDM_API_END
}

int fdmgpu_nscube_time_index(fdmgpu_nscube* h, int* t) {
    FDM_API_BEGIN
    if (!h || !t) FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    with_plan(h, [&](auto& s) { *t = s.time_index; });
    FDM_API_END
}

int fdmgpu_nscube_destroy(fdmgpu_nscube* h) {
    FDM_API_BEGIN
    delete h;
    FDM_API_END
}

}  // extern "C"
