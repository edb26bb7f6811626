// Tridiagonal, residual and combine kernels of the GB300 Poisson solver.
#pragma once

#include "common.cuh"

namespace fdmgpu {

// Maximum line length of the constant-coefficient tridiagonal kernel
// (kTriCk * kTriMaxCk).
constexpr int kTriCk = 16;
constexpr int kTriMaxCk = 64;

// Solves, for every line l of a batch, the Dirichlet system
//     u[i-1] + b_l u[i] + u[i+1] = gscale * g[i],  i = 0..n-1,  u[-1] = u[n] = 0,
// in place, with b_l = -2 - (lamA[l % A] + lamB[l / A]) * h2.  This is the
// 1-D operator (u[i-1] - 2u[i] + u[i+1])/h^2 - lambda shifted by the modes of
// the other axes, i.e. what the reference inverts with DST_z, the division by
// -(lm_z+lm_y+lm_x) and the inverse DST_z (src/lapl_cube.cpp:13-30, :70-84,
// :124-141), and what LaplRect inverts with gtsv per y-mode
// (src/lapl_rect.cpp:44-61, :85-92).
//
// One thread per line, Thomas elimination.  The forward sweep writes d'
// in place; the pivots c'_i = 1/(b - c'_{i-1}) depend only on the line's b,
// so the backward sweep recomputes them from checkpoints taken every kTriCk
// rows instead of storing them.  Loads and stores go kTriCk rows at a time
// so each thread keeps kTriCk independent memory operations in flight.
// Line base = (l % A) * sa + (l / A) * sb; element stride st.
template <typename T>
__global__ void __launch_bounds__(128) k_tridiag_const(T* W, int nlines, int n, int A, long long sa,
                                                       long long sb, long long st, long long vstride,
                                                       const T* lamA, const T* lamB, T h2, T gscale) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nlines) return;
    const int la = l % A, lb = l / A;
    T lam = T(0);
    if (lamA) lam += lamA[la];
    if (lamB) lam += lamB[lb];
    const T b = T(-2) - lam * h2;
    T* p = W + (long long)blockIdx.y * vstride + la * sa + lb * sb;

    T ck[kTriMaxCk];
    T cp = T(0), dp = T(0);
    const int nblk = (n + kTriCk - 1) / kTriCk;
    for (int blk = 0; blk < nblk; blk++) {
        const int i0 = blk * kTriCk;
        ck[blk] = cp;
        T g[kTriCk];
#pragma unroll
        for (int q = 0; q < kTriCk; q++)
            if (i0 + q < n) g[q] = p[(i0 + q) * st];
#pragma unroll
        for (int q = 0; q < kTriCk; q++) {
            if (i0 + q < n) {
                const T r = T(1) / (b - cp);
                cp = r;
                dp = (g[q] * gscale - dp) * r;
                g[q] = dp;
            }
        }
#pragma unroll
        for (int q = 0; q < kTriCk; q++)
            if (i0 + q < n) p[(i0 + q) * st] = g[q];
    }
    T u = T(0);
    for (int blk = nblk - 1; blk >= 0; blk--) {
        const int i0 = blk * kTriCk;
        T c = ck[blk];
        T cc[kTriCk], d[kTriCk];
#pragma unroll
        for (int q = 0; q < kTriCk; q++) {
            if (i0 + q < n) {
                c = T(1) / (b - c);
                cc[q] = c;
                d[q] = p[(i0 + q) * st];
            }
        }
#pragma unroll
        for (int q = kTriCk - 1; q >= 0; q--) {
            if (i0 + q < n) {
                u = d[q] - cc[q] * u;
                d[q] = u;
            }
        }
#pragma unroll
        for (int q = 0; q < kTriCk; q++)
            if (i0 + q < n) p[(i0 + q) * st] = d[q];
    }
}

// General tridiagonal systems, system-interleaved: element i of system s at
// [i*nsys + s].  lower[0] and upper[n-1] are ignored.  Thomas elimination
// without pivoting (as solve_tdiag_linear_my, src/asp_gauss.cpp:185-207);
// the modified upper diagonal goes to `cwork`, the solution to b.
template <typename T>
__global__ void k_tridiag_general(int n, int nsys, const T* lower, const T* diag, const T* upper, T* b,
                                  T* cwork) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    T cp = T(0), dp = T(0);
    for (int i = 0; i < n; i++) {
        const long long o = (long long)i * nsys + s;
        const T lo = i > 0 ? lower[o] : T(0);
        const T den = diag[o] - lo * cp;
        const T r = T(1) / den;
        cp = (i < n - 1) ? upper[o] * r : T(0);
        dp = (b[o] - lo * dp) * r;
        cwork[o] = cp;
        b[o] = dp;
    }
    T u = T(0);
    for (int i = n - 1; i >= 0; i--) {
        const long long o = (long long)i * nsys + s;
        u = b[o] - cwork[o] * u;
        b[o] = u;
    }
}

// r = f - inv_s * A(uhi + ulo) for the 7-point operator
// A u = cx(u[j-1] - 2u + u[j+1]) + cy(...) + cz(...), zero outside the box.
// FP64 arithmetic; r rounded to FP32.  ulo may be null.
__global__ void k_residual_f64(const double* __restrict__ f, const float* __restrict__ uhi,
                               const float* __restrict__ ulo, float* __restrict__ r, int nx, int ny, int nz,
                               long long vstride, double inv_s, double cx, double cy, double cz) {
    const long long vol = (long long)nx * ny * nz;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= vol) return;
    const long long off = (long long)blockIdx.y * vstride;
    const int j = idx % nx;
    const long long t = idx / nx;
    const int k = t % ny;
    const int i = t / ny;
    const long long sy = nx, sz = (long long)nx * ny;
    auto U = [&](long long o) -> double {
        double v = (double)uhi[off + o];
        if (ulo) v += (double)ulo[off + o];
        return v;
    };
    const double uc = U(idx);
    const double xm = j > 0 ? U(idx - 1) : 0.0, xp = j < nx - 1 ? U(idx + 1) : 0.0;
    const double ym = k > 0 ? U(idx - sy) : 0.0, yp = k < ny - 1 ? U(idx + sy) : 0.0;
    const double zm = i > 0 ? U(idx - sz) : 0.0, zp = i < nz - 1 ? U(idx + sz) : 0.0;
    const double au = cx * ((xm + xp) - 2.0 * uc) + cy * ((ym + yp) - 2.0 * uc) + cz * ((zm + zp) - 2.0 * uc);
    r[off + idx] = (float)(f[off + idx] - inv_s * au);
}

// Last refinement sweep: out = uhi + ulo_in + c in FP64; otherwise
// ulo_out = ulo_in + c in FP32 (ulo_in may be null = zero).
// Accumulates ||c||^2 and ||u||^2 per volume into norms[2*v], norms[2*v+1].
__global__ void k_combine(const float* __restrict__ uhi, const float* ulo_in, const float* __restrict__ c,
                          double* __restrict__ out, float* ulo_out, long long vol, long long vstride, int last,
                          double* __restrict__ norms) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long off = (long long)blockIdx.y * vstride;
    double cc = 0.0, uu = 0.0;
    if (idx < vol) {
        const float cf = c[off + idx];
        const float lo = ulo_in ? ulo_in[off + idx] : 0.f;
        const double ch = (double)cf;
        const double u = (double)uhi[off + idx] + (double)lo + ch;
        if (last) out[off + idx] = u;
        else ulo_out[off + idx] = lo + cf;
        cc = ch * ch;
        uu = u * u;
    }
    for (int o = 16; o > 0; o >>= 1) {
        cc += __shfl_down_sync(0xffffffffu, cc, o);
        uu += __shfl_down_sync(0xffffffffu, uu, o);
    }
    __shared__ double red[2][32];
    const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
    if (ln == 0) { red[0][w] = cc; red[1][w] = uu; }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        cc = ln < nw ? red[0][ln] : 0.0;
        uu = ln < nw ? red[1][ln] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            cc += __shfl_down_sync(0xffffffffu, cc, o);
            uu += __shfl_down_sync(0xffffffffu, uu, o);
        }
        if (ln == 0) {
            atomicAdd(&norms[2 * blockIdx.y], cc);
            atomicAdd(&norms[2 * blockIdx.y + 1], uu);
        }
    }
}

}  // namespace fdmgpu
