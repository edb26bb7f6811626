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

// Partitioned tridiagonal solve along z for the (x-mode, y-mode) lines of
// a batch of volumes (x fastest, line stride nx*ny): the same Dirichlet
// systems as k_tridiag_const,
//     u[i-1] + b u[i] + u[i+1] = gscale * g[i],  b = -2 - (lamx[x] + lamy[y]) h2,
// for n = P(m+1) - 1 rows (n+1 and m+1 powers of two).  The line is cut by
// P-1 separator rows (row c(m+1)+m) into P blocks of m rows.  Warp c of the
// CTA owns block c for 32 consecutive x: it loads its m rows coalesced into
// registers and solves the block with zero ends (v) and the responses to a
// unit value at either end (beta at the right end; by persymmetry of the
// constant-coefficient block the left-end response is beta reversed).  The
// separator values then satisfy a constant-coefficient tridiagonal system of
// P-1 unknowns,
//     beta_0 s[c-1] + (b + 2 beta_{m-1}) s[c] + beta_0 s[c+1]
//         = g(sep_c) - v^c_{m-1} - v^{c+1}_0,
// which one lane per column solves from shared memory; each block then adds
// the end responses and stores.  Every value is read and written once.
template <typename T, int m>
constexpr int zpart_max_threads() { return m * sizeof(T) >= 31 * 4 ? 256 : 512; }

template <typename T, int m>
__global__ void __launch_bounds__(zpart_max_threads<T, m>()) k_zsolve_part(T* W, int nx, int ny, int P, long long vstride,
                                                     const T* lamx, const T* lamy, T h2, T gscale) {
    extern __shared__ __align__(16) unsigned char zsm[];
    T* s_vf = reinterpret_cast<T*>(zsm);  // [P][32] first row of v per block
    T* s_vl = s_vf + P * 32;               // [P][32] last row of v
    T* s_g = s_vl + P * 32;                // [P][32] separator right-hand sides
    T* s_u = s_g + P * 32;                 // [P][32] separator solutions
    const int lane = threadIdx.x & 31;
    const int c = threadIdx.x >> 5;
    const int ntx = (nx + 31) >> 5;
    const int y = blockIdx.x / ntx;
    const int x = ((blockIdx.x - y * ntx) << 5) + lane;
    const bool act = x < nx;
    const long long st = (long long)nx * ny;
    T* p = W + (long long)blockIdx.y * vstride + (long long)y * nx + (act ? x : 0);
    const T b = act ? T(-2) - (lamx[x] + lamy[y]) * h2 : T(-4);
    const int r0 = c * (m + 1);

    T v[m], cp[m], be[m];
#pragma unroll
    for (int i = 0; i < m; i++) v[i] = act ? p[(r0 + i) * st] : T(0);
    T gsep = T(0);
    if (c < P - 1 && act) gsep = p[(r0 + m) * st];
    // forward elimination
    T prev_c = T(0), prev_d = T(0);
#pragma unroll
    for (int i = 0; i < m; i++) {
        const T r = T(1) / (b - prev_c);
        cp[i] = r;
        prev_d = (v[i] * gscale - prev_d) * r;
        v[i] = prev_d;
        prev_c = r;
    }
    // back substitution for v and the right-end response beta
    T bv = -cp[m - 1];
    be[m - 1] = bv;
#pragma unroll
    for (int i = m - 2; i >= 0; i--) {
        v[i] = v[i] - cp[i] * v[i + 1];
        bv = -cp[i] * bv;
        be[i] = bv;
    }
    s_vf[c * 32 + lane] = v[0];
    s_vl[c * 32 + lane] = v[m - 1];
    s_g[c * 32 + lane] = gsep * gscale;
    __syncthreads();
    if (c == 0 && P > 1) {
        // separators: constant-coefficient Thomas, P-1 rows
        const T lo = be[0], dg = b + T(2) * be[m - 1];
        T pc = T(0), pd = T(0);
        for (int k = 0; k < P - 1; k++) {
            const T rhs = s_g[k * 32 + lane] - s_vl[k * 32 + lane] - s_vf[(k + 1) * 32 + lane];
            const T r = T(1) / (dg - lo * pc);
            pc = lo * r;
            pd = (rhs - lo * pd) * r;
            s_u[k * 32 + lane] = pd;  // d' for now
            s_vf[k * 32 + lane] = pc;  // c' (v_first of block k is no longer needed)
        }
        T u = T(0);
        for (int k = P - 2; k >= 0; k--) {
            u = s_u[k * 32 + lane] - s_vf[k * 32 + lane] * u;
            s_u[k * 32 + lane] = u;
        }
    }
    __syncthreads();
    const T ul = c > 0 ? s_u[(c - 1) * 32 + lane] : T(0);
    const T ur = c < P - 1 ? s_u[c * 32 + lane] : T(0);
    if (act) {
#pragma unroll
        for (int i = 0; i < m; i++) p[(r0 + i) * st] = v[i] + be[m - 1 - i] * ul + be[i] * ur;
        if (c < P - 1) p[(r0 + m) * st] = ur;
    }
}

// The same partitioned solve with every mode-dependent factor read from a
// table built once per plan (zsolve_table_host): for mode (x, y) the block
// pivot reciprocals cp[0..m-1], the right-end response beta[0..m-1] and the
// separator system's pivot reciprocals rc[0..P-2] and multipliers
// pc[0..P-2], stored value-major (tab[v * modes + mode]) so lanes read
// consecutive modes.  With no divisions left the kernel is FMA chains plus
// coalesced loads; at 255^2 modes the FP32 table is 15.6 MB and stays in L2.
// MINB: resident CTAs per SM the register allocation is held to.
template <typename T, int m, int MINB = 2>
__global__ void __launch_bounds__(512, MINB) k_zsolve_tab(T* W, int nx, int ny, int P, long long vstride,
                                                    const T* __restrict__ tab, T gscale) {
    extern __shared__ __align__(16) unsigned char zsm[];
    T* s_vf = reinterpret_cast<T*>(zsm);
    T* s_vl = s_vf + P * 32;
    T* s_g = s_vl + P * 32;
    T* s_u = s_g + P * 32;
    const int lane = threadIdx.x & 31;
    const int c = threadIdx.x >> 5;
    const int ntx = (nx + 31) >> 5;
    const int y = blockIdx.x / ntx;
    const int x = ((blockIdx.x - y * ntx) << 5) + lane;
    const bool act = x < nx;
    const int modes = nx * ny;
    const int mode = y * nx + (act ? x : 0);
    const int st = nx * ny;
    const int r0 = c * (m + 1);
    T* p = W + (long long)blockIdx.y * vstride + (long long)r0 * st + (long long)y * nx + (act ? x : 0);

    T v[m], cp[m];
#pragma unroll
    for (int i = 0; i < m; i++) v[i] = act ? p[i * st] : T(0);
#pragma unroll
    for (int i = 0; i < m; i++) cp[i] = tab[(size_t)i * modes + mode];
    T gsep = T(0);
    if (c < P - 1 && act) gsep = p[m * st];
    T prev = T(0);
#pragma unroll
    for (int i = 0; i < m; i++) {
        prev = (v[i] * gscale - prev) * cp[i];
        v[i] = prev;
    }
#pragma unroll
    for (int i = m - 2; i >= 0; i--) v[i] = v[i] - cp[i] * v[i + 1];
    s_vf[c * 32 + lane] = v[0];
    s_vl[c * 32 + lane] = v[m - 1];
    s_g[c * 32 + lane] = gsep * gscale;
    const T* be = tab + (size_t)m * modes + mode;
    // warp c copies separator row c's factors into shared memory before the
    // barrier, so their latency overlaps the block solves
    T* s_rc = s_u + P * 32;
    T* s_pc = s_rc + P * 32;
    if (c < P - 1) {
        s_rc[c * 32 + lane] = tab[(size_t)(2 * m + c) * modes + mode];
        s_pc[c * 32 + lane] = tab[(size_t)(2 * m + P - 1 + c) * modes + mode];
    }
    __syncthreads();
    if (c == 0 && P > 1) {
        const T lo = be[0];
        T d = T(0);
        for (int k = 0; k < P - 1; k++) {
            const T rhs = s_g[k * 32 + lane] - s_vl[k * 32 + lane] - s_vf[(k + 1) * 32 + lane];
            d = (rhs - lo * d) * s_rc[k * 32 + lane];
            s_u[k * 32 + lane] = d;
        }
        T u = T(0);
        for (int k = P - 2; k >= 0; k--) {
            u = s_u[k * 32 + lane] - s_pc[k * 32 + lane] * u;
            s_u[k * 32 + lane] = u;
        }
    }
    __syncthreads();
    const T ul = c > 0 ? s_u[(c - 1) * 32 + lane] : T(0);
    const T ur = c < P - 1 ? s_u[c * 32 + lane] : T(0);
    if (act) {
#pragma unroll
        for (int i = 0; i < m; i++) cp[i] = be[(size_t)i * modes];
#pragma unroll
        for (int i = 0; i < m; i++) p[i * st] = v[i] + cp[m - 1 - i] * ul + cp[i] * ur;
        if (c < P - 1) p[m * st] = ur;
    }
}

}  // namespace fdmgpu
