// DST-I line transforms for the GB300 Poisson solver.
//
// Computes, for every line x[1..n] of a batch (N = n+1 = 2^q),
//     F[k] = scale * sum_{j=1}^{n} x[j] sin(pi j k / N),   k = 1..n,
// which is the transform of the reference's FFT<T>::sFFT (src/fft.cpp:294-365)
// with its `dx` argument as `scale`.  The reference computes it with the
// Samarskii-Nikolaev real recursion, one line per OpenMP thread.  Here a line
// is owned by a group of kGroup threads and goes through
//   1. the sine-weight fold y_j = sin(pi j/N)(x_j + x_{N-j}) + (x_j - x_{N-j})/2
//      that turns the DST into a real DFT of length N,
//   2. a radix-4 (+ one radix-2) Stockham complex FFT of length M = N/2 in
//      shared memory (the real DFT packed as y_{2m} + i y_{2m+1}),
//   3. the real-DFT unpack, where F[2k] = -Im Y_k and the odd outputs are a
//      prefix sum F[2k+1] = F[2k-1] + Re Y_k (segmented warp scan).
// Twiddle and weight tables are computed in FP64 on the host and rounded to
// the compute type once.
//
// Shared-memory layouts are skewed (one pad slot every 16 complex / 32 real
// entries) so that the contiguous per-thread blocks of the unpack and prefix
// sum fall into distinct banks.
#pragma once

#include "common.cuh"
#include "dd.cuh"

namespace fdmgpu {

constexpr int kGroup = 8;  // threads per line

template <typename T>
struct SineTables {
    const vec2_t<T>* tw;    // e^{-2 pi i k / M}, k = 0..M-1
    const vec2_t<T>* post;  // e^{-2 pi i k / N}, k = 0..M-1
    const T* wpre;          // sin(pi j / N), j = 0..N-1
    int N, M;
};

// complex slots per line of a Stockham buffer: holds M entries skewed by
// k + k/16, and is 8 (mod 16) so the two lines of a half-warp use disjoint
// bank pairs
__host__ __device__ inline int sine_line_stride(int M) {
    int S = M + M / 16 + 1;
    while (S % 16 != 8) S++;
    return S;
}
__host__ __device__ __forceinline__ int skew_c(int k) { return k + (k >> 4); }
// reals per line of the staging view (x[0..N] / F[1..N-1], skewed by i/32);
// odd, so transposed accesses by consecutive threads hit distinct banks
__host__ __device__ inline int sine_stage_stride(int N) {
    int SX = N + N / 32 + 2;
    if (SX % 2 == 0) SX++;
    return SX;
}
__host__ __device__ __forceinline__ int skew_r(int i) { return i + (i >> 5); }

template <typename T>
__host__ __device__ inline size_t sine_smem_bytes(int N, int L) {
    return 2ull * L * sine_line_stride(N / 2) * sizeof(vec2_t<T>);
}

// x / d for 0 <= x < 2^31 by multiply-high (Granlund-Montgomery round-up
// method).
struct FastDiv {
    unsigned d, m, s;
    FastDiv() : d(1), m(0), s(0) {}
    explicit FastDiv(unsigned div) : d(div) {
        s = 0;
        while ((1u << s) < d) s++;
        m = (unsigned)((((unsigned long long)1 << 32) * ((1ull << s) - d)) / d + 1);
    }
    __device__ __forceinline__ unsigned div(unsigned x) const { return (__umulhi(x, m) + x) >> s; }
};

// s + e += v with the rounding error of the addition kept in e (TwoSum);
// plain addition for FP64.
template <typename T>
__device__ __forceinline__ void acc_add(T& s, T& e, T v);
template <>
__device__ __forceinline__ void acc_add<float>(float& s, float& e, float v) {
    const ff t = two_sum(s, v);
    s = t.h;
    e = __fadd_rn(e, t.l);
}
template <>
__device__ __forceinline__ void acc_add<double>(double& s, double& e, double v) {
    s += v;
}

// Runs the transform of every line held by this CTA.  On entry the staging
// view of buffer B holds x[1..n] of line l at stage(B) + l*SX + skew_r(j)
// (entries 0 and N zero).  On exit the unscaled result F[1..n] sits in the
// staging view of the buffer returned, same skewed indexing.  All threads of
// the CTA must call it.
template <typename T>
__device__ T* sine_block(vec2_t<T>* A, vec2_t<T>* B, const SineTables<T>& tb, int l, int g) {
    using T2 = vec2_t<T>;
    const int N = tb.N, M = tb.M;
    const int S = sine_line_stride(M), SX = sine_stage_stride(N);

    // 1. fold + pack
    {
        const T* X = reinterpret_cast<const T*>(B) + (size_t)l * SX;
        T2* Al = A + (size_t)l * S;
        const T half = T(0.5);
        for (int m = g; m < M; m += kGroup) {
            const int j0 = 2 * m, j1 = 2 * m + 1;
            T y0 = T(0);
            if (m > 0) {
                T a = X[skew_r(j0)], b = X[skew_r(N - j0)];
                y0 = ldg(tb.wpre + j0) * (a + b) + half * (a - b);
            }
            T a = X[skew_r(j1)], b = X[skew_r(N - j1)];
            T y1 = ldg(tb.wpre + j1) * (a + b) + half * (a - b);
            T2 v; v.x = y0; v.y = y1;
            Al[m] = v;  // M == 1: no passes, and skew_c(0) == 0
        }
    }
    __syncthreads();

    // 2. Stockham passes, A -> B -> A ...; the last pass writes skewed
    T2* src = A;
    T2* dst = B;
    for (int Ns = 1; Ns < M;) {
        const int R = ((M / Ns) % 4 == 0) ? 4 : 2;
        const int MR = M / R;
        const int twstep = M / (Ns * R);
        const bool last = Ns * R == M;
        const T2* s = src + (size_t)l * S;
        T2* d = dst + (size_t)l * S;
        for (int j = g; j < MR; j += kGroup) {
            const int k = j & (Ns - 1);
            const int base = (j - k) * R + k;
            if (R == 4) {
                T2 v0 = s[j], v1 = s[j + MR], v2 = s[j + 2 * MR], v3 = s[j + 3 * MR];
                if (k) {
                    v1 = cmul<T>(v1, ldg(tb.tw + k * twstep));
                    v2 = cmul<T>(v2, ldg(tb.tw + 2 * k * twstep));
                    v3 = cmul<T>(v3, ldg(tb.tw + 3 * k * twstep));
                }
                T2 a0 = cadd<T>(v0, v2), a1 = csub<T>(v0, v2);
                T2 b0 = cadd<T>(v1, v3), b1 = cmul_mi<T>(csub<T>(v1, v3));
                if (last) {
                    d[skew_c(base)] = cadd<T>(a0, b0);
                    d[skew_c(base + Ns)] = cadd<T>(a1, b1);
                    d[skew_c(base + 2 * Ns)] = csub<T>(a0, b0);
                    d[skew_c(base + 3 * Ns)] = csub<T>(a1, b1);
                } else {
                    d[base] = cadd<T>(a0, b0);
                    d[base + Ns] = cadd<T>(a1, b1);
                    d[base + 2 * Ns] = csub<T>(a0, b0);
                    d[base + 3 * Ns] = csub<T>(a1, b1);
                }
            } else {
                T2 v0 = s[j], v1 = s[j + MR];
                if (k) v1 = cmul<T>(v1, ldg(tb.tw + k * twstep));
                const int o0 = last ? skew_c(base) : base;
                const int o1 = last ? skew_c(base + Ns) : base + Ns;
                d[o0] = cadd<T>(v0, v1);
                d[o1] = csub<T>(v0, v1);
            }
        }
        __syncwarp();
        T2* t = src; src = dst; dst = t;
        Ns *= R;
    }
    __syncthreads();

    // 3. unpack + odd-output prefix sum; results into the other buffer
    const T2* C = src + (size_t)l * S;
    T* F = reinterpret_cast<T*>(dst) + (size_t)l * SX;
    const int kb = (M + kGroup - 1) / kGroup;
    const int k0 = g * kb;
    const int k1 = min(M, k0 + kb);
    // The odd outputs are a running sum of M terms; it is accumulated with
    // an error term (float-float for FP32) so the rounding does not grow with
    // the line length.
    T sum = T(0), sum_e = T(0);
    for (int k = k0; k < k1; k++) {
        const T2 ck = C[skew_c(k)];
        const T2 cm = C[skew_c((M - k) & (M - 1))];
        T ex = T(0.5) * (ck.x + cm.x), ey = T(0.5) * (ck.y - cm.y);
        T ox = T(0.5) * (ck.y + cm.y), oy = T(-0.5) * (ck.x - cm.x);
        const T2 w = ldg(tb.post + k);
        T yr = ex + (w.x * ox - w.y * oy);
        T yi = ey + (w.x * oy + w.y * ox);
        if (k == 0) yr *= T(0.5);
        else F[skew_r(2 * k)] = -yi;
        F[skew_r(2 * k + 1)] = yr;
        acc_add<T>(sum, sum_e, yr);
    }
    // exclusive scan of the per-thread totals across the line's group
    T incl = sum, incl_e = sum_e;
#pragma unroll
    for (int off = 1; off < kGroup; off <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, incl, off, kGroup);
        T te = __shfl_up_sync(0xffffffffu, incl_e, off, kGroup);
        if (g >= off) {
            acc_add<T>(incl, incl_e, t);
            incl_e += te;
        }
    }
    T run = incl, run_e = incl_e;
    acc_add<T>(run, run_e, -sum);
    run_e -= sum_e;
    for (int k = k0; k < k1; k++) {
        acc_add<T>(run, run_e, F[skew_r(2 * k + 1)]);
        F[skew_r(2 * k + 1)] = run + run_e;
    }
    __syncthreads();
    return reinterpret_cast<T*>(dst);
}

// What a pass does around the transform.
enum SineMode {
    kPlain = 0,    // load Tin -> T, store T -> Tout
    kRound = 1,    // load FP64 -> FP32 by integer rounding (first pass of the mixed solve)
    kResidual = 2, // load r = f - A(uhi + ulo) in float-float (first pass of a refinement sweep)
    kCombine = 3   // store u = uhi + ulo + c to FP64, or ulo += c (last pass of a sweep)
};

struct SineFused {
    // kResidual
    const double* f;
    const float* uhi;
    const float* ulo;
    ff cx, cy, cz;        // stencil coefficients 1/h^2 / S as float pairs
    float cxf, cyf, czf;  // the same rounded to float (for A ulo)
    int iso;              // cx == cy == cz: one coefficient times the 6-neighbour sum
    // kCombine
    double* out64;
    float* ulo_out;  // when set: ulo += c (the float low part of u, kept for a further sweep)
    int last;        // write u = uhi + ulo + c to the FP64 output
    double* norms;  // per volume: ||c||^2, ||u||^2
    // optional per-volume pointers (device arrays indexed by blockIdx.y) for
    // the user-facing input (kRound / kPlain loads, the residual's f) and
    // output (kPlain stores, kCombine's FP64 result); null = volumes back to
    // back from the kernel's base pointer
    const void* const* vin;
    void* const* vout;
};

struct SineGeom {
    int nx, ny, nz;
    long long vstride;
    int L, Lshift;
    FastDiv div_n;   // by the line length n
    FastDiv div_ny;  // rows -> (z, y)
};

constexpr int kLoadBatch = 8;

// r = f - A(uhi + ulo) at one interior point (x fastest index idx), zero
// outside the box.  A U is formed exactly enough in float-float; A ulo in
// FP32 (it is ~1e-7 of A U).
__device__ __forceinline__ float residual_at(const SineFused& fu, long long idx, int x, int y, int z, int nx,
                                             int ny, int nz) {
    const long long sy = nx, sz = (long long)nx * ny;
    const float* U = fu.uhi;
    const float uc = U[idx];
    const float xm = x > 0 ? U[idx - 1] : 0.f, xp = x < nx - 1 ? U[idx + 1] : 0.f;
    const float ym = y > 0 ? U[idx - sy] : 0.f, yp = y < ny - 1 ? U[idx + sy] : 0.f;
    const float zm = z > 0 ? U[idx - sz] : 0.f, zp = z < nz - 1 ? U[idx + sz] : 0.f;
    const ff fsp = f64_split(fu.f[idx]);
    const float u2 = uc + uc;  // exact
    ff dx = ff_add_f(two_sum(xm, xp), -u2);
    ff dy = ff_add_f(two_sum(ym, yp), -u2);
    ff dz = ff_add_f(two_sum(zm, zp), -u2);
    ff au = ff_add(ff_add(ff_mul(dx, fu.cx), ff_mul(dy, fu.cy)), ff_mul(dz, fu.cz));
    float alo = 0.f;
    if (fu.ulo) {
        const float* V = fu.ulo;
        const float vc = V[idx];
        const float vxm = x > 0 ? V[idx - 1] : 0.f, vxp = x < nx - 1 ? V[idx + 1] : 0.f;
        const float vym = y > 0 ? V[idx - sy] : 0.f, vyp = y < ny - 1 ? V[idx + sy] : 0.f;
        const float vzm = z > 0 ? V[idx - sz] : 0.f, vzp = z < nz - 1 ? V[idx + sz] : 0.f;
        alo = fu.cxf * ((vxm + vxp) - 2.f * vc) + fu.cyf * ((vym + vyp) - 2.f * vc) + fu.czf * ((vzm + vzp) - 2.f * vc);
    }
    ff r = ff_add(fsp, ff{-au.h, -au.l});
    return (r.h + (r.l - alo));
}

// r = f - A(uhi + ulo) for every interior point of a batch of volumes,
// float-float as residual_at, written as FP32.  A thread takes kResX
// consecutive x of one row: the row's values (with one halo on each side)
// are loaded once and shared for the x-neighbours; the y and z neighbours
// are coalesced along x and served by L1/L2.  gridDim.y indexes the volume.
constexpr int kResX = 4;

__device__ __forceinline__ float ff_residual(const ff& fsp, float uc, float xm, float xp, float ym, float yp,
                                             float zm, float zp, const SineFused& fu, float alo) {
    const float u2 = uc + uc;
    ff dx = ff_add_f(two_sum(xm, xp), -u2);
    ff dy = ff_add_f(two_sum(ym, yp), -u2);
    ff dz = ff_add_f(two_sum(zm, zp), -u2);
    ff au = ff_add(ff_add(ff_mul(dx, fu.cx), ff_mul(dy, fu.cy)), ff_mul(dz, fu.cz));
    ff r = ff_add(fsp, ff{-au.h, -au.l});
    return r.h + (r.l - alo);
}

// Isotropic stencil: A u = c (sum of the 6 neighbours - 6 u).  The sum is
// accumulated as a float plus a float error term (TwoSum per addition), then
// joined with -6u and multiplied by c in float-float.
__device__ __forceinline__ float ff_residual_iso(const ff& fsp, float uc, float xm, float xp, float ym, float yp,
                                                 float zm, float zp, const ff& c, float alo) {
    ff t = two_sum(xm, xp);
    float e = t.l;
    t = two_sum(t.h, ym);
    e = __fadd_rn(e, t.l);
    t = two_sum(t.h, yp);
    e = __fadd_rn(e, t.l);
    t = two_sum(t.h, zm);
    e = __fadd_rn(e, t.l);
    t = two_sum(t.h, zp);
    e = __fadd_rn(e, t.l);
    const ff u6 = two_prod(6.f, uc);
    t = two_sum(t.h, -u6.h);
    e = __fadd_rn(e, __fsub_rn(t.l, u6.l));
    const ff sg = fast_two_sum(t.h, e);
    const ff au = ff_mul(sg, c);
    const ff r = ff_add(fsp, ff{-au.h, -au.l});
    return r.h + (r.l - alo);
}

__global__ void __launch_bounds__(256) k_residual(SineFused fu, float* __restrict__ r, int nx, int ny, int nz,
                                                  long long vstride, int segs, FastDiv div_segs, FastDiv div_ny) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int rows = ny * nz;
    if (t >= rows * segs) return;
    const long long voff = (long long)blockIdx.y * vstride;
    const int row = div_segs.div(t), seg = t - row * segs;
    const int z = div_ny.div(row), y = row - z * ny;
    const int x0 = seg * kResX;
    const long long rb = (long long)row * nx;
    const long long sy = nx, sz = (long long)nx * ny;
    const float* U = fu.uhi + voff;
    const float* V = fu.ulo ? fu.ulo + voff : nullptr;
    const double* F = fu.vin ? (const double*)fu.vin[blockIdx.y] : fu.f + voff;
    float c[kResX + 2];
#pragma unroll
    for (int q = 0; q < kResX + 2; q++) {
        const int x = x0 - 1 + q;
        c[q] = (x >= 0 && x < nx) ? U[rb + x] : 0.f;
    }
    float ym[kResX], yp[kResX], zm[kResX], zp[kResX];
    double fv[kResX];
#pragma unroll
    for (int q = 0; q < kResX; q++) {
        const int x = x0 + q;
        const bool in = x < nx;
        const long long i = rb + x;
        ym[q] = (in && y > 0) ? U[i - sy] : 0.f;
        yp[q] = (in && y < ny - 1) ? U[i + sy] : 0.f;
        zm[q] = (in && z > 0) ? U[i - sz] : 0.f;
        zp[q] = (in && z < nz - 1) ? U[i + sz] : 0.f;
        fv[q] = in ? F[i] : 0.0;
    }
#pragma unroll
    for (int q = 0; q < kResX; q++) {
        const int x = x0 + q;
        if (x >= nx) break;
        const long long i = rb + x;
        float alo = 0.f;
        if (V) {
            const float vc = V[i];
            const float vxm = x > 0 ? V[i - 1] : 0.f, vxp = x < nx - 1 ? V[i + 1] : 0.f;
            const float vym = y > 0 ? V[i - sy] : 0.f, vyp = y < ny - 1 ? V[i + sy] : 0.f;
            const float vzm = z > 0 ? V[i - sz] : 0.f, vzp = z < nz - 1 ? V[i + sz] : 0.f;
            alo = fu.cxf * ((vxm + vxp) - 2.f * vc) + fu.cyf * ((vym + vyp) - 2.f * vc) +
                  fu.czf * ((vzm + vzp) - 2.f * vc);
        }
        r[voff + i] = fu.iso ? ff_residual_iso(f64_split(fv[q]), c[q + 1], c[q], c[q + 2], ym[q], yp[q], zm[q], zp[q],
                                               fu.cx, alo)
                             : ff_residual(f64_split(fv[q]), c[q + 1], c[q], c[q + 2], ym[q], yp[q], zm[q], zp[q], fu,
                                           alo);
    }
}

// One DST pass over every line along x (AXIS 0, rows) or along y (AXIS 1,
// columns) of a batch of nz*ny*nx volumes (x fastest), out-of-place or
// in-place.  Rows: a CTA takes L consecutive rows.  Columns: a CTA takes a
// tile of L consecutive x at one z, all y.  gridDim.y indexes the volume.
template <typename Tin, typename T, typename Tout, int AXIS, int MODE>
__global__ void __launch_bounds__(256) k_sine_pass(const Tin* in, Tout* out, SineGeom geo, SineTables<T> tb,
                                                   T scale, SineFused fu) {
    using T2 = vec2_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = tb.M, N = tb.N, L = geo.L;
    const int nx = geo.nx, ny = geo.ny, nz = geo.nz;
    T2* A = reinterpret_cast<T2*>(smem_raw);
    T2* B = A + (size_t)L * sine_line_stride(M);
    T* XB = reinterpret_cast<T*>(B);
    const int SX = sine_stage_stride(N);
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    const int l = tid / kGroup, g = tid % kGroup;
    const long long voff = (long long)blockIdx.y * geo.vstride;

    int n, row0 = 0, nact, x0 = 0, z = 0;
    if (AXIS == 0) {
        n = nx;
        row0 = blockIdx.x * L;
        nact = min(L, ny * nz - row0);
    } else {
        n = ny;
        const int ntx = (nx + L - 1) >> geo.Lshift;
        z = blockIdx.x / ntx;
        x0 = (blockIdx.x - z * ntx) << geo.Lshift;
        nact = min(L, nx - x0);
    }

    for (int i = tid; i < L; i += nthr) {
        XB[(size_t)i * SX] = T(0);
        XB[(size_t)i * SX + skew_r(N)] = T(0);
    }
    // per-volume user pointers, when given, replace base + volume offset
    const Tin* inv = fu.vin ? (const Tin*)fu.vin[blockIdx.y] - voff : in;
    if (AXIS == 0) {
        const int total = nact * n;
        const long long base = voff + (long long)row0 * n;
        for (int e0 = tid; e0 < total; e0 += kLoadBatch * nthr) {
            T v[kLoadBatch];
            if (MODE == kResidual) {
#pragma unroll 2
                for (int q = 0; q < kLoadBatch; q++) {
                    const int e = e0 + q * nthr;
                    if (e < total) {
                        const int r = geo.div_n.div(e), c = e - r * n;
                        const int R = row0 + r;
                        const int zz = geo.div_ny.div(R), yy = R - zz * ny;
                        SineFused f2 = fu;
                        f2.f += voff;
                        f2.uhi += voff;
                        if (f2.ulo) f2.ulo += voff;
                        v[q] = T(residual_at(f2, (long long)R * n + c, c, yy, zz, nx, ny, nz));
                    }
                }
            } else {
#pragma unroll
                for (int q = 0; q < kLoadBatch; q++) {
                    const int e = e0 + q * nthr;
                    if (e < total) {
                        if (MODE == kRound) v[q] = T(f64_to_f32((double)inv[base + e]));
                        else v[q] = T(inv[base + e]);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kLoadBatch; q++) {
                const int e = e0 + q * nthr;
                if (e < total) {
                    const int r = geo.div_n.div(e), c = e - r * n;
                    XB[(size_t)r * SX + skew_r(c + 1)] = v[q];
                }
            }
        }
        for (int e = nact * SX + tid; e < L * SX; e += nthr) XB[e] = T(0);
    } else {
        const int total = n << geo.Lshift;
        const long long base = voff + ((long long)z * ny) * nx + x0;
        for (int e0 = tid; e0 < total; e0 += kLoadBatch * nthr) {
            T v[kLoadBatch];
#pragma unroll
            for (int q = 0; q < kLoadBatch; q++) {
                const int e = e0 + q * nthr;
                const int y = e >> geo.Lshift, c = e & (L - 1);
                v[q] = T(0);
                if (e < total && c < nact) {
                    if (MODE == kRound) v[q] = T(f64_to_f32((double)inv[base + (long long)y * nx + c]));
                    else v[q] = T(inv[base + (long long)y * nx + c]);
                }
            }
#pragma unroll
            for (int q = 0; q < kLoadBatch; q++) {
                const int e = e0 + q * nthr;
                if (e < total) {
                    const int y = e >> geo.Lshift, c = e & (L - 1);
                    XB[(size_t)c * SX + skew_r(y + 1)] = v[q];
                }
            }
        }
    }
    __syncthreads();

    const T* F = sine_block<T>(A, B, tb, l, g);

    if (AXIS == 0) {
        const int total = nact * n;
        const long long base = voff + (long long)row0 * n;
        if (MODE == kCombine) {
            float cc = 0.f, uu = 0.f;
            for (int e = tid; e < total; e += nthr) {
                const int r = geo.div_n.div(e), c = e - r * n;
                const float cv = (float)(scale * F[(size_t)r * SX + skew_r(c + 1)]);
                const long long idx = base + e;
                const float h = fu.uhi[idx];
                const float lo = fu.ulo ? fu.ulo[idx] : 0.f;
                ff s = two_sum(h, lo);
                s = ff_add_f(s, cv);
                if (fu.last) (fu.vout ? (double*)fu.vout[blockIdx.y] - voff : fu.out64)[idx] = ff_to_f64(s);
                if (fu.ulo_out) fu.ulo_out[idx] = lo + cv;
                cc += cv * cv;
                uu += s.h * s.h;
            }
            // per-CTA reduction, one FP64 atomic per CTA and quantity
            for (int o = 16; o > 0; o >>= 1) {
                cc += __shfl_down_sync(0xffffffffu, cc, o);
                uu += __shfl_down_sync(0xffffffffu, uu, o);
            }
            __shared__ float red[2][32];
            const int w = tid >> 5, ln = tid & 31;
            if (ln == 0) { red[0][w] = cc; red[1][w] = uu; }
            __syncthreads();
            if (w == 0) {
                const int nw = nthr >> 5;
                cc = ln < nw ? red[0][ln] : 0.f;
                uu = ln < nw ? red[1][ln] : 0.f;
                for (int o = 16; o > 0; o >>= 1) {
                    cc += __shfl_down_sync(0xffffffffu, cc, o);
                    uu += __shfl_down_sync(0xffffffffu, uu, o);
                }
                if (ln == 0 && fu.norms) {
                    atomicAdd(&fu.norms[2 * blockIdx.y], (double)cc);
                    atomicAdd(&fu.norms[2 * blockIdx.y + 1], (double)uu);
                }
            }
        } else {
            Tout* ov = fu.vout ? (Tout*)fu.vout[blockIdx.y] - voff : out;
            for (int e = tid; e < total; e += nthr) {
                const int r = geo.div_n.div(e), c = e - r * n;
                ov[base + e] = Tout(scale * F[(size_t)r * SX + skew_r(c + 1)]);
            }
        }
    } else {
        const int total = n << geo.Lshift;
        const long long base = voff + ((long long)z * ny) * nx + x0;
        for (int e = tid; e < total; e += nthr) {
            const int y = e >> geo.Lshift, c = e & (L - 1);
            if (c < nact) out[base + (long long)y * nx + c] = Tout(scale * F[(size_t)c * SX + skew_r(y + 1)]);
        }
    }
}

}  // namespace fdmgpu
