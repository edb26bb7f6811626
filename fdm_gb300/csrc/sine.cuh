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
//      prefix sum F[2k+1] = F[2k-1] + Re Y_k, done with a segmented warp scan.
// Twiddle and weight tables are computed in FP64 on the host and rounded to
// the compute type once.
#pragma once

#include "common.cuh"

namespace fdmgpu {

constexpr int kGroup = 8;  // threads per line

template <typename T>
struct SineTables {
    const vec2_t<T>* tw;    // e^{-2 pi i k / M}, k = 0..M-1
    const vec2_t<T>* post;  // e^{-2 pi i k / N}, k = 0..M-1
    const T* wpre;          // sin(pi j / N), j = 0..N-1
    int N, M;
};

// Complex elements per line in each of the two shared buffers.  The +8 pad
// makes consecutive lines start 8 complex elements apart modulo 16, so the
// two lines of a half-warp never share a bank pair.
__host__ __device__ inline int sine_line_stride(int M) { return M + 8; }

// Reals per line in the staging view of the buffers (x[0..N], F[1..N-1]).
// N+1 is odd, so a column-wise (transposed) access by consecutive threads
// hits distinct banks.
__host__ __device__ inline int sine_stage_stride(int N) { return N + 1; }

template <typename T>
__host__ __device__ inline size_t sine_smem_bytes(int N, int L) {
    return 2ull * L * sine_line_stride(N / 2) * sizeof(vec2_t<T>);
}

// Runs the transform of every line held by this CTA.  On entry the staging
// view of buffer B holds x[1..n] of line l at stage(B) + l*SX + 1 (entries 0
// and N must be zero).  On exit the result F[1..n] (unscaled) sits in the
// staging view of the buffer returned.  All threads of the CTA must call it.
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
                T a = X[j0], b = X[N - j0];
                y0 = ldg(tb.wpre + j0) * (a + b) + half * (a - b);
            }
            T a = X[j1], b = X[N - j1];
            T y1 = ldg(tb.wpre + j1) * (a + b) + half * (a - b);
            T2 v; v.x = y0; v.y = y1;
            Al[m] = v;
        }
    }
    __syncthreads();

    // 2. Stockham passes, A -> B -> A ...
    T2* src = A;
    T2* dst = B;
    for (int Ns = 1; Ns < M;) {
        const int R = ((M / Ns) % 4 == 0) ? 4 : 2;
        const int MR = M / R;
        const int twstep = M / (Ns * R);
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
                d[base] = cadd<T>(a0, b0);
                d[base + Ns] = cadd<T>(a1, b1);
                d[base + 2 * Ns] = csub<T>(a0, b0);
                d[base + 3 * Ns] = csub<T>(a1, b1);
            } else {
                T2 v0 = s[j], v1 = s[j + MR];
                if (k) v1 = cmul<T>(v1, ldg(tb.tw + k * twstep));
                d[base] = cadd<T>(v0, v1);
                d[base + Ns] = csub<T>(v0, v1);
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
    T sum = T(0);
    for (int k = k0; k < k1; k++) {
        const T2 ck = C[k];
        const T2 cm = C[(M - k) & (M - 1)];
        T ex = T(0.5) * (ck.x + cm.x), ey = T(0.5) * (ck.y - cm.y);
        T ox = T(0.5) * (ck.y + cm.y), oy = T(-0.5) * (ck.x - cm.x);
        const T2 w = ldg(tb.post + k);
        T yr = ex + (w.x * ox - w.y * oy);
        T yi = ey + (w.x * oy + w.y * ox);
        if (k == 0) yr *= T(0.5);
        else F[2 * k] = -yi;
        F[2 * k + 1] = yr;
        sum += yr;
    }
    T incl = sum;
#pragma unroll
    for (int off = 1; off < kGroup; off <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, incl, off, kGroup);
        if (g >= off) incl += t;
    }
    T run = incl - sum;
    for (int k = k0; k < k1; k++) {
        run += F[2 * k + 1];
        F[2 * k + 1] = run;
    }
    __syncthreads();
    return reinterpret_cast<T*>(dst);
}

// One DST pass over every line along x (AXIS 0, rows) or along y (AXIS 1,
// columns) of a batch of nz*ny*nx volumes (x fastest), out-of-place or
// in-place.  Rows: a CTA takes L consecutive rows.  Columns: a CTA takes a
// tile of L consecutive x at one z, all y.  gridDim.y indexes the volume.
// Loads convert Tin -> T, stores T -> Tout after multiplying by `scale`.
template <typename Tin, typename T, typename Tout, int AXIS>
__global__ void __launch_bounds__(256) k_sine_pass(const Tin* in, Tout* out,
                                                   int nx, int ny, int nz, long long vstride,
                                                   SineTables<T> tb, T scale, int L, int Lshift) {
    using T2 = vec2_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = tb.M, N = tb.N;
    T2* A = reinterpret_cast<T2*>(smem_raw);
    T2* B = A + (size_t)L * sine_line_stride(M);
    T* XB = reinterpret_cast<T*>(B);
    const int SX = sine_stage_stride(N);
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    const int l = tid / kGroup, g = tid % kGroup;
    const long long voff = (long long)blockIdx.y * vstride;
    in += voff;
    out += voff;

    int n, row0 = 0, nact, x0 = 0, z = 0;
    if (AXIS == 0) {
        n = nx;
        const int lines = ny * nz;
        row0 = blockIdx.x * L;
        nact = min(L, lines - row0);
    } else {
        n = ny;
        const int ntx = (nx + L - 1) >> Lshift;
        z = blockIdx.x / ntx;
        x0 = (blockIdx.x - z * ntx) << Lshift;
        nact = min(L, nx - x0);
    }

    // zero the ends of every staged line
    for (int i = tid; i < L; i += nthr) {
        XB[(size_t)i * SX] = T(0);
        XB[(size_t)i * SX + N] = T(0);
    }
    if (AXIS == 0) {
        const int total = nact * n;
        const Tin* src = in + (long long)row0 * n;
        for (int e = tid; e < total; e += nthr) {
            const int r = e / n, c = e - r * n;
            XB[(size_t)r * SX + c + 1] = T(src[e]);
        }
        for (int e = nact * SX + tid; e < L * SX; e += nthr) XB[e] = T(0);
    } else {
        const int total = n << Lshift;
        const Tin* src = in + ((long long)z * ny) * nx + x0;
        for (int e = tid; e < total; e += nthr) {
            const int y = e >> Lshift, c = e & (L - 1);
            T v = T(0);
            if (c < nact) v = T(src[(long long)y * nx + c]);
            XB[(size_t)c * SX + y + 1] = v;
        }
    }
    __syncthreads();

    const T* F = sine_block<T>(A, B, tb, l, g);

    if (AXIS == 0) {
        const int total = nact * n;
        Tout* dstp = out + (long long)row0 * n;
        for (int e = tid; e < total; e += nthr) {
            const int r = e / n, c = e - r * n;
            dstp[e] = Tout(scale * F[(size_t)r * SX + c + 1]);
        }
    } else {
        const int total = n << Lshift;
        Tout* dstp = out + ((long long)z * ny) * nx + x0;
        for (int e = tid; e < total; e += nthr) {
            const int y = e >> Lshift, c = e & (L - 1);
            if (c < nact) dstp[(long long)y * nx + c] = Tout(scale * F[(size_t)c * SX + y + 1]);
        }
    }
}

}  // namespace fdmgpu
