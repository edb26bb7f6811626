// Periodic real transforms of lines of n = 2^q points, the periodic
// LaplCube's building block (FFT<T>::pFFT_1 and FFT<T>::pFFT,
// src/fft.cpp:108-212), in the reference's coefficient layout:
//
//   forward (values -> coefficients, pFFT_1):
//     S[k]   = scale * sum_j f_j cos(2 pi j k / n),  k = 0 .. n/2
//     S[n-k] = scale * sum_j f_j sin(2 pi j k / n),  k = 1 .. n/2-1
//   inverse (coefficients -> values, pFFT):
//     f_j = scale * ( S[0]/2 + sum_{k=1}^{n/2-1} (S[k] cos + S[n-k] sin)(2 pi j k / n)
//                     + S[n/2]/2 cos(pi j) )
//
// Both go through one complex FFT of n/2 points per line (the even and odd
// samples packed as real and imaginary parts), done as a radix-2 Stockham
// loop in shared memory, plus the usual split / merge step.  Lines have any
// element stride: line L starts at (L / A) * B + (L % A) * C and steps by D
// (x-lines: A = 1, B = n, D = 1; y-lines: A = nx, B = nx*ny, C = 1,
// D = nx; z-lines: A = nx*ny, B = volume, C = 1, D = nx*ny).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace fdmgpu {

struct PLineGeom {
    long long lines;
    long long A, B, C, D;
};

__device__ __forceinline__ long long pline_base(const PLineGeom& g, long long L) {
    return (L / g.A) * g.B + (L % g.A) * g.C;
}

// lines per block: at most 2048 / n (at least 1; 32 KB of shared memory in
// FP64), 256 threads; fewer when that leaves most SMs without a block (small
// transforms)
__host__ __device__ constexpr int pfft_lines_per_block(int n) { return n >= 2048 ? 1 : 2048 / n; }

inline int pfft_lines_per_block(int n, long long lines, int sms) {
    int lpb = pfft_lines_per_block(n);
    while (lpb > 1 && (lines + lpb - 1) / lpb < 2LL * sms) lpb /= 2;
    return lpb;
}

template <typename T>
size_t pfft_smem_bytes(int n, int lpb) {
    // two complex buffers of n/2 points per line (Stockham ping-pong); the
    // real staging of n values aliases the second one
    return (size_t)lpb * 2 * (size_t)(n / 2 > 0 ? n / 2 : 1) * 2 * sizeof(T);
}

// tw[t] = e^{-2 pi i t / n}, t < n; LPB lines per block
template <typename T, bool INV>
__global__ void __launch_bounds__(256)
    k_pfft(const T* in, T* out, PLineGeom g, int n, int LPB, const vec2_t<T>* __restrict__ tw, T scale) {
    using T2 = vec2_t<T>;
    extern __shared__ __align__(16) unsigned char pf_raw[];
    const int M = n / 2;
    T2* bufA = reinterpret_cast<T2*>(pf_raw);
    T2* bufB = bufA + (size_t)LPB * M;
    T* stage = reinterpret_cast<T*>(bufB);  // n reals per line
    const int tid = threadIdx.x;
    const long long L0 = (long long)blockIdx.x * LPB;
    const int nl = (int)min((long long)LPB, g.lines - L0);
    const int tot = LPB * n;

    // ---- load: coalesced along x for unit-stride lines, across lines otherwise
    for (int e = tid; e < tot; e += blockDim.x) {
        int l, j;
        if (g.D == 1) { l = e / n; j = e - l * n; }
        else { j = e / LPB; l = e - j * LPB; }
        T v = T(0);
        if (l < nl) v = in[pline_base(g, L0 + l) + (long long)j * g.D];
        stage[l * n + j] = v;
    }
    __syncthreads();
    // ---- complex input of the n/2-point FFT
    for (int e = tid; e < LPB * M; e += blockDim.x) {
        const int l = e / M, m = e - l * M;
        const T* s = stage + l * n;
        T2 z;
        if (!INV) {
            z.x = s[2 * m];
            z.y = s[2 * m + 1];
        } else {
            // H_k = S_k - i S_{n-k} (H_0 = S_0, H_M = S_M); Y_k = (H_k + conj H_{M-k})
            // + i e^{+2 pi i k/n} (H_k - conj H_{M-k})
            const int k = m, kc = M - m;
            T2 hk, hc;
            hk.x = s[k];
            hk.y = (k == 0) ? T(0) : -s[n - k];
            hc.x = s[kc];
            hc.y = (kc == M) ? T(0) : -s[n - kc];
            hc.y = -hc.y;  // conjugate
            const T2 w = tw[k];  // e^{-2 pi i k/n}; e^{+...} = conj(w)
            T2 d, a;
            a.x = hk.x + hc.x; a.y = hk.y + hc.y;
            d.x = hk.x - hc.x; d.y = hk.y - hc.y;
            // i * conj(w) * d
            const T rx = w.x * d.x + w.y * d.y, ry = w.x * d.y - w.y * d.x;
            z.x = a.x - ry;
            z.y = a.y + rx;
        }
        bufA[l * M + m] = z;
    }
    __syncthreads();
    // ---- radix-2 Stockham, sign -1 forward, +1 inverse
    T2* src = bufA;
    T2* dst = bufB;
    for (int Ls = 1; Ls < M; Ls *= 2) {
        const int step = n / (2 * Ls);  // twiddle index stride
        for (int e = tid; e < LPB * (M / 2); e += blockDim.x) {
            const int l = e / (M / 2), b = e - l * (M / 2);
            const int j = b % Ls, k = b / Ls;
            T2 w = tw[j * step];
            if (INV) w.y = -w.y;
            const T2 u = src[l * M + k * Ls + j];
            const T2 v = src[l * M + k * Ls + j + M / 2];
            const T2 wv = cmul<T>(w, v);
            dst[l * M + 2 * k * Ls + j] = cadd<T>(u, wv);
            dst[l * M + 2 * k * Ls + j + Ls] = csub<T>(u, wv);
        }
        __syncthreads();
        T2* t = src;
        src = dst;
        dst = t;
    }
    // src holds the n/2-point transform; the staging (aliasing bufB) is free
    // only if src is bufA: copy back first otherwise
    if (src != bufA) {
        for (int e = tid; e < LPB * M; e += blockDim.x) bufA[e] = src[e];
        __syncthreads();
    }
    // ---- split (forward) / unpack (inverse) into the staging
    if (!INV) {
        for (int e = tid; e < LPB * (M + 1); e += blockDim.x) {
            const int l = e / (M + 1), k = e - l * (M + 1);
            const T2* Z = bufA + l * M;
            const T2 zk = Z[k % M];
            T2 zc = Z[(M - k) % M];
            zc.y = -zc.y;
            const T2 w = tw[k % n];
            T2 a, d;
            a.x = T(0.5) * (zk.x + zc.x); a.y = T(0.5) * (zk.y + zc.y);
            d.x = T(0.5) * (zk.x - zc.x); d.y = T(0.5) * (zk.y - zc.y);
            // F = a - i w d
            const T2 wd = cmul<T>(w, d);
            const T Fx = a.x + wd.y, Fy = a.y - wd.x;
            T* s = stage + l * n;
            s[k] = scale * Fx;
            if (k >= 1 && k <= M - 1) s[n - k] = -scale * Fy;
        }
    } else {
        for (int e = tid; e < LPB * M; e += blockDim.x) {
            const int l = e / M, m = e - l * M;
            const T2 z = bufA[l * M + m];
            T* s = stage + l * n;
            s[2 * m] = T(0.5) * scale * z.x;
            s[2 * m + 1] = T(0.5) * scale * z.y;
        }
    }
    __syncthreads();
    // ---- store
    for (int e = tid; e < tot; e += blockDim.x) {
        int l, j;
        if (g.D == 1) { l = e / n; j = e - l * n; }
        else { j = e / LPB; l = e - j * LPB; }
        if (l < nl) out[pline_base(g, L0 + l) + (long long)j * g.D] = stage[l * n + j];
    }
}

}  // namespace fdmgpu
