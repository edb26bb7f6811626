// Register-resident DST-I line transforms for N = 16 .. 512.
//
// Same transform and contract as k_sine_pass (sine.cuh): for every line
// x[1..n] (N = n+1), F[k] = scale * sum_j x[j] sin(pi j k / N), with the
// fold -> complex FFT of M = N/2 -> real unpack + prefix sum formulation.
// The complex FFT is done as two register passes instead of log4(M)
// shared-memory passes:
//     M = R1 * R2, G = R2 threads per line;
//     pass 1: thread g loads c[j1*R2 + g] (folded on the fly from the staged
//             line), does a DFT of length R1 in registers and multiplies by
//             w_M^(g*k1);
//     one transpose through shared memory;
//     pass 2: each thread does R1/G DFTs of length R2 in registers, giving
//             C[k1 + R1*k2].
// Every line uses one shared region: the staged input, the transpose, C and
// the staged output reuse it in turn.  Staged entry i sits at i + i/32 (one
// pad slot per 32, so the per-thread blocks of the unpack fall into distinct
// banks); in the column pass it is also XOR-swizzled with the line index so
// that consecutive threads walking across lines hit distinct banks.
#pragma once

#include "sine.cuh"

namespace fdmgpu {

template <int N> struct RgCfg;
template <> struct RgCfg<16> { static constexpr int R1 = 4, R2 = 2; };
template <> struct RgCfg<32> { static constexpr int R1 = 4, R2 = 4; };
template <> struct RgCfg<64> { static constexpr int R1 = 8, R2 = 4; };
template <> struct RgCfg<128> { static constexpr int R1 = 8, R2 = 8; };
template <> struct RgCfg<256> { static constexpr int R1 = 16, R2 = 8; };
template <> struct RgCfg<512> { static constexpr int R1 = 16, R2 = 16; };

template <int N>
struct RgGeom {
    static constexpr int M = N / 2;
    static constexpr int R1 = RgCfg<N>::R1, R2 = RgCfg<N>::R2;
    static constexpr int G = R2;           // threads per line
    static constexpr int L = 256 / G;      // lines per CTA
    static constexpr int D2 = R1 / G;      // length-R2 DFTs per thread in pass 2
    static constexpr int STAGE = N + N / 32 + 32;
    static constexpr int TR = R1 * (R2 + 1);
    static constexpr int CB = M + M / 16 + 1;
    static constexpr int CPLX = (TR > CB ? TR : CB) + 8;
    static constexpr int LS0 = STAGE > 2 * CPLX ? STAGE : 2 * CPLX;
    static constexpr int LS = (LS0 + 31) / 32 * 32;  // reals per line region
};

// cos / sin of 2 pi m / 16
__device__ __forceinline__ constexpr double c16(int m) {
    return m == 0 ? 1.0 : m == 1 ? 0.92387953251128674 : m == 2 ? 0.70710678118654757 : m == 3 ? 0.38268343236508984
         : m == 4 ? 0.0 : m == 5 ? -0.38268343236508973 : m == 6 ? -0.70710678118654746 : -0.92387953251128674;
}
__device__ __forceinline__ constexpr double s16(int m) {
    return m == 0 ? 0.0 : m == 1 ? 0.38268343236508978 : m == 2 ? 0.70710678118654746 : m == 3 ? 0.92387953251128674
         : m == 4 ? 1.0 : m == 5 ? 0.92387953251128674 : m == 6 ? 0.70710678118654757 : 0.38268343236508989;
}

// b * e^{-2 pi i m / R} for a compile-time m (after unrolling), 0 <= m < R/2
template <typename T, int R>
__device__ __forceinline__ vec2_t<T> twid(vec2_t<T> b, int m) {
    using T2 = vec2_t<T>;
    if (m == 0) return b;
    const int m16 = m * (16 / R);
    if (m16 == 4) {  // -i
        T2 r; r.x = b.y; r.y = -b.x; return r;
    }
    const T c = (T)c16(m16), s = (T)s16(m16);
    T2 r;
    r.x = b.x * c + b.y * s;
    r.y = b.y * c - b.x * s;
    return r;
}

__device__ __forceinline__ constexpr int bitrev(int i, int bits) {
    int r = 0;
    for (int b = 0; b < bits; b++) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}

// in-place forward DFT of length R (2, 4, 8, 16) in registers, natural order
template <typename T, int R>
__device__ __forceinline__ void dft_reg(vec2_t<T>* v) {
    using T2 = vec2_t<T>;
    constexpr int bits = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int j = bitrev(i, bits);
        if (i < j) {
            T2 t = v[i]; v[i] = v[j]; v[j] = t;
        }
    }
#pragma unroll
    for (int s = 1; s < R; s <<= 1) {
#pragma unroll
        for (int k = 0; k < R; k += 2 * s) {
#pragma unroll
            for (int j = 0; j < s; j++) {
                const T2 a = v[k + j];
                const T2 b = twid<T, R>(v[k + j + s], j * (R / (2 * s)));
                v[k + j] = cadd<T>(a, b);
                v[k + j + s] = csub<T>(a, b);
            }
        }
    }
}

// staged position of entry i of line l; the XOR swizzle is needed only
// when consecutive threads walk across lines (the column pass)
template <int N, int AXIS>
__device__ __forceinline__ int rg_pos(int l, int i) {
    if (AXIS == 1) return l * RgGeom<N>::LS + ((i + (i >> 5)) ^ (l & 31));
    return l * RgGeom<N>::LS + i + (i >> 5);
}

template <typename Tin, typename T, typename Tout, int AXIS, int MODE, int N>
__global__ void __launch_bounds__(256) k_sine_rg(const Tin* in, Tout* out, SineGeom geo, SineTables<T> tb, T scale,
                                                 SineFused fu) {
    using T2 = vec2_t<T>;
    using Gm = RgGeom<N>;
    constexpr int M = Gm::M, R1 = Gm::R1, R2 = Gm::R2, G = Gm::G, L = Gm::L, D2 = Gm::D2, LS = Gm::LS;
    constexpr int n = N - 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* S = reinterpret_cast<T*>(smem_raw);
    const int nx = geo.nx, ny = geo.ny, nz = geo.nz;
    const int tid = threadIdx.x;
    constexpr int nthr = L * G;
    const int l = tid / G, g = tid % G;
    const long long voff = (long long)blockIdx.y * geo.vstride;

    int row0 = 0, nact, x0 = 0, z = 0;
    if (AXIS == 0) {
        row0 = blockIdx.x * L;
        nact = min(L, ny * nz - row0);
    } else {
        const int ntx = (nx + L - 1) / L;
        z = blockIdx.x / ntx;
        x0 = (blockIdx.x - z * ntx) * L;
        nact = min(L, nx - x0);
    }

    // ---- load phase: staged lines x[1..n], x[0] = x[N] = 0
    for (int i = tid; i < L; i += nthr) {
        S[rg_pos<N, AXIS>(i, 0)] = T(0);
        S[rg_pos<N, AXIS>(i, N)] = T(0);
    }
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
                        const int r = e / n, c = e - r * n;
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
                        if (MODE == kRound) v[q] = T(f64_to_f32((double)in[base + e]));
                        else v[q] = T(in[base + e]);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kLoadBatch; q++) {
                const int e = e0 + q * nthr;
                if (e < total) {
                    const int r = e / n, c = e - r * n;
                    S[rg_pos<N, AXIS>(r, c + 1)] = v[q];
                }
            }
        }
        for (int e = nact * n + tid; e < L * n; e += nthr) {
            const int r = e / n, c = e - r * n;
            S[rg_pos<N, AXIS>(r, c + 1)] = T(0);
        }
    } else {
        const int total = n * L;
        const long long base = voff + ((long long)z * ny) * nx + x0;
        for (int e0 = tid; e0 < total; e0 += kLoadBatch * nthr) {
            T v[kLoadBatch];
#pragma unroll
            for (int q = 0; q < kLoadBatch; q++) {
                const int e = e0 + q * nthr;
                const int y = e / L, c = e - y * L;
                v[q] = T(0);
                if (e < total && c < nact) {
                    if (MODE == kRound) v[q] = T(f64_to_f32((double)in[base + (long long)y * nx + c]));
                    else v[q] = T(in[base + (long long)y * nx + c]);
                }
            }
#pragma unroll
            for (int q = 0; q < kLoadBatch; q++) {
                const int e = e0 + q * nthr;
                if (e < total) {
                    const int y = e / L, c = e - y * L;
                    S[rg_pos<N, AXIS>(c, y + 1)] = v[q];
                }
            }
        }
    }
    __syncthreads();

    // ---- pass 1: fold + DFT_R1 + twiddle
    T2 v[R1];
    {
        const T half = T(0.5);
#pragma unroll
        for (int j1 = 0; j1 < R1; j1++) {
            const int m = j1 * R2 + g;
            const int a0 = 2 * m, a1 = 2 * m + 1;
            T y0 = T(0);
            if (m > 0) {
                const T a = S[rg_pos<N, AXIS>(l, a0)], b = S[rg_pos<N, AXIS>(l, N - a0)];
                y0 = ldg(tb.wpre + a0) * (a + b) + half * (a - b);
            }
            const T a = S[rg_pos<N, AXIS>(l, a1)], b = S[rg_pos<N, AXIS>(l, N - a1)];
            const T y1 = ldg(tb.wpre + a1) * (a + b) + half * (a - b);
            v[j1].x = y0;
            v[j1].y = y1;
        }
        dft_reg<T, R1>(v);
        if (g) {
#pragma unroll
            for (int k1 = 1; k1 < R1; k1++) v[k1] = cmul<T>(v[k1], ldg(tb.tw + ((g * k1) & (M - 1))));
        }
    }
    __syncthreads();  // every line has read its staged input; the regions are reused below

    T2* Cl = reinterpret_cast<T2*>(S + (size_t)l * LS) + 8 * (l & 1);
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) Cl[k1 * (R2 + 1) + g] = v[k1];
    __syncwarp();

    // ---- pass 2: D2 DFTs of length R2 per thread
    T2 u[D2][R2];
#pragma unroll
    for (int d = 0; d < D2; d++) {
        const int k1 = g * D2 + d;
#pragma unroll
        for (int j2 = 0; j2 < R2; j2++) u[d][j2] = Cl[k1 * (R2 + 1) + j2];
        dft_reg<T, R2>(u[d]);
    }
    __syncwarp();
#pragma unroll
    for (int d = 0; d < D2; d++) {
        const int k1 = g * D2 + d;
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) Cl[skew_c(k1 + R1 * k2)] = u[d][k2];
    }
    __syncwarp();

    // ---- unpack + prefix sum over this thread's block of R1 consecutive k
    T ev[R1], od[R1];
#pragma unroll
    for (int t = 0; t < R1; t++) {
        const int k = g * R1 + t;
        const T2 ck = Cl[skew_c(k)];
        const T2 cm = Cl[skew_c((M - k) & (M - 1))];
        const T ex = T(0.5) * (ck.x + cm.x), ey = T(0.5) * (ck.y - cm.y);
        const T ox = T(0.5) * (ck.y + cm.y), oy = T(-0.5) * (ck.x - cm.x);
        const T2 w = ldg(tb.post + k);
        T yr = ex + (w.x * ox - w.y * oy);
        const T yi = ey + (w.x * oy + w.y * ox);
        if (k == 0) yr *= T(0.5);
        ev[t] = -yi;
        od[t] = yr;
    }
    // running sum of the odd terms: local inclusive prefix, then the
    // exclusive offset from the lanes before (segmented shuffle scan)
#pragma unroll
    for (int t = 1; t < R1; t++) od[t] += od[t - 1];
    T incl = od[R1 - 1];
#pragma unroll
    for (int off = 1; off < G; off <<= 1) {
        const T t = __shfl_up_sync(0xffffffffu, incl, off, G);
        if (g >= off) incl += t;
    }
    const T excl = incl - od[R1 - 1];
#pragma unroll
    for (int t = 0; t < R1; t++) od[t] += excl;
    __syncthreads();  // every line has read its C; staged outputs overwrite the regions
#pragma unroll
    for (int t = 0; t < R1; t++) {
        const int k = g * R1 + t;
        if (k > 0) S[rg_pos<N, AXIS>(l, 2 * k)] = ev[t];
        S[rg_pos<N, AXIS>(l, 2 * k + 1)] = od[t];
    }
    __syncthreads();

    // ---- store phase
    if (AXIS == 0) {
        const int total = nact * n;
        const long long base = voff + (long long)row0 * n;
        if (MODE == kCombine) {
            float cc = 0.f, uu = 0.f;
            for (int e = tid; e < total; e += nthr) {
                const int r = e / n, c = e - r * n;
                const float cv = (float)(scale * S[rg_pos<N, AXIS>(r, c + 1)]);
                const long long idx = base + e;
                const float h = fu.uhi[idx];
                const float lo = fu.ulo ? fu.ulo[idx] : 0.f;
                ff s2 = two_sum(h, lo);
                s2 = ff_add_f(s2, cv);
                if (fu.last) fu.out64[idx] = ff_to_f64(s2);
                else fu.ulo_out[idx] = lo + cv;
                cc += cv * cv;
                uu += s2.h * s2.h;
            }
            for (int o = 16; o > 0; o >>= 1) {
                cc += __shfl_down_sync(0xffffffffu, cc, o);
                uu += __shfl_down_sync(0xffffffffu, uu, o);
            }
            __shared__ float red[2][32];
            const int w = tid >> 5, ln = tid & 31;
            if (ln == 0) { red[0][w] = cc; red[1][w] = uu; }
            __syncthreads();
            if (w == 0) {
                constexpr int nw = nthr >> 5;
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
            for (int e = tid; e < total; e += nthr) {
                const int r = e / n, c = e - r * n;
                out[base + e] = Tout(scale * S[rg_pos<N, AXIS>(r, c + 1)]);
            }
        }
    } else {
        const int total = n * L;
        const long long base = voff + ((long long)z * ny) * nx + x0;
        for (int e = tid; e < total; e += nthr) {
            const int y = e / L, c = e - y * L;
            if (c < nact) out[base + (long long)y * nx + c] = Tout(scale * S[rg_pos<N, AXIS>(c, y + 1)]);
        }
    }
}

template <typename T, int N>
constexpr size_t rg_smem_bytes() {
    return (size_t)RgGeom<N>::L * RgGeom<N>::LS * sizeof(T);
}

}  // namespace fdmgpu
