// Register-resident DST-I line transforms for N = 16 .. 512.
//
// Same transform and contract as k_sine_pass (sine.cuh): for every line
// x[1..n] (N = n+1), F[k] = scale * sum_j x[j] sin(pi j k / N), with the
// fold -> complex FFT of M = N/2 -> real unpack + prefix sum formulation.
//
//   load:   the thread that loads x_j also loads x_{N-j} and writes the two
//           folded values y_j, y_{N-j}; lines are stored as M complex slots
//           c_m = (y_{2m}, y_{2m+1});
//   pass 1: M = R1 * R2, G = R2 threads per line; thread g takes
//           c[j1*R2 + g], does a DFT of length R1 in registers and multiplies
//           by w_M^(g*k1);
//   one transpose through shared memory;
//   pass 2: each thread does R1/G DFTs of length R2 in registers, giving
//           C[k1 + R1*k2];
//   unpack: Y_k and Y_{M-k} both come from the pair (C_k, C_{M-k})
//           (Y_{M-k} = conj(E_k - w_k O_k)), so each C is read once; thread
//           g owns k in [g*E, (g+1)*E) of the first half and their mirrors;
//           the odd outputs are a running sum over k, done as a local prefix
//           plus a forward shuffle scan for the first half and a backward one
//           for the mirrored blocks of the second half.
// Each line owns one region of complex slots used in turn by the packed
// input, the transpose, C and the packed output (F_{2k}, F_{2k+1}), so the
// phases inside a line need only warp-level synchronisation.
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

// NT: threads per CTA (256; 128 or 64 for the lines of up to 64 points of
// volumes too small to give every SM two CTAs of 256)
template <int N, int AXIS, int NT = 256>
struct RgGeom {
    static constexpr int M = N / 2;
    static constexpr int R1 = RgCfg<N>::R1, R2 = RgCfg<N>::R2;
    static constexpr int G = R2;              // threads per line
    static constexpr int L = NT / G;          // lines per CTA
    static constexpr int D2 = R1 / G;         // length-R2 DFTs per thread in pass 2
    static constexpr int E = M / (2 * G);     // unpack pairs per thread
    static constexpr int TR = R1 * (R2 + 1);  // transpose slots
    static constexpr int CS = M + M / 16 + 1; // skewed C / packed-output slots
    static constexpr int RS0 = TR > CS ? (TR > M ? TR : M) : (CS > M ? CS : M);
    // line stride in slots: 8 (mod 16) for the row pass so the two lines of
    // a half-warp use disjoint bank pairs; odd for the column pass, whose
    // load and store walk across lines.  Pass 2 and the unpack still meet
    // two-way conflicts between the two lines of a half-warp (they want an
    // odd, resp. 4 (mod 8), offset between them).  A layout without padding
    // whose views XOR the slot with a per-line mask removes most of them
    // (37 % fewer shared-memory wavefronts at 256 points in a bank model),
    // but measured slower on GB300 (x pass 1.56 -> 1.72 ms, y pass 1.45 ->
    // 1.52 ms per 16 x 255^3 pair) while the passes were bound by integer
    // index arithmetic.
    static constexpr int LS2 = AXIS == 0 ? ((RS0 + 7) / 16 * 16 + 8) : (RS0 | 1);
};

// Slot swizzles of the two layouts private to the line transform, FP32
// only (chosen for 8-byte slots): B, the transpose between its passes
// (entry (k1, j) at slot k1 (R2+1) + (j ^ mask): the XOR stays inside the
// row of R2 entries), and C (entry k at slot sk(k) ^ mask, pass 2 to the
// unpack).  The masks are keyed on bits 0 and 1 of the line's index.  The
// lines that share a half-warp want different offsets between them in
// different phases (pass 1 and its transpose write 16 banks, pass 2 an odd
// number of slots, the unpack 8 (mod 16) slots), which no single line
// stride gives; these masks give the fewest shared-memory wavefronts in a
// bank model of every phase (FP32 rows of 256 points: 1792 -> 1168 for the
// two layouts), and on GB300 the plane pass of 255^3 x 16 went from 2.88
// to 2.81 ms, the x passes about 1 % faster.  Column passes keep plain
// layouts: a swizzled column layout at the row stride (3328 -> 2450
// modelled wavefronts) needed more than 48 registers and ran 3-5 % slower
// at 4 CTAs per SM than the plain one at 5.  What works instead: the FP32
// column passes of 128 and 256 points hand their lines to the transform in
// an order that puts a half-warp's two lines 8 lines apart, and use the row
// masks (y pass 0.61 -> 0.59 ms, FP64-rounding y pass 0.86 -> 0.82 ms per
// 16 x 255^3 launch; 127^3 solves 3 % faster), and shift the packed output
// of odd positions (OOFF of rg_line_fft: y pass 0.59 -> 0.56 ms).
template <typename T, int N, int AXIS>
struct RgSwz {
    static constexpr int B0 = 0, B1 = 0, C0 = 0, C1 = 0;
};
template <int N>
struct RgSwzRow {
    static constexpr int B0 = N == 256 ? 1 : 0, B1 = N == 64 ? 1 : 0;
    static constexpr int C0 = N == 256 ? 5 : (N == 128 || N == 64) ? 2 : 0, C1 = N == 64 ? 1 : N == 32 ? 5 : 0;
};
template <> struct RgSwz<float, 256, 0> : RgSwzRow<256> {};
template <> struct RgSwz<float, 128, 0> : RgSwzRow<128> {};
template <> struct RgSwz<float, 64, 0> : RgSwzRow<64> {};
template <> struct RgSwz<float, 32, 0> : RgSwzRow<32> {};
template <> struct RgSwz<float, 32, 1> {
    static constexpr int B0 = 1, B1 = 2, C0 = 0, C1 = 0;
};

// largest s ^ m over s < n and every mask m whose bits lie within those of
// mmax rounded up to 2^k - 1
__host__ __device__ constexpr int swz_max(int n, int mmax) {
    int cover = 0;
    while (cover < mmax) cover = 2 * cover + 1;
    int r = 0;
    for (int s = 0; s < n; s++)
        for (int m = 0; m <= cover; m++) r = (s ^ m) > r ? (s ^ m) : r;
    return r;
}

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

// skewed slot of entry k of C / the packed output: one pad slot per 16
__device__ __forceinline__ int sk(int k) { return k + (k >> 4); }

// The transform of one line held in its slots Ls (AXIS's layout): on entry
// the folded values y_0..y_{N-1} as M complex slots c_m = (y_{2m}, y_{2m+1}),
// on exit the unscaled F_1..F_n with entry i as component i&1 of slot
// sk(i>>1).  Called by the G threads of the line (g = 0..G-1), which must
// belong to one warp; the phases inside need only warp synchronisation.
// line: the line's index in the CTA (selects the swizzle of RgSwz; SWZ =
// false keeps both private layouts plain).
template <typename T, int N, int AXIS, bool SWZ = true, int OOFF = 0>
__device__ __forceinline__ void rg_line_fft(vec2_t<T>* Ls, int g, int line, const SineTables<T>& tb) {
    using T2 = vec2_t<T>;
    using Gm = RgGeom<N, AXIS>;
    using Sw = RgSwz<T, N, AXIS>;
    constexpr int M = Gm::M, R1 = Gm::R1, R2 = Gm::R2, G = Gm::G, D2 = Gm::D2, E = Gm::E;
    static_assert(swz_max(R2, Sw::B0 | Sw::B1) < R2 && swz_max(Gm::CS, Sw::C0 | Sw::C1) < Gm::LS2,
                  "a swizzled slot stays inside its row of the transpose (B) and inside its line (C)");
    const int mB = SWZ ? (((line & 1) ? Sw::B0 : 0) ^ ((line & 2) ? Sw::B1 : 0)) : 0;
    const int mC = SWZ ? (((line & 1) ? Sw::C0 : 0) ^ ((line & 2) ? Sw::C1 : 0)) : 0;
    // ---- pass 1: DFT_R1 + twiddle
    T2 v[R1];
#pragma unroll
    for (int j1 = 0; j1 < R1; j1++) v[j1] = Ls[j1 * R2 + g];
    dft_reg<T, R1>(v);
    if (g) {
#pragma unroll
        for (int k1 = 1; k1 < R1; k1++) v[k1] = cmul<T>(v[k1], ldg(tb.tw + ((g * k1) & (M - 1))));
    }
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) Ls[k1 * (R2 + 1) + (g ^ mB)] = v[k1];
    __syncwarp();

    // ---- pass 2: D2 DFTs of length R2 per thread
    T2 u[D2][R2];
#pragma unroll
    for (int d = 0; d < D2; d++) {
        const int k1 = g * D2 + d;
#pragma unroll
        for (int j2 = 0; j2 < R2; j2++) u[d][j2] = Ls[k1 * (R2 + 1) + (j2 ^ mB)];
        dft_reg<T, R2>(u[d]);
    }
    __syncwarp();
#pragma unroll
    for (int d = 0; d < D2; d++) {
        const int k1 = g * D2 + d;
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) Ls[sk(k1 + R1 * k2) ^ mC] = u[d][k2];
    }
    __syncwarp();

    // ---- unpack: pairs (k, M-k) for k in [g*E, g*E + E)
    T ra[E], ia[E], rb[E], ib[E];
    T rmid = T(0), imid = T(0);
#pragma unroll
    for (int t = 0; t < E; t++) {
        const int k = g * E + t;
        const T2 ck = Ls[sk(k) ^ mC];
        if (k == 0) {
            ra[t] = T(0.5) * (ck.x + ck.y);  // Re Y_0, halved in the running sum
            ia[t] = T(0);
            const T2 cmid = Ls[sk(M / 2) ^ mC];
            rmid = cmid.x;
            imid = -cmid.y;
            rb[t] = T(0);
            ib[t] = T(0);
        } else {
            const T2 cm = Ls[sk(M - k) ^ mC];
            const T ex = T(0.5) * (ck.x + cm.x), ey = T(0.5) * (ck.y - cm.y);
            const T ox = T(0.5) * (ck.y + cm.y), oy = T(-0.5) * (ck.x - cm.x);
            const T2 w = ldg(tb.post + k);
            const T wx = w.x * ox - w.y * oy, wy = w.x * oy + w.y * ox;
            ra[t] = ex + wx;
            ia[t] = ey + wy;
            rb[t] = ex - wx;    // Re Y_{M-k}
            ib[t] = wy - ey;    // Im Y_{M-k}
        }
    }
    // running sums: first half in ascending k (blocks g = 0..G-1), then
    // Y_{M/2}, then the mirrored blocks in ascending k (g = G-1..0, each
    // walked from t = E-1 down to t = 0)
    T pa[E], pb[E];
    pa[0] = ra[0];
#pragma unroll
    for (int t = 1; t < E; t++) pa[t] = pa[t - 1] + ra[t];
    pb[E - 1] = rb[E - 1];
#pragma unroll
    for (int t = E - 2; t >= 0; t--) pb[t] = pb[t + 1] + rb[t];
    const T ta = pa[E - 1], tbk = pb[0];
    T inca = ta;
#pragma unroll
    for (int off = 1; off < G; off <<= 1) {
        const T x = __shfl_up_sync(0xffffffffu, inca, off, G);
        if (g >= off) inca += x;
    }
    T incb = tbk;
#pragma unroll
    for (int off = 1; off < G; off <<= 1) {
        const T x = __shfl_down_sync(0xffffffffu, incb, off, G);
        if (g + off < G) incb += x;
    }
    const T s1 = __shfl_sync(0xffffffffu, inca, G - 1, G);
    const T rm = __shfl_sync(0xffffffffu, rmid, 0, G);
    const T exa = inca - ta, exb = incb - tbk;
    const T bbase = s1 + rm + exb;
    // an odd line's packed output starts OOFF slots later (0: plain)
    const int mO = (line & 1) ? OOFF : 0;
    static_assert(Gm::CS + OOFF <= Gm::LS2 || OOFF == 0, "the shifted output stays inside its line");
    __syncwarp();
#pragma unroll
    for (int t = 0; t < E; t++) {
        const int k = g * E + t;
        T2 fa;
        fa.x = -ia[t];
        fa.y = exa + pa[t];
        Ls[sk(k) + mO] = fa;
        if (k > 0) {
            T2 fb;
            fb.x = -ib[t];
            fb.y = bbase + pb[t];
            Ls[sk(M - k) + mO] = fb;
        }
    }
    if (g == 0) {
        T2 fm;
        fm.x = -imid;
        fm.y = s1 + rmid;
        Ls[sk(M / 2) + mO] = fm;
    }
}

// Adds the CTA's sums of ||c||^2 and ||u||^2 to norms[2v], norms[2v+1]
// (v = blockIdx.y).  All threads of the CTA call it.
__device__ __forceinline__ void norms_reduce(float cc, float uu, double* norms, int tid, int nthr) {
    for (int o = 16; o > 0; o >>= 1) {
        cc += __shfl_down_sync(0xffffffffu, cc, o);
        uu += __shfl_down_sync(0xffffffffu, uu, o);
    }
    __shared__ float red[2][32];
    const int w = tid >> 5, ln = tid & 31;
    if (ln == 0) {
        red[0][w] = cc;
        red[1][w] = uu;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = nthr >> 5;
        cc = ln < nw ? red[0][ln] : 0.f;
        uu = ln < nw ? red[1][ln] : 0.f;
        for (int o = 16; o > 0; o >>= 1) {
            cc += __shfl_down_sync(0xffffffffu, cc, o);
            uu += __shfl_down_sync(0xffffffffu, uu, o);
        }
        if (ln == 0 && norms) {
            atomicAdd(&norms[2 * blockIdx.y], (double)cc);
            atomicAdd(&norms[2 * blockIdx.y + 1], (double)uu);
        }
    }
}

// column pass, one line per lane: item pairs loaded per batch of the fold
constexpr int kColFoldBatch = 8;    // FP32 input
constexpr int kColFoldBatch64 = 8;  // FP64 input (kRound)
// column combine pass with a low part: packed slots whose loads go ahead
constexpr int kCombineAhead = 4;

template <typename Tin, typename T, typename Tout, int AXIS, int MODE, int N, int NT = 256>
__device__ __forceinline__ void sine_rg_body(const Tin* in, Tout* out, const SineGeom& geo, const SineTables<T>& tb,
                                             T scale, const SineFused& fu) {
    using T2 = vec2_t<T>;
    using Gm = RgGeom<N, AXIS, NT>;
    // the lane-per-line column path and the paired row store walk 8 warps
    static_assert(NT == 256 || N <= 64, "CTAs of fewer than 256 threads are for lines of up to 64 points");
    constexpr int M = Gm::M, G = Gm::G, L = Gm::L;
    constexpr int LS2 = Gm::LS2;
    constexpr int n = N - 1;
    constexpr int ITEMS = M + 1;  // fold items per line: j = 0..M
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* S = reinterpret_cast<T2*>(smem_raw);
    T* Sr = reinterpret_cast<T*>(smem_raw);
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

    // ---- load + fold: item (line, j) reads x_j and x_{N-j} and writes
    // y_j = w_j (a+b) + (a-b)/2 and y_{N-j} = w_j (a+b) - (a-b)/2
    constexpr bool kCol32 = AXIS == 1 && L == 32 && NT == 256 && MODE != kResidual;
    // FP32 column transforms in the row-like line order (below), with the
    // packed output of odd positions shifted by kColOut slots; not the
    // 256-point combine pass (at its 48 registers the swizzles spill, and
    // it measured 2 % slower)
    constexpr bool kColRemap = kCol32 && sizeof(T) == 4 && !(MODE == kCombine && N == 256);
    constexpr int kColOut = kColRemap ? (N == 256 ? 4 : 2) : 0;
    const int lane = tid & 31, wid = tid >> 5;
    if constexpr (kCol32) {
        // column pass with one line per lane: warp w takes the items j =
        // w + 8q of its 32 lines, so an address is a per-thread base plus q
        // steps of 8 rows
        constexpr int QN = (ITEMS + 7) / 8;
        const bool act = lane < nact;
        const Tin* p = (fu.vin ? (const Tin*)fu.vin[blockIdx.y] : in + voff) + ((long long)z * ny) * nx + x0 + lane;
        T* xo = Sr + 2 * lane * LS2;  // this lane's line: folded entry j at xo[j]
        const long long s8 = 8LL * nx;
        const Tin* pa = p + (long long)(wid - 1) * nx;  // x_j sits in row j - 1
        const Tin* pb = p + (long long)(n - wid) * nx;  // x_{N-j} in row n - j
        // loads in flight per thread: FB pairs (FP32 input: all but one
        // batch of the line's items ahead of their use)
        constexpr int FB = sizeof(Tin) == 4 ? kColFoldBatch : kColFoldBatch64;
#pragma unroll
        for (int q0 = 0; q0 < QN; q0 += FB) {
            T av[FB], bv[FB];
#pragma unroll
            for (int qq = 0; qq < FB; qq++) {
                const int q = q0 + qq, j = wid + 8 * q;
                T a = T(0), b = T(0);
                if (q < QN && j <= M && (q > 0 || wid > 0) && act) {
                    if (MODE == kRound) {
                        a = T(f64_to_f32((double)pa[q * s8]));
                        b = T(f64_to_f32((double)pb[-q * s8]));
                    } else {
                        a = T(pa[q * s8]);
                        b = T(pb[-q * s8]);
                    }
                }
                av[qq] = a;
                bv[qq] = b;
            }
#pragma unroll
            for (int qq = 0; qq < FB; qq++) {
                const int q = q0 + qq, j = wid + 8 * q;
                if (q < QN && j <= M) {
                    const T w = ldg(tb.wpre + j);
                    const T sm = w * (av[qq] + bv[qq]), df = T(0.5) * (av[qq] - bv[qq]);
                    xo[j] = sm + df;  // j = 0: w_0 = 0 and a = b = 0
                    if (j != M && j != 0) xo[N - j] = sm - df;
                }
            }
        }
    } else {
        const T half = T(0.5);
        constexpr int total = L * ITEMS;
        for (int e0 = tid; e0 < total; e0 += 4 * nthr) {
            T av[4], bv[4];
            int lv[4], jv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int e = e0 + q * nthr;
                int line, j;
                if (AXIS == 0) {
                    line = e / ITEMS;
                    j = e - line * ITEMS;
                } else {
                    j = e / L;
                    line = e - j * L;
                }
                lv[q] = line;
                jv[q] = j;
                T a = T(0), b = T(0);
                if (e < total && line < nact && j >= 1) {
                    if (AXIS == 0) {
                        const int R = row0 + line;
                        if (MODE == kResidual) {
                            const int zz = geo.div_ny.div(R), yy = R - zz * ny;
                            SineFused f2 = fu;
                            f2.f = fu.vin ? (const double*)fu.vin[blockIdx.y] : fu.f + voff;
                            f2.uhi += voff;
                            if (f2.ulo) f2.ulo += voff;
                            const long long rb = (long long)R * n;
                            a = T(residual_at(f2, rb + j - 1, j - 1, yy, zz, nx, ny, nz));
                            b = T(residual_at(f2, rb + n - j, n - j, yy, zz, nx, ny, nz));
                        } else {
                            const Tin* p = (fu.vin ? (const Tin*)fu.vin[blockIdx.y] : in + voff) + (long long)R * n;
                            if (MODE == kRound) {
                                a = T(f64_to_f32((double)p[j - 1]));
                                b = T(f64_to_f32((double)p[n - j]));
                            } else {
                                a = T(p[j - 1]);
                                b = T(p[n - j]);
                            }
                        }
                    } else {
                        const Tin* p = (fu.vin ? (const Tin*)fu.vin[blockIdx.y] : in + voff) + ((long long)z * ny) * nx + x0 +
                                       line;
                        if (MODE == kRound) {
                            a = T(f64_to_f32((double)p[(long long)(j - 1) * nx]));
                            b = T(f64_to_f32((double)p[(long long)(n - j) * nx]));
                        } else {
                            a = T(p[(long long)(j - 1) * nx]);
                            b = T(p[(long long)(n - j) * nx]);
                        }
                    }
                }
                av[q] = a;
                bv[q] = b;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int e = e0 + q * nthr;
                if (e < total) {
                    const int line = lv[q], j = jv[q];
                    T* base = Sr + 2 * (size_t)line * LS2;
                    if (j == 0) {
                        base[0] = T(0);
                    } else {
                        const T w = ldg(tb.wpre + j);
                        const T sm = w * (av[q] + bv[q]), df = half * (av[q] - bv[q]);
                        base[j] = sm + df;
                        if (j != M) base[N - j] = sm - df;
                    }
                }
            }
        }
    }
    __syncthreads();

    if constexpr (kColRemap) {
        // the transform takes the lines in an order whose two lines per
        // half-warp sit 8 lines apart, 8 LS2 = 8 (mod 16) slots, as two
        // consecutive rows do, so the rows' slot swizzles apply (a bank
        // model of the transform: 2560 -> 1936 wavefronts per CTA at 256
        // points); the fold and store phases keep a line per lane
        static_assert(G == 8 && L == 32 && (8 * LS2) % 16 == 8, "line order for 8 threads per line");
        static_assert(swz_max(Gm::CS, RgSwz<T, N, 0>::C0 | RgSwz<T, N, 0>::C1) < LS2,
                      "a swizzled slot stays inside its column line");
        const int pl = ((l >> 1) & 7) + 8 * (l & 1) + 16 * (l >> 4);
        static_assert(Gm::CS + kColOut <= LS2, "the shifted output stays inside its column line");
        rg_line_fft<T, N, 0, true, kColOut>(S + (size_t)pl * LS2, g, l, tb);
    } else {
        rg_line_fft<T, N, AXIS>(S + (size_t)l * LS2, g, l, tb);
    }
    __syncthreads();

    // ---- store phase: entry i of line l is component i&1 of slot sk(i>>1).
    // Element e of the CTA's output goes to point idx of the volume (x
    // fastest); so is its offset in shared memory.
    const int total = AXIS == 0 ? nact * n : n * L;
    auto locate = [&](int e, long long& idx, int& so) -> bool {
        if (AXIS == 0) {
            const int r = e / n, i = e - r * n + 1;
            idx = (long long)row0 * n + e;
            so = 2 * (r * LS2 + sk(i >> 1)) + (i & 1);
            return e < total;
        } else {
            const int y = e / L, c = e - y * L, i = y + 1;
            idx = ((long long)z * ny + y) * nx + x0 + c;
            so = 2 * (c * LS2 + sk(i >> 1)) + (i & 1);
            return e < total && c < nact;
        }
    };
    // FP32 lines of 128 and 256 points read F_2k and F_2k+1 of a line as one
    // float2 (packed slot k) and store the two entries
    constexpr bool kPair = sizeof(T) == 4 && (N == 128 || N == 256);
    if constexpr (kCol32 && kPair) {
        // column pass, one line per lane: warp w stores the packed slots k =
        // w + 8q (slot sk(k) = w + 8q + q/2), entries 2k and 2k+1 to rows
        // y = 2k-1 and 2k
        constexpr int QS = M / 8;
        const bool act = lane < nact;
        // lines at odd transform positions (bit 3 of the line) hold their
        // packed output kColOut slots later
        const T2* src = S + lane * LS2 + wid + (kColRemap && (lane & 8) ? kColOut : 0);
        const long long s16 = 16LL * nx;
        const long long base = ((long long)z * ny + 2 * wid - 1) * nx + x0 + lane;  // row 2k-1 at q = 0
        if constexpr (MODE == kCombine) {
            float cc = 0.f, uu = 0.f;
            double* o64 = (fu.vout ? (double*)fu.vout[blockIdx.y] : fu.out64 + voff) + base;
            const float* uh = fu.uhi + voff + base;
            const float* ul = fu.ulo ? fu.ulo + voff + base : nullptr;
            float* ulo_out = fu.ulo_out ? fu.ulo_out + voff + base : nullptr;
            if (!ul) {
                // no low part (the first sweep): u = uhi + c as the float
                // pair two_sum(uhi, c), the value the general form below
                // gives with ulo = 0; the uhi loads of half the slots are
                // issued before any is used
                constexpr int QH = QS / 2;
#pragma unroll
                for (int q0 = 0; q0 < QS; q0 += QH) {
                    float hv[2 * QH];
#pragma unroll
                    for (int a = 0; a < 2 * QH; a++) {
                        const int q = q0 + (a >> 1), h = a & 1;
                        const bool ok = act && (h || q > 0 || wid > 0);
                        hv[a] = ok ? uh[q * s16 + h * nx] : 0.f;
                    }
#pragma unroll
                    for (int qq = 0; qq < QH; qq++) {
                        const int q = q0 + qq;
                        if (!act) continue;
                        const T2 f2 = src[8 * q + (q >> 1)];
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            if (!h && q == 0 && wid == 0) continue;
                            const long long o = q * s16 + h * nx;
                            const float cv = (float)(scale * (h ? f2.y : f2.x));
                            const ff s2 = two_sum(__fadd_rn(hv[2 * qq + h], 0.f), cv);
                            if (fu.last) o64[o] = ff_to_f64(s2);
                            if (ulo_out) ulo_out[o] = __fadd_rn(0.f, cv);
                            cc += cv * cv;
                            uu += s2.h * s2.h;
                        }
                    }
                }
                norms_reduce(cc, uu, fu.norms, tid, nthr);
                return;
            }
            // with a low part: the loads of kCombineAhead slots issued
            // before any of them is used
            constexpr int QC = kCombineAhead;
#pragma unroll
            for (int q0 = 0; q0 < QS; q0 += QC) {
                float hv[2 * QC], lw[2 * QC];
#pragma unroll
                for (int a = 0; a < 2 * QC; a++) {
                    const int q = q0 + (a >> 1), h = a & 1;
                    const long long o = q * s16 + h * nx;
                    const bool ok = act && (h || q > 0 || wid > 0);
                    hv[a] = ok ? uh[o] : 0.f;
                    lw[a] = ok ? ul[o] : 0.f;
                }
#pragma unroll
                for (int qq = 0; qq < QC; qq++) {
                    const int q = q0 + qq;
                    if (!act) continue;
                    const T2 f2 = src[8 * q + (q >> 1)];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (!h && q == 0 && wid == 0) continue;
                        const int a = 2 * qq + h;
                        const long long o = q * s16 + h * nx;
                        const float cv = (float)(scale * (h ? f2.y : f2.x));
                        ff s2 = two_sum(hv[a], lw[a]);
                        s2 = ff_add_f(s2, cv);
                        if (fu.last) o64[o] = ff_to_f64(s2);
                        if (ulo_out) ulo_out[o] = lw[a] + cv;
                        cc += cv * cv;
                        uu += s2.h * s2.h;
                    }
                }
            }
            norms_reduce(cc, uu, fu.norms, tid, nthr);
        } else {
            Tout* ob = (fu.vout ? (Tout*)fu.vout[blockIdx.y] : out + voff) + base;
            if (act) {
#pragma unroll
                for (int q = 0; q < QS; q++) {
                    const T2 f2 = src[8 * q + (q >> 1)];
                    if (q > 0 || wid > 0) ob[q * s16] = Tout(scale * f2.x);
                    ob[q * s16 + nx] = Tout(scale * f2.y);
                }
            }
        }
    } else if constexpr (AXIS == 0 && kPair && MODE != kCombine) {
        // row pass: warp w stores lines w, w+8, ...; lane c the packed slots
        // k = c + 32q (slot sk(k) = c + c/16 + 34q), entries to x = 2k-1, 2k
        Tout* ob = (fu.vout ? (Tout*)fu.vout[blockIdx.y] : out + voff) + (long long)row0 * n + 2 * lane;
#pragma unroll
        for (int li = 0; li < L / 8; li++) {
            const int r = wid + 8 * li;
            if (r >= nact) continue;
            const T2* src = S + r * LS2 + lane + (lane >> 4);
            Tout* dst = ob + (long long)r * n;
#pragma unroll
            for (int q = 0; q < M / 32; q++) {
                const T2 f2 = src[34 * q];
                if (q > 0 || lane > 0) dst[64 * q - 1] = Tout(scale * f2.x);
                dst[64 * q] = Tout(scale * f2.y);
            }
        }
    } else if (MODE == kCombine) {
        float cc = 0.f, uu = 0.f;
        double* o64 = fu.vout ? (double*)fu.vout[blockIdx.y] : fu.out64 + voff;
        // batches of 4 elements per thread: the uhi / ulo loads of a batch
        // are issued before any of them is used
        for (int e0 = tid; e0 < total; e0 += 4 * nthr) {
            float hv[4], lv[4];
            long long ix[4];
            int so[4];
            bool ok[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                ok[q] = locate(e0 + q * nthr, ix[q], so[q]);
                hv[q] = 0.f;
                lv[q] = 0.f;
                if (ok[q]) {
                    hv[q] = fu.uhi[voff + ix[q]];
                    if (fu.ulo) lv[q] = fu.ulo[voff + ix[q]];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (ok[q]) {
                    const float cv = (float)(scale * Sr[so[q]]);
                    // no low part: two_sum(u_hi, c), the value of the general
                    // form with u_lo = 0, bit for bit
                    ff s2;
                    if (fu.ulo) s2 = ff_add_f(two_sum(hv[q], lv[q]), cv);
                    else s2 = two_sum(__fadd_rn(hv[q], 0.f), cv);
                    if (fu.last) o64[ix[q]] = ff_to_f64(s2);
                    if (fu.ulo_out) fu.ulo_out[voff + ix[q]] = lv[q] + cv;
                    cc += cv * cv;
                    uu += s2.h * s2.h;
                }
            }
        }
        norms_reduce(cc, uu, fu.norms, tid, nthr);
    } else {
        Tout* ob = fu.vout ? (Tout*)fu.vout[blockIdx.y] : out + voff;
        for (int e = tid; e < total; e += nthr) {
            long long idx;
            int so;
            if (locate(e, idx, so)) ob[idx] = Tout(scale * Sr[so]);
        }
    }
}

template <typename Tin, typename T, typename Tout, int AXIS, int MODE, int N, int NT = 256>
__global__ void __launch_bounds__(NT) k_sine_rg(const Tin* in, Tout* out, SineGeom geo, SineTables<T> tb, T scale,
                                                SineFused fu) {
    sine_rg_body<Tin, T, Tout, AXIS, MODE, N, NT>(in, out, geo, tb, scale, fu);
}

// The same kernel held to 64 registers (4 CTAs of 256 threads per SM): for
// the FP32 x-line passes of 256 and 512 points, whose unconstrained
// allocation (70-78 registers) leaves 3 CTAs per SM and which run faster
// at the higher occupancy without spilling.
template <typename Tin, typename T, typename Tout, int AXIS, int MODE, int N>
__global__ void __launch_bounds__(256, 4) k_sine_rg_occ(const Tin* in, Tout* out, SineGeom geo, SineTables<T> tb,
                                                        T scale, SineFused fu) {
    sine_rg_body<Tin, T, Tout, AXIS, MODE, N>(in, out, geo, tb, scale, fu);
}

// The FP32 column pass of 256 points held to 48 registers (5 CTAs of 256
// threads per SM, no spills): 2.86 -> 2.84 ms per 16 x 255^3 step of its
// four launches; 6 CTAs (40 registers) spill and take 3.22 ms.
template <typename Tin, typename T, typename Tout, int AXIS, int MODE, int N>
__global__ void __launch_bounds__(256, 5) k_sine_rg_occ5(const Tin* in, Tout* out, SineGeom geo, SineTables<T> tb,
                                                         T scale, SineFused fu) {
    sine_rg_body<Tin, T, Tout, AXIS, MODE, N>(in, out, geo, tb, scale, fu);
}

template <typename T, int AXIS, int N>
constexpr bool rg_use_occ() {
    return sizeof(T) == 4 && AXIS == 0 && N >= 256;
}

template <typename T, int AXIS, int N>
constexpr bool rg_use_occ5() {
    return sizeof(T) == 4 && AXIS == 1 && N == 256;
}

template <typename T, int N, int AXIS, int NT = 256>
constexpr size_t rg_smem_bytes() {
    return (size_t)RgGeom<N, AXIS, NT>::L * RgGeom<N, AXIS, NT>::LS2 * sizeof(vec2_t<T>);
}

}  // namespace fdmgpu
