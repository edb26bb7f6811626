// One pass per y-mode plane of the mixed-precision Poisson pipeline: the
// DST along x, the tridiagonal solve along z and the inverse DST along x.
//
// For y-mode ky of a batch of FP32 volumes (x fastest: rows of nx, planes of
// nx*ny), the rows (z, ky), z = 0..nz-1, go through
//   1. the DST along x of every row (the x-line transform of sine_rg.cuh),
//   2. per x-mode i the Dirichlet tridiagonal system along z
//          u[z-1] + b u[z] + u[z+1] = gs * g[z],  b = -2 - (lx_i + ly_ky) hz^2,
//      which inverts what the reference does with DST_z, the division by
//      -(lm_z + lm_y + lm_x) and the inverse DST_z (src/lapl_cube.cpp:13-30,
//      :70-84, :124-141).  It is partitioned as k_zsolve_tab does it: P =
//      (nz+1)/16 blocks of 15 rows and P-1 separator rows, every factor read
//      from the per-mode table that the plan builds in FP64,
//   3. the inverse DST along x, stored back in place;
// one read and one write of the plane instead of three passes over the
// volume (x, z, inverse x) with a write and a read between each.
//
// A 255 x 255 FP32 plane (254 KB) is larger than one CTA's shared memory, so
// a cluster of C CTAs owns a plane: CTA r holds the L rows z = rL..rL+L-1
// (L = the lines per CTA of the x-line transform; the last CTA has L-1
// rows), which are the z blocks rB..rB+B-1 (B = L/16) with their separators.
// Only the separator system crosses CTAs.  Each CTA publishes its blocks'
// end values and its separators' right-hand sides in its own shared memory;
// after a cluster barrier, CTA r solves the P-1 separator unknowns of its
// share of the x-modes from those values (read from the peers' shared
// memory) and writes each solution into the shared memory of the CTAs whose
// blocks end on it; after a second barrier every CTA finishes its blocks
// locally.  The cluster barriers are hardware barriers of co-scheduled CTAs;
// no CTA leaves before the second one, so no peer memory is read after its
// owner exits.
#pragma once

#include <cooperative_groups.h>

#include "sine_rg.cuh"

namespace fdmgpu {

struct PlaneGeom {
    int nx, ny, nz;
    long long vstride;  // elements per volume
    int modes;          // nx * ny: the z table's stride between values
};

template <int N>
struct PlaneCfg {
    using Gm = RgGeom<N, 0>;
    static constexpr int L = Gm::L;      // rows per CTA
    static constexpr int B = L / 16;     // z blocks per CTA
    static constexpr int XS = 256;       // floats per x-mode array row (>= n)
    static constexpr size_t smem() {
        return (size_t)2 * L * Gm::LS2 * sizeof(float) + (size_t)(4 * B + 1) * XS * sizeof(float);
    }
};

// W: the batch of volumes (in place), grid (C * ny, volumes), 256 threads, a
// cluster of C CTAs along x.  gs: the forward x scale times the z-solve's
// right-hand-side scale; sc_inv: the inverse x scale; tab: the per-mode z
// factor table of k_zsolve_tab (block pivots, right-end responses,
// separator pivots and multipliers, value-major over nx*ny modes).
// The x transforms use the row swizzles of RgSwz (layouts B and C only, so
// the plane's own views of the folded input and packed output are plain).
constexpr bool kPlaneSwz = true;
// rows whose loads a warp issues together in the fold phase
constexpr int kPlaneFoldLines = 2;

template <int N, int C, int MINB>
__global__ void __launch_bounds__(256, MINB) k_plane_xz(float* __restrict__ W, PlaneGeom geo, SineTables<float> tb,
                                                        float gs, float sc_inv, const float* __restrict__ tab) {
    namespace cg = cooperative_groups;
    using T2 = float2;
    using Gm = RgGeom<N, 0>;
    using Pc = PlaneCfg<N>;
    constexpr int M = Gm::M, G = Gm::G, L = Gm::L, LS2 = Gm::LS2;
    constexpr int n = N - 1, ITEMS = M + 1, nthr = L * G;
    constexpr int m = 15, B = Pc::B, XS = Pc::XS;
    constexpr int P = C * B;             // z blocks of the plane
    constexpr int MPC = (n + C - 1) / C;  // x-modes whose separator system a CTA solves
    static_assert(nthr == 256 && n < XS && MPC <= 256 && P <= 16, "plane layout");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* S = reinterpret_cast<T2*>(smem_raw);
    float* Sr = reinterpret_cast<float*>(smem_raw);
    float* xf = Sr + 2 * L * LS2;  // [B][XS] first value of each block's zero-end solution
    float* xl = xf + B * XS;       // [B][XS] its last value
    float* xg = xl + B * XS;       // [B][XS] separator right-hand sides (times gs)
    float* xs = xg + B * XS;       // [B+1][XS] separator solutions s[rB-1 .. rB+B-1]

    cg::cluster_group cl = cg::this_cluster();
    const int r = (int)cl.block_rank();
    const int ky = blockIdx.x / C;
    const int nx = geo.nx, ny = geo.ny, nz = geo.nz;
    const int tid = threadIdx.x, l = tid / G, g = tid % G;
    const int z0 = r * L;
    const int nact = min(L, nz - z0);
    const long long rstride = (long long)ny * nx;  // between consecutive z rows
    float* row0 = W + (long long)blockIdx.y * geo.vstride + ((long long)z0 * ny + ky) * nx;

    // The fold and store phases run one warp per line: lane c takes the
    // items j = c + 32k (and lane 0 also j = M), so every global and shared
    // address is a per-thread base plus a compile-time offset.  In the fold
    // input entry j of the line at position p is float 2 p LS2 + j; in the
    // packed output entry i is float 2 p LS2 + 2 sk(i>>1) + (i&1), which is
    // c + 34k for i = c + 32k and fb - 34k for i = N - c - 32k (fb below).
    // Warp w folds, transforms and stores the rows w + 8j (j < LPW), kept at
    // positions LPW w + j: the transform's G threads of position p belong to
    // warp p / LPW, so between fold, transform and store only the warp
    // synchronises.  Row q of the CTA sits at position rowpos(q).
    const int lane = tid & 31, wid = tid >> 5;
    constexpr int KJ = M / 32;  // full rounds of 32 items per line (j < M)
    constexpr int LPW = L / 8;  // lines per warp
    static_assert(LPW * G == 32, "a warp's transform threads hold its own rows");
    auto rowpos = [](int q) { return LPW * (q & 7) + (q >> 3); };
    const int hh = (lane + 1) >> 1;
    const int fb = 2 * (M + M / 16 - hh - (hh > 0 ? 1 : 0)) + (lane & 1);
    static_assert(M % 32 == 0 && L % 8 == 0, "warp-per-line phases");

    // ---- 1. load + fold, then the DST along x; the loads of kPlaneFoldLines
    // rows are issued before any of them is folded
    constexpr int PL = kPlaneFoldLines;
    static_assert(LPW % PL == 0, "rows per warp in whole load batches");
#pragma unroll
    for (int l0 = 0; l0 < LPW; l0 += PL) {
        float a[PL][KJ], b[PL][KJ], am[PL];
#pragma unroll
        for (int pl = 0; pl < PL; pl++) {
            const int line = wid + 8 * (l0 + pl);
            const float* p = row0 + line * rstride;
            const bool in = line < nact;
#pragma unroll
            for (int k = 0; k < KJ; k++) {
                const bool ok = in && (k > 0 || lane > 0);
                a[pl][k] = ok ? p[lane + 32 * k - 1] : 0.f;
                b[pl][k] = ok ? p[n - lane - 32 * k] : 0.f;
            }
            am[pl] = in ? p[M - 1] : 0.f;
        }
#pragma unroll
        for (int pl = 0; pl < PL; pl++) {
            const int li = l0 + pl;
            const int line = wid + 8 * li;
            float* xo = Sr + 2 * (LPW * wid + li) * LS2;
            if (line < nact) {
#pragma unroll
                for (int k = 0; k < KJ; k++) {
                    const int j = lane + 32 * k;
                    const float w = ldg(tb.wpre + j);
                    const float sm = w * (a[pl][k] + b[pl][k]), df = 0.5f * (a[pl][k] - b[pl][k]);
                    xo[j] = sm + df;  // j = 0: both are 0
                    if (k > 0 || lane > 0) xo[N - j] = sm - df;
                }
                if (lane == 0) xo[M] = ldg(tb.wpre + M) * (am[pl] + am[pl]);
            } else {
                // the row past the plane's end (last CTA): a zero line
#pragma unroll
                for (int k = 0; k < 2 * KJ; k++) xo[lane + 32 * k] = 0.f;
            }
        }
    }
    __syncwarp();
    rg_line_fft<float, N, 0, kPlaneSwz>(S + l * LS2, g, l, tb);
    __syncthreads();

    // ---- 2. z blocks: thread t owns x-mode i = t of every local block
    // (thread 0 none).  Entry i of row q sits at Sr[2*(rowpos(q)*LS2 +
    // sk(i>>1)) + (i&1)], float i + 2 (i >> 5) of the row, so the 32 modes
    // of a warp are 32 consecutive floats (one wavefront); tm = i - 1 indexes
    // the mode's table column and its slots of xf, xl, xg and xs.
    const int t = tid;
    const bool mode_ok = t >= 1 && t <= n;
    const int i = t;
    const int tm0 = mode_ok ? t - 1 : 0;
    const int fo = 2 * sk(i >> 1) + (i & 1);
    const int modes = geo.modes;
    const int tmode = ky * nx + tm0;
    constexpr int RS = 2 * LS2;  // floats between rows
    if (mode_ok) {
        float cp[m];
#pragma unroll
        for (int k = 0; k < m; k++) cp[k] = tab[(size_t)k * modes + tmode];
#pragma unroll
        for (int b = 0; b < B; b++) {
            const int gb = r * B + b;
            float* col = Sr + fo;
            float v[m];
#pragma unroll
            for (int k = 0; k < m; k++) v[k] = col[rowpos(16 * b + k) * RS];
            float prev = 0.f;
#pragma unroll
            for (int k = 0; k < m; k++) {
                prev = (v[k] * gs - prev) * cp[k];
                v[k] = prev;
            }
#pragma unroll
            for (int k = m - 2; k >= 0; k--) v[k] = v[k] - cp[k] * v[k + 1];
#pragma unroll
            for (int k = 0; k < m; k++) col[rowpos(16 * b + k) * RS] = v[k];
            xf[b * XS + tm0] = v[0];
            xl[b * XS + tm0] = v[m - 1];
            xg[b * XS + tm0] = gb < P - 1 ? col[rowpos(16 * b + m) * RS] * gs : 0.f;
        }
    }
    // the plane's outer ends: s[-1] = s[P-1] = 0
    if (r == 0) xs[tid] = 0.f;
    if (r == C - 1) xs[B * XS + tid] = 0.f;
    cl.sync();

    // ---- 3. separator systems of this CTA's x-modes
    if (P > 1 && tid < MPC) {
        const int tm = r * MPC + tid;
        if (tm < n) {
            const int mm = ky * nx + tm;
            float d[P > 1 ? P - 1 : 1];
#pragma unroll
            for (int q = 0; q < P - 1; q++) {
                // separator q lies between block q and block q + 1
                const int c1 = q / B, b1 = q % B, c2 = (q + 1) / B, b2 = (q + 1) % B;
                const float* g1 = cl.map_shared_rank(xg, c1);
                const float* l1 = cl.map_shared_rank(xl, c1);
                const float* f2 = cl.map_shared_rank(xf, c2);
                d[q] = g1[b1 * XS + tm] - l1[b1 * XS + tm] - f2[b2 * XS + tm];
            }
            const float lo = tab[(size_t)m * modes + mm];
            float acc = 0.f;
#pragma unroll
            for (int q = 0; q < P - 1; q++) {
                acc = (d[q] - lo * acc) * tab[(size_t)(2 * m + q) * modes + mm];
                d[q] = acc;
            }
            float u = 0.f;
#pragma unroll
            for (int q = P - 2; q >= 0; q--) {
                u = d[q] - tab[(size_t)(2 * m + P - 1 + q) * modes + mm] * u;
                d[q] = u;
            }
            // s[q] ends block q on the right and block q+1 on the left: slot
            // q - (c B - 1) of xs in the CTA c that holds each of them
#pragma unroll
            for (int q = 0; q < P - 1; q++) {
                const int c1 = q / B, c2 = (q + 1) / B;
                cl.map_shared_rank(xs, c1)[(q - (c1 * B - 1)) * XS + tm] = d[q];
                if (c2 != c1) cl.map_shared_rank(xs, c2)[(q - (c2 * B - 1)) * XS + tm] = d[q];
            }
        }
    }
    cl.sync();

    // ---- 4. finish the blocks: u = v + beta_rev * s_left + beta * s_right
    if (mode_ok) {
        float be[m];
#pragma unroll
        for (int k = 0; k < m; k++) be[k] = tab[(size_t)(m + k) * modes + tmode];
#pragma unroll
        for (int b = 0; b < B; b++) {
            const int gb = r * B + b;
            const float ul = xs[b * XS + tm0], ur = xs[(b + 1) * XS + tm0];
            float* col = Sr + fo;
#pragma unroll
            for (int k = 0; k < m; k++) {
                float& e = col[rowpos(16 * b + k) * RS];
                e = e + be[m - 1 - k] * ul + be[k] * ur;
            }
            if (gb < P - 1) col[rowpos(16 * b + m) * RS] = ur;
        }
    }
    __syncthreads();

    // ---- 5. inverse DST along x: fold from the packed output into the fold
    // input of the same line (a warp reads the whole line first: the two
    // layouts overlap)
#pragma unroll
    for (int li = 0; li < LPW; li++) {
        float* base = Sr + 2 * (LPW * wid + li) * LS2;
        float a[KJ], b[KJ];
#pragma unroll
        for (int k = 0; k < KJ; k++) {
            const bool ok = k > 0 || lane > 0;
            a[k] = ok ? base[lane + 34 * k] : 0.f;
            b[k] = ok ? base[fb - 34 * k] : 0.f;
        }
        const float am = base[2 * (M / 2 + M / 32)];
        __syncwarp();
#pragma unroll
        for (int k = 0; k < KJ; k++) {
            const int j = lane + 32 * k;
            const float w = ldg(tb.wpre + j);
            const float sm = w * (a[k] + b[k]), df = 0.5f * (a[k] - b[k]);
            base[j] = sm + df;
            if (k > 0 || lane > 0) base[N - j] = sm - df;
        }
        if (lane == 0) base[M] = ldg(tb.wpre + M) * (am + am);
    }
    __syncwarp();
    rg_line_fft<float, N, 0, kPlaneSwz>(S + l * LS2, g, l, tb);
    __syncwarp();

    // ---- 6. store the rows: slot k = c + 32q of a line holds F_2k and
    // F_2k+1, which go to x = 2k-1 and 2k
#pragma unroll
    for (int li = 0; li < LPW; li++) {
        const int line = wid + 8 * li;
        if (line >= nact) continue;
        const T2* src = S + (LPW * wid + li) * LS2 + lane + (lane >> 4);
        float* dst = row0 + line * rstride + 2 * lane;
#pragma unroll
        for (int q = 0; q < M / 32; q++) {
            const T2 f2 = src[34 * q];
            if (q > 0 || lane > 0) dst[64 * q - 1] = sc_inv * f2.x;
            dst[64 * q] = sc_inv * f2.y;
        }
    }
}

}  // namespace fdmgpu
