// LaplCube / LaplRect plans and their C ABI (declared in include/fdmgpu.h).
//
// Plain form (any dtype): DST-x, DST-y on the user's output buffer in place,
// then one constant-coefficient tridiagonal solve per (x-mode, y-mode) along
// z, then the inverse DST-y and DST-x.  The z-tridiagonal replaces the
// reference's DST_z / divide / inverse DST_z (src/lapl_cube.cpp:13-30,
// :70-84, :124-141); it inverts the same operator, so results agree to
// round-off.  No scratch memory.
//
// Mixed form (FP64 arrays): the same pipeline in FP32 gives u0; then each
// refinement sweep forms r = f - A u / S from the FP32/FP64 state in FP64,
// solves for the correction in FP32 and accumulates.  S is the reference's
// overall scale (prod_a h_a N_a / l_a, 1 for the usual l = (n+1)h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <deque>
#include <map>
#include <vector>

#include "internal.h"
#include "poisson.h"
#include "sine.cuh"
#include "sine_rg.cuh"
#include "sine_tc.cuh"
#include "plane_xz.cuh"
#include "pfft.cuh"
#include "solve_kernels.cuh"

namespace fdmgpu {

// ---------------------------------------------------------------------------
// per-axis tables
// ---------------------------------------------------------------------------
template <typename T>
struct AxisTables {
    int N = 0, M = 0;
    DevBuf tw, post, wpre;

    void build(int N_) {
        N = N_;
        M = N / 2;
        using T2 = vec2_t<T>;
        std::vector<T2> htw(M > 0 ? M : 1), hpost(M > 0 ? M : 1);
        std::vector<T> hw(N);
        for (int k = 0; k < M; k++) {
            const double a = 2.0 * M_PI * k / M, b = 2.0 * M_PI * k / N;
            htw[k].x = (T)std::cos(a);
            htw[k].y = (T)(-std::sin(a));
            hpost[k].x = (T)std::cos(b);
            hpost[k].y = (T)(-std::sin(b));
        }
        for (int j = 0; j < N; j++) hw[j] = (T)std::sin(M_PI * j / N);
        FDM_CUDA(cudaMemcpy(tw.get(htw.size() * sizeof(T2)), htw.data(), htw.size() * sizeof(T2),
                            cudaMemcpyHostToDevice));
        FDM_CUDA(cudaMemcpy(post.get(hpost.size() * sizeof(T2)), hpost.data(), hpost.size() * sizeof(T2),
                            cudaMemcpyHostToDevice));
        FDM_CUDA(cudaMemcpy(wpre.get(hw.size() * sizeof(T)), hw.data(), hw.size() * sizeof(T),
                            cudaMemcpyHostToDevice));
    }
    SineTables<T> view() const {
        SineTables<T> v;
        v.tw = (const vec2_t<T>*)tw.p;
        v.post = (const vec2_t<T>*)post.p;
        v.wpre = (const T*)wpre.p;
        v.N = N;
        v.M = M;
        return v;
    }
};

// Dirichlet eigenvalues 4/h^2 sin^2(j pi / (2(n+1))), j = 1..n at [j-1]
// (src/lapl_cube.cpp:145-172), uploaded in type T.
template <typename T>
static void upload_lambda(DevBuf& buf, int n, double h) {
    std::vector<T> v(n);
    for (int j = 1; j <= n; j++) {
        const double s = std::sin(j * M_PI * 0.5 / (n + 1));
        v[j - 1] = (T)(4. / (h * h) * (s * s));
    }
    FDM_CUDA(cudaMemcpy(buf.get(n * sizeof(T)), v.data(), n * sizeof(T), cudaMemcpyHostToDevice));
}

// ---------------------------------------------------------------------------
// periodic LaplCube: twiddles, eigenvalues, the transform launcher and the
// divide
// ---------------------------------------------------------------------------
template <typename T>
static void upload_ptwiddles(DevBuf& buf, int n) {
    std::vector<vec2_t<T>> v(n);
    for (int t = 0; t < n; t++) {
        const double a = -2.0 * M_PI * t / n;
        v[t].x = (T)std::cos(a);
        v[t].y = (T)std::sin(a);
    }
    FDM_CUDA(cudaMemcpy(buf.get(n * sizeof(vec2_t<T>)), v.data(), n * sizeof(vec2_t<T>), cudaMemcpyHostToDevice));
}

// lm[p] = 4/h^2 sin^2(p pi / n), p = 0..n-1 (src/lapl_cube.cpp:150, periodic)
template <typename T>
static void upload_plambda(DevBuf& buf, int n, double h) {
    std::vector<T> v(n);
    for (int p = 0; p < n; p++) {
        const double s = std::sin(p * M_PI / n);
        v[p] = (T)(4. / (h * h) * (s * s));
    }
    FDM_CUDA(cudaMemcpy(buf.get(n * sizeof(T)), v.data(), n * sizeof(T), cudaMemcpyHostToDevice));
}

// streaming multiprocessors of the current device (looked up once per
// device)
static int sm_count() {
    static PerDevice<int> sms;
    return sms.get([] {
        int v = 0;
        FDM_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, current_device()));
        return v > 0 ? v : 1;
    });
}

template <typename T, bool INV>
static void launch_pfft(const T* in, T* out, const PLineGeom& g, int n, const void* tw, double scale,
                        cudaStream_t st) {
    const int LPB = pfft_lines_per_block(n, g.lines, sm_count());
    const unsigned grid = (unsigned)((g.lines + LPB - 1) / LPB);
    FDM_TIMED(INV ? "pfft_inverse" : "pfft_forward", st);
    k_pfft<T, INV><<<grid, 256, pfft_smem_bytes<T>(n, LPB), st>>>(in, out, g, n, LPB, (const vec2_t<T>*)tw,
                                                                  (T)scale);
    FDM_LAUNCH_CHECK();
}

// W /= -(lz[i] + ly[k] + lx[j]) (in T, as the reference's k2), zero mode := 0
template <typename T>
__global__ void k_pdivide(T* W, int nx, int ny, int nz, long long total, const T* lx, const T* ly, const T* lz) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const long long vol = (long long)nx * ny * nz;
    const long long r = e % vol;
    const int j = (int)(r % nx), k = (int)((r / nx) % ny), i = (int)(r / ((long long)nx * ny));
    const T k2 = lz[i] + ly[k] + lx[j];
    W[e] = (i == 0 && k == 0 && j == 0) ? T(0) : W[e] / -k2;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static const size_t kSineSmemBudget = 96 * 1024;

template <typename T>
static int pick_lines(int N) {
    int L = 32;
    while (L > 1 && sine_smem_bytes<T>(N, L) > kSineSmemBudget) L >>= 1;
    return L;
}

template <typename Tin, typename T, typename Tout, int AXIS, int MODE>
constexpr const char* sine_name() {
    return AXIS == 1 ? (MODE == kRound      ? "sine_y_round"
                        : MODE == kCombine ? "sine_y_combine"
                        : sizeof(T) == 8   ? "sine_y_f64"
                        : sizeof(Tout) == 8 ? "sine_y_f32_out64"
                                            : "sine_y_f32")
           : MODE == kRound    ? "sine_x_round"
           : MODE == kResidual ? "sine_x_resid"
           : MODE == kCombine  ? "sine_x_combine"
           : sizeof(T) == 8    ? "sine_x_f64"
           : sizeof(Tout) == 8 ? "sine_x_f32_out64"
                               : "sine_x_f32";
}

template <typename Tin, typename T, typename Tout, int AXIS, int MODE, int N, int NT = 256>
static void launch_rg_nt(const Tin* in, Tout* out, int nx, int ny, int nz, int nvol, const SineTables<T>& tb,
                         double scale, cudaStream_t st, const SineFused& fu, const SineGeom& geo) {
    constexpr int L = RgGeom<N, AXIS, NT>::L;
    constexpr size_t smem = rg_smem_bytes<T, N, AXIS, NT>();
    const auto kern = [] {
        if constexpr (NT != 256) return k_sine_rg<Tin, T, Tout, AXIS, MODE, N, NT>;
        else if constexpr (rg_use_occ5<T, AXIS, N>()) return k_sine_rg_occ5<Tin, T, Tout, AXIS, MODE, N>;
        else if constexpr (rg_use_occ<T, AXIS, N>()) return k_sine_rg_occ<Tin, T, Tout, AXIS, MODE, N>;
        else return k_sine_rg<Tin, T, Tout, AXIS, MODE, N>;
    }();
    static PerDevice<bool> attr_set;
    attr_set.get([kern] {
        FDM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return true;
    });
    unsigned gx;
    if (AXIS == 0) gx = (unsigned)((ny * (long long)nz + L - 1) / L);
    else gx = (unsigned)(nz * ((nx + L - 1) / L));
    dim3 grid(gx, nvol);
    FDM_TIMED((sine_name<Tin, T, Tout, AXIS, MODE>()), st);
    kern<<<grid, NT, smem, st>>>(in, out, geo, tb, (T)scale, fu);
    FDM_LAUNCH_CHECK();
}

// Lines of up to 64 points in volumes too small to give every SM two CTAs
// of 256 threads run in CTAs of 128 or 64 (fewer lines per CTA, more CTAs):
// a 63^3 volume's 3969 lines make 62 CTAs of 64 lines, on 62 of 152 SMs.
// rule_vols > 0: decide as for that many volumes (a caller whose launches
// serve varying numbers of volumes keeps one CTA size, and so the same
// rounding, for all).
template <typename Tin, typename T, typename Tout, int AXIS, int MODE, int N>
static void launch_rg(const Tin* in, Tout* out, int nx, int ny, int nz, int nvol, const SineTables<T>& tb,
                      double scale, cudaStream_t st, const SineFused& fu, SineGeom geo, int rule_vols) {
    if constexpr (N <= 64) {
        const long long lines =
            (AXIS == 0 ? (long long)ny * nz : (long long)nx * nz) * (rule_vols > 0 ? rule_vols : nvol);
        const long long want = 2LL * sm_count();
        if (lines / RgGeom<N, AXIS, 256>::L < want) {
            if (lines / RgGeom<N, AXIS, 128>::L >= want)
                return launch_rg_nt<Tin, T, Tout, AXIS, MODE, N, 128>(in, out, nx, ny, nz, nvol, tb, scale, st, fu,
                                                                      geo);
            return launch_rg_nt<Tin, T, Tout, AXIS, MODE, N, 64>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo);
        }
    }
    launch_rg_nt<Tin, T, Tout, AXIS, MODE, N, 256>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo);
}

// ---------------------------------------------------------------------------
// Tensor-core DST (N = 32, 64, 128): the pre-swizzled TF32 high / low image of
// the zero-padded sine matrix, and the launcher
// ---------------------------------------------------------------------------
static std::vector<float> tc_sine_image(int N) {
    const int n = N - 1;
    std::vector<float> img((size_t)2 * N * N, 0.f);
    float* hi = img.data();
    float* lo = img.data() + (size_t)N * N;
    for (int r = 0; r < n; r++)
        for (int k = 0; k < n; k++) {
            // sin(pi m / N) with m = (r+1)(k+1) reduced mod 2N
            const int m = ((r + 1) * (k + 1)) % (2 * N);
            const double v = std::sin(M_PI * (double)m / (double)N);
            const float h = tc_tf32((float)v);
            const uint32_t o = tc_sw128(N, r, k) / 4;
            hi[o] = h;
            lo[o] = tc_tf32((float)(v - (double)h));
        }
    return img;
}

static bool tc_supported(int N) { return N == 32 || N == 64 || N == 128; }

template <int N, int AXIS>
static auto tc_kernel() {
    if constexpr (N == 128) return k_sine_tc128<AXIS>;
    else return k_sine_tc<N, AXIS>;
}

template <int N, int AXIS>
static void launch_tc_n(const float* in, float* out, const SineTcGeom& g, const float* img, float scale, int* err,
                        cudaStream_t st) {
    using C = TcCfg<N>;
    const auto kern = tc_kernel<N, AXIS>();
    static PerDevice<int> grid_caps;
    const int grid_cap = grid_caps.get([kern] {
        FDM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::kSmem));
        FDM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        // resident CTAs per SM from the kernel's own registers and shared
        // memory, and tensor memory (512 columns per SM across CTAs)
        const int dev = current_device();
        int sms = 0, smem_sm = 0, regs_sm = 0;
        FDM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FDM_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        FDM_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
        cudaFuncAttributes fa;
        FDM_CUDA(cudaFuncGetAttributes(&fa, kern));
        const int smem_cta = C::kSmem + (int)fa.sharedSizeBytes + 1024;  // + the per-CTA reservation
        const int regs_cta = ((fa.numRegs + 7) / 8 * 8) * kTcThreads;
        int per_sm = std::min(smem_sm / smem_cta, regs_sm / std::max(regs_cta, 1));
        per_sm = std::max(1, std::min(per_sm, 512 / N));
        return per_sm * sms;
    });
    // as many CTAs as the tiles need in the fewest rounds, spread evenly
    const long long tiles = (g.lines + C::M - 1) / C::M;
    const long long rounds = (tiles + grid_cap - 1) / grid_cap;
    const unsigned grid = (unsigned)((tiles + rounds - 1) / std::max<long long>(rounds, 1));
    if (grid == 0) return;
    FDM_TIMED(AXIS == 0 ? "sine_x_tc" : "sine_y_tc", st);
    kern<<<grid, kTcThreads, C::kSmem, st>>>(in, out, g, img, scale, err);
    FDM_LAUNCH_CHECK();
}

// DST of lines of N-1 FP32 values on the tensor cores.  AXIS 0: `lines`
// contiguous lines; AXIS 1: lines along y of planes of (N-1) x nx values,
// `lines` = planes * nx.
template <int AXIS>
static void launch_sine_tc(int N, const float* in, float* out, long long lines, int nx, const float* img,
                           double scale, int* err, cudaStream_t st) {
    SineTcGeom g;
    g.lines = lines;
    g.nx = AXIS == 0 ? N - 1 : nx;
    g.plane = (long long)nx * (N - 1);
    if (N == 32) return launch_tc_n<32, AXIS>(in, out, g, img, (float)scale, err, st);
    if (N == 64) return launch_tc_n<64, AXIS>(in, out, g, img, (float)scale, err, st);
    if (N == 128) return launch_tc_n<128, AXIS>(in, out, g, img, (float)scale, err, st);
    FDM_FAIL(FDMGPU_ESIZE, "tensor-core DST supports N = 32, 64, 128 (got %d)", N);
}

template <typename Tin, typename T, typename Tout, int AXIS, int MODE = kPlain>
static void launch_sine(const Tin* in, Tout* out, int nx, int ny, int nz, int nvol, const SineTables<T>& tb,
                        double scale, cudaStream_t st, const SineFused* fused = nullptr, int rule_vols = 0) {
    SineGeom geo;
    geo.nx = nx; geo.ny = ny; geo.nz = nz;
    geo.vstride = (long long)nx * ny * nz;
    geo.div_n = FastDiv((unsigned)(AXIS == 0 ? nx : ny));
    geo.div_ny = FastDiv((unsigned)ny);
    SineFused fu;
    memset(&fu, 0, sizeof(fu));
    if (fused) fu = *fused;
    switch (tb.N) {
        case 16: return launch_rg<Tin, T, Tout, AXIS, MODE, 16>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo, rule_vols);
        case 32: return launch_rg<Tin, T, Tout, AXIS, MODE, 32>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo, rule_vols);
        case 64: return launch_rg<Tin, T, Tout, AXIS, MODE, 64>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo, rule_vols);
        case 128: return launch_rg<Tin, T, Tout, AXIS, MODE, 128>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo, rule_vols);
        case 256: return launch_rg<Tin, T, Tout, AXIS, MODE, 256>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo, rule_vols);
        case 512: return launch_rg<Tin, T, Tout, AXIS, MODE, 512>(in, out, nx, ny, nz, nvol, tb, scale, st, fu, geo, rule_vols);
        default: break;
    }
    // other lengths: the shared-memory Stockham kernel
    const int L = pick_lines<T>(tb.N);
    int Lshift = 0;
    while ((1 << Lshift) < L) Lshift++;
    const size_t smem = sine_smem_bytes<T>(tb.N, L);
    static PerDevice<bool> attr_set;
    attr_set.get([] {
        FDM_CUDA(cudaFuncSetAttribute(k_sine_pass<Tin, T, Tout, AXIS, MODE>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSineSmemBudget + 1024)));
        return true;
    });
    unsigned gx;
    if (AXIS == 0) gx = (unsigned)((ny * (long long)nz + L - 1) / L);
    else gx = (unsigned)(nz * ((nx + L - 1) / L));
    dim3 grid(gx, nvol);
    geo.L = L;
    geo.Lshift = Lshift;
    FDM_TIMED((sine_name<Tin, T, Tout, AXIS, MODE>()), st);
    k_sine_pass<Tin, T, Tout, AXIS, MODE><<<grid, L * kGroup, smem, st>>>(in, out, geo, tb, (T)scale, fu);
    FDM_LAUNCH_CHECK();
}

template <typename T>
static void launch_tridiag(T* W, int nlines, int n, int A, long long sa, long long sb, long long st_,
                           long long vstride, int nvol, const T* lamA, const T* lamB, double h2, double gscale,
                           cudaStream_t st) {
    dim3 grid((nlines + 127) / 128, nvol);
    FDM_TIMED(sizeof(T) == 8 ? "tridiag_f64" : "tridiag_f32", st);
    k_tridiag_const<T><<<grid, 128, 0, st>>>(W, nlines, n, A, sa, sb, st_, vstride, lamA, lamB, (T)h2, (T)gscale);
    FDM_LAUNCH_CHECK();
}

template <typename T, int m>
static void launch_zpart(T* W, int nx, int ny, int P, long long vstride, int nvol, const T* lamx, const T* lamy,
                         double h2, double gscale, cudaStream_t st) {
    const size_t smem = (size_t)4 * P * 32 * sizeof(T);
    dim3 grid((unsigned)(ny * ((nx + 31) / 32)), nvol);
    FDM_TIMED(sizeof(T) == 8 ? "zsolve_f64" : "zsolve_f32", st);
    k_zsolve_part<T, m><<<grid, 32 * P, smem, st>>>(W, nx, ny, P, vstride, lamx, lamy, (T)h2, (T)gscale);
    FDM_LAUNCH_CHECK();
}

// Tridiagonal solves along z of every (x-mode, y-mode) line: the partitioned
// kernel when the line splits into at most 16 blocks of 2^k-1 rows, the
// one-thread-per-line kernel otherwise.
template <typename T>
static void zsolve_lines(T* W, int nx, int ny, int nz, int nvol, const T* lamx, const T* lamy, double h2,
                         double gscale, cudaStream_t st) {
    const int mmax = 15;
    const int m = nz < mmax ? nz : mmax;
    const int P = (nz + 1) / (m + 1);
    const long long vs = (long long)nx * ny * nz;
    const int maxP = (m * (int)sizeof(T) >= 31 * 4 ? 256 : 512) / 32;
    if (P <= maxP && (m + 1) * P == nz + 1) {
        switch (m) {
            case 1: return launch_zpart<T, 1>(W, nx, ny, P, vs, nvol, lamx, lamy, h2, gscale, st);
            case 3: return launch_zpart<T, 3>(W, nx, ny, P, vs, nvol, lamx, lamy, h2, gscale, st);
            case 7: return launch_zpart<T, 7>(W, nx, ny, P, vs, nvol, lamx, lamy, h2, gscale, st);
            case 15: return launch_zpart<T, 15>(W, nx, ny, P, vs, nvol, lamx, lamy, h2, gscale, st);
            case 31:
                if (sizeof(T) == 4) return launch_zpart<T, sizeof(T) == 4 ? 31 : 15>(W, nx, ny, P, vs, nvol, lamx,
                                                                                     lamy, h2, gscale, st);
                break;
            default: break;
        }
    }
    launch_tridiag<T>(W, nx * ny, nz, nx, 1, nx, (long long)nx * ny, vs, nvol, lamx, lamy, h2, gscale, st);
}

static void launch_residual(const SineFused& fr, float* W, int nx, int ny, int nz, int nvol, cudaStream_t st) {
    const long long vol = (long long)nx * ny * nz;
    const int segs = (nx + kResX - 1) / kResX;
    const long long threads = (long long)ny * nz * segs;
    dim3 grid((unsigned)((threads + 255) / 256), nvol);
    FDM_TIMED("residual_ff", st);
    k_residual<<<grid, 256, 0, st>>>(fr, W, nx, ny, nz, vol, segs, FastDiv((unsigned)segs), FastDiv((unsigned)ny));
    FDM_LAUNCH_CHECK();
}

// Block / separator factors of the partitioned z-solve for every
// (x-mode, y-mode), computed in FP64 and stored in T (layout: k_zsolve_tab).
// Returns false when the line length does not split (the kernel without a
// table is used then).
template <typename T>
static bool zsolve_table_host(DevBuf& buf, int nx, int ny, int nz, const std::vector<double>& lamx,
                              const std::vector<double>& lamy, double h2, int* m_out, int* P_out) {
    const int m = nz < 15 ? nz : 15;
    const int P = (nz + 1) / (m + 1);
    if ((m + 1) * P != nz + 1 || P > 16) return false;
    const int modes = nx * ny;
    const int nv = 2 * m + 2 * (P - 1);
    std::vector<T> t((size_t)nv * modes);
    std::vector<double> cp(m), be(m);
    for (int k = 0; k < ny; k++)
        for (int j = 0; j < nx; j++) {
            const int mode = k * nx + j;
            const double b = -2.0 - (lamx[j] + lamy[k]) * h2;
            double c = 0.0;
            for (int i = 0; i < m; i++) {
                c = 1.0 / (b - c);
                cp[i] = c;
            }
            be[m - 1] = -cp[m - 1];
            for (int i = m - 2; i >= 0; i--) be[i] = -cp[i] * be[i + 1];
            for (int i = 0; i < m; i++) {
                t[(size_t)i * modes + mode] = (T)cp[i];
                t[(size_t)(m + i) * modes + mode] = (T)be[i];
            }
            const double lo = be[0], dg = b + 2.0 * be[m - 1];
            double pc = 0.0;
            for (int q = 0; q < P - 1; q++) {
                const double r = 1.0 / (dg - lo * pc);
                pc = lo * r;
                t[(size_t)(2 * m + q) * modes + mode] = (T)r;
                t[(size_t)(2 * m + P - 1 + q) * modes + mode] = (T)pc;
            }
        }
    FDM_CUDA(cudaMemcpy(buf.get(t.size() * sizeof(T)), t.data(), t.size() * sizeof(T), cudaMemcpyHostToDevice));
    *m_out = m;
    *P_out = P;
    return true;
}

template <typename T>
static void zsolve_tab_launch(T* W, int nx, int ny, int nz, int nvol, const T* tab, int m, int P, double gscale,
                              cudaStream_t st) {
    const size_t smem = (size_t)6 * P * 32 * sizeof(T);
    dim3 grid((unsigned)(ny * ((nx + 31) / 32)), nvol);
    const long long vs = (long long)nx * ny * nz;
    FDM_TIMED(sizeof(T) == 8 ? "zsolve_f64" : "zsolve_f32", st);
    switch (m) {
        case 1: k_zsolve_tab<T, 1><<<grid, 32 * P, smem, st>>>(W, nx, ny, P, vs, tab, (T)gscale); break;
        case 3: k_zsolve_tab<T, 3><<<grid, 32 * P, smem, st>>>(W, nx, ny, P, vs, tab, (T)gscale); break;
        case 7: k_zsolve_tab<T, 7><<<grid, 32 * P, smem, st>>>(W, nx, ny, P, vs, tab, (T)gscale); break;
        default:
            // FP32 blocks of 15 rows at 3 CTAs of 512 threads per SM (40
            // registers, 24 bytes spilled): 1.27 -> 1.13 ms per 16 x 255^3
            // step of its two launches
            if constexpr (sizeof(T) == 4)
                k_zsolve_tab<T, 15, 3><<<grid, 32 * P, smem, st>>>(W, nx, ny, P, vs, tab, (T)gscale);
            else
                k_zsolve_tab<T, 15><<<grid, 32 * P, smem, st>>>(W, nx, ny, P, vs, tab, (T)gscale);
            break;
    }
    FDM_LAUNCH_CHECK();
}

// Fused plane pass (k_plane_xz): rows per CTA and cluster size for an
// x-line of N points and nz rows; false when the plane does not split into
// 1, 2, 4 or 8 CTAs of whole z blocks.
static bool plane_split(int N, int nz, int* C) {
    int L = 0;
    switch (N) {
        case 64: L = PlaneCfg<64>::L; break;
        case 128: L = PlaneCfg<128>::L; break;
        case 256: L = PlaneCfg<256>::L; break;
        default: return false;
    }
    if ((nz + 1) % L != 0 || nz + 1 > 256) return false;  // at most 16 z blocks of 16 rows
    const int c = (nz + 1) / L;
    if (c != 1 && c != 2 && c != 4 && c != 8) return false;
    *C = c;
    return true;
}

template <int N, int C>
static void launch_plane_n(float* W, const PlaneGeom& g, int nvol, const SineTables<float>& tb, float gs, float sci,
                           const float* tab, cudaStream_t st) {
  if constexpr (PlaneCfg<N>::B * C > 16) {
    FDM_FAIL(FDMGPU_ESIZE, "plane pass: more than 16 z blocks");
  } else {
    // 4 CTAs of 256 threads per SM (64 registers) fit next to their shared
    // memory (47 KB at N = 256)
    const auto kern = k_plane_xz<N, C, 4>;
    constexpr size_t smem = PlaneCfg<N>::smem();
    static PerDevice<bool> attr_set;
    attr_set.get([kern] {
        FDM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        return true;
    });
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(C * g.ny), (unsigned)nvol, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    FDM_TIMED("plane_xz_f32", st);
    FDM_CUDA(cudaLaunchKernelEx(&cfg, kern, W, g, tb, gs, sci, tab));
  }
}

template <int N>
static void launch_plane_c(int C, float* W, const PlaneGeom& g, int nvol, const SineTables<float>& tb, float gs,
                           float sci, const float* tab, cudaStream_t st) {
    switch (C) {
        case 1: return launch_plane_n<N, 1>(W, g, nvol, tb, gs, sci, tab, st);
        case 2: return launch_plane_n<N, 2>(W, g, nvol, tb, gs, sci, tab, st);
        case 4: return launch_plane_n<N, 4>(W, g, nvol, tb, gs, sci, tab, st);
        case 8: return launch_plane_n<N, 8>(W, g, nvol, tb, gs, sci, tab, st);
        default: FDM_FAIL(FDMGPU_ESIZE, "plane pass: cluster of %d CTAs", C);
    }
}

// Forward DST along x, z solve and inverse DST along x of every y-mode plane
// of nvol FP32 volumes in place (scales: fwd along x times gscale of the z
// right-hand side, inv along x).
static void launch_plane(float* W, int nx, int ny, int nz, int nvol, const SineTables<float>& tb, double fwd,
                         double gscale, double inv, const float* tab, cudaStream_t st) {
    int C = 0;
    if (!plane_split(nx + 1, nz, &C)) FDM_FAIL(FDMGPU_ESIZE, "plane pass: unsupported %dx%d", nx, nz);
    PlaneGeom g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.vstride = (long long)nx * ny * nz;
    g.modes = nx * ny;
    const float gs = (float)(fwd * gscale), sci = (float)inv;
    switch (nx + 1) {
        case 64: return launch_plane_c<64>(C, W, g, nvol, tb, gs, sci, tab, st);
        case 128: return launch_plane_c<128>(C, W, g, nvol, tb, gs, sci, tab, st);
        case 256: return launch_plane_c<256>(C, W, g, nvol, tb, gs, sci, tab, st);
        default: FDM_FAIL(FDMGPU_ESIZE, "plane pass: x line of %d points", nx + 1);
    }
}

static std::vector<double> lambda_host(int n, double h) {
    std::vector<double> v(n);
    for (int j = 1; j <= n; j++) {
        const double s = std::sin(j * M_PI * 0.5 / (n + 1));
        v[j - 1] = 4. / (h * h) * (s * s);
    }
    return v;
}

// Conditioning limit of the mixed-precision solve.  kappa = (sum over the
// axes of the largest eigenvalue) / (sum of the smallest) of the discrete
// operator.  Measured on GB300 with one refinement sweep at tol 1e-10:
// 255^3 (kappa 2.7e4) reaches 2e-12 on smooth and 1.6e-11 on white-noise
// data; axes of 1023 points (kappa 1.5e5 to 4.2e5) stall between 1e-10 and
// 1e-7 however many sweeps run, because the second differences cancel more
// digits (1/h^2 ~ 1e6) than the float-float residual carries and the FP32
// tridiagonal z-solve of 1023 rows loses more than the refinement recovers.
// Plans above the limit run the FP64 solver instead.
constexpr double kMixedKappaMax = 3.0e4;

static double lapl_kappa(int nx, int ny, int nz, double hx, double hy, double hz) {
    auto lam = [](int n, double h, int j) {
        const double s = std::sin(j * M_PI * 0.5 / (n + 1));
        return 4. / (h * h) * (s * s);
    };
    const double hi = lam(nx, hx, nx) + lam(ny, hy, ny) + lam(nz, hz, nz);
    const double lo = lam(nx, hx, 1) + lam(ny, hy, 1) + lam(nz, hz, 1);
    return hi / lo;
}

static void check_grid_y(int nrhs) {
    if (nrhs < 1 || nrhs > 65535) FDM_FAIL(FDMGPU_EINVAL, "nrhs must be in [1, 65535], got %d", nrhs);
}

static bool pow2_interior(int n) { return n >= 1 && n <= FDMGPU_MAX_N && ilog2_exact(n + 1) > 0; }
static bool pow2_periodic(int n) { return n >= 2 && n <= 512 && ilog2_exact(n) > 0; }

// ---------------------------------------------------------------------------
// LaplCube
// ---------------------------------------------------------------------------
struct CubePlan {
    int dtype, nx, ny, nz;
    double dx, dy, dz, lx, ly, lz;
    int precision = FDMGPU_PLAIN;
    double tol = 1e-10;
    int max_sweeps = 3;
    double scx, scy, slx, sly;  // forward / inverse DST scales
    double hx_eff, hz_eff;      // spacings whose eigenvalues the reference uses
    double zfac, S;
    AxisTables<double> tx64, ty64;
    AxisTables<float> tx32, ty32;
    DevBuf lamx64, lamy64, lamx32, lamy32;
    DevBuf work32, uhi, ulo, norms, work64;
    DevBuf ztab64, ztab32;  // partitioned z-solve factors per mode
    int zmode = 1;          // 1: table-driven z-solve when the line splits, 0: factors computed per solve
    int dst_tc = -1;        // bit 0 / bit 1: plain FP32 DST passes along x / y on the tensor cores (32-, 64-,
                            // 128-point axes); -1: default_tc_mask()
    int pipeline = 1;       // mixed form: 1 = DST-y, fused x-z plane pass, DST-y where the plane splits
                            // (plane_split); 0 = the five passes x, y, z, y, x
    bool periodic = false;  // all three axes periodic (real FFTs, divide, inverse FFTs)
    bool mixed_ok = true;   // within the mixed solve's conditioning limit (kMixedKappaMax)
    DevBuf ptw_x, ptw_y, ptw_z, plam_x, plam_y, plam_z;
    DevBuf tc_img_x, tc_img_y, tc_err;
    int zm64 = 0, zP64 = 0, zm32 = 0, zP32 = 0;
    DevBuf hin, hout;
    int last_sweeps = 0, last_nrhs = 0;
    cudaStream_t last_stream = 0;
    // host-batch pipeline: copy-in, compute and copy-out streams, a ring of
    // device slots and the events that order their reuse
    static constexpr int kRing = 3;
    cudaStream_t pst[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev_in[kRing] = {}, ev_comp[kRing] = {}, ev_out[kRing] = {};
    DevBuf ring_in, ring_out;

    ~CubePlan() {
        for (int i = 0; i < kRing; i++) {
            if (ev_in[i]) cudaEventDestroy(ev_in[i]);
            if (ev_comp[i]) cudaEventDestroy(ev_comp[i]);
            if (ev_out[i]) cudaEventDestroy(ev_out[i]);
        }
        for (auto& q : pst)
            if (q) cudaStreamDestroy(q);
    }

    // nrhs host volumes: chunk i is copied in on stream 0 while chunk i-1 is
    // solved on stream 1 and chunk i-2 is copied out on stream 2.
    void solve_host_pipelined(void* ans, const void* rhs, int nrhs) {
        if (!pst[0]) {
            for (auto& q : pst) FDM_CUDA(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
            for (int i = 0; i < kRing; i++) {
                FDM_CUDA(cudaEventCreateWithFlags(&ev_in[i], cudaEventDisableTiming));
                FDM_CUDA(cudaEventCreateWithFlags(&ev_comp[i], cudaEventDisableTiming));
                FDM_CUDA(cudaEventCreateWithFlags(&ev_out[i], cudaEventDisableTiming));
            }
        }
        const size_t eb = dtype == FDMGPU_F64 ? sizeof(double) : sizeof(float);
        const size_t vb = (size_t)vol() * eb;
        char* din = (char*)ring_in.get(vb * kRing);
        char* dout = (char*)ring_out.get(vb * kRing);
        // the slots may still be in use by a previous call on these streams
        for (auto& q : pst) FDM_CUDA(cudaStreamSynchronize(q));
        bool used[kRing] = {false, false, false};
        for (int i = 0; i < nrhs; i++) {
            const int s = i % kRing;
            char* si = din + s * vb;
            char* so = dout + s * vb;
            if (used[s]) FDM_CUDA(cudaStreamWaitEvent(pst[0], ev_comp[s], 0));
            FDM_CUDA(cudaMemcpyAsync(si, (const char*)rhs + (size_t)i * vb, vb, cudaMemcpyHostToDevice, pst[0]));
            FDM_CUDA(cudaEventRecord(ev_in[s], pst[0]));
            FDM_CUDA(cudaStreamWaitEvent(pst[1], ev_in[s], 0));
            if (used[s]) FDM_CUDA(cudaStreamWaitEvent(pst[1], ev_out[s], 0));
            solve_device(so, si, 1, pst[1]);
            FDM_CUDA(cudaEventRecord(ev_comp[s], pst[1]));
            FDM_CUDA(cudaStreamWaitEvent(pst[2], ev_comp[s], 0));
            FDM_CUDA(cudaMemcpyAsync((char*)ans + (size_t)i * vb, so, vb, cudaMemcpyDeviceToHost, pst[2]));
            FDM_CUDA(cudaEventRecord(ev_out[s], pst[2]));
            used[s] = true;
        }
        FDM_CUDA(cudaStreamSynchronize(pst[2]));
        FDM_CUDA(cudaStreamSynchronize(pst[1]));
        last_stream = pst[1];
        last_nrhs = 1;
    }

    // periodic plan (LaplCube<T,check,periodic^3>, src/lapl_cube.h:58-100):
    // the reference shares lm_y with x (resp. z) when the point counts match
    void init_periodic() {
        slx = std::sqrt(2. / lx);
        sly = std::sqrt(2. / ly);
        if (dtype == FDMGPU_F64) {
            upload_ptwiddles<double>(ptw_x, nx);
            upload_ptwiddles<double>(ptw_y, ny);
            upload_ptwiddles<double>(ptw_z, nz);
            upload_plambda<double>(plam_y, ny, dy);
            upload_plambda<double>(plam_x, nx, nx == ny ? dy : dx);
            upload_plambda<double>(plam_z, nz, nz == ny ? dy : dz);
        } else {
            upload_ptwiddles<float>(ptw_x, nx);
            upload_ptwiddles<float>(ptw_y, ny);
            upload_ptwiddles<float>(ptw_z, nz);
            upload_plambda<float>(plam_y, ny, dy);
            upload_plambda<float>(plam_x, nx, nx == ny ? dy : dx);
            upload_plambda<float>(plam_z, nz, nz == ny ? dy : dz);
        }
    }

    // forward transforms z, y, x (scale h*sqrt(2/l)), divide, inverse x, y,
    // z (scale sqrt(2/l)), as src/lapl_cube.cpp:9-142 orders them
    template <typename T>
    void run_periodic(T* ans, const T* rhs, int nrhs, cudaStream_t st) {
        const double slz = std::sqrt(2. / lz);
        const long long v = vol();
        PLineGeom gx{(long long)nrhs * nz * ny, 1, nx, 0, 1};
        PLineGeom gy{(long long)nrhs * nz * nx, nx, (long long)nx * ny, 1, nx};
        PLineGeom gz{(long long)nrhs * nx * ny, (long long)nx * ny, v, 1, (long long)nx * ny};
        launch_pfft<T, false>(rhs, ans, gz, nz, ptw_z.p, dz * slz, st);
        launch_pfft<T, false>(ans, ans, gy, ny, ptw_y.p, dy * sly, st);
        launch_pfft<T, false>(ans, ans, gx, nx, ptw_x.p, dx * slx, st);
        {
            const long long total = v * nrhs;
            FDM_TIMED("pdivide", st);
            k_pdivide<T><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(ans, nx, ny, nz, total, (const T*)plam_x.p,
                                                                           (const T*)plam_y.p, (const T*)plam_z.p);
            FDM_LAUNCH_CHECK();
        }
        launch_pfft<T, true>(ans, ans, gx, nx, ptw_x.p, slx, st);
        launch_pfft<T, true>(ans, ans, gy, ny, ptw_y.p, sly, st);
        launch_pfft<T, true>(ans, ans, gz, nz, ptw_z.p, slz, st);
    }

    void init() {
        if (periodic) {
            init_periodic();
            return;
        }
        slx = std::sqrt(2. / lx);
        sly = std::sqrt(2. / ly);
        const double slz = std::sqrt(2. / lz);
        scx = dx * slx;
        scy = dy * sly;
        // The reference shares lm_y with x (resp. z) when the point counts
        // match, whatever the spacing (src/lapl_cube.cpp:165, :171).
        hx_eff = (nx == ny) ? dy : dx;
        hz_eff = (nz == ny) ? dy : dz;
        zfac = dz * slz * slz * (nz + 1) / 2.0;
        S = (dx * slx * slx * (nx + 1) / 2.0) * (dy * sly * sly * (ny + 1) / 2.0) * zfac;
        kappa = lapl_kappa(nx, ny, nz, hx_eff, dy, hz_eff);
        mixed_ok = kappa <= kMixedKappaMax;
        if (dtype == FDMGPU_F64) {
            tx64.build(nx + 1);
            ty64.build(ny + 1);
            upload_lambda<double>(lamx64, nx, hx_eff);
            upload_lambda<double>(lamy64, ny, dy);
        } else {
            tx32.build(nx + 1);
            ty32.build(ny + 1);
            upload_lambda<float>(lamx32, nx, hx_eff);
            upload_lambda<float>(lamy32, ny, dy);
        }
    }

    void ensure_mixed_tables() {
        if (!tx32.N) {
            tx32.build(nx + 1);
            ty32.build(ny + 1);
            upload_lambda<float>(lamx32, nx, hx_eff);
            upload_lambda<float>(lamy32, ny, dy);
        }
    }

    long long vol() const { return (long long)nx * ny * nz; }

    // plain FP32 DST pass along AXIS, on the tensor cores when enabled for
    // the axis and it has 32, 64 or 128 points
    template <int AXIS>
    void sine32(const float* in, float* out, int nrhs, double scale, cudaStream_t st) {
        const int N = (AXIS == 0 ? nx : ny) + 1;
        if (((tc_mask() >> AXIS) & 1) && tc_supported(N)) {
            DevBuf& img = AXIS == 0 ? tc_img_x : tc_img_y;
            if (!img.p) {
                std::vector<float> h = tc_sine_image(N);
                img.get(h.size() * sizeof(float));
                FDM_CUDA(cudaMemcpy(img.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
            }
            if (!tc_err.p) {
                tc_err.get(sizeof(int));
                FDM_CUDA(cudaMemset(tc_err.p, 0, sizeof(int)));
            }
            const long long lines = (long long)nrhs * nz * (AXIS == 0 ? ny : nx);
            launch_sine_tc<AXIS>(N, in, out, lines, nx, (const float*)img.p, scale, (int*)tc_err.p, st);
            return;
        }
        launch_sine<float, float, float, AXIS>(in, out, nx, ny, nz, nrhs, (AXIS == 0 ? tx32 : ty32).view(), scale, st);
    }

    template <typename Tin, typename T, int MODE = kPlain>
    void forward_xy(const Tin* in, T* W, int nrhs, const AxisTables<T>& tx, const AxisTables<T>& ty,
                    cudaStream_t st, const SineFused* fu = nullptr) {
        launch_sine<Tin, T, T, 0, MODE>(in, W, nx, ny, nz, nrhs, tx.view(), scx, st, fu);
        launch_sine<T, T, T, 1>(W, W, nx, ny, nz, nrhs, ty.view(), scy, st);
    }
    template <typename T>
    void zsolve(T* W, int nrhs, const DevBuf& lx_, const DevBuf& ly_, cudaStream_t st) {
        DevBuf& tab = sizeof(T) == 8 ? ztab64 : ztab32;
        int& zm = sizeof(T) == 8 ? zm64 : zm32;
        int& zP = sizeof(T) == 8 ? zP64 : zP32;
        if (!tab.p && zm == 0) {
            if (!zsolve_table_host<T>(tab, nx, ny, nz, lambda_host(nx, hx_eff), lambda_host(ny, dy), hz_eff * hz_eff,
                                      &zm, &zP))
                zm = -1;
        }
        if (zm > 0 && zmode == 1) {
            zsolve_tab_launch<T>(W, nx, ny, nz, nrhs, (const T*)tab.p, zm, zP, zfac * hz_eff * hz_eff, st);
            return;
        }
        zsolve_lines<T>(W, nx, ny, nz, nrhs, (const T*)lx_.p, (const T*)ly_.p, hz_eff * hz_eff,
                        zfac * hz_eff * hz_eff, st);
    }

    // the FP32 z factor table (built on first use); false when the z line
    // does not split into blocks
    bool ztab32_ready() {
        if (!ztab32.p && zm32 == 0) {
            if (!zsolve_table_host<float>(ztab32, nx, ny, nz, lambda_host(nx, hx_eff), lambda_host(ny, dy),
                                          hz_eff * hz_eff, &zm32, &zP32))
                zm32 = -1;
        }
        return zm32 > 0;
    }

    // whether the mixed solve runs the three-pass pipeline with the fused
    // x-z plane pass
    bool plane_ok() {
        int C = 0;
        return pipeline == 1 && zmode == 1 && !(tc_mask() & 1) && plane_split(nx + 1, nz, &C) && ztab32_ready() &&
               zm32 == 15;
    }

    // Tensor-core DST passes of a mixed plan whose schedule was not set:
    // 32-point x axes (they never take the plane pipeline, whose x lines
    // have 64 to 256 points) and 32-point y axes of plans that run the five
    // passes.  Measured on GB300 (mixed, tol 1e-10): 31^3 x 64 at 522 k
    // solves/s with both axes on the tensor cores against 449 k with FFTs,
    // and the batch tuner kept the x axis on the tensor cores for every
    // 31-point-x group of its 512-volume batch; with the plane pipeline the
    // y axis ties (63^3 x 16: 95.1 k against 95.0 k), so the FFT stays.
    int default_tc_mask() const {
        if (precision != FDMGPU_MIXED || dtype != FDMGPU_F64 || periodic) return 0;
        int m = nx + 1 == 32 ? 1 : 0;
        int C = 0;
        const bool planes = pipeline == 1 && zmode == 1 && !(m & 1) && plane_split(nx + 1, nz, &C);
        if (ny + 1 == 32 && !planes) m |= 2;
        return m;
    }
    int tc_mask() const { return dst_tc >= 0 ? dst_tc : default_tc_mask(); }

    // Times every schedule of the mixed form on the caller's right-hand
    // sides (pipeline, z-solve variant, tensor-core axes) and keeps the
    // fastest whose accuracy is assured: with a refinement sweep, a variant
    // with per-solve z factors or tensor-core passes must predict
    // 10 e^(sweeps+1) <= tol from its measured first-sweep estimate e (as the
    // batch tuner does); without a sweep (tol >= 1e-5, above the FP32 and
    // split-TF32 inner solves' errors) per-solve factors do not qualify.
    // Synchronises st.  Returns the chosen schedule's time per call in ms.
    double tune(void* ans, const void* rhs, int nrhs, cudaStream_t st) {
        if (precision != FDMGPU_MIXED || !mixed_ok || periodic) return 0.0;
        ensure_mixed_tables();
        const int tc_axes = (tc_supported(nx + 1) ? 1 : 0) | (tc_supported(ny + 1) ? 2 : 0);
        const int sweeps = sweeps_for_tol();
        cudaEvent_t a, b;
        FDM_CUDA(cudaEventCreate(&a));
        FDM_CUDA(cudaEventCreate(&b));
        double best = 1e30;
        const int p0 = pipeline, z0 = zmode, t0 = dst_tc;  // restored if a candidate fails
        int bp = pipeline, bz = zmode, bt = tc_mask();
        try {
            for (int pl = 1; pl >= 0; pl--)
                for (int zm = 1; zm >= 0; zm--)
                    for (int tc = 0; tc <= 3; tc++) {
                        if (tc & ~tc_axes) continue;
                        int C = 0;
                        // a plane schedule that cannot take planes is the five-pass one
                        if (pl == 1 && (zm == 0 || (tc & 1) || !plane_split(nx + 1, nz, &C))) continue;
                        if (zm == 0 && sweeps == 0) continue;
                        pipeline = pl;
                        zmode = zm;
                        dst_tc = tc;
                        solve_device(ans, rhs, nrhs, st);  // warm-up: tables and scratch of this schedule
                        FDM_CUDA(cudaEventRecord(a, st));
                        solve_device(ans, rhs, nrhs, st);
                        FDM_CUDA(cudaEventRecord(b, st));
                        FDM_CUDA(cudaEventSynchronize(b));
                        float ms = 0.f;
                        FDM_CUDA(cudaEventElapsedTime(&ms, a, b));
                        if ((zm == 0 || tc != 0) && sweeps > 0) {
                            const double e = first_sweep_est(nrhs, st);
                            if (10.0 * std::pow(e, sweeps + 1) > tol) continue;
                        }
                        if (ms < best) {
                            best = ms;
                            bp = pl;
                            bz = zm;
                            bt = tc;
                        }
                    }
        } catch (...) {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            pipeline = p0;
            zmode = z0;
            dst_tc = t0;
            throw;
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        pipeline = bp;
        zmode = bz;
        dst_tc = bt;
        return best;
    }

    void solve_device(void* ans, const void* rhs, int nrhs, cudaStream_t st) {
        check_grid_y(nrhs);
        last_est.clear();
        last_stream = st;
        last_nrhs = nrhs;
        if (periodic) {
            last_sweeps = 0;
            if (dtype == FDMGPU_F64) run_periodic<double>((double*)ans, (const double*)rhs, nrhs, st);
            else run_periodic<float>((float*)ans, (const float*)rhs, nrhs, st);
            return;
        }
        if (precision == FDMGPU_PLAIN || !mixed_ok) {
            // a mixed plan beyond the conditioning limit solves in FP64
            last_sweeps = precision == FDMGPU_PLAIN ? 0 : -1;
            if (dtype == FDMGPU_F64) run_plain<double>((double*)ans, (const double*)rhs, nrhs, tx64, ty64, lamx64,
                                                       lamy64, st);
            else run_plain<float>((float*)ans, (const float*)rhs, nrhs, tx32, ty32, lamx32, lamy32, st);
            return;
        }
        run_mixed((double*)ans, (const double*)rhs, nrhs, st);
    }

    template <typename T>
    void run_plain(T* ans, const T* rhs, int nrhs, const AxisTables<T>& tx, const AxisTables<T>& ty,
                   const DevBuf& lx_, const DevBuf& ly_, cudaStream_t st) {
        forward_xy<T, T>(rhs, ans, nrhs, tx, ty, st);
        zsolve<T>(ans, nrhs, lx_, ly_, st);
        launch_sine<T, T, T, 1>(ans, ans, nx, ny, nz, nrhs, ty.view(), sly, st);
        launch_sine<T, T, T, 0>(ans, ans, nx, ny, nz, nrhs, tx.view(), slx, st);
    }

    int sweeps_for_tol() const {
        int s = tol >= 1e-5 ? 0 : (tol >= 1e-11 ? 1 : 2);
        return s < max_sweeps ? s : max_sweeps;
    }

    static ff split_host(double v) {
        const float h = (float)v;
        return ff{h, (float)(v - (double)h)};
    }

    // Model of the error left after a refinement sweep.  Sweep k measures
    // e_k = ||c_k|| / ||u||, the relative size of its correction, which is
    // the error of the solution before it.  The error after it is the larger
    // of rho e_k, rho the contraction of a sweep, and the floor the
    // float-float residual allows, kFloorPerKappa times the operator's
    // eigenvalue ratio kappa.  From two sweeps rho = e_k / e_{k-1}; after the
    // first, rho = kRhoPerErr e_1 (an FP32 inner solve that leaves a relative
    // error e on u leaves a multiple of e on the rougher correction).
    // Measured on GB300 over 16 cases (31^3 to 255^3, anisotropic spacings,
    // smooth and white-noise data; relative L2 against the FP64 form): error
    // after one sweep / e_1^2 between 2.5 and 44.  Error after two sweeps /
    // kappa: 1.1e-17 to 6.7e-17 on those cases, but up to 2.0e-16 over 44
    // more (elongated boxes such as 31 x 255 x 31 and 255 x 31 x 31, with FFT
    // and with tensor-core DST passes).  The constants keep a margin of 2.3
    // and 1.5 over the largest.
    static constexpr double kRhoPerErr = 100.0;
    static constexpr double kFloorPerKappa = 3e-16;
    double kappa = 0.0;  // largest over smallest eigenvalue, summed over the axes
    double est_after(double ek, double ekm1, int k) const {
        if (ek <= 0.0) return kFloorPerKappa * kappa;
        const double rho = k >= 2 && ekm1 > 0.0 ? std::min(1.0, ek / ekm1) : std::min(1.0, kRhoPerErr * ek);
        return std::max(rho * ek, kFloorPerKappa * kappa);
    }
    // estimates of the nrhs right-hand sides from their norms after `sweeps`
    // sweeps (host copy of the norms buffer, layout [sweep][rhs][c2, u2])
    void estimates_from_norms(const double* v, int nrhs, int sweeps, double* est) const {
        for (int i = 0; i < nrhs; i++) {
            if (sweeps <= 0) {
                est[i] = -1.0;
                continue;
            }
            auto e = [&](int k) {  // e_k, k = 1..sweeps
                const double c2 = v[(size_t)2 * nrhs * (k - 1) + 2 * i], u2 = v[(size_t)2 * nrhs * (k - 1) + 2 * i + 1];
                return u2 > 0 ? std::sqrt(c2 / u2) : 0.0;
            };
            est[i] = est_after(e(sweeps), sweeps >= 2 ? e(sweeps - 1) : 0.0, sweeps);
        }
    }
    int refine_adaptive = 0;       // 1: extra sweeps while an estimate exceeds tol (synchronises)
    int rule_vols = 0;             // > 0: line transforms choose their CTA size as for this many volumes
    std::vector<double> last_est;  // per RHS, filled by an adaptive solve

    // final estimates of the last solve (synchronises st)
    std::vector<double> final_estimates(int nrhs, int sweeps, cudaStream_t st) const {
        std::vector<double> out(nrhs, -1.0);
        if (sweeps <= 0 || !norms.p) return out;
        std::vector<double> v((size_t)2 * nrhs * sweeps);
        FDM_CUDA(cudaStreamSynchronize(st));
        FDM_CUDA(cudaMemcpy(v.data(), norms.p, v.size() * sizeof(double), cudaMemcpyDeviceToHost));
        estimates_from_norms(v.data(), nrhs, sweeps, out.data());
        return out;
    }

    // The passes of one mixed pipeline: `first` takes the FP64 right-hand
    // sides to the FP32 work volume one pass short of the solution, `last`
    // applies that final pass (T_out = the FP64 output or UH), `inner` takes
    // the residual in W to the correction one pass short, `combine` applies
    // the final pass and adds the correction.
    template <typename First, typename Last, typename Inner, typename Combine>
    void sweep_loop(double* ans, const double* rhs, int nrhs, cudaStream_t st, const void* const* vin,
                    void* const* vout, First first, Last last, Inner inner, Combine combine) {
        const long long V = vol() * nrhs;
        const int sweeps = sweeps_for_tol();
        last_sweeps = sweeps;
        last_est.clear();
        float* W = (float*)work32.get(V * sizeof(float));
        first(W);
        if (sweeps == 0) {
            SineFused fo;
            memset(&fo, 0, sizeof(fo));
            fo.vout = vout;
            last(W, (double*)ans, (float*)nullptr, fo);
            return;
        }
        const bool adaptive = refine_adaptive && max_sweeps > sweeps;
        const int cap = adaptive ? max_sweeps : sweeps;
        float* UH = (float*)uhi.get(V * sizeof(float));
        float* UL = (sweeps > 1 || adaptive) ? (float*)ulo.get(V * sizeof(float)) : nullptr;
        double* NR = (double*)norms.get((size_t)2 * nrhs * cap * sizeof(double));
        FDM_CUDA(cudaMemsetAsync(NR, 0, (size_t)2 * nrhs * cap * sizeof(double), st));
        {
            SineFused fo;
            memset(&fo, 0, sizeof(fo));
            last(W, (double*)nullptr, UH, fo);
        }
        // r = f - A u / S: the inner solve multiplies by S again, so it
        // returns the correction S A^-1 f - u
        const double cx = 1.0 / (hx_eff * hx_eff) / S, cy = 1.0 / (dy * dy) / S, cz = 1.0 / (hz_eff * hz_eff) / S;
        auto sweep = [&](int s, bool is_last, bool keep) {
            SineFused fr;
            memset(&fr, 0, sizeof(fr));
            fr.f = rhs;
            fr.vin = vin;
            fr.uhi = UH;
            fr.ulo = s >= 2 ? UL : nullptr;
            fr.cx = split_host(cx); fr.cy = split_host(cy); fr.cz = split_host(cz);
            fr.cxf = (float)cx; fr.cyf = (float)cy; fr.czf = (float)cz;
            fr.iso = (cx == cy && cy == cz) ? 1 : 0;
            launch_residual(fr, W, nx, ny, nz, nrhs, st);
            inner(W);
            SineFused fc;
            memset(&fc, 0, sizeof(fc));
            fc.uhi = UH;
            fc.ulo = s >= 2 ? UL : nullptr;
            fc.out64 = ans;
            fc.vout = vout;
            fc.ulo_out = (!is_last || keep) ? UL : nullptr;
            fc.last = is_last ? 1 : 0;
            fc.norms = NR + (size_t)2 * nrhs * (s - 1);
            combine(W, fc);
        };
        for (int s = 1; s <= sweeps; s++) sweep(s, s == sweeps, adaptive);
        if (!adaptive) return;
        // closed loop: more sweeps while a right-hand side's estimated
        // remaining error exceeds tol
        int done = sweeps;
        for (;;) {
            last_est = final_estimates(nrhs, done, st);
            const double worst = *std::max_element(last_est.begin(), last_est.end());
            if (worst <= tol || done >= cap) break;
            done++;
            sweep(done, true, done < cap);
            last_sweeps = done;
        }
    }

    // Mixed solve of nrhs volumes.  With vin / vout (device arrays of nrhs
    // user pointers) the FP64 input and output volumes are addressed through
    // them and rhs / ans are not used; the FP32 scratch stays contiguous.
    // With the fused plane pass: DST-y, the x-z plane pass, inverse DST-y
    // (the x and y transforms commute, so it is the same operator as the x,
    // y, z, y, x order of the five-pass form).
    void run_mixed(double* ans, const double* rhs, int nrhs, cudaStream_t st, const void* const* vin = nullptr,
                   void* const* vout = nullptr) {
        ensure_mixed_tables();
        if (plane_ok()) {
            const float* tab = (const float*)ztab32.p;
            const double gscale = zfac * hz_eff * hz_eff;
            sweep_loop(
                ans, rhs, nrhs, st, vin, vout,
                [&](float* W) {
                    SineFused fin;
                    memset(&fin, 0, sizeof(fin));
                    fin.vin = vin;
                    launch_sine<double, float, float, 1, kRound>(rhs, W, nx, ny, nz, nrhs, ty32.view(), scy, st, &fin);
                    launch_plane(W, nx, ny, nz, nrhs, tx32.view(), scx, gscale, slx, tab, st);
                },
                [&](float* W, double* o64, float* o32, const SineFused& fo) {
                    if (o64) launch_sine<float, float, double, 1>(W, o64, nx, ny, nz, nrhs, ty32.view(), sly, st, &fo);
                    else launch_sine<float, float, float, 1>(W, o32, nx, ny, nz, nrhs, ty32.view(), sly, st);
                },
                [&](float* W) {
                    launch_sine<float, float, float, 1>(W, W, nx, ny, nz, nrhs, ty32.view(), scy, st);
                    launch_plane(W, nx, ny, nz, nrhs, tx32.view(), scx, gscale, slx, tab, st);
                },
                [&](float* W, const SineFused& fc) {
                    launch_sine<float, float, float, 1, kCombine>(W, (float*)nullptr, nx, ny, nz, nrhs, ty32.view(),
                                                                  sly, st, &fc);
                });
            return;
        }
        sweep_loop(
            ans, rhs, nrhs, st, vin, vout,
            [&](float* W) {
                SineFused fin;
                memset(&fin, 0, sizeof(fin));
                fin.vin = vin;
                launch_sine<double, float, float, 0, kRound>(rhs, W, nx, ny, nz, nrhs, tx32.view(), scx, st, &fin);
                sine32<1>(W, W, nrhs, scy, st);
                zsolve<float>(W, nrhs, lamx32, lamy32, st);
                sine32<1>(W, W, nrhs, sly, st);
            },
            [&](float* W, double* o64, float* o32, const SineFused& fo) {
                if (o64) launch_sine<float, float, double, 0>(W, o64, nx, ny, nz, nrhs, tx32.view(), slx, st, &fo);
                else sine32<0>(W, o32, nrhs, slx, st);
            },
            [&](float* W) {
                sine32<0>(W, W, nrhs, scx, st);
                sine32<1>(W, W, nrhs, scy, st);
                zsolve<float>(W, nrhs, lamx32, lamy32, st);
                sine32<1>(W, W, nrhs, sly, st);
            },
            [&](float* W, const SineFused& fc) {
                launch_sine<float, float, float, 0, kCombine>(W, (float*)nullptr, nx, ny, nz, nrhs, tx32.view(), slx,
                                                              st, &fc);
            });
    }

    // Plain FP64 solve through pointer tables: first pass from the user
    // volumes into contiguous FP64 scratch, last pass back out.
    void run_plain_ptrs(const void* const* vin, void* const* vout, int nrhs, cudaStream_t st, double* Wext = nullptr) {
        const long long V = vol() * nrhs;
        double* W = Wext ? Wext : (double*)work64.get(V * sizeof(double));
        const int rv = rule_vols;
        SineFused fin;
        memset(&fin, 0, sizeof(fin));
        fin.vin = vin;
        launch_sine<double, double, double, 0>(nullptr, W, nx, ny, nz, nrhs, tx64.view(), scx, st, &fin, rv);
        launch_sine<double, double, double, 1>(W, W, nx, ny, nz, nrhs, ty64.view(), scy, st, nullptr, rv);
        zsolve<double>(W, nrhs, lamx64, lamy64, st);
        launch_sine<double, double, double, 1>(W, W, nx, ny, nz, nrhs, ty64.view(), sly, st, nullptr, rv);
        SineFused fo;
        memset(&fo, 0, sizeof(fo));
        fo.vout = vout;
        launch_sine<double, double, double, 0>(W, nullptr, nx, ny, nz, nrhs, tx64.view(), slx, st, &fo, rv);
    }

    // Largest first-sweep correction estimate ||c||/||u|| over the nrhs
    // volumes of the last mixed solve on st (synchronises st): the relative
    // error of the FP32 inner solve.  0 when the last solve ran no sweep.
    double first_sweep_est(int nrhs, cudaStream_t st) {
        if (last_sweeps <= 0 || !norms.p) return 0.0;
        FDM_CUDA(cudaStreamSynchronize(st));
        std::vector<double> v((size_t)2 * nrhs);
        FDM_CUDA(cudaMemcpy(v.data(), norms.p, v.size() * sizeof(double), cudaMemcpyDeviceToHost));
        double e = 0.0;
        for (int i = 0; i < nrhs; i++)
            if (v[2 * i + 1] > 0) e = std::max(e, std::sqrt(v[2 * i] / v[2 * i + 1]));
        return e;
    }

    size_t scratch_bytes() const {
        return work32.bytes + work64.bytes + uhi.bytes + ulo.bytes + norms.bytes + hin.bytes + hout.bytes + ztab32.bytes +
               ztab64.bytes + ring_in.bytes + ring_out.bytes;
    }
};

// ---------------------------------------------------------------------------
// LaplRect / LaplRectFFT2
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_divide2d(T* W, int nx, int ny, long long vstride, const T* lamx, const T* lamy, int hack) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)nx * ny) return;
    const int j = idx % nx, k = idx / nx;
    T* p = W + (long long)blockIdx.y * vstride + idx;
    // doubly periodic: the reference sets the (0, 0) mode to 1
    // ("hack for double-period", src/lapl_rect.cpp:169-172)
    *p = (hack && idx == 0) ? T(1) : *p / (-lamy[k] * T(1) - lamx[j]);
}

struct RectPlan {
    int dtype, method, nx, ny;
    // bit 1: y periodic (the reference's F::head), bit 0: x periodic
    // (F::tail::head; LaplRectFFT2 only: LaplRect's tridiagonal x ignores it)
    int flags = 0;
    double dx, dy, lx, ly;
    AxisTables<double> tx64, ty64;
    AxisTables<float> tx32, ty32;
    DevBuf lamx64, lamy64, lamx32, lamy32;
    DevBuf ptw_x, ptw_y;  // periodic transforms' twiddles
    DevBuf hin, hout;

    bool py() const { return (flags & 2) != 0; }
    bool px() const { return (flags & 1) != 0 && method == FDMGPU_RECT_FFT2; }

    template <typename T>
    void init_t(AxisTables<T>& tx, AxisTables<T>& ty, DevBuf& lamx, DevBuf& lamy) {
        if (py()) {
            upload_ptwiddles<T>(ptw_y, ny);
            upload_plambda<T>(lamy, ny, dy);  // lm_y = 4/dy^2 sin^2(k pi/ny), src/lapl_rect.cpp:16
        } else {
            ty.build(ny + 1);
            upload_lambda<T>(lamy, ny, dy);
        }
        if (method != FDMGPU_RECT_FFT2) return;
        if (px()) {
            upload_ptwiddles<T>(ptw_x, nx);
            upload_plambda<T>(lamx, nx, dx);  // src/lapl_rect.cpp:30
        } else {
            tx.build(nx + 1);
            // lm_y stands in for lm_x only without periodic flags (src/lapl_rect.cpp:35-40)
            upload_lambda<T>(lamx, nx, (flags == 0 && nx == ny) ? dy : dx);
        }
    }

    void init() {
        if (dtype == FDMGPU_F64) init_t<double>(tx64, ty64, lamx64, lamy64);
        else init_t<float>(tx32, ty32, lamx32, lamy32);
    }

    template <typename T>
    void run(T* ans, const T* rhs, int nrhs, const AxisTables<T>& tx, const AxisTables<T>& ty, const DevBuf& lamx,
             const DevBuf& lamy, cudaStream_t st) {
        const double sly = std::sqrt(2. / ly), slx = std::sqrt(2. / lx);
        const long long vs = (long long)nx * ny;
        // periodic lines: along y, line L = (volume, column) starts at
        // (L / nx) * vs + L % nx with stride nx; along x, rows of nx
        const PLineGeom gy{(long long)nrhs * nx, nx, vs, 1, nx};
        const PLineGeom gx{(long long)nrhs * ny, 1, nx, 0, 1};
        if (py()) launch_pfft<T, false>(rhs, ans, gy, ny, ptw_y.p, dy * sly, st);
        else launch_sine<T, T, T, 1>(rhs, ans, nx, ny, 1, nrhs, ty.view(), dy * sly, st);
        if (method == FDMGPU_RECT_TRIDIAG) {
            // per y-mode k: (u[j-1] - 2u[j] + u[j+1])/dx^2 - lm_y[k] u[j] = g[j]
            launch_tridiag<T>(ans, ny, nx, 1, 0, nx, 1, vs, nrhs, nullptr, (const T*)lamy.p, dx * dx, dx * dx, st);
        } else {
            if (px()) launch_pfft<T, false>(ans, ans, gx, nx, ptw_x.p, dx * slx, st);
            else launch_sine<T, T, T, 0>(ans, ans, nx, ny, 1, nrhs, tx.view(), dx * slx, st);
            {
                dim3 grid((unsigned)((vs + 255) / 256), nrhs);
                FDM_TIMED("divide2d", st);
                k_divide2d<T><<<grid, 256, 0, st>>>(ans, nx, ny, vs, (const T*)lamx.p, (const T*)lamy.p,
                                                    (px() && py()) ? 1 : 0);
                FDM_LAUNCH_CHECK();
            }
            if (px()) launch_pfft<T, true>(ans, ans, gx, nx, ptw_x.p, slx, st);
            else launch_sine<T, T, T, 0>(ans, ans, nx, ny, 1, nrhs, tx.view(), slx, st);
        }
        if (py()) launch_pfft<T, true>(ans, ans, gy, ny, ptw_y.p, sly, st);
        else launch_sine<T, T, T, 1>(ans, ans, nx, ny, 1, nrhs, ty.view(), sly, st);
    }

    void solve_device(void* ans, const void* rhs, int nrhs, cudaStream_t st) {
        check_grid_y(nrhs);
        if (dtype == FDMGPU_F64) run<double>((double*)ans, (const double*)rhs, nrhs, tx64, ty64, lamx64, lamy64, st);
        else run<float>((float*)ans, (const float*)rhs, nrhs, tx32, ty32, lamx32, lamy32, st);
    }
};

}  // namespace fdmgpu

using namespace fdmgpu;

struct fdmgpu_lapl_cube {
    CubePlan plan;
};

namespace fdmgpu {

// ---------------------------------------------------------------------------
// Batched solves of uneven sizes
//
// Right-hand sides are grouped by geometry; each group owns a CubePlan (its
// tables and contiguous FP32 scratch) and reads / writes the user volumes
// through device arrays of pointers, so nothing is gathered or scattered.
// A group's schedule -- right-hand sides per pipeline launch (chunk) and the
// z-solve variant -- is picked by timing the candidates on the group's own
// data (tune).  The first solve after tuning captures every group's
// pipeline, each on its own stream forked from one origin stream, into a
// single CUDA graph; later solves are one graph launch.
// ---------------------------------------------------------------------------
struct BatchGroup {
    int nx, ny, nz;
    double g[6];
    std::vector<int> members;
    std::unique_ptr<CubePlan> plan;
    int chunk = 0;  // right-hand sides per pipeline launch (0: all)
    int zmode = 1;
    DevBuf ptr_in, ptr_out;  // device arrays of the members' user pointers
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    double tuned_ms = 0.0;
};

struct BatchPlan {
    int count = 0, precision = FDMGPU_MIXED;
    double tol = 1e-10;
    std::deque<BatchGroup> groups;  // never relocates its elements
    cudaStream_t origin = nullptr;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches_per_solve = 0;
    std::vector<const void*> in_host;
    std::vector<void*> out_host;

    ~BatchPlan() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto& gr : groups) {
            if (gr.done) cudaEventDestroy(gr.done);
            if (gr.st) cudaStreamDestroy(gr.st);
        }
        if (fork) cudaEventDestroy(fork);
        if (origin) cudaStreamDestroy(origin);
    }

    void init(const int* n3, const double* h3, const double* l3) {
        for (int i = 0; i < count; i++) {
            const int nx = n3[3 * i], ny = n3[3 * i + 1], nz = n3[3 * i + 2];
            int found = -1;
            for (size_t k = 0; k < groups.size(); k++) {
                const BatchGroup& gr = groups[k];
                if (gr.nx == nx && gr.ny == ny && gr.nz == nz && gr.g[0] == h3[3 * i] && gr.g[1] == h3[3 * i + 1] &&
                    gr.g[2] == h3[3 * i + 2] && gr.g[3] == l3[3 * i] && gr.g[4] == l3[3 * i + 1] &&
                    gr.g[5] == l3[3 * i + 2]) {
                    found = (int)k;
                    break;
                }
            }
            if (found < 0) {
                groups.emplace_back();
                BatchGroup& gr = groups.back();
                gr.nx = nx; gr.ny = ny; gr.nz = nz;
                for (int a = 0; a < 3; a++) {
                    gr.g[a] = h3[3 * i + a];
                    gr.g[3 + a] = l3[3 * i + a];
                }
                found = (int)groups.size() - 1;
            }
            groups[found].members.push_back(i);
        }
        FDM_CUDA(cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking));
        FDM_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        for (auto& gr : groups) {
            gr.plan.reset(new CubePlan());
            CubePlan& c = *gr.plan;
            c.dtype = FDMGPU_F64;
            c.nx = gr.nx; c.ny = gr.ny; c.nz = gr.nz;
            c.dx = gr.g[0]; c.dy = gr.g[1]; c.dz = gr.g[2];
            c.lx = gr.g[3]; c.ly = gr.g[4]; c.lz = gr.g[5];
            c.precision = precision;
            c.tol = tol;
            c.init();
            gr.chunk = (int)gr.members.size();
            gr.ptr_in.get(gr.members.size() * sizeof(void*));
            gr.ptr_out.get(gr.members.size() * sizeof(void*));
            FDM_CUDA(cudaStreamCreateWithFlags(&gr.st, cudaStreamNonBlocking));
            FDM_CUDA(cudaEventCreateWithFlags(&gr.done, cudaEventDisableTiming));
        }
    }

    // copies the members' user pointers into each group's device arrays
    void upload_pointers(void* const* ans, const void* const* rhs, cudaStream_t st) {
        if ((int)in_host.size() == count && std::equal(in_host.begin(), in_host.end(), rhs) &&
            std::equal(out_host.begin(), out_host.end(), ans))
            return;  // the device arrays already hold these pointers
        in_host.clear();
        out_host.clear();
        for (auto& gr : groups) {
            std::vector<const void*> pin(gr.members.size());
            std::vector<void*> pout(gr.members.size());
            for (size_t k = 0; k < gr.members.size(); k++) {
                pin[k] = rhs[gr.members[k]];
                pout[k] = ans[gr.members[k]];
                if (!pin[k] || !pout[k]) FDM_FAIL(FDMGPU_EINVAL, "null volume pointer for right-hand side %d", gr.members[k]);
            }
            FDM_CUDA(cudaMemcpyAsync(gr.ptr_in.p, pin.data(), pin.size() * sizeof(void*), cudaMemcpyHostToDevice, st));
            FDM_CUDA(cudaMemcpyAsync(gr.ptr_out.p, pout.data(), pout.size() * sizeof(void*), cudaMemcpyHostToDevice,
                                     st));
        }
        FDM_CUDA(cudaStreamSynchronize(st));  // host vectors go out of scope
        in_host.assign(rhs, rhs + count);
        out_host.assign(ans, ans + count);
    }

    // enqueues group gr's pipeline on stream st with its current schedule
    void enqueue_group(BatchGroup& gr, cudaStream_t st) {
        CubePlan& c = *gr.plan;
        c.zmode = gr.zmode;
        const int m = (int)gr.members.size();
        const int ch = gr.chunk > 0 ? gr.chunk : m;
        const void* const* vin = (const void* const*)gr.ptr_in.p;
        void* const* vout = (void* const*)gr.ptr_out.p;
        for (int s0 = 0; s0 < m; s0 += ch) {
            const int k = std::min(ch, m - s0);
            if (precision == FDMGPU_MIXED && c.mixed_ok) c.run_mixed(nullptr, nullptr, k, st, vin + s0, vout + s0);
            else c.run_plain_ptrs(vin + s0, vout + s0, k, st);
        }
    }

    // time each schedule candidate of every group on its data; keep the best
    // that keeps the tolerance.  Candidates: right-hand sides per launch
    // sequence x z-solve variant (factor table / per-solve factors) x DST
    // passes per axis (FFT / tensor cores, for 32-, 64-, 128-point axes).  A
    // variant is
    // accurate enough when its first-sweep correction estimate e (the FP32
    // solve's relative error) predicts 10 e^(sweeps+1) <= tol; with no sweep
    // only the default variants qualify.
    void tune() {
        cudaEvent_t a, b;
        FDM_CUDA(cudaEventCreate(&a));
        FDM_CUDA(cudaEventCreate(&b));
        for (auto& gr : groups) {
            const int m = (int)gr.members.size();
            int chunks[4] = {m, 8, 2, 1};
            double best = 1e30;
            int bc = m, bz = 1, bt = 0;
            const bool mixed = precision == FDMGPU_MIXED;
            const int sweeps = mixed ? gr.plan->sweeps_for_tol() : -1;
            const int tc_axes = mixed ? ((tc_supported(gr.nx + 1) ? 1 : 0) | (tc_supported(gr.ny + 1) ? 2 : 0)) : 0;
            for (int tc = 0; tc <= 3; tc++) {
                if (tc & ~tc_axes) continue;
                for (int zm = 1; zm >= 0; zm--) {
                    const bool is_default = zm == 1 && tc == 0;
                    if (!is_default && mixed && sweeps == 0) continue;
                    for (int ci = 0; ci < 4; ci++) {
                        const int ch = chunks[ci];
                        if (ch > m || (ci > 0 && ch == chunks[ci - 1])) continue;
                        gr.chunk = ch;
                        gr.zmode = zm;
                        gr.plan->dst_tc = tc;
                        enqueue_group(gr, gr.st);  // warm-up: allocates scratch and tables
                        FDM_CUDA(cudaEventRecord(a, gr.st));
                        enqueue_group(gr, gr.st);
                        FDM_CUDA(cudaEventRecord(b, gr.st));
                        FDM_CUDA(cudaEventSynchronize(b));
                        float ms = 0.f;
                        FDM_CUDA(cudaEventElapsedTime(&ms, a, b));
                        if (!is_default && mixed && ci == 0) {
                            // whole group in one launch sequence: the norms
                            // cover every member
                            const double e = gr.plan->first_sweep_est(m, gr.st);
                            if (10.0 * std::pow(e, sweeps + 1) > tol) break;
                        }
                        if (ms < best) {
                            best = ms;
                            bc = ch;
                            bz = zm;
                            bt = tc;
                        }
                    }
                }
            }
            gr.chunk = bc;
            gr.zmode = bz;
            gr.plan->dst_tc = bt;
            gr.tuned_ms = best;
            enqueue_group(gr, gr.st);  // scratch for the chosen schedule exists before capture
        }
        FDM_CUDA(cudaDeviceSynchronize());
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        drop_graph();
    }

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }

    void capture() {
        // eager pass first: every scratch buffer and table of the chosen
        // schedules is allocated outside the capture
        for (auto& gr : groups) enqueue_group(gr, gr.st);
        FDM_CUDA(cudaDeviceSynchronize());
        const unsigned long long l0 = fdmgpu_launch_count();
        FDM_CUDA(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
        try {
            FDM_CUDA(cudaEventRecord(fork, origin));
            for (auto& gr : groups) {
                FDM_CUDA(cudaStreamWaitEvent(gr.st, fork, 0));
                enqueue_group(gr, gr.st);
                FDM_CUDA(cudaEventRecord(gr.done, gr.st));
                FDM_CUDA(cudaStreamWaitEvent(origin, gr.done, 0));
            }
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(origin, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        FDM_CUDA(cudaStreamEndCapture(origin, &graph));
        FDM_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        launches_per_solve = (int)(fdmgpu_launch_count() - l0);
    }

    void solve(void* const* ans, const void* const* rhs, cudaStream_t st) {
        upload_pointers(ans, rhs, origin);
        if (!exec) capture();
        FDM_CUDA(cudaEventRecord(fork, st));
        FDM_CUDA(cudaStreamWaitEvent(origin, fork, 0));
        FDM_CUDA(cudaGraphLaunch(exec, origin));
        FDM_CUDA(cudaEventRecord(fork, origin));
        FDM_CUDA(cudaStreamWaitEvent(st, fork, 0));
    }
};

}  // namespace fdmgpu

struct fdmgpu_batch {
    BatchPlan plan;
};
struct fdmgpu_lapl_rect {
    RectPlan plan;
};

namespace fdmgpu {

// ---------------------------------------------------------------------------
// LaplCyl3FFT2: Poisson in a cylindrical annulus (src/lapl_cyl.h:178-262,
// src/lapl_cyl.cpp:10-166).  Arrays (nphi, nz, nr), r fastest.  Periodic
// transform along phi, DST (Dirichlet z) or periodic transform (periodic z)
// along z, then per (phi-mode, z-mode) a radial tridiagonal system with
// variable coefficients, eliminated without row swaps (the reference's
// LAPACK gttrf / gttrs; the matrices are diagonally dominant so partial
// pivoting does not swap); the elimination factors are prepared once per
// plan, laid out [j][system] so that the threads of a warp (consecutive
// systems) read them coalesced.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_cyl_rsolve(T* W, long long nsys, int nr, const T* __restrict__ fact, const T* __restrict__ piv,
                             const T* __restrict__ up) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    T* b = W + s * nr;
    const long long ns = nsys;
    T prev = b[0];
    for (int j = 0; j + 1 < nr; j++) {
        const T f = fact[(long long)j * ns + s];
        const T cur = b[j + 1] - f * prev;
        b[j + 1] = cur;
        prev = cur;
    }
    T x = b[nr - 1] / piv[(long long)(nr - 1) * ns + s];
    b[nr - 1] = x;
    for (int j = nr - 2; j >= 0; j--) {
        x = (b[j] - up[j] * x) / piv[(long long)j * ns + s];
        b[j] = x;
    }
}

struct CylPlan {
    int dtype = FDMGPU_F64;
    bool periodic_z = false;
    int nr, nz, nphi;
    double dr, dz, r0, lr, lz;
    AxisTables<double> tz64;
    AxisTables<float> tz32;
    DevBuf tw_phi, tw_z, fact, piv, up;

    long long vol() const { return (long long)nphi * nz * nr; }
    long long nsys() const { return (long long)nphi * nz; }

    template <typename T>
    void build() {
        const double dphi = 2 * M_PI / nphi, dphi2 = dphi * dphi, dr2 = dr * dr, dz2 = dz * dz;
        const int zpoints = periodic_z ? nz : nz + 1;
        std::vector<T> lm_phi(nphi), lm_z(nz);
        for (int i = 0; i < nphi; i++) {
            const double sn = std::sin(i * dphi * 0.5);
            lm_phi[i] = (T)(4.0 / dphi2 * (sn * sn));
        }
        for (int kk = 0; kk < nz; kk++) {
            // z1..zn: 1..nz (Dirichlet), 0..nz-1 (periodic)
            const int k = periodic_z ? kk : kk + 1;
            const double sn = periodic_z ? std::sin(k * M_PI / zpoints) : std::sin(k * M_PI * 0.5 / zpoints);
            lm_z[kk] = (T)(4. / dz2 * (sn * sn));
        }
        const long long ns = nsys();
        std::vector<T> hf((size_t)nr * ns), hp((size_t)nr * ns), hu(nr), hl(nr);
        for (int j = 1; j <= nr; j++) {
            const double r = r0 + j * dr;
            hl[j - 1] = (T)((r - 0.5 * dr) / dr2 / r);
            hu[j - 1] = (T)((r + 0.5 * dr) / dr2 / r);
        }
        for (int i = 0; i < nphi; i++)
            for (int kk = 0; kk < nz; kk++) {
                const long long sidx = (long long)i * nz + kk;
                // D_j = -2/dr^2 - lm_phi/r/r - lm_z (src/lapl_cyl.cpp:142), LU without swaps
                T dd = 0;
                for (int j = 1; j <= nr; j++) {
                    const double r = r0 + j * dr;
                    const T d = (T)(-2 / dr2 - lm_phi[i] / r / r - lm_z[kk]);
                    if (j == 1) {
                        dd = d;
                    } else {
                        const T f = hl[j - 1] / dd;
                        hf[(size_t)(j - 2) * ns + sidx] = f;
                        dd = d - f * hu[j - 2];
                    }
                    hp[(size_t)(j - 1) * ns + sidx] = dd;
                }
            }
        FDM_CUDA(cudaMemcpy(fact.get(hf.size() * sizeof(T)), hf.data(), hf.size() * sizeof(T), cudaMemcpyHostToDevice));
        FDM_CUDA(cudaMemcpy(piv.get(hp.size() * sizeof(T)), hp.data(), hp.size() * sizeof(T), cudaMemcpyHostToDevice));
        FDM_CUDA(cudaMemcpy(up.get(hu.size() * sizeof(T)), hu.data(), hu.size() * sizeof(T), cudaMemcpyHostToDevice));
        upload_ptwiddles<T>(tw_phi, nphi);
        if (periodic_z) upload_ptwiddles<T>(tw_z, nz);
        else if (sizeof(T) == 8) tz64.build(nz + 1);
        else tz32.build(nz + 1);
    }

    void init() {
        if (dtype == FDMGPU_F64) build<double>();
        else build<float>();
    }

    template <typename T>
    void run(T* ans, const T* rhs, int nrhs, cudaStream_t st) {
        const double inv_sqrt_pi = 0.56418958354775629;  // the reference's SQRT_M_1_PI
        const double dphi = 2 * M_PI / nphi, slz = std::sqrt(2. / lz);
        const long long v = vol(), plane = (long long)nz * nr;
        PLineGeom gphi{(long long)nrhs * plane, plane, v, 1, plane};
        PLineGeom gz{(long long)nrhs * nphi * nr, nr, plane, 1, nr};
        launch_pfft<T, false>(rhs, ans, gphi, nphi, tw_phi.p, (double)(T)(dphi * inv_sqrt_pi), st);
        if (periodic_z) launch_pfft<T, false>(ans, ans, gz, nz, tw_z.p, dz * slz, st);
        else launch_sine<T, T, T, 1>(ans, ans, nr, nz, nphi, nrhs, table<T>().view(), dz * slz, st);
        {
            const long long ns = nsys();
            FDM_TIMED("cyl_rsolve", st);
            for (int v0 = 0; v0 < nrhs; v0++) {
                k_cyl_rsolve<T><<<(unsigned)((ns + 127) / 128), 128, 0, st>>>(ans + v0 * v, ns, nr, (const T*)fact.p,
                                                                              (const T*)piv.p, (const T*)up.p);
                FDM_LAUNCH_CHECK();
            }
        }
        if (periodic_z) launch_pfft<T, true>(ans, ans, gz, nz, tw_z.p, slz, st);
        else launch_sine<T, T, T, 1>(ans, ans, nr, nz, nphi, nrhs, table<T>().view(), slz, st);
        launch_pfft<T, true>(ans, ans, gphi, nphi, tw_phi.p, (double)(T)inv_sqrt_pi, st);
    }

    template <typename T>
    const AxisTables<T>& table() const;

    void solve_device(void* ans, const void* rhs, int nrhs, cudaStream_t st) {
        check_grid_y(nrhs);
        if (dtype == FDMGPU_F64) run<double>((double*)ans, (const double*)rhs, nrhs, st);
        else run<float>((float*)ans, (const float*)rhs, nrhs, st);
    }
};
template <>
const AxisTables<double>& CylPlan::table<double>() const { return tz64; }
template <>
const AxisTables<float>& CylPlan::table<float>() const { return tz32; }

}  // namespace fdmgpu

struct fdmgpu_lapl_cyl {
    CylPlan plan;
};

namespace fdmgpu {

// ---------------------------------------------------------------------------
// Mixed-precision solve that allocates nothing
//
// Some callers cannot allocate device memory when they solve: an application
// whose device memory is owned by its own pool or by another framework's
// allocator (a cudaMalloc behind that allocator's back can fail or fragment
// it), a time-stepping loop that must not stall in the allocator after
// start-up, or a host program that forbids dynamic device allocation once it
// is initialised.  fdmgpu_lapl_cube_solve_mixed_noalloc serves them: it runs
// the same kernels as the mixed solve of fdmgpu_lapl_cube_solve_device, but
// its tables, FP32 work volumes and norms live in the fixed array below,
// which exists once per device for as long as the library is loaded.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[FDMGPU_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kMaxDevices];

// Device address of the array on the current device.  The first call on a
// device looks it up with cudaGetSymbolAddress (which also loads the module
// there); later calls reuse the address.
static unsigned char* noalloc_scratch() {
    const int dev = current_device();
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            FDM_FAIL(FDMGPU_ECUDA, "cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    return (unsigned char*)g_noalloc_ptr[dev];
}

// DST tables (rounded to FP32 from FP64 values) and Dirichlet eigenvalues
// 4/h^2 sin^2(j pi / (2(n+1))) of one axis, written into the array.
__global__ void k_noalloc_tables(float2* tw, float2* post, float* wpre, float* lam, int N, double h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int M = N / 2, n = N - 1;
    double s, c;
    if (i < M) {
        sincospi(2.0 * i / M, &s, &c);
        tw[i] = make_float2((float)c, (float)(-s));
        sincospi(2.0 * i / N, &s, &c);
        post[i] = make_float2((float)c, (float)(-s));
    }
    if (i < N) wpre[i] = (float)sinpi((double)i / N);
    if (i < n) {
        const double sv = sinpi((i + 1) * 0.5 / (n + 1));
        lam[i] = (float)(4.0 / (h * h) * (sv * sv));
    }
}

// Per-mode factors of the partitioned z-solve, the table zsolve_table_host
// builds for a handle (layout of k_zsolve_tab: block pivot reciprocals,
// right-end responses, separator pivot reciprocals and multipliers, value
// major), computed here on the device in FP64 and stored in FP32.  The
// eigenvalues are 4/h^2 sin^2(j pi / (2(n+1))) of x (spacing hx) and y
// (spacing hy); h2 is the z spacing squared.  Products and sums are rounded
// one by one (no contraction), as the host computes them.
__global__ void k_noalloc_ztable(float* tab, int nx, int ny, int m, int P, double hx, double hy, double h2) {
    const int modes = nx * ny;
    const int mode = blockIdx.x * blockDim.x + threadIdx.x;
    if (mode >= modes) return;
    const int j = mode % nx, k = mode / nx;
    const double sx = sinpi((j + 1) * 0.5 / (nx + 1)), sy = sinpi((k + 1) * 0.5 / (ny + 1));
    const double lx = __dmul_rn(4. / (hx * hx), __dmul_rn(sx, sx));
    const double ly = __dmul_rn(4. / (hy * hy), __dmul_rn(sy, sy));
    const double b = __dsub_rn(-2.0, __dmul_rn(__dadd_rn(lx, ly), h2));
    double cp[15], be[15];
    double c = 0.0;
    for (int i = 0; i < m; i++) {
        c = 1.0 / __dsub_rn(b, c);
        cp[i] = c;
    }
    be[m - 1] = -cp[m - 1];
    for (int i = m - 2; i >= 0; i--) be[i] = __dmul_rn(-cp[i], be[i + 1]);
    for (int i = 0; i < m; i++) {
        tab[(size_t)i * modes + mode] = (float)cp[i];
        tab[(size_t)(m + i) * modes + mode] = (float)be[i];
    }
    const double lo = be[0], dg = __dadd_rn(b, __dmul_rn(2.0, be[m - 1]));
    double pc = 0.0;
    for (int q = 0; q < P - 1; q++) {
        const double r = 1.0 / __dsub_rn(dg, __dmul_rn(lo, pc));
        pc = __dmul_rn(lo, r);
        tab[(size_t)(2 * m + q) * modes + mode] = (float)r;
        tab[(size_t)(2 * m + P - 1 + q) * modes + mode] = (float)pc;
    }
}

// Block length m and block count P of the table-driven z-solve for nz rows
// (the split zsolve_table_host uses); false when the line does not split
// into at most 16 blocks of 2^k - 1 rows.
static bool ztable_split(int nz, int* m, int* P) {
    *m = nz < 15 ? nz : 15;
    *P = (nz + 1) / (*m + 1);
    return (*m + 1) * *P == nz + 1 && *P <= 16;
}

struct NoallocAxis {
    float2 *tw, *post;
    float *wpre, *lam;
};

static size_t noalloc_align(size_t v) { return (v + 255) & ~(size_t)255; }

static size_t noalloc_axis_bytes(int N) {
    const int M = N / 2 > 0 ? N / 2 : 1;
    return noalloc_align(M * sizeof(float2)) * 2 + noalloc_align(N * sizeof(float)) * 2;
}

static NoallocAxis noalloc_axis(unsigned char*& p, int N) {
    const int M = N / 2 > 0 ? N / 2 : 1;
    NoallocAxis a;
    a.tw = (float2*)p; p += noalloc_align(M * sizeof(float2));
    a.post = (float2*)p; p += noalloc_align(M * sizeof(float2));
    a.wpre = (float*)p; p += noalloc_align(N * sizeof(float));
    a.lam = (float*)p; p += noalloc_align(N * sizeof(float));
    return a;
}

static void noalloc_solve(double dx, double dy, double dz, double lx, double ly, double lz, int nx, int ny, int nz,
                          double tol, double* ans, const double* rhs, int nrhs, cudaStream_t st) {
    // geometry as CubePlan::init
    const double slx = std::sqrt(2. / lx), sly = std::sqrt(2. / ly), slz = std::sqrt(2. / lz);
    const double scx = dx * slx, scy = dy * sly;
    const double hx_eff = (nx == ny) ? dy : dx;
    const double hz_eff = (nz == ny) ? dy : dz;
    const double zfac = dz * slz * slz * (nz + 1) / 2.0;
    const double S = (dx * slx * slx * (nx + 1) / 2.0) * (dy * sly * sly * (ny + 1) / 2.0) * zfac;
    int sweeps = tol >= 1e-5 ? 0 : (tol >= 1e-11 ? 1 : 2);
    if (lapl_kappa(nx, ny, nz, hx_eff, dy, hz_eff) > kMixedKappaMax)
        FDM_FAIL(FDMGPU_ENOTSUP,
                 "%dx%dx%d is beyond the mixed-precision conditioning limit (kappa %.3g > %.3g): the handle API "
                 "solves such sizes in FP64",
                 nx, ny, nz, lapl_kappa(nx, ny, nz, hx_eff, dy, hz_eff), kMixedKappaMax);

    const long long V = (long long)nx * ny * nz * nrhs;
    // the per-mode z factor table of a handle's mixed plan, when the line
    // splits (otherwise both solve with factors computed per solve)
    int zm = 0, zP = 0;
    const bool ztab = ztable_split(nz, &zm, &zP);
    const size_t tab_bytes = ztab ? noalloc_align((size_t)(2 * zm + 2 * (zP - 1)) * nx * ny * sizeof(float)) : 0;
    const size_t need = noalloc_axis_bytes(nx + 1) + noalloc_axis_bytes(ny + 1) + tab_bytes +
                        noalloc_align((size_t)2 * nrhs * (sweeps > 0 ? sweeps : 1) * sizeof(double)) +
                        noalloc_align((size_t)V * sizeof(float)) * (sweeps == 0 ? 1 : (sweeps > 1 ? 3 : 2));
    if (need > (size_t)FDMGPU_NOALLOC_SCRATCH_BYTES)
        FDM_FAIL(FDMGPU_EBUDGET,
                 "the solve needs %zu bytes of scratch; the no-allocation entry point has %u (nrhs=%d of %dx%dx%d)",
                 need, (unsigned)FDMGPU_NOALLOC_SCRATCH_BYTES, nrhs, nx, ny, nz);

    unsigned char* p = noalloc_scratch();
    NoallocAxis ax = noalloc_axis(p, nx + 1);
    NoallocAxis ay = noalloc_axis(p, ny + 1);
    float* ZT = ztab ? (float*)p : nullptr;
    p += tab_bytes;
    double* NR = (double*)p;
    p += noalloc_align((size_t)2 * nrhs * (sweeps > 0 ? sweeps : 1) * sizeof(double));
    float* W = (float*)p;
    p += noalloc_align((size_t)V * sizeof(float));
    float* UH = sweeps > 0 ? (float*)p : nullptr;
    if (sweeps > 0) p += noalloc_align((size_t)V * sizeof(float));
    float* UL = sweeps > 1 ? (float*)p : nullptr;

    {
        FDM_TIMED("noalloc_tables", st);
        k_noalloc_tables<<<(nx + 1 + 255) / 256, 256, 0, st>>>(ax.tw, ax.post, ax.wpre, ax.lam, nx + 1, hx_eff);
        FDM_LAUNCH_CHECK();
    }
    {
        FDM_TIMED("noalloc_tables", st);
        k_noalloc_tables<<<(ny + 1 + 255) / 256, 256, 0, st>>>(ay.tw, ay.post, ay.wpre, ay.lam, ny + 1, dy);
        FDM_LAUNCH_CHECK();
    }
    if (ztab) {
        FDM_TIMED("noalloc_tables", st);
        k_noalloc_ztable<<<(nx * ny + 127) / 128, 128, 0, st>>>(ZT, nx, ny, zm, zP, hx_eff, dy, hz_eff * hz_eff);
        FDM_LAUNCH_CHECK();
    }
    auto view = [](const NoallocAxis& a, int N) {
        SineTables<float> v;
        v.tw = a.tw; v.post = a.post; v.wpre = a.wpre; v.N = N; v.M = N / 2;
        return v;
    };
    const SineTables<float> tx = view(ax, nx + 1), ty = view(ay, ny + 1);
    const double h2 = hz_eff * hz_eff, gscale = zfac * hz_eff * hz_eff;
    auto zsolve = [&](float* w) {
        if (ztab) zsolve_tab_launch<float>(w, nx, ny, nz, nrhs, ZT, zm, zP, gscale, st);
        else zsolve_lines<float>(w, nx, ny, nz, nrhs, ax.lam, ay.lam, h2, gscale, st);
    };

    launch_sine<double, float, float, 0, kRound>(rhs, W, nx, ny, nz, nrhs, tx, scx, st);
    launch_sine<float, float, float, 1>(W, W, nx, ny, nz, nrhs, ty, scy, st);
    zsolve(W);
    launch_sine<float, float, float, 1>(W, W, nx, ny, nz, nrhs, ty, sly, st);
    if (sweeps == 0) {
        launch_sine<float, float, double, 0>(W, ans, nx, ny, nz, nrhs, tx, slx, st);
        return;
    }
    // the norms must start at zero on every call: the array keeps the last
    // call's contents
    FDM_CUDA(cudaMemsetAsync(NR, 0, (size_t)2 * nrhs * sweeps * sizeof(double), st));
    launch_sine<float, float, float, 0>(W, UH, nx, ny, nz, nrhs, tx, slx, st);
    const double cx = 1.0 / (hx_eff * hx_eff) / S, cy = 1.0 / (dy * dy) / S, cz = 1.0 / (hz_eff * hz_eff) / S;
    for (int s = 1; s <= sweeps; s++) {
        SineFused fr;
        memset(&fr, 0, sizeof(fr));
        fr.f = rhs;
        fr.uhi = UH;
        fr.ulo = s >= 2 ? UL : nullptr;
        fr.cx = CubePlan::split_host(cx); fr.cy = CubePlan::split_host(cy); fr.cz = CubePlan::split_host(cz);
        fr.cxf = (float)cx; fr.cyf = (float)cy; fr.czf = (float)cz;
        fr.iso = (cx == cy && cy == cz) ? 1 : 0;
        launch_residual(fr, W, nx, ny, nz, nrhs, st);
        launch_sine<float, float, float, 0>(W, W, nx, ny, nz, nrhs, tx, scx, st);
        launch_sine<float, float, float, 1>(W, W, nx, ny, nz, nrhs, ty, scy, st);
        zsolve(W);
        launch_sine<float, float, float, 1>(W, W, nx, ny, nz, nrhs, ty, sly, st);
        SineFused fc;
        memset(&fc, 0, sizeof(fc));
        fc.uhi = UH;
        fc.ulo = s >= 2 ? UL : nullptr;
        fc.out64 = ans;
        fc.ulo_out = s < sweeps ? UL : nullptr;
        fc.last = s == sweeps ? 1 : 0;
        fc.norms = NR + (size_t)2 * nrhs * (s - 1);
        launch_sine<float, float, float, 0, kCombine>(W, (float*)nullptr, nx, ny, nz, nrhs, tx, slx, st, &fc);
    }
}

void cube_solve_device(fdmgpu_lapl_cube* h, void* ans, const void* rhs, int nrhs, cudaStream_t st) {
    h->plan.solve_device(ans, rhs, nrhs, st);
}

void cube_solve_ptrs(fdmgpu_lapl_cube* h, const void* const* d_in, void* const* d_out, int nvol, double* scratch,
                     cudaStream_t st) {
    CubePlan& c = h->plan;
    if (c.dtype != FDMGPU_F64 || c.periodic) FDM_FAIL(FDMGPU_ENOTSUP, "pointer-table solves are FP64 Dirichlet");
    check_grid_y(nvol);
    c.last_stream = st;
    c.last_nrhs = nvol;
    c.last_sweeps = 0;
    c.run_plain_ptrs(d_in, d_out, nvol, st, scratch);
}

void cube_set_rule_volumes(fdmgpu_lapl_cube* h, int vols) { h->plan.rule_vols = vols > 0 ? vols : 0; }

int cube_norms_async(fdmgpu_lapl_cube* h, double* host, int nrhs, cudaStream_t st) {
    const CubePlan& c = h->plan;
    if (c.last_sweeps <= 0 || !c.norms.p) return c.last_sweeps;
    FDM_CUDA(cudaMemcpyAsync(host, c.norms.p, (size_t)2 * nrhs * c.last_sweeps * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
    return c.last_sweeps;
}

void cube_estimates(const fdmgpu_lapl_cube* h, const double* norms_host, int sweeps, int nrhs, double* est) {
    h->plan.estimates_from_norms(norms_host, nrhs, sweeps, est);
}

void cyl_solve_device(fdmgpu_lapl_cyl* h, void* ans, const void* rhs, int nrhs, cudaStream_t st) {
    h->plan.solve_device(ans, rhs, nrhs, st);
}
}  // namespace fdmgpu

// twiddles e^{-2 pi i t / n} of the periodic 3-D transforms, one table per
// (device, element type, n), kept for the life of the process
static const void* pfft3d_twiddles(int dtype, int n) {
    static std::mutex mu;
    static std::map<long long, std::unique_ptr<DevBuf>> cache;
    int dev = 0;
    FDM_CUDA(cudaGetDevice(&dev));
    const long long key = ((long long)dev << 32) | ((long long)dtype << 16) | n;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second->p;
    std::unique_ptr<DevBuf> b(new DevBuf());
    if (dtype == FDMGPU_F64) upload_ptwiddles<double>(*b, n);
    else upload_ptwiddles<float>(*b, n);
    const void* p = b->p;
    cache.emplace(key, std::move(b));
    return p;
}

// FFT<T>::pFFT_1_3d / pFFT_3d (src/fft.cpp:214-292): the periodic transform
// along x (fastest), then y, then z of `count` cubes of n^3, scale dx on
// every pass
template <typename T, bool INV>
static void pfft3d_run(const T* in, T* out, int n, int count, double dx, const void* tw, cudaStream_t st) {
    const long long n2 = (long long)n * n, lines = (long long)count * n2;
    PLineGeom gx{lines, 1, n, 0, 1};
    PLineGeom gy{lines, n, n2, 1, n};
    PLineGeom gz{lines, n2, n2 * n, 1, n2};
    launch_pfft<T, INV>(in, out, gx, n, tw, dx, st);
    launch_pfft<T, INV>(out, out, gy, n, tw, dx, st);
    launch_pfft<T, INV>(out, out, gz, n, tw, dx, st);
}

static size_t elem_size(int dtype) { return dtype == FDMGPU_F64 ? sizeof(double) : sizeof(float); }

// Diagnostic: the integer FP64 <-> float conversions of the mixed path
// beside the hardware conversions and the FP64 sum of a float pair.
__global__ void k_dd_check(const double* x, const float* ph, const float* pl, long long n, float* f32, float* f32_hw,
                           float* split_hi, float* split_lo, double* w, double* w_hw) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = x[i];
    f32[i] = f64_to_f32(d);
    f32_hw[i] = __double2float_rn(d);
    const ff s = f64_split(d);
    split_hi[i] = s.h;
    split_lo[i] = s.l;
    w[i] = ff_to_f64(ff{ph[i], pl[i]});
    w_hw[i] = __dadd_rn((double)ph[i], (double)pl[i]);
}

extern "C" {

int fdmgpu_lapl_cube_create(fdmgpu_lapl_cube** h, int dtype, int bc_flags, double dx, double dy, double dz,
                            double lx, double ly, double lz, int nx, int ny, int nz) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle pointer");
    *h = nullptr;
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    if (bc_flags != FDMGPU_DIRICHLET && bc_flags != FDMGPU_PERIODIC)
        FDM_FAIL(FDMGPU_ENOTSUP, "boundary flags %d: all Dirichlet (0) or all periodic (7)", bc_flags);
    const bool periodic = bc_flags == FDMGPU_PERIODIC;
    if (periodic) {
        if (!pow2_periodic(nx) || !pow2_periodic(ny) || !pow2_periodic(nz))
            FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: periodic n must be a power of two in [2, 512] "
                                   "(got %d,%d,%d)", nx, ny, nz);
    } else if (!pow2_interior(nx) || !pow2_interior(ny) || !pow2_interior(nz)) {
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: n+1 must be a power of two and n <= %d (got %d,%d,%d)",
                 FDMGPU_MAX_N, nx, ny, nz);
    }
    if (!(dx > 0 && dy > 0 && dz > 0 && lx > 0 && ly > 0 && lz > 0))
        FDM_FAIL(FDMGPU_EINVAL, "spacings and lengths must be positive");
    std::unique_ptr<fdmgpu_lapl_cube> p(new fdmgpu_lapl_cube());
    CubePlan& c = p->plan;
    c.dtype = dtype; c.nx = nx; c.ny = ny; c.nz = nz;
    c.dx = dx; c.dy = dy; c.dz = dz; c.lx = lx; c.ly = ly; c.lz = lz;
    c.periodic = periodic;
    c.init();
    *h = p.release();
    FDM_API_END
}

int fdmgpu_lapl_cube_set_precision(fdmgpu_lapl_cube* h, int precision, double tol, int max_sweeps) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (precision != FDMGPU_PLAIN && precision != FDMGPU_MIXED) FDM_FAIL(FDMGPU_EINVAL, "bad precision %d", precision);
    if (precision == FDMGPU_MIXED && h->plan.dtype != FDMGPU_F64)
        FDM_FAIL(FDMGPU_ENOTSUP, "mixed precision needs FP64 arrays");
    if (precision == FDMGPU_MIXED && h->plan.periodic)
        FDM_FAIL(FDMGPU_ENOTSUP, "the periodic LaplCube is plain precision only");
    h->plan.precision = precision;
    h->plan.tol = tol > 0 ? tol : 1e-10;
    h->plan.max_sweeps = max_sweeps >= 0 ? max_sweeps : 3;
    FDM_API_END
}

int fdmgpu_lapl_cube_solve_device(fdmgpu_lapl_cube* h, void* d_ans, const void* d_rhs, int nrhs, void* stream) {
    FDM_API_BEGIN
    if (!h || !d_ans || !d_rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    h->plan.solve_device(d_ans, d_rhs, nrhs, (cudaStream_t)stream);
    FDM_API_END
}

int fdmgpu_lapl_cube_solve(fdmgpu_lapl_cube* h, void* ans, const void* rhs) {
    FDM_API_BEGIN
    if (!h || !ans || !rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    CubePlan& c = h->plan;
    const size_t bytes = (size_t)c.vol() * elem_size(c.dtype);
    void* din = c.hin.get(bytes);
    void* dout = c.hout.get(bytes);
    FDM_CUDA(cudaMemcpy(din, rhs, bytes, cudaMemcpyHostToDevice));
    c.solve_device(dout, din, 1, 0);
    FDM_CUDA(cudaMemcpy(ans, dout, bytes, cudaMemcpyDeviceToHost));
    FDM_API_END
}

int fdmgpu_lapl_cube_solve_host_batch(fdmgpu_lapl_cube* h, void* ans, const void* rhs, int nrhs) {
    FDM_API_BEGIN
    if (!h || !ans || !rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (nrhs < 1) FDM_FAIL(FDMGPU_EINVAL, "nrhs must be positive");
    h->plan.solve_host_pipelined(ans, rhs, nrhs);
    FDM_API_END
}

int fdmgpu_lapl_cube_last_info(fdmgpu_lapl_cube* h, int* sweeps, double* est, int nrhs) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    CubePlan& c = h->plan;
    FDM_CUDA(cudaStreamSynchronize(c.last_stream));
    if (sweeps) *sweeps = c.last_sweeps;
    if (est) {
        if (nrhs > c.last_nrhs) FDM_FAIL(FDMGPU_EINVAL, "asked for %d estimates, last solve had %d", nrhs, c.last_nrhs);
        const std::vector<double> e = (int)c.last_est.size() == c.last_nrhs
                                          ? c.last_est
                                          : c.final_estimates(c.last_nrhs, c.last_sweeps, c.last_stream);
        for (int i = 0; i < nrhs; i++) est[i] = e[i];
    }
    FDM_API_END
}

int fdmgpu_lapl_cube_scratch_bytes(fdmgpu_lapl_cube* h, size_t* bytes) {
    FDM_API_BEGIN
    if (!h || !bytes) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    *bytes = h->plan.scratch_bytes();
    FDM_API_END
}

int fdmgpu_lapl_cube_destroy(fdmgpu_lapl_cube* h) {
    FDM_API_BEGIN
    delete h;
    FDM_API_END
}

int fdmgpu_batch_create(fdmgpu_batch** h, int count, const int* n3, const double* h3, const double* l3,
                        int precision, double tol) {
    FDM_API_BEGIN
    if (!h || !n3 || !h3 || !l3) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    *h = nullptr;
    if (count < 1) FDM_FAIL(FDMGPU_EINVAL, "count must be positive");
    if (precision != FDMGPU_PLAIN && precision != FDMGPU_MIXED) FDM_FAIL(FDMGPU_EINVAL, "bad precision %d", precision);
    for (int i = 0; i < count; i++) {
        for (int a = 0; a < 3; a++) {
            if (!pow2_interior(n3[3 * i + a]))
                FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: right-hand side %d has n=%d", i, n3[3 * i + a]);
            if (!(h3[3 * i + a] > 0 && l3[3 * i + a] > 0))
                FDM_FAIL(FDMGPU_EINVAL, "right-hand side %d: spacings and lengths must be positive", i);
        }
    }
    std::unique_ptr<fdmgpu_batch> p(new fdmgpu_batch());
    p->plan.count = count;
    p->plan.precision = precision;
    p->plan.tol = tol > 0 ? tol : 1e-10;
    p->plan.init(n3, h3, l3);
    *h = p.release();
    FDM_API_END
}

int fdmgpu_batch_tune(fdmgpu_batch* h, void* const* d_ans, const void* const* d_rhs) {
    FDM_API_BEGIN
    if (!h || !d_ans || !d_rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    h->plan.upload_pointers(d_ans, d_rhs, h->plan.origin);
    h->plan.tune();
    FDM_API_END
}

int fdmgpu_batch_solve(fdmgpu_batch* h, void* const* d_ans, const void* const* d_rhs, void* stream) {
    FDM_API_BEGIN
    if (!h || !d_ans || !d_rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    h->plan.solve(d_ans, d_rhs, (cudaStream_t)stream);
    FDM_API_END
}

int fdmgpu_batch_info(fdmgpu_batch* h, int* groups, int* launches_per_solve) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (groups) *groups = (int)h->plan.groups.size();
    if (launches_per_solve) *launches_per_solve = h->plan.launches_per_solve;
    FDM_API_END
}

int fdmgpu_batch_schedule(fdmgpu_batch* h, int group, int* n3, int* members, int* chunk, int* ztable, int* dst_tc,
                          double* tuned_ms) {
    FDM_API_BEGIN
    if (!h || group < 0 || group >= (int)h->plan.groups.size()) FDM_FAIL(FDMGPU_EINVAL, "bad handle or group");
    const BatchGroup& gr = h->plan.groups[group];
    if (n3) { n3[0] = gr.nx; n3[1] = gr.ny; n3[2] = gr.nz; }
    if (members) *members = (int)gr.members.size();
    if (chunk) *chunk = gr.chunk;
    if (ztable) *ztable = gr.zmode;
    if (dst_tc) *dst_tc = gr.plan->tc_mask();
    if (tuned_ms) *tuned_ms = gr.tuned_ms;
    FDM_API_END
}

int fdmgpu_batch_destroy(fdmgpu_batch* h) {
    FDM_API_BEGIN
    delete h;
    FDM_API_END
}

int fdmgpu_lapl_cyl_create(fdmgpu_lapl_cyl** h, int dtype, int periodic_z, double dr, double dz, double r0,
                           double lr, double lz, int nr, int nz, int nphi) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle pointer");
    *h = nullptr;
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    if (!pow2_periodic(nphi)) FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: nphi=%d", nphi);
    if (periodic_z ? !pow2_periodic(nz) : !pow2_interior(nz))
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: nz=%d (periodic %d)", nz, periodic_z);
    if (nr < 1 || nr > 4096) FDM_FAIL(FDMGPU_ESIZE, "nr must be in [1, 4096], got %d", nr);
    if (!(dr > 0 && dz > 0 && r0 >= 0 && lr > 0 && lz > 0)) FDM_FAIL(FDMGPU_EINVAL, "bad geometry");
    std::unique_ptr<fdmgpu_lapl_cyl> p(new fdmgpu_lapl_cyl());
    CylPlan& c = p->plan;
    c.dtype = dtype; c.periodic_z = periodic_z != 0;
    c.nr = nr; c.nz = nz; c.nphi = nphi;
    c.dr = dr; c.dz = dz; c.r0 = r0; c.lr = lr; c.lz = lz;
    c.init();
    *h = p.release();
    FDM_API_END
}

int fdmgpu_lapl_cyl_solve(fdmgpu_lapl_cyl* h, void* ans, const void* rhs) {
    FDM_API_BEGIN
    if (!h || !ans || !rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    CylPlan& c = h->plan;
    const size_t bytes = (size_t)c.vol() * (c.dtype == FDMGPU_F64 ? 8 : 4);
    DevBuf din, dout;
    FDM_CUDA(cudaMemcpy(din.get(bytes), rhs, bytes, cudaMemcpyHostToDevice));
    c.solve_device(dout.get(bytes), din.p, 1, 0);
    FDM_CUDA(cudaMemcpy(ans, dout.p, bytes, cudaMemcpyDeviceToHost));
    FDM_API_END
}

int fdmgpu_lapl_cyl_solve_device(fdmgpu_lapl_cyl* h, void* d_ans, const void* d_rhs, int nrhs, void* stream) {
    FDM_API_BEGIN
    if (!h || !d_ans || !d_rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    h->plan.solve_device(d_ans, d_rhs, nrhs, (cudaStream_t)stream);
    FDM_API_END
}

int fdmgpu_lapl_cyl_destroy(fdmgpu_lapl_cyl* h) {
    FDM_API_BEGIN
    delete h;
    FDM_API_END
}

int fdmgpu_lapl_rect_create_flags(fdmgpu_lapl_rect** h, int dtype, int method, int flags, double dx, double dy,
                                  double lx, double ly, int nx, int ny) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle pointer");
    *h = nullptr;
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    if (method != FDMGPU_RECT_TRIDIAG && method != FDMGPU_RECT_FFT2) FDM_FAIL(FDMGPU_EINVAL, "bad method %d", method);
    if (flags != 0 && flags != 2 && flags != 3)
        FDM_FAIL(FDMGPU_ENOTSUP, "flags %d: the reference instantiates none (0), y periodic (2) and both (3), "
                                 "src/lapl_rect.cpp:209-238", flags);
    const bool py = (flags & 2) != 0, px = (flags & 1) != 0 && method == FDMGPU_RECT_FFT2;
    if (py ? !pow2_periodic(ny) : !pow2_interior(ny))
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: %s (ny=%d)",
                 py ? "periodic ny must be a power of two in [2, 512]" : "ny+1 must be a power of two", ny);
    if (method == FDMGPU_RECT_FFT2 && (px ? !pow2_periodic(nx) : !pow2_interior(nx)))
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: %s (nx=%d)",
                 px ? "periodic nx must be a power of two in [2, 512]" : "nx+1 must be a power of two", nx);
    if (nx < 1 || nx > kTriCk * kTriMaxCk) FDM_FAIL(FDMGPU_ESIZE, "nx must be in [1, %d]", kTriCk * kTriMaxCk);
    if (!(dx > 0 && dy > 0 && lx > 0 && ly > 0)) FDM_FAIL(FDMGPU_EINVAL, "spacings and lengths must be positive");
    std::unique_ptr<fdmgpu_lapl_rect> p(new fdmgpu_lapl_rect());
    RectPlan& r = p->plan;
    r.dtype = dtype; r.method = method; r.nx = nx; r.ny = ny; r.flags = flags;
    r.dx = dx; r.dy = dy; r.lx = lx; r.ly = ly;
    r.init();
    *h = p.release();
    FDM_API_END
}

int fdmgpu_lapl_rect_create(fdmgpu_lapl_rect** h, int dtype, int method, double dx, double dy, double lx, double ly,
                            int nx, int ny) {
    return fdmgpu_lapl_rect_create_flags(h, dtype, method, 0, dx, dy, lx, ly, nx, ny);
}

int fdmgpu_lapl_rect_solve_device(fdmgpu_lapl_rect* h, void* d_ans, const void* d_rhs, int nrhs, void* stream) {
    FDM_API_BEGIN
    if (!h || !d_ans || !d_rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    h->plan.solve_device(d_ans, d_rhs, nrhs, (cudaStream_t)stream);
    FDM_API_END
}

int fdmgpu_lapl_rect_solve(fdmgpu_lapl_rect* h, void* ans, const void* rhs) {
    FDM_API_BEGIN
    if (!h || !ans || !rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    RectPlan& r = h->plan;
    const size_t bytes = (size_t)r.nx * r.ny * elem_size(r.dtype);
    void* din = r.hin.get(bytes);
    void* dout = r.hout.get(bytes);
    FDM_CUDA(cudaMemcpy(din, rhs, bytes, cudaMemcpyHostToDevice));
    r.solve_device(dout, din, 1, 0);
    FDM_CUDA(cudaMemcpy(ans, dout, bytes, cudaMemcpyDeviceToHost));
    FDM_API_END
}

int fdmgpu_lapl_rect_destroy(fdmgpu_lapl_rect* h) {
    FDM_API_BEGIN
    delete h;
    FDM_API_END
}

int fdmgpu_lapl_cube_solve_mixed_noalloc(double dx, double dy, double dz, double lx, double ly, double lz, int nx,
                                         int ny, int nz, double tol, void* d_ans, const void* d_rhs, int nrhs,
                                         void* stream) {
    FDM_API_BEGIN
    if (!d_ans || !d_rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (!pow2_interior(nx) || !pow2_interior(ny) || !pow2_interior(nz))
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: n+1 must be a power of two and n <= %d (got %d,%d,%d)",
                 FDMGPU_MAX_N, nx, ny, nz);
    if (!(dx > 0 && dy > 0 && dz > 0 && lx > 0 && ly > 0 && lz > 0))
        FDM_FAIL(FDMGPU_EINVAL, "spacings and lengths must be positive");
    check_grid_y(nrhs);
    noalloc_solve(dx, dy, dz, lx, ly, lz, nx, ny, nz, tol > 0 ? tol : 1e-10, (double*)d_ans, (const double*)d_rhs,
                  nrhs, (cudaStream_t)stream);
    FDM_API_END
}

int fdmgpu_sine_device(int dtype, int N, int nlines, double scale, void* d_out, const void* d_in, void* stream) {
    FDM_API_BEGIN
    if (!d_out || !d_in) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (N < 2 || N - 1 > FDMGPU_MAX_N || ilog2_exact(N) < 0)
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: N=%d", N);
    if (nlines < 1) FDM_FAIL(FDMGPU_EINVAL, "nlines must be positive");
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == FDMGPU_F64) {
        AxisTables<double> t;
        t.build(N);
        launch_sine<double, double, double, 0>((const double*)d_in, (double*)d_out, N - 1, nlines, 1, 1, t.view(),
                                               scale, st);
        FDM_CUDA(cudaStreamSynchronize(st));
    } else if (dtype == FDMGPU_F32) {
        AxisTables<float> t;
        t.build(N);
        launch_sine<float, float, float, 0>((const float*)d_in, (float*)d_out, N - 1, nlines, 1, 1, t.view(), scale,
                                            st);
        FDM_CUDA(cudaStreamSynchronize(st));
    } else {
        FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    }
    FDM_API_END
}

int fdmgpu_pfft3d_device(int dtype, int n, int inverse, double dx, void* d_out, const void* d_in, int count,
                         void* stream) {
    FDM_API_BEGIN
    if (!d_out || !d_in) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (!pow2_periodic(n)) FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: N must be a power of two in [2, 512], got %d", n);
    if (count < 1) FDM_FAIL(FDMGPU_EINVAL, "count must be positive");
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    cudaStream_t st = (cudaStream_t)stream;
    const void* tw = pfft3d_twiddles(dtype, n);
    if (dtype == FDMGPU_F64) {
        if (inverse) pfft3d_run<double, true>((const double*)d_in, (double*)d_out, n, count, dx, tw, st);
        else pfft3d_run<double, false>((const double*)d_in, (double*)d_out, n, count, dx, tw, st);
    } else {
        if (inverse) pfft3d_run<float, true>((const float*)d_in, (float*)d_out, n, count, dx, tw, st);
        else pfft3d_run<float, false>((const float*)d_in, (float*)d_out, n, count, dx, tw, st);
    }
    FDM_API_END
}

int fdmgpu_pfft_device(int dtype, int N, int inverse, int nlines, double dx, void* d_out, const void* d_in,
                       void* stream) {
    FDM_API_BEGIN
    if (!d_out || !d_in) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (!pow2_periodic(N)) FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: N must be a power of two in [2, 512], got %d", N);
    if (nlines < 1) FDM_FAIL(FDMGPU_EINVAL, "nlines must be positive");
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    cudaStream_t st = (cudaStream_t)stream;
    const void* tw = pfft3d_twiddles(dtype, N);
    const PLineGeom g{nlines, 1, N, 0, 1};
    if (dtype == FDMGPU_F64) {
        if (inverse) launch_pfft<double, true>((const double*)d_in, (double*)d_out, g, N, tw, dx, st);
        else launch_pfft<double, false>((const double*)d_in, (double*)d_out, g, N, tw, dx, st);
    } else {
        if (inverse) launch_pfft<float, true>((const float*)d_in, (float*)d_out, g, N, tw, dx, st);
        else launch_pfft<float, false>((const float*)d_in, (float*)d_out, g, N, tw, dx, st);
    }
    FDM_API_END
}

int fdmgpu_pfft3d(int dtype, int n, int inverse, double dx, void* out, const void* in) {
    FDM_API_BEGIN
    if (!out || !in) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (!pow2_periodic(n)) FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N) failed: N must be a power of two in [2, 512], got %d", n);
    const size_t bytes = (size_t)n * n * n * (dtype == FDMGPU_F64 ? sizeof(double) : sizeof(float));
    DevBuf din, dout;
    FDM_CUDA(cudaMemcpy(din.get(bytes), in, bytes, cudaMemcpyHostToDevice));
    const int rc = fdmgpu_pfft3d_device(dtype, n, inverse, dx, dout.get(bytes), din.p, 1, nullptr);
    if (rc) return rc;
    FDM_CUDA(cudaMemcpy(out, dout.p, bytes, cudaMemcpyDeviceToHost));
    FDM_API_END
}

int fdmgpu_sine_tc_device(int N, int axis, int nx, long long count, double scale, void* d_out, const void* d_in,
                          void* stream) {
    FDM_API_BEGIN
    if (!d_out || !d_in) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (!tc_supported(N)) FDM_FAIL(FDMGPU_ESIZE, "tensor-core DST supports N = 32, 64, 128 (got %d)", N);
    if (count < 1 || (axis != 0 && axis != 1) || (axis == 1 && nx < 1))
        FDM_FAIL(FDMGPU_EINVAL, "bad axis, nx or count");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float> h = tc_sine_image(N);
    DevBuf img, err;
    img.get(h.size() * sizeof(float));
    err.get(sizeof(int));
    FDM_CUDA(cudaMemcpy(img.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    FDM_CUDA(cudaMemset(err.p, 0, sizeof(int)));
    if (axis == 0)
        launch_sine_tc<0>(N, (const float*)d_in, (float*)d_out, count, N - 1, (const float*)img.p, scale,
                          (int*)err.p, st);
    else
        launch_sine_tc<1>(N, (const float*)d_in, (float*)d_out, count * nx, nx, (const float*)img.p, scale,
                          (int*)err.p, st);
    FDM_CUDA(cudaStreamSynchronize(st));
    int failed = 0;
    FDM_CUDA(cudaMemcpy(&failed, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (failed) FDM_FAIL(FDMGPU_ETIMEOUT, "tensor-core DST: the wait for the MMAs gave up");
    FDM_API_END
}

int fdmgpu_check_bounded_wait(unsigned spins) {
    FDM_API_BEGIN
    if (spins < 1 || spins > (1u << 20)) FDM_FAIL(FDMGPU_EINVAL, "spins must be in [1, 2^20]");
    DevBuf flag;
    flag.get(sizeof(int));
    FDM_CUDA(cudaMemset(flag.p, 0xff, sizeof(int)));
    k_bounded_wait_check<<<1, 32>>>(spins, (int*)flag.p);
    FDM_LAUNCH_CHECK();
    int gave_up = -1;
    FDM_CUDA(cudaMemcpy(&gave_up, flag.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (gave_up == 1) FDM_FAIL(FDMGPU_ETIMEOUT, "bounded wait gave up after %u tries (nothing arrived)", spins);
    if (gave_up != 0) FDM_FAIL(FDMGPU_ECUDA, "bounded-wait check did not run");
    FDM_API_END
}

int fdmgpu_lapl_cube_set_schedule(fdmgpu_lapl_cube* h, int ztable, int dst_tc) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if ((ztable != 0 && ztable != 1) || dst_tc < 0 || dst_tc > 3) FDM_FAIL(FDMGPU_EINVAL, "ztable 0/1, dst_tc 0..3");
    h->plan.zmode = ztable;
    h->plan.dst_tc = dst_tc;
    FDM_API_END
}

int fdmgpu_lapl_cube_tune(fdmgpu_lapl_cube* h, void* d_ans, const void* d_rhs, int nrhs, void* stream,
                          double* ms) {
    FDM_API_BEGIN
    if (!h || !d_ans || !d_rhs) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (nrhs < 1) FDM_FAIL(FDMGPU_EINVAL, "nrhs must be positive");
    const double t = h->plan.tune(d_ans, d_rhs, nrhs, (cudaStream_t)stream);
    if (ms) *ms = t;
    FDM_API_END
}

int fdmgpu_lapl_cube_get_schedule(fdmgpu_lapl_cube* h, int* pipeline, int* ztable, int* dst_tc) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (pipeline) *pipeline = h->plan.pipeline;
    if (ztable) *ztable = h->plan.zmode;
    if (dst_tc) *dst_tc = h->plan.tc_mask();
    FDM_API_END
}

int fdmgpu_lapl_cube_set_refinement(fdmgpu_lapl_cube* h, int adaptive) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (adaptive != 0 && adaptive != 1) FDM_FAIL(FDMGPU_EINVAL, "adaptive must be 0 or 1");
    h->plan.refine_adaptive = adaptive;
    FDM_API_END
}

int fdmgpu_lapl_cube_set_pipeline(fdmgpu_lapl_cube* h, int pipeline) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (pipeline != FDMGPU_PIPE_FIVE_PASS && pipeline != FDMGPU_PIPE_PLANES)
        FDM_FAIL(FDMGPU_EINVAL, "pipeline must be FDMGPU_PIPE_FIVE_PASS or FDMGPU_PIPE_PLANES");
    h->plan.pipeline = pipeline;
    FDM_API_END
}

int fdmgpu_lapl_cube_pipeline_in_use(fdmgpu_lapl_cube* h, int* pipeline) {
    FDM_API_BEGIN
    if (!h || !pipeline) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    CubePlan& p = h->plan;
    *pipeline = (!p.periodic && p.dtype == FDMGPU_F64 && p.precision == FDMGPU_MIXED && p.mixed_ok && p.plane_ok())
                    ? FDMGPU_PIPE_PLANES
                    : FDMGPU_PIPE_FIVE_PASS;
    FDM_API_END
}

int fdmgpu_lapl_cube_device_status(fdmgpu_lapl_cube* h, int* failed) {
    FDM_API_BEGIN
    if (!h || !failed) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    *failed = 0;
    if (h->plan.tc_err.p) {
        FDM_CUDA(cudaDeviceSynchronize());
        FDM_CUDA(cudaMemcpy(failed, h->plan.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    }
    FDM_API_END
}

int fdmgpu_tridiag_device(int dtype, int n, int nsys, const void* d_lower, const void* d_diag, const void* d_upper,
                          void* d_b, void* stream) {
    FDM_API_BEGIN
    if (!d_lower || !d_diag || !d_upper || !d_b) FDM_FAIL(FDMGPU_EINVAL, "null argument");
    if (n < 1 || nsys < 1) FDM_FAIL(FDMGPU_EINVAL, "n and nsys must be positive");
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf work;
    const int blocks = (nsys + 127) / 128;
    FDM_TIMED("tridiag_general", st);
    if (dtype == FDMGPU_F64) {
        double* cw = (double*)work.get((size_t)n * nsys * sizeof(double));
        k_tridiag_general<double><<<blocks, 128, 0, st>>>(n, nsys, (const double*)d_lower, (const double*)d_diag,
                                                          (const double*)d_upper, (double*)d_b, cw);
    } else if (dtype == FDMGPU_F32) {
        float* cw = (float*)work.get((size_t)n * nsys * sizeof(float));
        k_tridiag_general<float><<<blocks, 128, 0, st>>>(n, nsys, (const float*)d_lower, (const float*)d_diag,
                                                         (const float*)d_upper, (float*)d_b, cw);
    } else {
        FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    }
    FDM_LAUNCH_CHECK();
    FDM_CUDA(cudaStreamSynchronize(st));
    FDM_API_END
}

int fdmgpu_check_dd_conversions(long long n, const double* d_x, const float* d_hi, const float* d_lo, float* d_f32,
                                float* d_f32_hw, float* d_split_hi, float* d_split_lo, double* d_f64, double* d_f64_hw,
                                void* stream) {
    FDM_API_BEGIN
    if (n < 0 || (n > 0 && (!d_x || !d_hi || !d_lo || !d_f32 || !d_f32_hw || !d_split_hi || !d_split_lo || !d_f64 ||
                            !d_f64_hw)))
        FDM_FAIL(FDMGPU_EINVAL, "bad argument");
    if (n == 0) return FDMGPU_OK;
    k_dd_check<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_x, d_hi, d_lo, n, d_f32, d_f32_hw,
                                                                              d_split_hi, d_split_lo, d_f64, d_f64_hw);
    FDM_LAUNCH_CHECK();
    FDM_API_END
}

}  // extern "C"
