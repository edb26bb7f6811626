// DST-I of short lines (N = 32, 64, 128: n = N-1 = 31, 63, 127 points) as a dense
// contraction on the 5th-generation tensor cores.
//
//   Y[l][k] = scale * sum_j X[l][j] sin(pi (j+1)(k+1) / N),  j, k < n
//
// is Y = X S with S symmetric (the reference computes the same transform
// with its real recursion, FFT<T>::sFFT, src/fft.cpp:294-365).  A CTA of
// 256 threads owns 128 lines at a time: the lines (M = 128) are the A
// operand, S (N x N, zero-padded at index n) the B operand, both K-major in
// shared memory in the 128-byte swizzled layout; one elected thread issues
// tcgen05.mma (kind::tf32, FP32 accumulators in tensor memory) and commits
// to an mbarrier; each warp then reads its 32 accumulator rows with
// tcgen05.ld.  FP32 accuracy comes from splitting both operands into TF32
// high and low parts: X S ~ Xh Sh + Xh Sl + Xl Sh (the dropped Xl Sl term
// and the TF32 rounding of the low parts are ~2^-22 relative).
//
// AXIS 0: lines along x (contiguous, stride n), AXIS 1: lines along y of
// each z-plane (stride nx), line index (plane, x).  In-place use is safe: a
// CTA reads all of its lines before it writes any of them.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fdmgpu {

struct SineTcGeom {
    long long lines;  // lines over all volumes
    int nx;           // AXIS 1: points per x-row (the line index is plane * nx + x)
    long long plane;  // AXIS 1: elements per z-plane (nx * n)
};

template <int N>
struct TcCfg {
    static constexpr int n = N - 1;
    static constexpr int M = 128;                          // lines per tile
    static constexpr int KB = N > 64 ? 64 : N;             // K values of the line tile held at a time
    static constexpr int NKB = N / KB;                     // K blocks per tile
    static constexpr int kSBytes = N * N * 4;              // one TF32 part of S
    static constexpr int kABytes = M * KB * 4;             // one TF32 part of a K block of the line tile
    static constexpr int kStage = M * n * 4;               // AXIS 0 output staging (reuses the A parts)
    static constexpr int kSmem = 1024 /*align*/ + 2 * kSBytes + 2 * kABytes + 64;
    static_assert(2 * kABytes >= kStage, "staging must fit in the A parts");
    static_assert(2 * kABytes >= M * (KB + 1) * 4, "K-block staging must fit in the A parts");
};

// byte offset of element (r, k) in a K-major, 128-byte-swizzled operand of
// `rows` rows: 8-row x 128-byte atoms, atom columns of 32 K values, the
// 16-byte chunk index XORed with the row within the atom
__host__ __device__ __forceinline__ uint32_t tc_sw128(int rows, int r, int k) {
    const uint32_t kb = (uint32_t)k >> 5, c = ((uint32_t)k >> 2) & 7, e = (uint32_t)k & 3;
    return kb * (uint32_t)rows * 128u + ((uint32_t)r >> 3) * 1024u + ((uint32_t)r & 7) * 128u +
           ((c ^ ((uint32_t)r & 7)) << 4) + (e << 2);
}

// TF32 rounding of an FP32 value (to nearest on the 13 dropped bits)
__host__ __device__ __forceinline__ float tc_tf32(float x) {
#ifdef __CUDA_ARCH__
    uint32_t u = __float_as_uint(x);
    u = (u + 0x1000u) & 0xFFFFE000u;
    return __uint_as_float(u);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;
    float y;
    memcpy(&y, &u, 4);
    return y;
#endif
}

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory operand descriptor: start address, SBO = 1024 (8-row
// groups), 128-byte swizzle, descriptor version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ bool tc_try_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
#endif

// Spin limit of the MMA-completion wait (each try_wait may itself suspend
// for a while); on expiry the kernel records a failure and returns.
constexpr unsigned kTcSpinLimit = 1u << 24;

constexpr int kTcThreads = 256;

// Diagnostic of the bounded wait the tensor-core kernels use: one thread
// waits on an mbarrier that nothing arrives at, with the same try_wait loop
// and a caller-given spin limit, and reports whether it gave up (1) or saw
// the phase complete (0).  It ends after `spins` tries either way.
__global__ void k_bounded_wait_check(unsigned spins, int* gave_up) {
#if defined(__CUDA_ARCH__)
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(&mbar)), "r"(1));
        unsigned n = 0;
        bool done = false;
        while (!(done = tc_try_wait(tc_smem(&mbar), 0)) && ++n < spins) {
        }
        *gave_up = done ? 0 : 1;
    }
#endif
}

template <int N, int AXIS>
__global__ void __launch_bounds__(kTcThreads, (N == 32 ? 3 : 2))
    k_sine_tc(const float* in, float* out, SineTcGeom g, const float* __restrict__ simg, float scale, int* err) {
#if defined(__CUDA_ARCH__)
    using C = TcCfg<N>;
    constexpr int n = C::n, M = C::M, T = kTcThreads;
    // each thread owns half a line of the tile: line r = tid % 128, values
    // k in [KH*h, KH*h + KH) with h = tid / 128
    constexpr int KH = N / 2;
    // AXIS 0 reads the tile as one contiguous, 16-byte aligned run of M*n
    // values: float4 loads
    constexpr int kF4 = (M * n / 4 + T - 1) / T;
    extern __shared__ unsigned char tc_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* s_hi = base;
    unsigned char* s_lo = base + C::kSBytes;
    unsigned char* a_hi = base + 2 * C::kSBytes;
    unsigned char* a_lo = a_hi + C::kABytes;
    float* raw_in = (float*)a_lo;   // AXIS 0: the tile as read, M*n values
    float* raw_out = (float*)a_hi;  // AXIS 0: the tile as written
    uint64_t* mbar = (uint64_t*)(a_hi + 2 * C::kABytes);
    uint32_t* tslot = (uint32_t*)(mbar + 1);
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r = tid & (M - 1), kh = (tid >> 7) * KH;
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(mbar)), "r"(1));
    }
    // S (both parts) arrives pre-swizzled: a straight 16-byte copy
    {
        const float4* src = (const float4*)simg;
        float4* dst = (float4*)s_hi;
        for (int i = tid; i < 2 * C::kSBytes / 16; i += T) dst[i] = __ldg(src + i);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)),
                     "r"(N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    // D f32, A/B tf32, K-major both, N columns, M = 128
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
    const uint32_t sa_hi = tc_smem(a_hi), sa_lo = tc_smem(a_lo), ss_hi = tc_smem(s_hi), ss_lo = tc_smem(s_lo);
    const uint32_t mb = tc_smem(mbar);
    const long long ntiles = (g.lines + M - 1) / M;
    uint32_t phase = 0;

    // the loads of a tile go to registers one tile ahead: they are in flight
    // while the previous tile's MMAs and epilogue run
    constexpr int kRegs = AXIS == 0 ? 4 * kF4 : KH;
    float v[kRegs];
    auto fetch = [&](long long tile) {
        const long long L0 = tile * M;
        const int rows = (int)(g.lines - L0 < M ? g.lines - L0 : M);
        if (AXIS == 0) {
            const float* src = in + L0 * n;
            const int cnt = rows * n;
#pragma unroll
            for (int j = 0; j < kF4; j++) {
                const int q = tid + j * T;
                float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                if (4 * q + 3 < cnt) {
                    x = __ldg((const float4*)src + q);
                } else if (4 * q < cnt) {
                    x.x = src[4 * q];
                    if (4 * q + 1 < cnt) x.y = src[4 * q + 1];
                    if (4 * q + 2 < cnt) x.z = src[4 * q + 2];
                }
                v[4 * j] = x.x; v[4 * j + 1] = x.y; v[4 * j + 2] = x.z; v[4 * j + 3] = x.w;
            }
        } else {
            const bool ok = r < rows;
            const long long L = L0 + r;
            const long long p = ok ? L / g.nx : 0;
            const float* src = in + p * g.plane + (ok ? L - p * g.nx : 0);
#pragma unroll
            for (int j = 0; j < KH; j++) {
                const int k = kh + j;
                v[j] = (ok && k < n) ? src[(long long)k * g.nx] : 0.f;
            }
        }
    };
    // 16-byte chunks of this thread's half line -> TF32 high / low parts
    auto put_half = [&](const float* w) {
        const uint32_t rowoff = ((uint32_t)r >> 3) * 1024u + ((uint32_t)r & 7) * 128u;
#pragma unroll
        for (int c = 0; c < KH / 4; c++) {
            const int k = kh + 4 * c;
            const uint32_t o = (uint32_t)(k >> 5) * (uint32_t)M * 128u + rowoff +
                               ((((uint32_t)k >> 2) & 7) ^ ((uint32_t)r & 7)) * 16u;
            float4 h, l;
            h.x = tc_tf32(w[4 * c]);     l.x = tc_tf32(w[4 * c] - h.x);
            h.y = tc_tf32(w[4 * c + 1]); l.y = tc_tf32(w[4 * c + 1] - h.y);
            h.z = tc_tf32(w[4 * c + 2]); l.z = tc_tf32(w[4 * c + 2] - h.z);
            h.w = tc_tf32(w[4 * c + 3]); l.w = tc_tf32(w[4 * c + 3] - h.w);
            *(float4*)(a_hi + o) = h;
            *(float4*)(a_lo + o) = l;
        }
    };
    if (blockIdx.x < ntiles) fetch(blockIdx.x);

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long L0 = tile * M;
        const int rows = (int)(g.lines - L0 < M ? g.lines - L0 : M);
        // ---- registers -> A (TF32 high and low parts), zero padding at k = n
        if (AXIS == 0) {
            // through the tile's raw image: linear in, half lines out
#pragma unroll
            for (int j = 0; j < kF4; j++) {
                const int q = tid + j * T;
                if (q < M * n / 4) ((float4*)raw_in)[q] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
            __syncthreads();
            float w[KH];
#pragma unroll
            for (int j = 0; j < KH; j++) w[j] = (kh + j < n) ? raw_in[r * n + kh + j] : 0.f;
            __syncthreads();
            put_half(w);
        } else {
            put_half(v);
        }
        tc_fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // ---- Y = Ah Sh + Ah Sl + Al Sh, K = N in steps of 8
        if (tid == 0) {
#pragma unroll 1
            for (int part = 0; part < 3; part++) {
                const uint32_t a = part == 2 ? sa_lo : sa_hi;
                const uint32_t b = part == 1 ? ss_lo : ss_hi;
#pragma unroll
                for (int s = 0; s < N / 8; s++) {
                    const int k0 = s * 8;
                    const uint32_t koff_a = (uint32_t)(k0 >> 5) * M * 128u + (uint32_t)((k0 & 31) >> 3) * 32u;
                    const uint32_t koff_b = (uint32_t)(k0 >> 5) * N * 128u + (uint32_t)((k0 & 31) >> 3) * 32u;
                    tc_mma_tf32(tmem, tc_desc(a + koff_a), tc_desc(b + koff_b), idesc, (part | s) != 0);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        if (tile + gridDim.x < ntiles) fetch(tile + gridDim.x);
        // ---- bounded wait for the MMAs
        {
            unsigned spins = 0;
            bool done = false;
            while (!(done = tc_try_wait(mb, phase)) && ++spins < kTcSpinLimit) {
            }
            if (!done) s_fail = 1;
        }
        phase ^= 1;
        tc_fence_after();
        __syncthreads();
        if (s_fail) break;
        // ---- accumulators -> output: warp w reads TMEM lanes 32(w%4).. and
        // half (w/4) of the columns
        const int er = (warp & 3) * 32 + lane;
        const long long L = L0 + er;
        const int cbeg = (warp >> 2) * (N / 2);
#pragma unroll 1
        for (int c0 = cbeg; c0 < cbeg + N / 2; c0 += 16) {
            float y[16];
            tc_ld16(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0, y);
            if (AXIS == 0) {
                // the tile as written (line stride n is odd: no bank conflicts)
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c0 + j < n) raw_out[er * n + c0 + j] = y[j] * scale;
            } else if (er < rows) {
                const long long p = L / g.nx;
                float* dst = out + p * g.plane + (L - p * g.nx);
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c0 + j < n) dst[(long long)(c0 + j) * g.nx] = y[j] * scale;
            }
        }
        tc_fence_before();
        __syncthreads();
        if (AXIS == 0) {
            const int cnt = rows * n;
            float* dst = out + L0 * n;
            for (int q = tid; 4 * q < cnt; q += T) {
                if (4 * q + 3 < cnt) {
                    ((float4*)dst)[q] = ((const float4*)raw_out)[q];
                } else {
                    for (int i = 4 * q; i < cnt; i++) dst[i] = raw_out[i];
                }
            }
            __syncthreads();
        }
        tc_fence_after();
    }
    if (s_fail && tid == 0) atomicExch(err, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(N));
#endif
}

// N = 128: the split-TF32 sine matrix (128 KB) stays in shared memory and
// the line tile goes through in two K blocks of 64 (64 KB for both parts);
// the MMAs of a block accumulate onto the previous block's in TMEM.  One
// CTA per SM (193 KB of shared memory).  Each K block is read coalesced
// into a padded staging image, then redistributed as half-rows (AXIS 0), or
// read straight into half-rows (AXIS 1); the next block's loads are in
// registers while the current block's MMAs run.
template <int AXIS>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_sine_tc128(const float* in, float* out, SineTcGeom g, const float* __restrict__ simg, float scale, int* err) {
#if defined(__CUDA_ARCH__)
    constexpr int N = 128;
    using C = TcCfg<N>;
    constexpr int n = C::n, M = C::M, T = kTcThreads, KB = C::KB, NKB = C::NKB;
    constexpr int KH = KB / 2;          // values of a half-row of one K block
    constexpr int KS = KB + 1;          // padded row stride of the AXIS 0 staging
    constexpr int kLd = M * KB / T;     // AXIS 0 loads per thread per K block
    extern __shared__ unsigned char tc_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* s_hi = base;
    unsigned char* s_lo = base + C::kSBytes;
    unsigned char* a_hi = base + 2 * C::kSBytes;
    unsigned char* a_lo = a_hi + C::kABytes;
    float* raw = (float*)a_hi;  // AXIS 0: one K block as read / the tile as written
    uint64_t* mbar = (uint64_t*)(a_hi + 2 * C::kABytes);
    uint32_t* tslot = (uint32_t*)(mbar + 1);
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r = tid & (M - 1), kh = (tid >> 7) * KH;
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(mbar)), "r"(1));
    }
    {
        const float4* src = (const float4*)simg;
        float4* dst = (float4*)s_hi;
        for (int i = tid; i < 2 * C::kSBytes / 16; i += T) dst[i] = __ldg(src + i);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)),
                     "r"(N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
    const uint32_t sa_hi = tc_smem(a_hi), sa_lo = tc_smem(a_lo), ss_hi = tc_smem(s_hi), ss_lo = tc_smem(s_lo);
    const uint32_t mb = tc_smem(mbar);
    const long long ntiles = (g.lines + M - 1) / M;
    uint32_t phase = 0;

    constexpr int kRegs = AXIS == 0 ? kLd : KH;
    float v[kRegs];
    // loads of K block kb of a tile into registers
    auto fetch = [&](long long tile, int kb) {
        const long long L0 = tile * M;
        const int rows = (int)(g.lines - L0 < M ? g.lines - L0 : M);
        if (AXIS == 0) {
#pragma unroll
            for (int j = 0; j < kLd; j++) {
                const int e = tid + j * T, line = e / KB, c = e - line * KB, k = kb * KB + c;
                v[j] = (line < rows && k < n) ? in[(L0 + line) * n + k] : 0.f;
            }
        } else {
            const bool ok = r < rows;
            const long long L = L0 + r;
            const long long p = ok ? L / g.nx : 0;
            const float* src = in + p * g.plane + (ok ? L - p * g.nx : 0);
#pragma unroll
            for (int j = 0; j < KH; j++) {
                const int k = kb * KB + kh + j;
                v[j] = (ok && k < n) ? src[(long long)k * g.nx] : 0.f;
            }
        }
    };
    // this thread's half-row of the current K block -> TF32 parts
    auto put_half = [&](const float* w) {
        const uint32_t rowoff = ((uint32_t)r >> 3) * 1024u + ((uint32_t)r & 7) * 128u;
#pragma unroll
        for (int c = 0; c < KH / 4; c++) {
            const int k = kh + 4 * c;  // within the block
            const uint32_t o = (uint32_t)(k >> 5) * (uint32_t)M * 128u + rowoff +
                               ((((uint32_t)k >> 2) & 7) ^ ((uint32_t)r & 7)) * 16u;
            float4 h, l;
            h.x = tc_tf32(w[4 * c]);     l.x = tc_tf32(w[4 * c] - h.x);
            h.y = tc_tf32(w[4 * c + 1]); l.y = tc_tf32(w[4 * c + 1] - h.y);
            h.z = tc_tf32(w[4 * c + 2]); l.z = tc_tf32(w[4 * c + 2] - h.z);
            h.w = tc_tf32(w[4 * c + 3]); l.w = tc_tf32(w[4 * c + 3] - h.w);
            *(float4*)(a_hi + o) = h;
            *(float4*)(a_lo + o) = l;
        }
    };
    if (blockIdx.x < ntiles) fetch(blockIdx.x, 0);

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long L0 = tile * M;
        const int rows = (int)(g.lines - L0 < M ? g.lines - L0 : M);
#pragma unroll 1
        for (int kb = 0; kb < NKB; kb++) {
            if (AXIS == 0) {
#pragma unroll
                for (int j = 0; j < kLd; j++) {
                    const int e = tid + j * T, line = e / KB, c = e - line * KB;
                    raw[line * KS + c] = v[j];
                }
                __syncthreads();
                float w[KH];
#pragma unroll
                for (int j = 0; j < KH; j++) w[j] = raw[r * KS + kh + j];
                __syncthreads();
                put_half(w);
            } else {
                put_half(v);
            }
            tc_fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
#pragma unroll 1
                for (int part = 0; part < 3; part++) {
                    const uint32_t a = part == 2 ? sa_lo : sa_hi;
                    const uint32_t b = part == 1 ? ss_lo : ss_hi;
#pragma unroll
                    for (int s = 0; s < KB / 8; s++) {
                        const int k0 = s * 8;               // within the block (A)
                        const int kg = kb * KB + k0;        // within S (B)
                        const uint32_t koff_a = (uint32_t)(k0 >> 5) * M * 128u + (uint32_t)((k0 & 31) >> 3) * 32u;
                        const uint32_t koff_b = (uint32_t)(kg >> 5) * N * 128u + (uint32_t)((kg & 31) >> 3) * 32u;
                        tc_mma_tf32(tmem, tc_desc(a + koff_a), tc_desc(b + koff_b), idesc, (kb | part | s) != 0);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                             : "memory");
            }
            if (kb + 1 < NKB) fetch(tile, kb + 1);
            else if (tile + gridDim.x < ntiles) fetch(tile + gridDim.x, 0);
            {
                unsigned spins = 0;
                bool done = false;
                while (!(done = tc_try_wait(mb, phase)) && ++spins < kTcSpinLimit) {
                }
                if (!done) s_fail = 1;
            }
            phase ^= 1;
            tc_fence_after();
            __syncthreads();
            if (s_fail) break;
        }
        if (s_fail) break;
        // ---- accumulators -> output: warp w reads lanes 32(w%4).. and half (w/4) of the columns
        const int er = (warp & 3) * 32 + lane;
        const long long L = L0 + er;
        const int cbeg = (warp >> 2) * (N / 2);
#pragma unroll 1
        for (int c0 = cbeg; c0 < cbeg + N / 2; c0 += 16) {
            float y[16];
            tc_ld16(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0, y);
            if (AXIS == 0) {
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c0 + j < n) raw[er * n + c0 + j] = y[j] * scale;
            } else if (er < rows) {
                const long long p = L / g.nx;
                float* dst = out + p * g.plane + (L - p * g.nx);
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (c0 + j < n) dst[(long long)(c0 + j) * g.nx] = y[j] * scale;
            }
        }
        tc_fence_before();
        __syncthreads();
        if (AXIS == 0) {
            const int cnt = rows * n;
            float* dst = out + L0 * n;
            for (int q = tid; 4 * q < cnt; q += T) {
                if (4 * q + 3 < cnt) {
                    ((float4*)dst)[q] = ((const float4*)raw)[q];
                } else {
                    for (int i = 4 * q; i < cnt; i++) dst[i] = raw[i];
                }
            }
            __syncthreads();
        }
        tc_fence_after();
    }
    if (s_fail && tid == 0) atomicExch(err, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(N));
#endif
}

}  // namespace fdmgpu
