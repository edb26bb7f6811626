// Particle-mesh N-body driver around the periodic LaplCube: the GPU form of
// the reference's NBody<T,check,CIC3<T>> (test/nbody.cpp:25-511).
//
// A step is calc_a_pm then move (test/nbody.cpp:134-143):
//   1. k_nb_cic     per body: cloud-in-cell corner and eight weights
//                   (CIC3<T>::distribute, src/interpolate.h:66-96), the cell
//                   indices NBody::move assigns, and the bin keys below;
//   2. counting sort of the bodies into bins, each bin in ascending body
//                   index (the order of the reference's cell lists):
//                   k_nb_scan_* (exclusive scan of the bin counts), k_nb_fill,
//                   k_nb_sort_small / k_nb_sort_big; k_nb_shares lays out the
//                   deposited bodies' CIC shares m M in that order;
//   3. k_nb_deposit per grid point: f = -M/l^3 plus the CIC shares of the
//                   bodies that distribute_masses visits, gathered in its
//                   order, and rhs = 4 G pi f / h^3 (test/nbody.cpp:275-305);
//   4. the periodic LaplCube solve of rhs into psi (poisson.cu);
//   5. k_nb_efield  E = -grad psi, Hockney's 4/3 blend of the 2nd and 4th
//                   order differences (test/nbody.cpp:327-342);
//   6. k_nb_pp      (local only) the short-range pair forces over the 27
//                   neighbour cells of the pp grid (test/nbody.cpp:353-419);
//   7. k_nb_accel   a = F + sum_corners E M (calc_accelerations, :431-470),
//                   fused with the velocity-Verlet move (:472-511).
// The sequence is captured into a CUDA graph after the first step.
//
// Bins.  distribute_masses (test/nbody.cpp:243-258) walks, for off = 0 then
// 1, only the cells whose three indices are all congruent to off mod 2 (two
// of the eight parity classes), each cell's bodies in index order.  Bodies
// are therefore binned by (pass, CIC corner cell), pass = that class or
// none; a grid point gathers pass 0 then pass 1 over the eight corner cells
// that cover it.  With the reference's own cell formula equal to the CIC
// corner (always in double; in float except where a quotient rounds onto a
// cell face) each point sees one non-empty bin per pass, summed in the
// reference's order, so the density is bit-identical to the reference's.
// The pp grid has its own bins (key offset 2 n^3).
//
// Arithmetic follows the reference's C++ types (T stored, double where a
// driver parameter enters) with explicit round-to-nearest operations, so no
// multiply-add is contracted where the reference's source has none.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "poisson.h"

namespace fdmgpu {
namespace nb {

template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
template <>
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
template <typename T>
__device__ __forceinline__ T sub_rn(T a, T b);
template <>
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
template <>
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// a / b in T: FP64 through cdiv, FP32 by the (fast) IEEE float division
__device__ __forceinline__ double tdiv(double a, CDiv d) { return cdiv(a, d); }
__device__ __forceinline__ float tdiv(float a, CDiv d) { return a / (float)d.b; }

__host__ __device__ __forceinline__ int wrap(int v, int n) {
    v %= n;
    return v < 0 ? v + n : v;
}
__host__ __device__ __forceinline__ int pack3(int z, int y, int x) { return (z << 20) | (y << 10) | x; }
__device__ __forceinline__ void unpack3(int p, int& z, int& y, int& x) {
    z = p >> 20;
    y = (p >> 10) & 1023;
    x = p & 1023;
}

template <typename T>
struct Params {
    T org[3];       // origin, in T
    T hT;           // h as the CIC3 argument (T)
    T lT;           // l as a pp image offset (T)
    T f0;           // -M / l / l / l, stored to T
    T beta;         // 4/3 in T
    double l, h, hpp;
    double dt, hdt, hdt2;  // dt, 0.5 dt, 0.5 dt dt
    double G, rcrit, rhs_scale, sqrtpi;
    CDiv dhT, dh, dhpp, drc, dsqrtpi;  // h in T (the CIC3 argument), h, l / npp, rcrit, sqrt(pi)
    // R^2 < r2_in exactly when sqrt(R^2) + 0.001 < rcrit in double (both
    // operations correctly rounded and monotone, so the range test of
    // apply_bi_bj is a threshold on R^2, found by bisection over doubles)
    double r2_in;
    int n, npp, N, local, sgn;
    int lists_empty;  // the cell lists hold no bodies: nothing deposits, no pair forces
    long long n3;
    long long dep_bins;  // 2 n^3
};

// SoA body arrays: component m of body b at [m * N + b]
template <typename T>
struct Bodies {
    T *x, *v, *a, *ap, *F, *mass;
};

// 1. CIC weights (body-major: M[b * 8 + 4 i + 2 k + j]), corner cell, list
// cells and the bin keys
template <typename T>
__global__ void __launch_bounds__(256) k_nb_cic(Bodies<T> B, Params<T> P, T* __restrict__ M, int* __restrict__ corner,
                                                int* __restrict__ pcell, int* __restrict__ key, int* __restrict__ count) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.N) return;
    const int N = P.N, n = P.n;
    int c[3], lc[3], pc[3] = {0, 0, 0};
    T w[3];
#pragma unroll
    for (int m = 0; m < 3; m++) {
        const T xx = sub_rn<T>(B.x[m * N + b], P.org[m]);
        const T q = tdiv(xx, P.dhT);
        const int ci = (int)floor(q);  // CIC3: int j = floor(x / h), h in T
        w[m] = tdiv(sub_rn<T>(xx, mul_rn<T>((T)ci, P.hT)), P.dhT);
        c[m] = wrap(ci, n);
        // NBody::move: floor((x - origin) / h) in double, the CIC quotient itself in FP64
        const double qd = sizeof(T) == 8 ? (double)q : cdiv((double)xx, P.dh);
        lc[m] = wrap((int)floor(qd), n);
        if (P.local) pc[m] = wrap((int)floor(cdiv((double)xx, P.dhpp)), P.npp);
    }
    // M[i][k][j] = w_z * w_y * w_x with w = (1 - r, r), left to right
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int bb = 0; bb < 2; bb++)
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const T wz = a ? w[2] : sub_rn<T>(T(1), w[2]);
                const T wy = bb ? w[1] : sub_rn<T>(T(1), w[1]);
                const T wx = cc ? w[0] : sub_rn<T>(T(1), w[0]);
                M[(long long)b * 8 + 4 * a + 2 * bb + cc] = mul_rn<T>(mul_rn<T>(wz, wy), wx);
            }
    corner[b] = pack3(c[2], c[1], c[0]);
    const int p0 = lc[0] & 1;
    const bool visited = !P.lists_empty && (lc[1] & 1) == p0 && (lc[2] & 1) == p0;
    int kd = -1;
    if (visited) {
        kd = (int)(p0 * P.n3 + ((long long)c[2] * n + c[1]) * n + c[0]);
        atomicAdd(&count[kd], 1);
    }
    key[b] = kd;
    if (P.local) {
        const int npp = P.npp;
        const int kp = P.lists_empty ? -1 : (int)(P.dep_bins + ((long long)pc[2] * npp + pc[1]) * npp + pc[0]);
        pcell[b] = pack3(pc[2], pc[1], pc[0]);
        key[N + b] = kp;
        if (kp >= 0) atomicAdd(&count[kp], 1);
    }
}

// 2a. exclusive scan of the bin counts: per-chunk scan, scan of the chunk
// totals, add-back.  A chunk is 1024 threads x 4 bins.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* smem, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) smem[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int s = lane < nw ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        if (lane < nw) smem[lane] = s;  // inclusive warp totals
    }
    __syncthreads();
    total = smem[(blockDim.x >> 5) - 1];
    const int base = warp ? smem[warp - 1] : 0;
    __syncthreads();
    return base + incl - v;
}

__global__ void __launch_bounds__(kScanThreads) k_nb_scan_local(const int* __restrict__ in, int* __restrict__ out,
                                                                int* __restrict__ partial, long long nbins) {
    __shared__ int smem[32];
    const long long base = (long long)blockIdx.x * kScanChunk + (long long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        v[i] = base + i < nbins ? in[base + i] : 0;
        s += v[i];
    }
    int total;
    int run = block_exclusive_scan(s, smem, total);
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < nbins) out[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

// one block: exclusive scan of the chunk totals in place; writes the grand
// total after the last bin and clears the big-bin counter of the sort
__global__ void __launch_bounds__(kScanThreads) k_nb_scan_partials(int* __restrict__ partial, int nchunks,
                                                                   int* __restrict__ end_slot,
                                                                   int* __restrict__ bigcount) {
    __shared__ int smem[32];
    int carry = 0;
    for (int b0 = 0; b0 < nchunks; b0 += kScanThreads) {
        const int i = b0 + threadIdx.x;
        const int v = i < nchunks ? partial[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, smem, total);
        if (i < nchunks) partial[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) {
        *end_slot = carry;
        *bigcount = 0;
    }
}

__global__ void __launch_bounds__(256) k_nb_scan_add(int* __restrict__ out, const int* __restrict__ partial,
                                                     long long nbins) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nbins) out[e] += partial[e / kScanChunk];
}

// 2b. place every body in its bins; the counts count back down to zero
__global__ void __launch_bounds__(256) k_nb_fill(const int* __restrict__ key, int N, int nkeys, const int* __restrict__ start,
                                                 int* __restrict__ count, int* __restrict__ sorted) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= N) return;
    for (int r = 0; r < nkeys; r++) {
        const int k = key[r * N + b];
        if (k < 0) continue;
        const int c = atomicSub(&count[k], 1);
        sorted[start[k] + c - 1] = b;
    }
}

// 2c. ascending body order inside each bin: insertion sort for bins of up
// to 32 bodies, larger bins handed to k_nb_sort_big
constexpr int kSmallBin = 32;

__global__ void __launch_bounds__(256) k_nb_sort_small(const int* __restrict__ start, long long nbins, int* __restrict__ sorted,
                                                       int* __restrict__ bigcount, int* __restrict__ biglist) {
    const long long bin = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (bin >= nbins) return;
    const int beg = start[bin], s = start[bin + 1] - beg;
    if (s <= 1) return;
    if (s > kSmallBin) {
        biglist[atomicAdd(bigcount, 1)] = (int)bin;
        return;
    }
    int* p = sorted + beg;
    for (int i = 1; i < s; i++) {
        const int v = p[i];
        int j = i - 1;
        while (j >= 0 && p[j] > v) {
            p[j + 1] = p[j];
            j--;
        }
        p[j + 1] = v;
    }
}

// Big bins (more than 32 bodies).  Each CTA takes a chunk of eight entries
// of the big-bin list: bins of up to kWarpSortMax bodies go one per warp
// (each body placed at its rank, counted by the lanes), larger ones to the
// whole CTA in turn: a bitonic network in shared memory up to kBitonicMax
// bodies (padded with INT_MAX to a power of two), a CTA-wide rank count
// beyond.
constexpr int kWarpSortMax = 256;
constexpr int kBitonicMax = 8192;
constexpr int kSortBigThreads = 256;

__device__ __forceinline__ void rank_place(const int* __restrict__ src, int* __restrict__ dst, int s, int e0,
                                           int stride) {
    for (int e = e0; e < s; e += stride) {
        const int v = src[e];
        int rank = 0;
        for (int t = 0; t < s; t++) rank += src[t] < v;
        dst[rank] = v;
    }
}

__global__ void __launch_bounds__(kSortBigThreads) k_nb_sort_big(const int* __restrict__ start, int* __restrict__ sorted,
                                                                 int* __restrict__ tmp, const int* __restrict__ bigcount,
                                                                 const int* __restrict__ biglist) {
    __shared__ int sk[kBitonicMax];
    constexpr int kWarps = kSortBigThreads / 32;
    const int nbig = *bigcount;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c0 = blockIdx.x * kWarps; c0 < nbig; c0 += gridDim.x * kWarps) {
        // small big bins: one per warp
        {
            const int w = c0 + warp;
            if (w < nbig) {
                const int bin = biglist[w];
                const int beg = start[bin], s = start[bin + 1] - beg;
                if (s <= kWarpSortMax) {
                    for (int e = lane; e < s; e += 32) tmp[beg + e] = sorted[beg + e];
                    __syncwarp();
                    rank_place(tmp + beg, sorted + beg, s, lane, 32);
                }
            }
        }
        // the chunk's larger bins, one after another with the whole CTA
        for (int q = 0; q < kWarps && c0 + q < nbig; q++) {
            const int bin = biglist[c0 + q];
            const int beg = start[bin], s = start[bin + 1] - beg;
            if (s <= kWarpSortMax) continue;
            if (s <= kBitonicMax) {
                int P = 512;
                while (P < s) P <<= 1;
                for (int e = threadIdx.x; e < P; e += blockDim.x) sk[e] = e < s ? sorted[beg + e] : INT_MAX;
                __syncthreads();
                for (int k = 2; k <= P; k <<= 1)
                    for (int jj = k >> 1; jj > 0; jj >>= 1) {
                        for (int e = threadIdx.x; e < P; e += blockDim.x) {
                            const int p = e ^ jj;
                            if (p > e) {
                                const int a = sk[e], b = sk[p];
                                const bool up = (e & k) == 0;
                                if ((a > b) == up) {
                                    sk[e] = b;
                                    sk[p] = a;
                                }
                            }
                        }
                        __syncthreads();
                    }
                for (int e = threadIdx.x; e < s; e += blockDim.x) sorted[beg + e] = sk[e];
            } else {
                for (int e = threadIdx.x; e < s; e += blockDim.x) tmp[beg + e] = sorted[beg + e];
                __syncthreads();
                rank_place(tmp + beg, sorted + beg, s, threadIdx.x, blockDim.x);
            }
            __syncthreads();
        }
    }
}

// 2d. the eight CIC shares m * M of every deposited body, laid out corner
// by corner in bin order, so the gather below walks contiguous memory
template <typename T>
__global__ void __launch_bounds__(256) k_nb_shares(const int* __restrict__ sorted, const int* __restrict__ ndep,
                                                   const T* __restrict__ mass, const T* __restrict__ M, int N,
                                                   T* __restrict__ share) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= *ndep) return;
    const int b = sorted[s];
    const T m = mass[b];
#pragma unroll
    for (int w = 0; w < 8; w++) share[(long long)w * N + s] = mul_rn<T>(m, M[(long long)b * 8 + w]);
}

// 3. density and right-hand side, gathered per grid point
template <typename T>
__global__ void __launch_bounds__(64) k_nb_deposit(Params<T> P, const T* __restrict__ share,
                                                    const int* __restrict__ start, T* __restrict__ f,
                                                    T* __restrict__ rhs) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= P.n3) return;
    const int n = P.n, N = P.N;
    const int j = (int)(e % n), k = (int)((e / n) % n), i = (int)(e / ((long long)n * n));
    // the sixteen bin bounds first (independent loads), then the bodies
    int lo[16], hi[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const int pass = q >> 3, a = (q >> 2) & 1, bb = (q >> 1) & 1, cc = q & 1;
        const long long bin = pass * P.n3 + ((long long)wrap(i - a, n) * n + wrap(k - bb, n)) * n + wrap(j - cc, n);
        lo[q] = start[bin];
        hi[q] = start[bin + 1];
    }
    T acc = P.f0;
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const T* sw = share + (long long)(q & 7) * N;
        for (int s = lo[q]; s < hi[q]; s++) acc = add_rn<T>(acc, sw[s]);
    }
    f[e] = acc;
    // 4 * G * M_PI * f / h / h / h in double
    rhs[e] = (T)cdiv(cdiv(cdiv(__dmul_rn(P.rhs_scale, (double)acc), P.dh), P.dh), P.dh);
}

// 5. E = -grad psi, periodic
template <typename T>
__global__ void __launch_bounds__(64) k_nb_efield(Params<T> P, const T* __restrict__ psi, T* __restrict__ E) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= P.n3) return;
    const int n = P.n;
    const int j = (int)(e % n), k = (int)((e / n) % n), i = (int)(e / ((long long)n * n));
    auto at = [&](int ii, int kk, int jj) {
        return psi[((long long)wrap(ii, n) * n + wrap(kk, n)) * n + wrap(jj, n)];
    };
    const T mbeta = -P.beta, obeta = sub_rn<T>(T(1), P.beta);
    T d1[3], d2[3];
    d1[0] = sub_rn<T>(at(i, k, j + 1), at(i, k, j - 1));
    d2[0] = sub_rn<T>(at(i, k, j + 2), at(i, k, j - 2));
    d1[1] = sub_rn<T>(at(i, k + 1, j), at(i, k - 1, j));
    d2[1] = sub_rn<T>(at(i, k + 2, j), at(i, k - 2, j));
    d1[2] = sub_rn<T>(at(i + 1, k, j), at(i - 1, k, j));
    d2[2] = sub_rn<T>(at(i + 2, k, j), at(i - 2, k, j));
#pragma unroll
    for (int m = 0; m < 3; m++) {
        // -beta*(d1)/2/h - (1-beta)*(d2)/4/h; halving and quartering are
        // exact scalings, the same in either form
        const double t1 = cdiv((double)mul_rn<T>(mul_rn<T>(mbeta, d1[m]), T(0.5)), P.dh);
        const double t2 = cdiv((double)mul_rn<T>(mul_rn<T>(obeta, d2[m]), T(0.25)), P.dh);
        E[m * P.n3 + e] = (T)__dsub_rn(t1, t2);
    }
}

// 6. short-range pair forces (local), per body in the reference's order.
// A thread owns a body and walks its candidates (the 27 neighbour cells,
// each cell's bodies in index order); only about one candidate in six lies
// within rcrit, so the pairs that do are queued per warp (ballot + prefix,
// which keeps each lane's pairs in its own candidate order) and their
// erfc / exp terms are evaluated 32 at a time, one pair per lane; each owner
// then adds its pairs' terms in queue order.  The result is the serial
// loop's, term for term, without paying the transcendental branch on every
// candidate of every lane.
constexpr int kPpWarps = 4;
constexpr int kPpQueue = 64;

template <typename T>
struct PpQueue {
    double R[kPpQueue];
    double t[3][kPpQueue];
    T d[3][kPpQueue];
    int bj[kPpQueue];
    unsigned char lane[kPpQueue];
};

template <typename T>
__device__ __forceinline__ void pp_flush(PpQueue<T>& q, int cnt, int lane, const Params<T>& P,
                                         const T* __restrict__ mass, T F[3]) {
    __syncwarp();
    if (lane < cnt) {
        const double R = __dadd_rn(sqrt(q.R[lane]), 0.001);  // the queue holds R^2
        // erfc(R/2/rcrit) + R/rcrit/sqrt(pi) * exp(-R*R/4/rcrit/rcrit)
        const double ex = exp(cdiv(cdiv(__dmul_rn(__dmul_rn(-R, R), 0.25), P.drc), P.drc));
        const double sh = __dadd_rn(erfc(cdiv(__dmul_rn(R, 0.5), P.drc)), __dmul_rn(cdiv(cdiv(R, P.drc), P.dsqrtpi), ex));
        const double mG = __dmul_rn((double)(-mass[q.bj[lane]]), P.G);
        const CDiv dR = cdiv_dev(R);
#pragma unroll
        for (int m = 0; m < 3; m++)
            q.t[m][lane] = __dmul_rn(cdiv(cdiv(cdiv(__dmul_rn(mG, (double)q.d[m][lane]), dR), dR), dR), sh);
    }
    __syncwarp();
    for (int e = 0; e < cnt; e++)
        if (q.lane[e] == lane)
#pragma unroll
            for (int m = 0; m < 3; m++) F[m] = (T)__dadd_rn((double)F[m], q.t[m][e]);
    __syncwarp();
}

template <typename T>
__global__ void __launch_bounds__(kPpWarps * 32) k_nb_pp(Bodies<T> B, Params<T> P, const int* __restrict__ pcell,
                                                        const int* __restrict__ start, const int* __restrict__ sorted) {
    __shared__ PpQueue<T> queues[kPpWarps];
    PpQueue<T>& q = queues[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int bi = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = bi < P.N;
    const int N = P.N, n = P.n, npp = P.npp;
    int pi = 0, pk = 0, pj = 0;
    T xi[3] = {T(0), T(0), T(0)};
    T F[3] = {T(0), T(0), T(0)};
    if (active) {
        unpack3(pcell[bi], pi, pk, pj);
#pragma unroll
        for (int m = 0; m < 3; m++) xi[m] = B.x[m * N + bi];
    }
    int cell = -1, s = 0, s1 = 0;  // candidate iterator: neighbour cell 0..26, position in its bin
    T off[3] = {T(0), T(0), T(0)};
    int qn = 0;  // queued pairs (the same in every lane)
    const unsigned lt = (1u << lane) - 1u;
    while (true) {
        bool has = false;
        int bj = -1;
        if (active) {
            while (s >= s1 && cell < 26) {
                cell++;
                const int i0 = cell / 9 - 1, k0 = (cell / 3) % 3 - 1, j0 = cell % 3 - 1;
                // image offsets as test/nbody.cpp:364-369 set them
                off[0] = (pk + k0 < 0) ? -P.lT : ((pk + k0 >= n) ? P.lT : T(0));
                off[1] = (pj + j0 < 0) ? -P.lT : ((pj + j0 >= n) ? P.lT : T(0));
                off[2] = (pi + i0 < 0) ? -P.lT : ((pi + i0 >= n) ? P.lT : T(0));
                const long long bin =
                    P.dep_bins + ((long long)wrap(pi + i0, npp) * npp + wrap(pk + k0, npp)) * npp + wrap(pj + j0, npp);
                s = start[bin];
                s1 = start[bin + 1];
            }
            if (s < s1) {
                bj = sorted[s++];
                has = true;
            }
        }
        if (!__any_sync(0xffffffffu, has)) break;
        bool inr = false;
        double R = 0;
        T d[3];
        if (has && bj != bi) {
#pragma unroll
            for (int m = 0; m < 3; m++) {
                d[m] = sub_rn<T>(xi[m], add_rn<T>(B.x[m * N + bj], off[m]));
                R = __dadd_rn(R, __dmul_rn((double)d[m], (double)d[m]));
            }
            inr = R < P.r2_in;  // sqrt(R^2) + 0.001 < rcrit, without the square root
        }
        const unsigned mask = __ballot_sync(0xffffffffu, inr);
        if (inr) {
            const int pos = qn + __popc(mask & lt);
            q.R[pos] = R;
#pragma unroll
            for (int m = 0; m < 3; m++) q.d[m][pos] = d[m];
            q.bj[pos] = bj;
            q.lane[pos] = (unsigned char)lane;
        }
        qn += __popc(mask);
        if (qn >= 32) {
            pp_flush<T>(q, 32, lane, P, B.mass, F);
            // keep the overflow, in order, at the front
            if (lane < qn - 32) {
                const int src = 32 + lane;
                q.R[lane] = q.R[src];
#pragma unroll
                for (int m = 0; m < 3; m++) q.d[m][lane] = q.d[m][src];
                q.bj[lane] = q.bj[src];
                q.lane[lane] = q.lane[src];
            }
            __syncwarp();
            qn -= 32;
        }
    }
    if (qn > 0) pp_flush<T>(q, qn, lane, P, B.mass, F);
    if (active)
#pragma unroll
        for (int m = 0; m < 3; m++) B.F[m * N + bi] = F[m];
}

// 7. accelerations, then (MOVE) the velocity-Verlet update
template <typename T, bool MOVE>
__global__ void __launch_bounds__(256) k_nb_accel(Bodies<T> B, Params<T> P, const T* __restrict__ M,
                                                  const int* __restrict__ corner, const T* __restrict__ E) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.N) return;
    const int N = P.N, n = P.n;
    int ci, ck, cj;
    unpack3(corner[b], ci, ck, cj);
    T acc[3];
#pragma unroll
    for (int m = 0; m < 3; m++) acc[m] = add_rn<T>(T(0), B.F[m * N + b]);
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int bb = 0; bb < 2; bb++)
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const long long e = ((long long)wrap(ci + a, n) * n + wrap(ck + bb, n)) * n + wrap(cj + cc, n);
                const T w = M[(long long)b * 8 + 4 * a + 2 * bb + cc];
#pragma unroll
                for (int m = 0; m < 3; m++) acc[m] = add_rn<T>(acc[m], mul_rn<T>(E[m * P.n3 + e], w));
            }
#pragma unroll
    for (int m = 0; m < 3; m++) B.a[m * N + b] = acc[m];
    if constexpr (MOVE) {
#pragma unroll
    for (int m = 0; m < 3; m++) {
        const T ap = B.ap[m * N + b];
        const double step = __dadd_rn(__dmul_rn(P.dt, (double)B.v[m * N + b]), __dmul_rn(P.hdt2, (double)ap));
        T x = (T)__dadd_rn((double)B.x[m * N + b], step);
        if (x < P.org[m]) x = (T)__dadd_rn((double)x, P.l);
        if ((double)x >= __dadd_rn((double)P.org[m], P.l)) x = (T)__dsub_rn((double)x, P.l);
        B.x[m * N + b] = x;
    }
#pragma unroll
    for (int m = 0; m < 3; m++) {
        const T ap = B.ap[m * N + b];
        const T s = add_rn<T>(acc[m], ap);
        B.v[m * N + b] = (T)__dadd_rn((double)B.v[m * N + b], __dmul_rn(P.hdt, (double)s));
        B.ap[m * N + b] = acc[m];
    }
    }
}

// calc_error's exact pair sum (test/nbody.cpp:145-170), bodies in index
// order through shared-memory tiles
constexpr int kDirectTile = 256;

template <typename T>
__global__ void __launch_bounds__(kDirectTile) k_nb_direct(Bodies<T> B, Params<T> P, T* __restrict__ Fout) {
    __shared__ T sx[3][kDirectTile];
    __shared__ T sm[kDirectTile];
    const int N = P.N;
    const int bi = blockIdx.x * blockDim.x + threadIdx.x;
    T xi[3] = {T(0), T(0), T(0)};
    if (bi < N)
        for (int m = 0; m < 3; m++) xi[m] = B.x[m * N + bi];
    T F[3] = {T(0), T(0), T(0)};
    const T sg = (T)P.sgn;
    for (int t0 = 0; t0 < N; t0 += kDirectTile) {
        const int j = t0 + threadIdx.x;
        if (j < N) {
            for (int m = 0; m < 3; m++) sx[m][threadIdx.x] = B.x[m * N + j];
            sm[threadIdx.x] = B.mass[j];
        }
        __syncthreads();
        const int cnt = min(kDirectTile, N - t0);
        if (bi < N)
            for (int u = 0; u < cnt; u++) {
                if (t0 + u == bi) continue;
                T d[3];
                double R = 0;
#pragma unroll
                for (int m = 0; m < 3; m++) {
                    d[m] = sub_rn<T>(xi[m], sx[m][u]);
                    R = __dadd_rn(R, __dmul_rn((double)d[m], (double)d[m]));
                }
                R = __dadd_rn(sqrt(R), 0.00001);
                const double mG = __dmul_rn((double)mul_rn<T>(sg, sm[u]), P.G);
                const CDiv dR = cdiv_dev(R);
#pragma unroll
                for (int m = 0; m < 3; m++)
                    F[m] = (T)__dadd_rn((double)F[m], cdiv(cdiv(cdiv(__dmul_rn(mG, (double)d[m]), dR), dR), dR));
            }
        __syncthreads();
    }
    if (bi < N)
        for (int m = 0; m < 3; m++) Fout[m * N + bi] = F[m];
}

// The smallest double R2 >= 0 with !(sqrt(R2) + 0.001 < rc): the pair test
// of apply_bi_bj (test/nbody.cpp:403-411) is then R2 < threshold.
static double pair_range_threshold(double rc) {
    auto inr = [rc](double r2) { return std::sqrt(r2) + 0.001 < rc; };
    if (!inr(0.0)) return 0.0;
    unsigned long long lo = 0, hi = 0x7ff0000000000000ull;  // bit patterns of 0 and +inf
    while (hi - lo > 1) {
        const unsigned long long mid = lo + (hi - lo) / 2;
        double v;
        std::memcpy(&v, &mid, sizeof v);
        if (inr(v)) lo = mid;
        else hi = mid;
    }
    double t;
    std::memcpy(&t, &hi, sizeof t);
    return t;
}

template <typename T>
struct Plan {
    Params<T> P{};
    int N = 0;
    double total_mass = 0;
    long long nbins = 0;
    int nkeys = 1;
    int nchunks = 0;
    long long steps_done = 0;
    int sms = 1;  // streaming multiprocessors (grid of the big-bin sort)
    // NBody's cell lists are filled by the constructor's random branch and by
    // every move, emptied at the end of calc_a_pm; the solar branch leaves
    // them empty, and so does calc_a_pm without a move (calc_error)
    bool lists_empty = false;
    cudaStream_t st = nullptr;
    DevBuf body_mem, work_mem, grid_mem;
    Bodies<T> B{};
    T *M = nullptr, *share = nullptr, *f = nullptr, *rhs = nullptr, *psi = nullptr, *E = nullptr;
    int *corner = nullptr, *pcell = nullptr, *key = nullptr, *count = nullptr, *start = nullptr, *partial = nullptr;
    int *bigcount = nullptr, *biglist = nullptr, *sorted = nullptr, *tmp = nullptr;
    fdmgpu_lapl_cube* lapl = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;

    ~Plan() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        if (lapl) fdmgpu_lapl_cube_destroy(lapl);
        if (st) cudaStreamDestroy(st);
    }

    static size_t al(size_t b) { return (b + 255) / 256 * 256; }

    void init(double x0, double y0, double z0, double l, int n, int npp, int N_, double dt, double G, int sgn, int local,
              double crit) {
        N = N_;
        P.org[0] = (T)x0; P.org[1] = (T)y0; P.org[2] = (T)z0;
        P.l = l;
        P.h = l / n;
        P.hpp = l / npp;
        P.hT = (T)P.h;
        P.lT = (T)l;
        P.beta = (T)(4. / 3.);
        P.dt = dt;
        P.hdt = 0.5 * dt;
        P.hdt2 = 0.5 * dt * dt;
        P.G = G;
        P.rcrit = P.hpp * (double)(T)crit;  // rcrit(hpp * crit), crit of type T
        P.rhs_scale = 4 * G * M_PI;
        P.sqrtpi = std::sqrt(M_PI);
        P.dhT = cdiv_of((double)P.hT);
        P.dh = cdiv_of(P.h);
        P.dhpp = cdiv_of(P.hpp);
        P.drc = cdiv_of(P.rcrit);
        P.r2_in = pair_range_threshold(P.rcrit);
        P.dsqrtpi = cdiv_of(P.sqrtpi);
        P.n = n; P.npp = npp; P.N = N; P.local = local; P.sgn = sgn;
        P.n3 = (long long)n * n * n;
        P.dep_bins = 2 * P.n3;
        nkeys = local ? 2 : 1;
        nbins = P.dep_bins + (local ? (long long)npp * npp * npp : 0);
        if (nbins >= (1LL << 30)) FDM_FAIL(FDMGPU_ESIZE, "too many cells: 2 n^3 + npp^3 = %lld", nbins);
        nchunks = (int)((nbins + kScanChunk - 1) / kScanChunk);

        char* p = (char*)body_mem.get(al(sizeof(T) * N) * 16);
        auto take = [&](size_t bytes) { char* q = p; p += al(bytes); return q; };
        B.x = (T*)take(sizeof(T) * 3 * N);
        B.v = (T*)take(sizeof(T) * 3 * N);
        B.a = (T*)take(sizeof(T) * 3 * N);
        B.ap = (T*)take(sizeof(T) * 3 * N);
        B.F = (T*)take(sizeof(T) * 3 * N);
        B.mass = (T*)take(sizeof(T) * N);
        FDM_CUDA(cudaMemset(body_mem.p, 0, body_mem.bytes));

        const size_t wbytes = al(sizeof(T) * 8 * N) * 2 + al(sizeof(int) * N) * 2 + al(sizeof(int) * 2 * N) +
                              al(sizeof(int) * nbins) + al(sizeof(int) * (nbins + 1)) + al(sizeof(int) * nchunks) +
                              al(sizeof(int)) + al(sizeof(int) * (2 * (size_t)N / (kSmallBin + 1) + 1)) +
                              al(sizeof(int) * 2 * N) * 2;
        p = (char*)work_mem.get(wbytes);
        M = (T*)take(sizeof(T) * 8 * N);
        share = (T*)take(sizeof(T) * 8 * N);
        corner = (int*)take(sizeof(int) * N);
        pcell = (int*)take(sizeof(int) * N);
        key = (int*)take(sizeof(int) * 2 * N);
        count = (int*)take(sizeof(int) * nbins);
        start = (int*)take(sizeof(int) * (nbins + 1));
        partial = (int*)take(sizeof(int) * nchunks);
        bigcount = (int*)take(sizeof(int));
        biglist = (int*)take(sizeof(int) * (2 * (size_t)N / (kSmallBin + 1) + 1));
        sorted = (int*)take(sizeof(int) * 2 * N);
        tmp = (int*)take(sizeof(int) * 2 * N);
        FDM_CUDA(cudaMemset(work_mem.p, 0, work_mem.bytes));

        p = (char*)grid_mem.get(al(sizeof(T) * P.n3) * 6);
        f = (T*)take(sizeof(T) * P.n3);
        rhs = (T*)take(sizeof(T) * P.n3);
        psi = (T*)take(sizeof(T) * P.n3);
        E = (T*)take(sizeof(T) * 3 * P.n3);
        FDM_CUDA(cudaMemset(grid_mem.p, 0, grid_mem.bytes));

        FDM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        int dev = 0;
        FDM_CUDA(cudaGetDevice(&dev));
        FDM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        // solver3(h, h, h, l, l, l, n, n, n), periodic in all three directions
        const int rc = fdmgpu_lapl_cube_create(&lapl, sizeof(T) == 8 ? FDMGPU_F64 : FDMGPU_F32, FDMGPU_PERIODIC, P.h,
                                               P.h, P.h, l, l, l, n, n, n);
        if (rc) throw Error{rc};
    }

    // NBody::G: init_points' solar branch replaces it before the first step
    void set_G(double g) {
        P.G = g;
        P.rhs_scale = 4 * g * M_PI;  // 4 * G * M_PI, left to right
    }

    void set_total_mass(double m) {
        total_mass = m;
        P.f0 = (T)(-m / P.l / P.l / P.l);
    }

    void enqueue(bool move) {
        const int T256 = 256;
        auto blocks = [](long long count, int per) { return (unsigned)((count + per - 1) / per); };
        {
            FDM_TIMED("nb_cic", st);
            k_nb_cic<T><<<blocks(N, T256), T256, 0, st>>>(B, P, M, corner, pcell, key, count);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("nb_scan_local", st);
            k_nb_scan_local<<<nchunks, kScanThreads, 0, st>>>(count, start, partial, nbins);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("nb_scan_partials", st);
            k_nb_scan_partials<<<1, kScanThreads, 0, st>>>(partial, nchunks, start + nbins, bigcount);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("nb_scan_add", st);
            k_nb_scan_add<<<blocks(nbins, T256), T256, 0, st>>>(start, partial, nbins);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("nb_fill", st);
            k_nb_fill<<<blocks(N, T256), T256, 0, st>>>(key, N, nkeys, start, count, sorted);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("nb_sort_small", st);
            k_nb_sort_small<<<blocks(nbins, T256), T256, 0, st>>>(start, nbins, sorted, bigcount, biglist);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("nb_sort_big", st);
            k_nb_sort_big<<<sms * 2, kSortBigThreads, 0, st>>>(start, sorted, tmp, bigcount, biglist);
            FDM_LAUNCH_CHECK();
        }
        {
            // deposited bodies occupy the first start[dep_bins] positions
            FDM_TIMED("nb_shares", st);
            k_nb_shares<T><<<blocks(N, T256), T256, 0, st>>>(sorted, start + P.dep_bins, B.mass, M, N, share);
            FDM_LAUNCH_CHECK();
        }
        {
            // 64-thread blocks: the mass grid is small (32^3 points at the
            // driver's defaults), so spread it over every SM
            FDM_TIMED("nb_deposit", st);
            k_nb_deposit<T><<<blocks(P.n3, 64), 64, 0, st>>>(P, share, start, f, rhs);
            FDM_LAUNCH_CHECK();
        }
        cube_solve_device(lapl, psi, rhs, 1, st);
        {
            FDM_TIMED("nb_efield", st);
            k_nb_efield<T><<<blocks(P.n3, 64), 64, 0, st>>>(P, psi, E);
            FDM_LAUNCH_CHECK();
        }
        if (P.local) {
            FDM_TIMED("nb_pp", st);
            k_nb_pp<T><<<blocks(N, kPpWarps * 32), kPpWarps * 32, 0, st>>>(B, P, pcell, start, sorted);
            FDM_LAUNCH_CHECK();
        }
        {
            FDM_TIMED("nb_accel", st);
            if (move) k_nb_accel<T, true><<<blocks(N, T256), T256, 0, st>>>(B, P, M, corner, E);
            else k_nb_accel<T, false><<<blocks(N, T256), T256, 0, st>>>(B, P, M, corner, E);
            FDM_LAUNCH_CHECK();
        }
    }

    void drop_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
    }

    // calc_a_pm without the move, eagerly
    void forces() {
        P.lists_empty = lists_empty ? 1 : 0;
        enqueue(false);
        P.lists_empty = 0;
        lists_empty = true;
    }

    void step(int k) {
        for (int s = 0; s < k; s++) {
            if (lists_empty || (!gexec && steps_done == 0)) {
                P.lists_empty = lists_empty ? 1 : 0;
                enqueue(true);
                P.lists_empty = 0;
                lists_empty = false;
            } else {
                if (!gexec) {
                    FDM_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                    try {
                        enqueue(true);
                    } catch (...) {
                        cudaGraph_t g = nullptr;
                        cudaStreamEndCapture(st, &g);
                        if (g) cudaGraphDestroy(g);
                        throw;
                    }
                    FDM_CUDA(cudaStreamEndCapture(st, &graph));
                    FDM_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
                }
                FDM_CUDA(cudaGraphLaunch(gexec, st));
            }
            steps_done++;
        }
    }
};

}  // namespace nb
}  // namespace fdmgpu

using namespace fdmgpu;

struct fdmgpu_nbody {
    int dtype = FDMGPU_F64;
    std::unique_ptr<nb::Plan<double>> d;
    std::unique_ptr<nb::Plan<float>> f;
};

namespace {

template <typename Fn>
void with_nb(fdmgpu_nbody* h, Fn&& fn) {
    if (h->d) fn(*h->d);
    else fn(*h->f);
}

// host staging of N x 3 (body-major, the reference's Body::x[3]) <-> SoA
template <typename T>
void upload3(T* dev, const void* host, int N, cudaStream_t st) {
    std::vector<T> s((size_t)3 * N);
    const T* h = (const T*)host;
    for (int b = 0; b < N; b++)
        for (int m = 0; m < 3; m++) s[(size_t)m * N + b] = h[3 * (size_t)b + m];
    FDM_CUDA(cudaMemcpyAsync(dev, s.data(), s.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    FDM_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
void download3(void* host, const T* dev, int N, cudaStream_t st) {
    std::vector<T> s((size_t)3 * N);
    FDM_CUDA(cudaMemcpyAsync(s.data(), dev, s.size() * sizeof(T), cudaMemcpyDeviceToHost, st));
    FDM_CUDA(cudaStreamSynchronize(st));
    T* h = (T*)host;
    for (int b = 0; b < N; b++)
        for (int m = 0; m < 3; m++) h[3 * (size_t)b + m] = s[(size_t)m * N + b];
}

template <typename T>
void set_bodies(nb::Plan<T>& s, const void* x, const void* v, const void* a, const void* ap, const void* mass) {
    const int N = s.N;
    std::vector<T> zero((size_t)3 * N, T(0));
    upload3<T>(s.B.x, x, N, s.st);
    upload3<T>(s.B.v, v, N, s.st);
    upload3<T>(s.B.a, a ? a : zero.data(), N, s.st);
    upload3<T>(s.B.ap, ap ? ap : zero.data(), N, s.st);
    FDM_CUDA(cudaMemcpyAsync(s.B.mass, mass, sizeof(T) * N, cudaMemcpyHostToDevice, s.st));
    FDM_CUDA(cudaMemsetAsync(s.B.F, 0, sizeof(T) * 3 * N, s.st));
    FDM_CUDA(cudaStreamSynchronize(s.st));
    double m = 0;  // mass += body.mass, in index order
    const T* mp = (const T*)mass;
    for (int b = 0; b < N; b++) m += mp[b];
    s.set_total_mass(m);
    s.lists_empty = false;
    s.drop_graph();  // f0 is a graph kernel argument
}

// init_points (test/nbody.cpp:515-590): the solar table, or N bodies drawn
// from the standard library's default engine and uniform distribution in T
// as the reference draws them (three coordinates, then the mass, per body)
template <typename T>
void init_points(nb::Plan<T>& s, double l, double vel, int solar, double* G) {
    const int N = s.N;
    std::vector<T> x((size_t)3 * N, T(0)), v((size_t)3 * N, T(0)), m(N, T(0));
    if (solar) {
        struct Row {
            double x, y, vx, vy, mass;
        };
        // Sun, Mercury, Venus, Earth, Moon, Mars, Jupiter, Saturn, Uranus, Neptune
        static const Row rows[10] = {{0, 0, 0, 0, 333333},       {0, 0.39, 1.58, 0, 0.038}, {0, 0.72, 1.17, 0, 0.82},
                                     {0, 1, 1, 0, 1},            {0, 1.00256, 1.03, 0, 0.012}, {0, 1.51, 0.8, 0, 0.1},
                                     {0, 5.2, 0.43, 0, 317},     {0, 9.3, 0.32, 0, 95},     {0, 19.3, 0.23, 0, 14.5},
                                     {0, 30, 0.18, 0, 16.7}};
        for (int b = 0; b < 10; b++) {
            x[3 * b] = (T)rows[b].x;
            x[3 * b + 1] = (T)rows[b].y;
            v[3 * b] = (T)rows[b].vx;
            v[3 * b + 1] = (T)rows[b].vy;
            m[b] = (T)rows[b].mass;
        }
        *G = 2.96e-6;
    } else {
        std::default_random_engine gen;
        std::uniform_real_distribution<T> dist(0.0, 1.0);
        for (int b = 0; b < N; b++) {
            for (int i = 0; i < 3; i++) x[3 * b + i] = (T)(l * dist(gen) + s.P.org[i]);
            m[b] = (T)(0.2 + 1.5 * dist(gen));
            T d = 0;  // blas::dot(3, x, 1, x, 1), left to right
            for (int i = 0; i < 3; i++) d += x[3 * b + i] * x[3 * b + i];
            const double R = std::sqrt(d);
            const double V = vel / std::sqrt(R);
            v[3 * b] = (T)(V * x[3 * b + 1]);
            v[3 * b + 1] = (T)(-V * x[3 * b]);
        }
    }
    set_bodies<T>(s, x.data(), v.data(), nullptr, nullptr, m.data());
    s.lists_empty = solar != 0;
}

}  // namespace

extern "C" {

int fdmgpu_nbody_create(fdmgpu_nbody** h, int dtype, double x0, double y0, double z0, double l, int n, int npp,
                        int nbodies, double dt, double G, double vel, int sgn, int local, int solar, double crit) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle pointer");
    *h = nullptr;
    if (dtype != FDMGPU_F64 && dtype != FDMGPU_F32) FDM_FAIL(FDMGPU_EINVAL, "bad dtype %d", dtype);
    if (n < 2 || n > 512 || ilog2_exact(n) < 0)
        FDM_FAIL(FDMGPU_ESIZE, "verify((1<<n) == N): the periodic mass grid needs n a power of two in [2, 512], got %d", n);
    if (npp < 1 || npp > 1023) FDM_FAIL(FDMGPU_ESIZE, "npp must be in [1, 1023], got %d", npp);
    const int N = solar ? 10 : nbodies;
    if (N < 1) FDM_FAIL(FDMGPU_EINVAL, "need at least one body, got %d", nbodies);
    if (N > (1 << 28)) FDM_FAIL(FDMGPU_ESIZE, "at most 2^28 bodies, got %d", N);
    if (!(l > 0) || !(dt > 0)) FDM_FAIL(FDMGPU_EINVAL, "l and dt must be positive");
    std::unique_ptr<fdmgpu_nbody> p(new fdmgpu_nbody());
    p->dtype = dtype;
    double g = G;
    if (dtype == FDMGPU_F64) {
        p->d.reset(new nb::Plan<double>());
        p->d->init(x0, y0, z0, l, n, npp, N, dt, G, sgn, local, crit);
        init_points(*p->d, l, vel, solar, &g);
        p->d->set_G(g);
    } else {
        p->f.reset(new nb::Plan<float>());
        p->f->init(x0, y0, z0, l, n, npp, N, dt, G, sgn, local, crit);
        init_points(*p->f, l, vel, solar, &g);
        p->f->set_G(g);
    }
    *h = p.release();
    FDM_API_END
}

int fdmgpu_nbody_info(fdmgpu_nbody* h, int* nbodies, double* G, double* total_mass, long long* steps_done) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    with_nb(h, [&](auto& s) {
        if (nbodies) *nbodies = s.N;
        if (G) *G = s.P.G;
        if (total_mass) *total_mass = s.total_mass;
        if (steps_done) *steps_done = s.steps_done;
    });
    FDM_API_END
}

int fdmgpu_nbody_set_bodies(fdmgpu_nbody* h, const void* x, const void* v, const void* a, const void* aprev,
                            const void* mass) {
    FDM_API_BEGIN
    if (!h || !x || !v || !mass) FDM_FAIL(FDMGPU_EINVAL, "null handle or array");
    if (h->d) set_bodies<double>(*h->d, x, v, a, aprev, mass);
    else set_bodies<float>(*h->f, x, v, a, aprev, mass);
    FDM_API_END
}

int fdmgpu_nbody_get_bodies(fdmgpu_nbody* h, void* x, void* v, void* a, void* aprev, void* mass, void* F) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    with_nb(h, [&](auto& s) {
        using T = std::remove_pointer_t<decltype(s.M)>;
        if (x) download3<T>(x, s.B.x, s.N, s.st);
        if (v) download3<T>(v, s.B.v, s.N, s.st);
        if (a) download3<T>(a, s.B.a, s.N, s.st);
        if (aprev) download3<T>(aprev, s.B.ap, s.N, s.st);
        if (F) download3<T>(F, s.B.F, s.N, s.st);
        if (mass) {
            FDM_CUDA(cudaMemcpyAsync(mass, s.B.mass, sizeof(T) * s.N, cudaMemcpyDeviceToHost, s.st));
            FDM_CUDA(cudaStreamSynchronize(s.st));
        }
    });
    FDM_API_END
}

int fdmgpu_nbody_step(fdmgpu_nbody* h, int steps) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (steps < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
    with_nb(h, [&](auto& s) {
        s.step(steps);
        FDM_CUDA(cudaStreamSynchronize(s.st));
    });
    FDM_API_END
}

int fdmgpu_nbody_step_async(fdmgpu_nbody* h, int steps) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    if (steps < 0) FDM_FAIL(FDMGPU_EINVAL, "negative step count");
    with_nb(h, [&](auto& s) { s.step(steps); });
    FDM_API_END
}

int fdmgpu_nbody_sync(fdmgpu_nbody* h) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    with_nb(h, [&](auto& s) { FDM_CUDA(cudaStreamSynchronize(s.st)); });
    FDM_API_END
}

int fdmgpu_nbody_calc_forces(fdmgpu_nbody* h) {
    FDM_API_BEGIN
    if (!h) FDM_FAIL(FDMGPU_EINVAL, "null handle");
    with_nb(h, [&](auto& s) {
        s.forces();
        FDM_CUDA(cudaStreamSynchronize(s.st));
    });
    FDM_API_END
}

int fdmgpu_nbody_direct_forces(fdmgpu_nbody* h, void* F) {
    FDM_API_BEGIN
    if (!h || !F) FDM_FAIL(FDMGPU_EINVAL, "null handle or output");
    with_nb(h, [&](auto& s) {
        using T = std::remove_pointer_t<decltype(s.M)>;
        DevBuf out;
        T* d = (T*)out.get(sizeof(T) * 3 * s.N);
        {
            FDM_TIMED("nb_direct", s.st);
            nb::k_nb_direct<T><<<(s.N + nb::kDirectTile - 1) / nb::kDirectTile, nb::kDirectTile, 0, s.st>>>(s.B, s.P, d);
            FDM_LAUNCH_CHECK();
        }
        download3<T>(F, d, s.N, s.st);
    });
    FDM_API_END
}

int fdmgpu_nbody_get_field(fdmgpu_nbody* h, int field, void* out, size_t count) {
    FDM_API_BEGIN
    if (!h || !out) FDM_FAIL(FDMGPU_EINVAL, "null handle or output");
    if (field < 0 || field > 3) FDM_FAIL(FDMGPU_EINVAL, "bad field %d", field);
    with_nb(h, [&](auto& s) {
        using T = std::remove_pointer_t<decltype(s.M)>;
        const size_t n3 = (size_t)s.P.n3;
        const size_t want = field == 3 ? 3 * n3 : n3;
        if (count != want) FDM_FAIL(FDMGPU_EINVAL, "field %d has %zu elements, got %zu", field, want, count);
        FDM_CUDA(cudaStreamSynchronize(s.st));
        if (field < 3) {
            const T* src = field == 0 ? s.f : (field == 1 ? s.rhs : s.psi);
            FDM_CUDA(cudaMemcpy(out, src, n3 * sizeof(T), cudaMemcpyDeviceToHost));
        } else {
            std::vector<T> tmp(3 * n3);
            FDM_CUDA(cudaMemcpy(tmp.data(), s.E, 3 * n3 * sizeof(T), cudaMemcpyDeviceToHost));
            T* o = (T*)out;
            for (size_t e = 0; e < n3; e++)
                for (int m = 0; m < 3; m++) o[3 * e + m] = tmp[m * n3 + e];
        }
    });
    FDM_API_END
}

int fdmgpu_nbody_destroy(fdmgpu_nbody* h) {
    FDM_API_BEGIN
    if (h) {
        with_nb(h, [&](auto& s) { cudaStreamSynchronize(s.st); });
        delete h;
    }
    FDM_API_END
}

}  // extern "C"
