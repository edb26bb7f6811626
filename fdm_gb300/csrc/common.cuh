// Shared helpers for the GB300 Poisson / NSCube kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fdmgpu {

template <typename T> struct vec2;
template <> struct vec2<float> { using type = float2; };
template <> struct vec2<double> { using type = double2; };
template <typename T> using vec2_t = typename vec2<T>::type;

template <typename T>
__device__ __forceinline__ vec2_t<T> cmul(vec2_t<T> a, vec2_t<T> b) {
    vec2_t<T> r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename T>
__device__ __forceinline__ vec2_t<T> cadd(vec2_t<T> a, vec2_t<T> b) {
    vec2_t<T> r; r.x = a.x + b.x; r.y = a.y + b.y; return r;
}
template <typename T>
__device__ __forceinline__ vec2_t<T> csub(vec2_t<T> a, vec2_t<T> b) {
    vec2_t<T> r; r.x = a.x - b.x; r.y = a.y - b.y; return r;
}
// multiply by -i
template <typename T>
__device__ __forceinline__ vec2_t<T> cmul_mi(vec2_t<T> a) {
    vec2_t<T> r; r.x = a.y; r.y = -a.x; return r;
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

// A divisor fixed for a whole run and its correctly rounded reciprocal
// (computed on the host, or by cdiv_dev on the device).
struct CDiv {
    double b, y;
};
inline CDiv cdiv_of(double b) { return CDiv{b, 1.0 / b}; }
__device__ __forceinline__ CDiv cdiv_dev(double b) { return CDiv{b, 1.0 / b}; }

// a / d.b correctly rounded, for finite a and quotients and remainders in
// the normal range: q0 = a*y within two ulps, then two remainder
// corrections r = a - b q (exact through the fused multiply-add) and
// q <- q + r y.  After the first q is faithful, and a faithful q with
// y = RN(1/b) corrects to RN(a/b) (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34,
// 1990; the correction theorem as stated in J.-M. Muller et al., Handbook
// of Floating-Point Arithmetic, ch. on division).  Five FP64 operations and
// no data-dependent slow path; a zero dividend returns its signed zero.
__device__ __forceinline__ double cdiv(double a, CDiv d) {
    const double q0 = a * d.y;
    double q = fma(fma(-q0, d.b, a), d.y, q0);
    q = fma(fma(-q, d.b, a), d.y, q);
    return (__double_as_longlong(a) << 1) == 0 ? q0 : q;
}

__host__ __device__ inline int ilog2_exact(int n) {
    int q = 0;
    if (n < 1) return -1;
    while ((1 << q) < n) q++;
    return (1 << q) == n ? q : -1;
}

}  // namespace fdmgpu
