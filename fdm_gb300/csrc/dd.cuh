// Double-FP32 ("float-float") arithmetic and exact FP64 <-> FP32-pair
// conversions done with FP32 and integer instructions only.
//
// GB300's FP64 pipe runs at about 1/58 of its FP32 rate, so the mixed
// Poisson path keeps FP64 arithmetic out of its per-point work: FP64 inputs
// are split into a pair of floats (hi, lo) with integer bit operations, the
// residual is formed in float-float arithmetic, and the FP64 output is
// assembled from a float pair by integer addition on the FP64 bit pattern.
//
// Float-float algorithms: Knuth's TwoSum, Dekker's Fast2Sum and the
// FMA-based TwoProduct (T. Ogita, S. M. Rump, S. Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26(6), 2005).  The __f*_rn intrinsics keep
// the compiler from contracting or reassociating the error terms.
#pragma once

#include <stdint.h>

namespace fdmgpu {

struct ff {
    float h, l;
};

// s + e == a + b exactly
__host__ __device__ __forceinline__ ff two_sum(float a, float b) {
#ifdef __CUDA_ARCH__
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
#else
    volatile float s = a + b;
    volatile float bb = s - a;
    volatile float e = (a - (s - bb)) + (b - bb);
#endif
    return ff{s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float e = __fsub_rn(b, __fsub_rn(s, a));
    return ff{s, e};
}

// p + e == a * b exactly
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);
    return ff{p, e};
}

// a + b, relative error ~2^-44
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.h, b.h);
    const float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
    return fast_two_sum(s.h, e);
}

__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = two_sum(a.h, b);
    const float e = __fadd_rn(s.l, a.l);
    return fast_two_sum(s.h, e);
}

// a * b, relative error ~2^-44
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = two_prod(a.h, b.h);
    float e = __fmaf_rn(a.h, b.l, p.l);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p.h, e);
}

// Nearest float to an FP64 value, by integer rounding of the bit pattern
// (round half away from zero; exact hardware conversion outside the normal
// float range).
__device__ __forceinline__ float f64_to_f32(double d) {
    const long long b = __double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 897 || e > 1149) return __double2float_rn(d);
    const long long r = (b & 0x7fffffffffffffffLL) + (1LL << 28);
    const int er = (int)(r >> 52);
    const unsigned bits = ((unsigned)(b >> 32) & 0x80000000u) | ((unsigned)(er - 896) << 23) |
                          ((unsigned)(r >> 29) & 0x7fffffu);
    return __uint_as_float(bits);
}

// (hi, lo) with hi + lo == d to ~2^-48 relative: hi is d rounded to a float,
// lo the rounded remainder.  Integer path for 2^-74 <= |d| < 2^127.
__device__ __forceinline__ ff f64_split(double d) {
    const long long b = __double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 949 || e > 1149) {
        const float h = __double2float_rn(d);
        return ff{h, __double2float_rn(d - (double)h)};
    }
    const long long mag = b & 0x7fffffffffffffffLL;
    const long long r = (mag + (1LL << 28)) & ~((1LL << 29) - 1);  // hi as an FP64 pattern
    const int er = (int)(r >> 52);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const float h = __uint_as_float(sign | ((unsigned)(er - 896) << 23) | ((unsigned)(r >> 29) & 0x7fffffu));
    const int delta = (int)(mag - r);  // |delta| <= 2^28, units of 2^(e-1075)
    float l = __int2float_rn(delta) * __uint_as_float((unsigned)(e - 948) << 23);
    if (sign) l = -l;
    return ff{h, l};
}

// FP64 value of h + l for a normalised pair (|l| <= ulp_f32(h)/2), built by
// integer addition on the FP64 bit pattern of h; exact to half an FP64 ulp.
__device__ __forceinline__ double ff_to_f64(ff v) {
    const unsigned hb = __float_as_uint(v.h);
    const int eh = (int)((hb >> 23) & 0xff);
    const unsigned lb = __float_as_uint(v.l);
    const int el = (int)((lb >> 23) & 0xff);
    if (eh == 0 || eh == 255) return (double)v.h + (double)v.l;
    long long D = ((long long)(eh + 896) << 52) | ((long long)(hb & 0x7fffffu) << 29);
    if (el != 0) {
        const long long ml = (long long)((lb & 0x7fffffu) | 0x800000u);
        const int sh = el - eh + 29;  // <= 5 for a normalised pair
        long long q;
        if (sh >= 0) q = ml << sh;
        else if (sh > -26) q = (ml + (1LL << (-sh - 1))) >> (-sh);
        else q = 0;
        if ((hb ^ lb) & 0x80000000u) {
            if ((hb & 0x7fffffu) == 0) q <<= 1;  // h a power of two: step into the lower binade
            D -= q;
        } else {
            D += q;
        }
    }
    D |= (long long)(hb & 0x80000000u) << 32;
    return __longlong_as_double(D);
}

}  // namespace fdmgpu
