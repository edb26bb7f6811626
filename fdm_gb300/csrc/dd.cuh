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

// The split and the FP64 assembly below cover zero, subnormal, huge, inf and
// NaN operands with integer operations as well.  A short FP64 fallback for
// those cases is compiled as predicated code that every element issues: it
// kept the FP64 pipe of the residual and final passes busy (36 % and 66 %
// active) although no element took it.  The plain rounding f64_to_f32 keeps
// its one-instruction hardware fallback, which costs less there than the
// integer form issued the same way.

// Exact FP64 bit pattern of the float with bit pattern fb (zero, subnormal,
// inf and NaN included).
__device__ __forceinline__ long long f32_to_f64_bits(unsigned fb) {
    const long long sign = (long long)(fb & 0x80000000u) << 32;
    const unsigned e = (fb >> 23) & 0xffu, m = fb & 0x7fffffu;
    if (e == 255u) return sign | (0x7ffLL << 52) | ((long long)m << 29);
    if (e != 0u) return sign | ((long long)(e + 896u) << 52) | ((long long)m << 29);
    if (m == 0u) return sign;
    const int p = 31 - __clz((int)m);  // leading bit of the subnormal mantissa, 0..22
    return sign | ((long long)(p + 874) << 52) | (((long long)m << (52 - p)) & 0xfffffffffffffLL);
}

// Round to nearest, ties to even, of the FP64 value with bit pattern b and
// biased exponent e when the float result is zero, subnormal, the top binade,
// inf or NaN (e < 897 or e > 1149): the hardware conversion's result.
__device__ __forceinline__ float f64_to_f32_edge(long long b, int e) {
    const unsigned sign = (unsigned)((unsigned long long)b >> 32) & 0x80000000u;
    const long long mag = b & 0x7fffffffffffffffLL;
    if (e == 2047) return __uint_as_float(mag > 0x7ff0000000000000LL ? 0x7fffffffu : (sign | 0x7f800000u));
    if (e > 1150) return __uint_as_float(sign | 0x7f800000u);
    if (e == 1150) {  // 2^127 <= |d| < 2^128: exponent 254, or inf when the rounding carries
        long long r = mag >> 29;
        const long long rem = mag & 0x1fffffffLL;
        if (rem > 0x10000000LL || (rem == 0x10000000LL && (r & 1))) r++;
        return __uint_as_float(sign | (unsigned)(r - (896LL << 23)));
    }
    // |d| < 2^-126: the result is a multiple of 2^-149
    const int shift = 926 - e;  // >= 30
    if (e == 0 || shift > 54) return __uint_as_float(sign);
    const long long m = (mag & 0xfffffffffffffLL) | (1LL << 52);
    long long q = m >> shift;
    const long long rem = m & ((1LL << shift) - 1), half = 1LL << (shift - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    return __uint_as_float(sign | (unsigned)q);  // q = 2^23 is the smallest normal
}

// Nearest float to an FP64 value, by integer rounding of the bit pattern:
// round half away from zero in the normal float range, the hardware
// conversion (ties to even) outside it.
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

// (hi, lo) of an FP64 pattern with biased exponent 949 <= e <= 1149
// (2^-74 <= |d| < 2^127): hi is d rounded to a float, lo the rounded
// remainder, hi + lo == d to ~2^-48 relative.
__device__ __forceinline__ ff f64_split_normal(long long b, int e) {
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

// f64_split outside 2^-74 <= |d| < 2^127.  Between 2^-126 and 2^-74 and
// between 2^127 and 2^191 the pair of d scaled by 2^(+-64) is scaled back
// (hi exact, lo rounded where it falls below the normal floats); below
// 2^-126 hi is d rounded to the float grid and lo is 0; above 2^191, for inf
// and for NaN hi is the hardware conversion and lo is -hi or NaN, the values
// of rn(d - hi).
__device__ __forceinline__ ff f64_split_edge(long long b, int e) {
    if (e >= 897 && e < 949) {
        const ff s = f64_split_normal(b + (64LL << 52), e + 64);
        return ff{__fmul_rn(s.h, 0x1p-64f), __fmul_rn(s.l, 0x1p-64f)};
    }
    if (e > 1149 && e < 1214) {
        const ff s = f64_split_normal(b - (64LL << 52), e - 64);
        const float h = __fmul_rn(s.h, 0x1p64f);
        return ff{h, (__float_as_uint(h) & 0x7fffffffu) == 0x7f800000u ? -h : __fmul_rn(s.l, 0x1p64f)};
    }
    const float h = f64_to_f32_edge(b, e);
    if (e < 897) return ff{h, 0.f};
    return ff{h, e == 2047 ? __uint_as_float(0x7fffffffu) : -h};
}

// (hi, lo) with hi + lo == d to ~2^-48 relative: hi is d rounded to a float,
// lo the rounded remainder.
__device__ __forceinline__ ff f64_split(double d) {
    const long long b = __double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 949 || e > 1149) return f64_split_edge(b, e);
    return f64_split_normal(b, e);
}

// FP64 value of h + l for a float h in the normal range and |l| <= ulp(h)/2
// (l finite: zero, subnormal or normal), built by integer addition on the
// FP64 bit pattern of h; exact to half an FP64 ulp.
__device__ __forceinline__ double ff_to_f64_normal(unsigned hb, unsigned lb) {
    const int eh = (int)((hb >> 23) & 0xff);
    const int el = (int)((lb >> 23) & 0xff);
    long long D = ((long long)(eh + 896) << 52) | ((long long)(hb & 0x7fffffu) << 29);
    // l = ml * 2^(el' - 150): a subnormal l has no implicit bit and el' = 1;
    // q, l in units of the FP64 ulp of h, stays below 2^30, so 32-bit shifts
    const unsigned ml = (lb & 0x7fffffu) | (el ? 0x800000u : 0u);
    if (ml != 0) {
        const int sh = (el ? el : 1) - eh + 29;  // <= 5 for a normalised pair
        unsigned q;
        if (sh >= 0) q = ml << sh;
        else if (sh > -26) q = (ml + (1u << (-sh - 1))) >> (-sh);
        else q = 0;
        if ((hb ^ lb) & 0x80000000u) {
            if ((hb & 0x7fffffu) == 0) q <<= 1;  // h a power of two: step into the lower binade
            D -= (long long)q;
        } else {
            D += (long long)q;
        }
    }
    D |= (long long)(hb & 0x80000000u) << 32;
    return __longlong_as_double(D);
}

// (double)h + (double)l when h is zero, subnormal, inf or NaN or l is inf or
// NaN, by integer (and exact FP32) operations: NaN for a NaN operand or
// inf - inf, the inf otherwise; with h zero or subnormal and l as well, the
// exact sum (a multiple of 2^-149 below 2^-125); with l in the normal range
// (not a normalised pair) l + h to half an FP64 ulp.
__device__ __forceinline__ double ff_to_f64_edge(unsigned hb, unsigned lb) {
    const unsigned ha = hb & 0x7fffffffu, la = lb & 0x7fffffffu;
    if (ha > 0x7f800000u || la > 0x7f800000u ||
        (ha == 0x7f800000u && la == 0x7f800000u && ((hb ^ lb) & 0x80000000u)))
        return __longlong_as_double(0x7fffffffffffffffLL);
    if (ha == 0x7f800000u) return __longlong_as_double(f32_to_f64_bits(hb));
    if (la == 0x7f800000u) return __longlong_as_double(f32_to_f64_bits(lb));
    if (la >= 0x00800000u) {
        // l normal, h zero or subnormal (not a normalised pair): l + h as the
        // normalised pair fast_two_sum gives, exactly equal to it
        const ff t = fast_two_sum(__uint_as_float(lb), __uint_as_float(hb));
        const unsigned tb = __float_as_uint(t.h);
        if ((tb & 0x7f800000u) != 0u) return ff_to_f64_normal(tb, __float_as_uint(t.l));
        return __longlong_as_double(f32_to_f64_bits(tb));  // l + h subnormal: exact, t.l == 0
    }
    // both zero or subnormal: integers in units of 2^-149
    const int s = ((hb & 0x80000000u) ? -(int)ha : (int)ha) + ((lb & 0x80000000u) ? -(int)la : (int)la);
    if (s == 0) return __longlong_as_double((long long)(hb & lb & 0x80000000u) << 32);
    // |s| < 2^24 is the bit pattern of the float |s| * 2^-149 (subnormal, or
    // the smallest normal binade)
    return __longlong_as_double(f32_to_f64_bits((s < 0 ? 0x80000000u : 0u) | (unsigned)(s < 0 ? -s : s)));
}

// FP64 value of h + l for a normalised pair (|l| <= ulp_f32(h)/2), exact to
// half an FP64 ulp, with integer operations only.
__device__ __forceinline__ double ff_to_f64(ff v) {
    const unsigned hb = __float_as_uint(v.h);
    const unsigned lb = __float_as_uint(v.l);
    const unsigned eh = (hb >> 23) & 0xffu;
    if (eh == 0u || eh == 255u || (lb & 0x7f800000u) == 0x7f800000u) return ff_to_f64_edge(hb, lb);
    return ff_to_f64_normal(hb, lb);
}

}  // namespace fdmgpu
