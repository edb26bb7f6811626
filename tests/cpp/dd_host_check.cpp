// Host build of fdm_gb300/csrc/dd.cuh: the integer FP64 <-> float conversions
// of the mixed solver checked against the host's IEEE conversions and FP64
// addition, over the whole exponent range (zero, subnormal doubles and
// floats, exact ties, the top float binade, overflow, inf, NaN).  The CUDA
// intrinsics dd.cuh calls are given their IEEE meaning here.  Prints one
// summary line; exit status 1 on any mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <utility>
#include <vector>

#define __host__
#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double d) { long long x; std::memcpy(&x, &d, 8); return x; }
static inline double __longlong_as_double(long long x) { double d; std::memcpy(&d, &x, 8); return d; }
static inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline unsigned __float_as_uint(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
static inline float __int2float_rn(int i) { return (float)i; }
static inline float __double2float_rn(double d) { return (float)d; }
static inline float __fadd_rn(float a, float b) { volatile float r = a + b; return r; }
static inline float __fsub_rn(float a, float b) { volatile float r = a - b; return r; }
static inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
static inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((unsigned)x); }
#include "../../fdm_gb300/csrc/dd.cuh"

using namespace fdmgpu;

static unsigned fbits(float f) { return __float_as_uint(f); }
static long long dbits(double d) { return __double_as_longlong(d); }
static bool same_f(float a, float b) { return (std::isnan(a) && std::isnan(b)) || fbits(a) == fbits(b); }
static bool same_d(double a, double b) { return (std::isnan(a) && std::isnan(b)) || dbits(a) == dbits(b); }
static double ulp_of(double x) { return std::fabs(std::nextafter(x, INFINITY) - x); }

int main() {
    std::mt19937_64 g(7);
    std::vector<double> xs;
    auto add = [&](double v) { xs.push_back(v); xs.push_back(-v); };
    const double specials[] = {0.0, 5e-324, 1e-310, std::ldexp(1.0, -150), std::ldexp(1.0, -149),
                               std::ldexp(3.0, -150), std::ldexp(5.0, -151), std::ldexp(1.0, -126),
                               std::nextafter(std::ldexp(1.0, -126), 0.0), std::ldexp(1.0, -127), std::ldexp(1.0, -74),
                               std::nextafter(std::ldexp(1.0, -74), 0.0), std::ldexp(1.0, 127),
                               std::nextafter(std::ldexp(1.0, 127), 0.0), std::ldexp(1.0, 128),
                               std::ldexp(1.0, 128) - std::ldexp(1.0, 103), std::ldexp(1.0, 128) - std::ldexp(1.0, 104),
                               std::nextafter(std::ldexp(1.0, 128) - std::ldexp(1.0, 103), 0.0), std::ldexp(1.0, 191),
                               std::ldexp(1.7, 190), 1.7976931348623157e308, INFINITY, NAN, 1.0, 3.0e-40, 1.0e-45,
                               7.0e-46};
    for (double v : specials) add(v);
    for (int e = -1080; e <= 1030; e++)
        for (int k = 0; k < 12; k++) {
            double m = 1.0 + (double)(g() >> 11) * std::ldexp(1.0, -53);
            if (k == 0) m = 1.0;
            if (k == 1) m = 1.0 + std::ldexp(1.0, -24);  // a tie of the float rounding
            if (k == 2) m = 1.0 + std::ldexp(3.0, -25);
            add(std::ldexp(m, e));
        }
    long bad_round = 0, bad_split = 0, bad_sum = 0;
    for (double x : xs) {
        const int e = (int)((dbits(x) >> 52) & 0x7ff);
        const float r = f64_to_f32(x), hw = (float)x;
        if (!same_f(r, hw)) {
            // inside the normal float range only exact ties may differ
            const bool edge = e < 897 || e > 1149;
            if (edge || std::fabs((double)hw - x) != std::fabs((double)r - x)) bad_round++;
        }
        const ff s = f64_split(x);
        const float h_hw = (float)x;
        const float l_hw = (float)(x - (double)h_hw);
        const double ax = std::fabs(x);
        if (std::isnan(x)) {
            if (!(std::isnan(s.h) && std::isnan(s.l))) bad_split++;
        } else if (std::isinf(x) || ax >= std::ldexp(1.0, 191) || std::isinf(s.h)) {
            if (!(same_f(s.h, h_hw) && same_f(s.l, l_hw))) bad_split++;
        } else if (ax < std::ldexp(1.0, -126)) {
            if (!(same_f(s.h, h_hw) && s.l == 0.0f)) bad_split++;
        } else if (std::fabs(x - ((double)s.h + (double)s.l)) > std::ldexp(ax, -48) + std::ldexp(1.0, -149)) {
            bad_split++;
        }
    }
    // FP64 value of float pairs: normalised pairs from the values above, every
    // combination of special floats, and normal lo beside zero / subnormal hi
    std::vector<std::pair<float, float>> ps;
    for (double x : xs) {
        const float h = (float)x;
        ps.push_back({h, std::isfinite(h) ? (float)(x - (double)h) : 0.0f});
    }
    const float sp[] = {0.f, -0.f, 1e-45f, -1e-45f, 3e-40f, -3e-40f, 1.1754942e-38f, 2.5e-38f, -1e-37f,
                        INFINITY, -INFINITY, NAN, 1.0f};
    for (float a : sp)
        for (float c : sp) ps.push_back({a, c});
    std::mt19937 g32(3);
    for (int it = 0; it < 200000; it++) {
        const unsigned hb = g32() & 0x807fffffu;
        unsigned lb = (g32() & 0x80000000u) | ((1u + g32() % 253u) << 23) | (g32() & 0x7fffffu);
        if (it % 3 == 0) lb = (lb & 0x807fffffu) | ((1u + g32() % 30u) << 23);
        ps.push_back({__uint_as_float(hb), __uint_as_float(lb)});
    }
    for (const auto& p : ps) {
        const float h = p.first, l = p.second;
        const double w = ff_to_f64(ff{h, l});
        const double hw = (double)h + (double)l;
        const unsigned eh = (fbits(h) >> 23) & 0xff, el = (fbits(l) >> 23) & 0xff;
        const bool swapped = eh == 0 && el != 0 && el != 255;
        if ((eh == 0 || eh == 255 || el == 255) && !swapped) {
            if (!same_d(w, hw) && !(w == 0.0 && hw == 0.0 && std::signbit(w) == std::signbit(hw))) bad_sum++;
        } else if (swapped || std::fabs((double)l) <= std::ldexp(std::fabs((double)h), -24)) {
            // within half an FP64 ulp of the exact sum: equal to the rounded
            // sum or, at a tie, its neighbour
            if (!(w == hw || std::fabs(w - hw) <= ulp_of(hw))) bad_sum++;
        }
    }
    std::printf("values %zu pairs %zu: bad rounding %ld, bad split %ld, bad pair sum %ld\n", xs.size(), ps.size(),
                bad_round, bad_split, bad_sum);
    return (bad_round || bad_split || bad_sum) ? 1 : 0;
}
