// lp_math.cuh — correctly rounded binary32 atan2, atan and exp on the device.
//
// The reference path feeds these values into discrete decisions (voxel bins, quadrants, the
// jump-convolution vote). glibc's float versions are not correctly rounded and differ between
// builds, so the device implements the one platform-independent definition: the binary32
// value nearest to the exact result (round to nearest, ties to even).
//
// Method (Ziv's two-step rounding test): evaluate in binary64 with the CUDA double functions
// (documented max error 2 ulp for atan2/atan, 1 ulp for exp); if that value lies further than
// 2^-49 relative from every binary32 rounding boundary, its rounding is the correct one.
// Otherwise re-evaluate in double-double arithmetic (about 2^-100 relative error) from the
// mathematical definitions below and round that:
//   exp(x)  = 2^k * exp(r),  r = x - k ln2 (|r| <= ln2/2), Taylor series of exp(r)
//   atan(t) = 4 atan(t''), t' = t / (1 + sqrt(1 + t^2)) applied twice (|t''| <= tan(pi/16)),
//             odd Taylor series; atan(t) = pi/2 - atan(1/t) for t > 1
//   atan2(y, x) from atan(min/max) with the quadrant identities.
// Double-double primitives are Dekker/Knuth error-free transformations (two_sum, two_prod
// with fma). Constants ln2, pi/2 and pi are split into double-double pairs (computed to 200
// bits with mpmath).
#pragma once
#include <cstdint>

namespace lpm
{
struct dd
{
    double hi, lo;
};

__device__ __forceinline__ dd two_sum(double a, double b)
{
    const double s = a + b;
    const double bb = s - a;
    const double e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ dd quick_two_sum(double a, double b)
{
    const double s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ dd two_prod(double a, double b)
{
    const double p = a * b;
    return {p, fma(a, b, -p)};
}
__device__ __forceinline__ dd dd_add(dd a, dd b)
{
    dd s = two_sum(a.hi, b.hi);
    const dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd dd_neg(dd a)
{
    return {-a.hi, -a.lo};
}
__device__ __forceinline__ dd dd_sub(dd a, dd b)
{
    return dd_add(a, dd_neg(b));
}
__device__ __forceinline__ dd dd_mul(dd a, dd b)
{
    dd p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd dd_mul_d(dd a, double b)
{
    dd p = two_prod(a.hi, b);
    p.lo += a.lo * b;
    return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd dd_div(dd a, dd b)
{
    const double q1 = a.hi / b.hi;
    dd r = dd_sub(a, dd_mul_d(b, q1));
    const double q2 = r.hi / b.hi;
    r = dd_sub(r, dd_mul_d(b, q2));
    const double q3 = r.hi / b.hi;
    dd q = quick_two_sum(q1, q2);
    return dd_add(q, dd{q3, 0.0});
}
__device__ __forceinline__ dd dd_sqrt(dd a)
{
    if (a.hi <= 0.0)
        return {0.0, 0.0};
    const double x = sqrt(a.hi);
    const dd x2 = two_prod(x, x);
    const double e = ((a.hi - x2.hi) - x2.lo + a.lo) / (2.0 * x);
    return quick_two_sum(x, e);
}

constexpr double kLn2Hi = 0x1.62e42fefa39efp-1;
constexpr double kLn2Lo = 0x1.abc9e3b39803fp-56;
constexpr double kPiHi = 0x1.921fb54442d18p+1;
constexpr double kPiLo = 0x1.1a62633145c07p-53;
constexpr double kPi2Hi = 0x1.921fb54442d18p+0;
constexpr double kPi2Lo = 0x1.1a62633145c07p-54;

// exp(x) in double-double for a binary32 argument (|x| < 104).
static __device__ __noinline__ dd dd_exp(float xf)
{
    const double x = static_cast<double>(xf);
    const double k = rint(x / kLn2Hi);
    // r = x - k*ln2, k integer with |k| < 160: k*ln2Hi is exact in double-double via two_prod
    dd r = dd_sub(dd{x, 0.0}, dd_add(two_prod(k, kLn2Hi), two_prod(k, kLn2Lo)));
    dd sum{1.0, 0.0};
    dd term{1.0, 0.0};
    for (int i = 1; i <= 27; ++i)
    {
        term = dd_mul(term, r);
        term = dd_div(term, dd{static_cast<double>(i), 0.0});
        sum = dd_add(sum, term);
    }
    const int ki = static_cast<int>(k);
    return {scalbn(sum.hi, ki), scalbn(sum.lo, ki)};
}

// atan(t) for t >= 0 in double-double.
static __device__ __noinline__ dd dd_atan_pos(dd t)
{
    bool invert = false;
    if (t.hi > 1.0)
    {
        t = dd_div(dd{1.0, 0.0}, t);
        invert = true;
    }
    for (int k = 0; k < 2; ++k)
    {
        const dd s = dd_sqrt(dd_add(dd{1.0, 0.0}, dd_mul(t, t)));
        t = dd_div(t, dd_add(dd{1.0, 0.0}, s));
    }
    const dd t2 = dd_mul(t, t);
    dd sum{0.0, 0.0};
    // odd series, highest term first: sum_{j=0}^{24} (-1)^j t^(2j+1) / (2j+1)
    for (int j = 24; j >= 0; --j)
    {
        const double c = ((j & 1) ? -1.0 : 1.0);
        const dd inv = dd_div(dd{c, 0.0}, dd{static_cast<double>(2 * j + 1), 0.0});
        sum = dd_add(dd_mul(sum, t2), inv);
    }
    sum = dd_mul(sum, t);
    sum = dd_mul_d(sum, 4.0);
    if (invert)
        sum = dd_sub(dd{kPi2Hi, kPi2Lo}, sum);
    return sum;
}

// Correct binary32 rounding of hi + lo (|lo| <= ulp(hi)/2).
__device__ __forceinline__ float round_dd(dd v)
{
    float f = __double2float_rn(v.hi);
    const double fd = static_cast<double>(f);
    if (fd == v.hi)
    {
        return f; // hi is a float; lo is far below half an ulp of it
    }
    // neighbour of f on the side of v.hi, and the midpoint between them
    const float g = (v.hi > fd) ? nextafterf(f, INFINITY) : nextafterf(f, -INFINITY);
    const double mid = 0.5 * (fd + static_cast<double>(g)); // exact in double
    if (v.hi == mid)
    {
        if (v.lo == 0.0)
            return f; // exact tie: __double2float_rn already chose the even one
        const bool beyond = (v.hi > fd) ? (v.lo > 0.0) : (v.lo < 0.0);
        return beyond ? g : f;
    }
    return f;
}

// True when the binary64 approximation v (relative error < 2^-50) might round differently
// from the exact value: v lies within 2^-49 |v| of a binary32 rounding boundary.
__device__ __forceinline__ bool near_boundary(double v)
{
    const float f = __double2float_rn(v);
    if (isinf(f) || v == 0.0)
        return false;
    const double fd = static_cast<double>(f);
    const float up = nextafterf(f, INFINITY), dn = nextafterf(f, -INFINITY);
    const double m_up = 0.5 * (fd + static_cast<double>(up));
    const double m_dn = 0.5 * (fd + static_cast<double>(dn));
    const double tol = fabs(v) * 0x1p-49;
    return fabs(v - m_up) <= tol || fabs(v - m_dn) <= tol;
}

__device__ __forceinline__ float cr_expf(float x)
{
    if (x < -104.0f)
        return 0.0f;
    if (x > 89.0f)
        return INFINITY;
    const double v = exp(static_cast<double>(x));
    if (!near_boundary(v))
        return __double2float_rn(v);
    return round_dd(dd_exp(x));
}

__device__ __forceinline__ float cr_atanf(float x)
{
    if (isnan(x))
        return x;
    const double v = atan(static_cast<double>(x));
    if (!near_boundary(v))
        return __double2float_rn(v);
    dd r = dd_atan_pos(dd{fabs(static_cast<double>(x)), 0.0});
    if (x < 0.0f)
        r = dd_neg(r);
    return round_dd(r);
}

__device__ __forceinline__ float cr_atan2f(float y, float x)
{
    const double v = atan2(static_cast<double>(y), static_cast<double>(x));
    if (!near_boundary(v) || isnan(v))
        return __double2float_rn(v);
    const double ax = fabs(static_cast<double>(x)), ay = fabs(static_cast<double>(y));
    dd r;
    if (ay <= ax)
        r = dd_atan_pos(dd_div(dd{ay, 0.0}, dd{ax, 0.0}));
    else
        r = dd_sub(dd{kPi2Hi, kPi2Lo}, dd_atan_pos(dd_div(dd{ax, 0.0}, dd{ay, 0.0})));
    if (signbit(x))
        r = dd_sub(dd{kPiHi, kPiLo}, r);
    if (signbit(y))
        r = dd_neg(r);
    return round_dd(r);
}

// The reference's own minimax atan2 (lidar_processing_lib/include/lidar_processing_lib/common.hpp:33-62):
// plain binary32 operations, no fused multiply-add (the library is built with --fmad=false).
__device__ __forceinline__ float atan2_approx(float y, float x)
{
    const float ax = fabsf(x);
    const float ay = fabsf(y);
    const float mx = fmaxf(ay, ax);
    const float mn = fminf(ay, ax);
    const float a = mn / mx;
    const float s = a * a;
    const float c = s * a;
    const float q = s * s;
    float r = 0.024840285F * q + 0.18681418F;
    const float t = -0.094097948F * q - 0.33213072F;
    r = r * s + t;
    r = r * c + a;
    if (ay > ax)
        r = 1.57079637F - r;
    if (x < 0)
        r = 3.14159274F - r;
    if (y < 0)
        r = -r;
    return r;
}
} // namespace lpm
