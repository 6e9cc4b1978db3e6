// lp_math.cuh — correctly rounded binary32 atan2, atan and exp on the device.
//
// The reference path feeds these values into discrete decisions (voxel bins, quadrants, the
// jump-convolution vote). glibc's float versions are not correctly rounded and differ between
// builds, so the device implements the one platform-independent definition: the binary32
// value nearest to the exact result (round to nearest, ties to even).
//
// Three stages, each used only when the one before cannot decide the rounding (Ziv's strategy):
//
// 1. float-float (FP32 units only; the GPU's FP64 rate is a small fraction of its FP32 rate):
//      exp(x)  = 2^m * 2^(j/64) * exp(r),  n = rint(64 x / ln2) = 64 m + j,
//                r = x - n ln2/64 (|r| <= ln2/128), exp(r) by its Taylor polynomial of degree 5
//                (P. T. P. Tang, "Table-driven implementation of the exponential function in IEEE
//                floating-point arithmetic", ACM TOMS 15(2), 1989),
//      atan(t) = atan(c) + atan((t - c) / (1 + t c)),  c = rint(128 t) / 128 (0 <= t <= 1),
//                atan(u) = u - u^3/3 + u^5/5 - u^7/7 (|u| <= 1/256);  atan(t) = pi/2 - atan(1/t)
//                above 1; atan2 from atan(min/max) with the quadrant identities.
//    Products and sums that must be exact use the error-free transformations of Dekker and Knuth
//    (two_sum, two_prod with fma). The result hi + lo is within 2^-36 of the exact value
//    (relative; the analysis beside each function gives about 2^-38); if that interval does not
//    contain a binary32 rounding boundary, hi + lo rounds like the exact value.
// 2. binary64 with the CUDA double functions (documented max error 2 ulp for atan2/atan, 1 ulp
//    for exp); if that value lies further than 2^-49 relative from every binary32 rounding
//    boundary, its rounding is the correct one.
// 3. double-double arithmetic (about 2^-100 relative error) from the mathematical definitions
//    below, then rounded:
//      exp(x)  = 2^k * exp(r),  r = x - k ln2 (|r| <= ln2/2), Taylor series of exp(r)
//      atan(t) = 4 atan(t''), t' = t / (1 + sqrt(1 + t^2)) applied twice (|t''| <= tan(pi/16)),
//                odd Taylor series; atan(t) = pi/2 - atan(1/t) for t > 1
//      atan2(y, x) from atan(min/max) with the quadrant identities.
// Constants ln2, pi/2 and pi are split into double-double pairs (computed to 200 bits with
// mpmath); the float-float tables are written by gen_math_tables.py.
#pragma once
#include <cstdint>

#include "lp_math_tables.cuh"

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

__device__ __forceinline__ float cr_expf_fp64(float x)
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

__device__ __forceinline__ float cr_atanf_fp64(float x)
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

__device__ __forceinline__ float cr_atan2f_fp64(float y, float x)
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

// ---------------------------------------------------------------------------------------------
// Stage 1: float-float evaluation.
// ---------------------------------------------------------------------------------------------
struct ff
{
    float hi, lo;
};

__device__ __forceinline__ ff two_sum_f(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ ff fast_two_sum_f(float a, float b) // |a| >= |b| or a == 0
{
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ ff two_prod_f(float a, float b)
{
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}

// Rounding test: v = hi + lo approximates y with |v - y| <= 2^-36 |y|. Writes the binary32
// nearest y and returns true when every value of that interval rounds to the same float; returns
// false (undecided) otherwise. hi + lo is first renormalised exactly (s = fl(hi + lo), e the
// remainder); y rounds to s when s + e stays, by more than the error bound, inside the rounding
// interval of s: half the gap to the neighbour on e's side (a quarter ulp below a power of two).
__device__ __forceinline__ bool ff_round(ff v, float* out)
{
    const ff n = fast_two_sum_f(v.hi, v.lo);
    const float s = n.hi, e = n.lo;
    const float as = fabsf(s);
    if (!(as >= 0x1p-100f && as <= 0x1p100f))
        return false;
    const uint32_t bits = __float_as_uint(as);
    const float up = __uint_as_float(bits + 1u) - as;                      // gap above |s|
    const float dn = ((bits & 0x7fffffu) == 0u) ? 0.5f * up : up;         // gap below |s|
    const bool away = (e > 0.0f) == (s > 0.0f);                           // e points away from 0
    const float half = 0.5f * (away ? up : dn);
    const float room = half - fabsf(e);       // exact or within 2^-24 of it (|e| <= half)
    if (room > as * 0x1p-35f)                 // twice the error bound: covers the rounding of room
    {
        *out = s;
        return true;
    }
    return false;
}

// exp(x) for -87 <= x <= 88.5 (normal results). Error (relative, before scaling by 2^m):
// reduction r = x - n ln2/64 in float-float, exact but for the ln2/64 tail and the float sums of
// small terms (< 2^-50); polynomial: 1 + r exact, r^2/2 exact product, the rest in float
// (< 2^-40 each for the two float sums, truncation 2^-54); table pair 2^-48; the float-float
// product with the table < 2^-40. Total below 2^-38.
__device__ __forceinline__ bool ff_expf(float x, float* out)
{
    const float nf = rintf(x * 92.332482616893656f); // 64 / ln2: it only chooses n
    const int n = static_cast<int>(nf);
    const int j = n & 63;
    const int m = (n - j) >> 6;
    const ff a = two_sum_f(x, -nf * kLn2By64Head);   // nf * head is exact (|n| < 2^14)
    const ff p2 = two_prod_f(nf, kLn2By64Mid);
    ff r = two_sum_f(a.hi, -p2.hi);
    r.lo = r.lo + ((a.lo - p2.lo) - nf * kLn2By64Tail);
    r = fast_two_sum_f(r.hi, r.lo);
    const float rh = r.hi, rl = r.lo;
    const ff q = two_prod_f(rh, rh);                  // r^2 (of the head)
    const float small = q.lo * 0.5f + rh * rl + q.hi * rh * (1.0f / 6.0f) + q.hi * q.hi * (1.0f / 24.0f) +
                        q.hi * q.hi * rh * (1.0f / 120.0f);
    const ff s1 = two_sum_f(1.0f, rh);
    const float t = q.hi * 0.5f + (rl + small);
    const ff e = fast_two_sum_f(s1.hi, s1.lo + t);     // exp(r)
    const float2 T = kExp2Tab[j];
    ff p = two_prod_f(e.hi, T.x);
    p.lo = p.lo + (e.hi * T.y + e.lo * T.x);
    float f;
    if (!ff_round(p, &f))
        return false;
    *out = scalbnf(f, m); // exact: the result is a normal float
    return true;
}

// atan(t) for t = th + tl in [0, 1] (tl = 0 or |tl| <= 2^-23 th). c = j/128, j = rint(128 th):
// th - c is exact (Sterbenz), 1 + t c is formed from an exact product; u = (t - c) / (1 + t c) in
// float-float (relative error < 2^-45), |u| <= 1/256; atan(u) = u - u^3/3 + u^5/5 - u^7/7 with
// the cubic and higher terms in float (< 2^-39.5 |u| with the u_lo contribution; |u| is at most
// atan(t) for j <= 1 and below it otherwise), truncation u^9/9 < 2^-66 |u|; table pair 2^-48;
// the final float sums < 2^-46. The result is within 2^-39 relative of atan(t).
__device__ __forceinline__ ff ff_atan_unit(float th, float tl)
{
    const float jf = fminf(fmaxf(rintf(th * 128.0f), 0.0f), 128.0f); // table bounds, whatever th is
    const int j = static_cast<int>(jf);
    const float c = jf * (1.0f / 128.0f);
    const ff nu = two_sum_f(th - c, tl);
    const ff pc = two_prod_f(th, c);
    ff d = two_sum_f(1.0f, pc.hi);
    d.lo = d.lo + (pc.lo + tl * c);
    d = fast_two_sum_f(d.hi, d.lo);
    const float q1 = nu.hi / d.hi;
    float rem = fmaf(-q1, d.hi, nu.hi); // exact
    rem = (rem + nu.lo) - q1 * d.lo;
    const float q2 = rem / d.hi;
    const ff u = fast_two_sum_f(q1, q2);
    const float u2 = u.hi * u.hi;
    const float corr = u.hi * u2 * (-1.0f / 3.0f) + u.hi * u2 * u2 * (1.0f / 5.0f) +
                       u.hi * u2 * u2 * u2 * (-1.0f / 7.0f) - u2 * u.lo;
    const float2 A = kAtanTab[j];
    const ff s = two_sum_f(A.x, u.hi);
    return fast_two_sum_f(s.hi, s.lo + (A.y + (u.lo + corr)));
}

// pi/2 - a or pi - a in float-float (a >= 0 no larger than the constant).
__device__ __forceinline__ ff ff_const_minus(float chi, float clo, ff a)
{
    const ff s = two_sum_f(chi, -a.hi);
    return fast_two_sum_f(s.hi, s.lo + (clo - a.lo));
}

__device__ __forceinline__ bool ff_atanf(float x, float* out)
{
    const float t = fabsf(x);
    if (!(t >= 0x1p-60f && t <= 0x1p60f))
        return false;
    ff r;
    if (t <= 1.0f)
        r = ff_atan_unit(t, 0.0f);
    else
    {
        const float q1 = 1.0f / t;
        const float rem = fmaf(-q1, t, 1.0f); // exact
        const ff inv = fast_two_sum_f(q1, rem / t);
        r = ff_const_minus(kPi2FHi, kPi2FLo, ff_atan_unit(inv.hi, inv.lo));
    }
    if (x < 0.0f)
        r = {-r.hi, -r.lo};
    return ff_round(r, out);
}

__device__ __forceinline__ bool ff_atan2f(float y, float x, float* out)
{
    const float ax = fabsf(x), ay = fabsf(y);
    // zeros, huge, tiny, inf, nan (each compared on its own: fminf/fmaxf would drop a nan)
    if (!(ax >= 0x1p-60f && ax <= 0x1p60f && ay >= 0x1p-60f && ay <= 0x1p60f))
        return false;
    const float mn = fminf(ax, ay), mx = fmaxf(ax, ay);
    const float q1 = mn / mx;
    const float rem = fmaf(-q1, mx, mn); // exact
    const ff t = fast_two_sum_f(q1, rem / mx);
    ff r = ff_atan_unit(t.hi, t.lo);
    if (ay > ax)
        r = ff_const_minus(kPi2FHi, kPi2FLo, r);
    if (x < 0.0f)
        r = ff_const_minus(kPiFHi, kPiFLo, r);
    if (y < 0.0f)
        r = {-r.hi, -r.lo};
    return ff_round(r, out);
}

__device__ __forceinline__ float cr_expf(float x)
{
    float f;
    if (x >= -87.0f && x <= 88.5f && ff_expf(x, &f))
        return f;
    return cr_expf_fp64(x);
}

__device__ __forceinline__ float cr_atanf(float x)
{
    float f;
    if (ff_atanf(x, &f))
        return f;
    return cr_atanf_fp64(x);
}

__device__ __forceinline__ float cr_atan2f(float y, float x)
{
    float f;
    if (ff_atan2f(y, x, &f))
        return f;
    return cr_atan2f_fp64(y, x);
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
