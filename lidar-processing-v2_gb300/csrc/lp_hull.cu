// lp_hull.cu — per-cluster convex hull and oriented bounding boxes.
//
// Reference: lidar_processing_lib/src/polygonizer.cpp and Processor::run's per-cluster gather
// (src/processor/src/processor.cpp:627-671). Persistent CTAs take clusters from a work queue
// (clusters above 512 members one CTA each, then the others one warp each). The cluster scatter
// has already written each member's x, y contiguously and the cluster's z range. Per cluster:
//   1. the members extreme in 16 directions (an inscribed polygon of members),
//   2. Quickhull refinement: the member farthest outside each polygon edge is inserted, for a
//      few rounds; members proven strictly inside leave the active set. Every polygon vertex is a
//      member, so a member strictly inside the polygon (an FP32 test with a 1e-5 relative margin,
//      far above its rounding error) cannot be a hull vertex,
//   3. sort of the remaining candidates by (x, y, member order), Andrew's monotone chain with the
//      reference's FP64 orientation predicate (polygonizer.cpp:45-50, 62-85) decided in FP32
//      wherever that is provably the same decision: the same output as the reference's chain over
//      all members,
//   4. local hull indices = rank of each hull vertex among the cluster's members in input
//      order (the reference gathers a cluster's points in obstacle order, processor.cpp:640),
//   5. rotating-calipers box (Shamos antipodal pairs, best area kept as a float exactly like
//      BoundingBox::area; comparisons screened in FP32) and the PCA box, one warp each (in the CTA
//      path while the other warps count the ranks).
#include <cfloat>
#include <mutex>

#include "lp_introsort.cuh"
#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_math.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
constexpr int kHullThreads = 256;
constexpr int kHullSmem = 1024; // candidates sorted in shared memory; larger sets use global scratch

template <typename T>
struct HPt
{
    T x, y;
    uint32_t key; // tie-break and identity: member input order
};

template <typename T>
__device__ __forceinline__ bool hpt_less(const HPt<T>& a, const HPt<T>& b)
{
    if (a.x < b.x)
        return true;
    if (b.x < a.x)
        return false;
    if (a.y < b.y)
        return true;
    if (b.y < a.y)
        return false;
    return a.key < b.key;
}

// polygonizer.cpp:45-50: counter-clockwise or collinear, evaluated in FP64 exactly as written
__device__ __forceinline__ bool ccw_or_colinear(double ax, double ay, double bx, double by, double cx, double cy)
{
    return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax) <= 0;
}

__device__ __forceinline__ uint32_t ford(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ unsigned long long warp_max64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t > v ? t : v;
    }
    return v;
}
__device__ __forceinline__ double warp_min_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ---------------------------------------------------------------------------------------------
// Shamos antipodal pairs (polygonizer.cpp:93-163) for the hull P[0..n), written to `pairs`.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double tri_area(double ax, double ay, double bx, double by, double cx, double cy)
{
    // areaOfTriangle, polygonizer.hpp:227-231
    return fabs((ax * (by - cy) + bx * (cy - ay) + cx * (ay - by)) * 0.5);
}

// Triangle-area comparisons of the pair walk, evaluated in FP64 exactly as the reference does.
struct AreaCmpFp64
{
    const double2* P;
    __device__ __forceinline__ double ad(int a, int b, int c) const
    {
        return tri_area(P[a].x, P[a].y, P[b].x, P[b].y, P[c].x, P[c].y);
    }
    __device__ __forceinline__ bool gt(int a1, int b1, int c1, int a2, int b2, int c2) const
    {
        return ad(a1, b1, c1) > ad(a2, b2, c2);
    }
    __device__ __forceinline__ bool eq(int a1, int b1, int c1, int a2, int b2, int c2) const
    {
        return ad(a1, b1, c1) == ad(a2, b2, c2);
    }
};

// The same comparisons decided in FP32 where the float areas differ by more than `tol`, else in
// FP64. Float areas use coordinates relative to (ox, oy): with every |local vertex| <= R the
// float area is within 1.02e-6 R^2 of the exact area of the (float-valued) vertices, and the FP64
// area of the reference within 1e-14 M R (M the largest |coordinate|). tol is at least twice the
// sum of both bounds, so a decision taken in FP32 is the one FP64 takes.
struct AreaCmpFiltered
{
    const double2* P;
    const float2* Pf; // the same vertices as floats (exact: they are float points)
    float ox, oy, tol;
    __device__ __forceinline__ float af(int a, int b, int c) const
    {
        const float ax = Pf[a].x - ox, ay = Pf[a].y - oy;
        const float bx = Pf[b].x - ox, by = Pf[b].y - oy;
        const float cx = Pf[c].x - ox, cy = Pf[c].y - oy;
        return fabsf((ax * (by - cy) + bx * (cy - ay) + cx * (ay - by)) * 0.5f);
    }
    __device__ __forceinline__ double ad(int a, int b, int c) const
    {
        return tri_area(P[a].x, P[a].y, P[b].x, P[b].y, P[c].x, P[c].y);
    }
    __device__ __forceinline__ bool gt(int a1, int b1, int c1, int a2, int b2, int c2) const
    {
        const float d = af(a1, b1, c1) - af(a2, b2, c2);
        if (d > tol)
            return true;
        if (d < -tol)
            return false;
        return ad(a1, b1, c1) > ad(a2, b2, c2);
    }
    __device__ __forceinline__ bool eq(int a1, int b1, int c1, int a2, int b2, int c2) const
    {
        if (fabsf(af(a1, b1, c1) - af(a2, b2, c2)) > tol)
            return false;
        return ad(a1, b1, c1) == ad(a2, b2, c2);
    }
};

template <typename Cmp>
__device__ int antipodal_pairs(const Cmp& cmp, int n, int2* pairs, int cap)
{
    int np = 0;
    if (n < 2)
        return 0;
    auto nx = [n](int i) { return (i + 1 == n) ? 0 : i + 1; };
    auto push = [&](int a, int b) {
        if (np < cap)
            pairs[np] = make_int2(a, b);
        ++np;
    };
    const int i0 = n - 1;
    int i = 0, j = 1;
    int guard = 0;
    // areaOfTriangle(i, i+1, j+1) > areaOfTriangle(i, i+1, j)
    while (cmp.gt(i, nx(i), nx(j), i, nx(i), j) && guard++ < 4 * n + 8)
        j = nx(j);
    const int j0 = j;
    guard = 0;
    while (i != j0 && guard++ < 4 * n + 8)
    {
        i = nx(i);
        push(i, j);
        int g2 = 0;
        while (cmp.gt(i, nx(i), nx(j), i, nx(i), j) && g2++ < 4 * n + 8)
        {
            j = nx(j);
            if (!(i == j0 && j == i0))
                push(i, j);
            else
                return np;
        }
        if (cmp.eq(j, nx(i), nx(j), i, nx(i), j))
        {
            if (!(i == j0 && j == i0))
                push(i, nx(j));
            else
                push(nx(i), j);
        }
    }
    return np;
}

__device__ __forceinline__ float warp_min_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Rotating calipers (polygonizer.cpp:165-278) by one warp: all lanes return the same box.
__device__ void calipers_warp(const double2* P, int n, const int2* pairs, int npairs, lp_bounding_box* out)
{
    const uint32_t lane = lane_id();
    lp_bounding_box box;
    for (int k = 0; k < 4; ++k)
        box.corners[k][0] = box.corners[k][1] = 0.0;
    box.area = 0.0f;
    box.angle_rad = 0.0f;
    box.is_valid = 0;
    if (n < 3)
    {
        if (lane == 0)
            *out = box;
        return;
    }
    double cx = 0.0, cy = 0.0;
    for (int k = 0; k < n; ++k)
    {
        cx += P[k].x;
        cy += P[k].y;
    }
    cx /= n;
    cy /= n;
    float best = __double2float_rn(DBL_MAX); // BoundingBox::area is a float: DBL_MAX -> +inf
    for (int pi = 0; pi < npairs; ++pi)
    {
        const int2 pr = pairs[pi];
        for (int e = 0; e < 2; ++e)
        {
            const int index = e == 0 ? pr.x : pr.y;
            for (int o = 0; o < 2; ++o)
            {
                int nb = index + (o == 0 ? -1 : 1);
                if (nb < 0)
                    nb += n;
                else if (nb >= n)
                    nb -= n;
                const double ex = P[nb].x - P[index].x;
                const double ey = P[nb].y - P[index].y;
                const double len = sqrt(ex * ex + ey * ey);
                if (len < 1.0e-6)
                    continue;
                const double ux = ex / len, uy = ey / len;
                double mnx = DBL_MAX, mxx = -DBL_MAX, mny = DBL_MAX, mxy = -DBL_MAX;
                for (int k = static_cast<int>(lane); k < n; k += 32)
                {
                    const double tx = P[k].x - cx, ty = P[k].y - cy;
                    const double rx = tx * ux + ty * uy;
                    const double ry = -tx * uy + ty * ux;
                    mnx = fmin(mnx, rx);
                    mxx = fmax(mxx, rx);
                    mny = fmin(mny, ry);
                    mxy = fmax(mxy, ry);
                }
                mnx = warp_min_d(mnx);
                mxx = warp_max_d(mxx);
                mny = warp_min_d(mny);
                mxy = warp_max_d(mxy);
                const double area = (mxx - mnx) * (mxy - mny);
                if (area < static_cast<double>(best))
                {
                    best = __double2float_rn(area);
                    box.area = best;
                    box.corners[0][0] = mnx * ux - mny * uy + cx;
                    box.corners[0][1] = mnx * uy + mny * ux + cy;
                    box.corners[1][0] = mxx * ux - mny * uy + cx;
                    box.corners[1][1] = mxx * uy + mny * ux + cy;
                    box.corners[2][0] = mxx * ux - mxy * uy + cx;
                    box.corners[2][1] = mxx * uy + mxy * ux + cy;
                    box.corners[3][0] = mnx * ux - mxy * uy + cx;
                    box.corners[3][1] = mnx * uy + mxy * ux + cy;
                    box.angle_rad = lpm::atan2_approx(__double2float_rn(uy), __double2float_rn(ux));
                    box.is_valid = 1;
                }
            }
        }
    }
    if (lane == 0)
        *out = box;
}

// Principal components of the 2x2 covariance as the reference gets them: V of Eigen 3.4's
// JacobiSVD (svd_.compute, polygonizer.cpp:326), in binary64 and in that library's operation order
// (this file is compiled without multiply-add contraction), so the axes are bit-identical to the
// host's. Steps: divide by the largest |coefficient|; while an off-diagonal entry exceeds
// max(DBL_MIN, 2 eps max|diagonal|), a left rotation symmetrises the (1, 0) block and a Jacobi
// rotation diagonalises it (W rotated on both sides, V on the right); columns ordered by
// descending |diagonal| with a strict comparison. Below the threshold nothing rotates, so a
// near-diagonal covariance keeps the identity axes. Sweeps stop after 64 (one or two in practice;
// the library loops until the test passes). Returns false for a non-finite covariance (the
// library's InvalidInput: the reference's box stays invalid, :327-330).
struct Rot2
{
    double c, s;
};

__device__ __forceinline__ void rot2_apply(double& x0, double& x1, double& y0, double& y1, Rot2 r)
{
    if (r.c == 1.0 && r.s == 0.0)
        return;
    const double a0 = x0, a1 = x1, b0 = y0, b1 = y1;
    x0 = r.c * a0 + r.s * b0;
    x1 = r.c * a1 + r.s * b1;
    y0 = -r.s * a0 + r.c * b0;
    y1 = -r.s * a1 + r.c * b1;
}

__device__ bool pca_axes(double sxx, double sxy, double syy, double& v00, double& v01, double& v10, double& v11)
{
    if (!(isfinite(sxx) && isfinite(sxy) && isfinite(syy)))
        return false;
    double scale = fmax(fmax(fabs(sxx), fabs(sxy)), fmax(fabs(sxy), fabs(syy)));
    if (scale == 0.0)
        scale = 1.0;
    double w00 = sxx / scale, w01 = sxy / scale, w10 = sxy / scale, w11 = syy / scale;
    v00 = 1.0, v01 = 0.0, v10 = 0.0, v11 = 1.0;
    const double precision = 2.0 * DBL_EPSILON;
    double max_diag = fmax(fabs(w00), fabs(w11));
    for (int sweep = 0; sweep < 64; ++sweep)
    {
        const double threshold = fmax(DBL_MIN, precision * max_diag);
        if (!(fabs(w10) > threshold || fabs(w01) > threshold))
            break;
        // block of the index pair (1, 0): m = [[W11, W10], [W01, W00]]
        double m00 = w11, m01 = w10, m10 = w01, m11 = w00;
        Rot2 r1{1.0, 0.0};
        const double t = m00 + m11, d = m10 - m01;
        if (!(fabs(d) < DBL_MIN))
        {
            const double u = t / d;
            const double tmp = sqrt(1.0 + u * u);
            r1 = Rot2{u / tmp, 1.0 / tmp};
        }
        rot2_apply(m00, m01, m10, m11, r1);
        Rot2 rr{1.0, 0.0}; // the Jacobi rotation of [[m00, m01], [m01, m11]]
        const double deno = 2.0 * fabs(m01);
        if (!(deno < DBL_MIN))
        {
            const double tau = (m00 - m11) / deno;
            const double w = sqrt(tau * tau + 1.0);
            const double tt = tau > 0.0 ? 1.0 / (tau + w) : 1.0 / (tau - w);
            const double sign_t = tt > 0.0 ? 1.0 : -1.0;
            const double n = 1.0 / sqrt(tt * tt + 1.0);
            rr = Rot2{n, -sign_t * (m01 / fabs(m01)) * fabs(tt) * n};
        }
        const Rot2 rl{r1.c * rr.c - r1.s * -rr.s, r1.c * -rr.s + r1.s * rr.c}; // r1 composed with rr^T
        const Rot2 rt{rr.c, -rr.s};
        rot2_apply(w10, w11, w00, w01, rl); // rows 1 and 0 of W
        rot2_apply(w01, w11, w00, w10, rt); // columns 1 and 0 of W
        rot2_apply(v01, v11, v00, v10, rt); // columns 1 and 0 of V
        max_diag = fmax(max_diag, fmax(fabs(w11), fabs(w00)));
    }
    if (fabs(w11) * scale > fabs(w00) * scale)
    {
        const double a = v00, b = v10;
        v00 = v01;
        v10 = v11;
        v01 = a;
        v11 = b;
    }
    return true;
}

// PCA box (polygonizer.cpp:280-362) in FP64 by one thread: mean, centred X^T X / (n - 1), the
// JacobiSVD axes, rotate, min/max, corners back to the original frame.
__device__ void pca_box(const double2* P, int n, lp_bounding_box* out)
{
    lp_bounding_box box;
    for (int k = 0; k < 4; ++k)
        box.corners[k][0] = box.corners[k][1] = 0.0;
    box.area = 0.0f;
    box.angle_rad = 0.0f;
    box.is_valid = 0;
    if (n >= 3)
    {
        double mx = 0.0, my = 0.0;
        for (int i = 0; i < n; ++i)
        {
            mx += P[i].x;
            my += P[i].y;
        }
        mx /= n;
        my /= n;
        double sxx = 0.0, sxy = 0.0, syy = 0.0;
        for (int i = 0; i < n; ++i)
        {
            const double dx = P[i].x - mx, dy = P[i].y - my;
            sxx += dx * dx;
            sxy += dx * dy;
            syy += dy * dy;
        }
        sxx /= (n - 1);
        sxy /= (n - 1);
        syy /= (n - 1);
        double v00, v01, v10, v11;
        if (pca_axes(sxx, sxy, syy, v00, v01, v10, v11))
        {
            double mnx = DBL_MAX, mxx = -DBL_MAX, mny = DBL_MAX, mxy = -DBL_MAX;
            for (int i = 0; i < n; ++i)
            {
                const double dx = P[i].x - mx, dy = P[i].y - my;
                const double rx = dx * v00 + dy * v10;
                const double ry = dx * v01 + dy * v11;
                mnx = fmin(mnx, rx);
                mxx = fmax(mxx, rx);
                mny = fmin(mny, ry);
                mxy = fmax(mxy, ry);
            }
            const double xs[4] = {mnx, mxx, mxx, mnx};
            const double ys[4] = {mny, mny, mxy, mxy};
            for (int k = 0; k < 4; ++k)
            {
                box.corners[k][0] = xs[k] * v00 + ys[k] * v01 + mx;
                box.corners[k][1] = xs[k] * v10 + ys[k] * v11 + my;
            }
            box.area = __double2float_rn((mxx - mnx) * (mxy - mny));
            box.angle_rad = __double2float_rn(atan2(v10, v00));
            box.is_valid = 1;
        }
    }
    *out = box;
}

// Sums of the x and of the y coordinates of P[0..n) as the reference's loop computes them in
// binary64 (left to right), by one warp; every lane returns both. Each term is a multiple of
// 2^g (g from its exponent and the trailing zeros of its significand) and below 2^t in
// magnitude; when log2(n) + max t - min g <= 53 every partial sum of any order is exact, so a warp
// tree gives the loop's result. Otherwise (tiny next to large coordinates) the loop runs as written.
__device__ __forceinline__ void sum_xy_fp64(const double2* P, int n, double& sx, double& sy)
{
    const uint32_t lane = lane_id();
    int tmax = -4096, gmin = 4096;
    bool ok = true;
    double px = 0.0, py = 0.0;
    auto scan = [&](double v) {
        const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v));
        const int e = static_cast<int>((u >> 52) & 0x7ffull);
        if ((u << 1) == 0ull)
            return; // zero
        if (e == 0 || e == 0x7ff)
        {
            ok = false; // subnormal, infinite or nan
            return;
        }
        const unsigned long long m = (u & 0xfffffffffffffull) | (1ull << 52);
        tmax = max(tmax, e - 1022);
        gmin = min(gmin, e - 1075 + (__ffsll(static_cast<long long>(m)) - 1));
    };
    for (int k = static_cast<int>(lane); k < n; k += 32)
    {
        scan(P[k].x);
        scan(P[k].y);
        px += P[k].x;
        py += P[k].y;
    }
    ok = __all_sync(0xffffffffu, ok);
    tmax = __reduce_max_sync(0xffffffffu, tmax);
    gmin = __reduce_min_sync(0xffffffffu, gmin);
    const int lg = 32 - __clz(n); // >= log2(n)
    if (ok && lg + tmax - gmin <= 53)
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            px += __shfl_xor_sync(0xffffffffu, px, o);
            py += __shfl_xor_sync(0xffffffffu, py, o);
        }
        sx = px;
        sy = py;
        return;
    }
    sx = 0.0;
    sy = 0.0;
    for (int k = 0; k < n; ++k)
    {
        sx += P[k].x;
        sy += P[k].y;
    }
}

// PCA box by one warp, every step in FP64 in the reference's order: the mean, the covariance sums
// (the principal axis is ill-conditioned exactly where they nearly cancel), the JacobiSVD axes
// (pca_axes, evaluated by every lane alike), the rotated extents (lanes stride over the vertices;
// min and max do not depend on order) and the corners. The box equals the single-thread pca_box
// bit for bit.
__device__ void pca_box_warp(const double2* P, int n, lp_bounding_box* out)
{
    const uint32_t lane = lane_id();
    lp_bounding_box box;
    for (int k = 0; k < 4; ++k)
        box.corners[k][0] = box.corners[k][1] = 0.0;
    box.area = 0.0f;
    box.angle_rad = 0.0f;
    box.is_valid = 0;
    if (n >= 3)
    {
        double sx, sy;
        sum_xy_fp64(P, n, sx, sy);
        // mx = sx / n and my = sy / n on lanes 0 and 1 (one division sequence)
        const double mq = ((lane & 1u) ? sy : sx) / static_cast<double>(n);
        const double mx = __shfl_sync(0xffffffffu, mq, 0), my = __shfl_sync(0xffffffffu, mq, 1);
        // the three covariance sums keep the reference's order: the products of vertex k come from
        // lane k mod 32, lanes 0, 1 and 2 accumulate sxx, sxy and syy in one instruction per step
        double acc = 0.0;
        for (int base = 0; base < n; base += 32)
        {
            const int k = base + static_cast<int>(lane);
            double txx = 0.0, txy = 0.0, tyy = 0.0;
            if (k < n)
            {
                const double dx = P[k].x - mx, dy = P[k].y - my;
                txx = dx * dx;
                txy = dx * dy;
                tyy = dy * dy;
            }
            const int cnt = min(32, n - base);
            for (int j = 0; j < cnt; ++j)
            {
                const double a0 = __shfl_sync(0xffffffffu, txx, j);
                const double a1 = __shfl_sync(0xffffffffu, txy, j);
                const double a2 = __shfl_sync(0xffffffffu, tyy, j);
                acc += (lane == 0u) ? a0 : ((lane == 1u) ? a1 : a2);
            }
        }
        const double cq = acc / static_cast<double>(n - 1);
        const double sxx = __shfl_sync(0xffffffffu, cq, 0), sxy = __shfl_sync(0xffffffffu, cq, 1),
                     syy = __shfl_sync(0xffffffffu, cq, 2);
        double v00, v01, v10, v11;
        if (pca_axes(sxx, sxy, syy, v00, v01, v10, v11))
        {
            double mnx = DBL_MAX, mxx = -DBL_MAX, mny = DBL_MAX, mxy = -DBL_MAX;
            for (int i = static_cast<int>(lane); i < n; i += 32)
            {
                const double dx = P[i].x - mx, dy = P[i].y - my;
                const double rx = dx * v00 + dy * v10;
                const double ry = dx * v01 + dy * v11;
                mnx = fmin(mnx, rx);
                mxx = fmax(mxx, rx);
                mny = fmin(mny, ry);
                mxy = fmax(mxy, ry);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
            {
                mnx = fmin(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
                mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
                mny = fmin(mny, __shfl_xor_sync(0xffffffffu, mny, o));
                mxy = fmax(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
            }
            const double xs[4] = {mnx, mxx, mxx, mnx};
            const double ys[4] = {mny, mny, mxy, mxy};
            for (int k = 0; k < 4; ++k)
            {
                box.corners[k][0] = xs[k] * v00 + ys[k] * v01 + mx;
                box.corners[k][1] = xs[k] * v10 + ys[k] * v11 + my;
            }
            box.area = __double2float_rn((mxx - mnx) * (mxy - mny));
            box.angle_rad = __double2float_rn(atan2(v10, v00));
            box.is_valid = 1;
        }
    }
    if (lane == 0)
        *out = box;
}

// FP64 rotated extents of P about (cx, cy) for the unit direction (ux, uy), by one warp.
__device__ __forceinline__ void extents_fp64(const double2* P, int n, double cx, double cy, double ux, double uy,
                                             double& mnx, double& mxx, double& mny, double& mxy)
{
    mnx = DBL_MAX, mxx = -DBL_MAX, mny = DBL_MAX, mxy = -DBL_MAX;
    for (int k = static_cast<int>(lane_id()); k < n; k += 32)
    {
        const double tx = P[k].x - cx, ty = P[k].y - cy;
        const double rx = tx * ux + ty * uy;
        const double ry = -tx * uy + ty * ux;
        mnx = fmin(mnx, rx);
        mxx = fmax(mxx, rx);
        mny = fmin(mny, ry);
        mxy = fmax(mxy, ry);
    }
    mnx = warp_min_d(mnx);
    mxx = warp_max_d(mxx);
    mny = warp_min_d(mny);
    mxy = warp_max_d(mxy);
}

// extents_fp64 for n <= 32 (vertex k on lane k). The FP32 projections of the float vertices about
// the float centroid along the float direction lie within tol / 2 of the FP64 ones, so a lane more
// than tol above the FP32 minimum cannot hold the FP64 minimum: only the lanes within tol of each
// FP32 extreme compare their FP64 values (usually one or two lanes instead of a five-level tree).
__device__ __forceinline__ double pick_min_fp64(double v, float f, float tol)
{
    const float m = warp_min_f(f);
    double r = DBL_MAX;
    for (uint32_t c = __ballot_sync(0xffffffffu, f <= m + tol); c != 0u; c &= c - 1u)
        r = fmin(r, __shfl_sync(0xffffffffu, v, __ffs(c) - 1));
    return r;
}
__device__ __forceinline__ double pick_max_fp64(double v, float f, float tol)
{
    const float m = warp_max_f(f);
    double r = -DBL_MAX;
    for (uint32_t c = __ballot_sync(0xffffffffu, f >= m - tol); c != 0u; c &= c - 1u)
        r = fmax(r, __shfl_sync(0xffffffffu, v, __ffs(c) - 1));
    return r;
}
__device__ __forceinline__ void extents_screened(const double2* P, const float2* Pf, int n, double cx, double cy,
                                                 double ux, double uy, float cxf, float cyf, float tol, double& mnx,
                                                 double& mxx, double& mny, double& mxy)
{
    const int lane = static_cast<int>(lane_id());
    const bool live = lane < n;
    const float uxf = __double2float_rn(ux), uyf = __double2float_rn(uy);
    double rx = 0.0, ry = 0.0;
    float fx = 0.0f, fy = 0.0f;
    if (live)
    {
        const double tx = P[lane].x - cx, ty = P[lane].y - cy;
        rx = tx * ux + ty * uy;
        ry = -tx * uy + ty * ux;
        const float sx = Pf[lane].x - cxf, sy = Pf[lane].y - cyf;
        fx = sx * uxf + sy * uyf;
        fy = -sx * uyf + sy * uxf;
    }
    mnx = pick_min_fp64(rx, live ? fx : INFINITY, tol);
    mxx = pick_max_fp64(rx, live ? fx : -INFINITY, tol);
    mny = pick_min_fp64(ry, live ? fy : INFINITY, tol);
    mxy = pick_max_fp64(ry, live ? fy : -INFINITY, tol);
}

// Rotating calipers with the candidate boxes screened in FP32 (same result as calipers_warp).
//
// The reference walks the edges named by the antipodal pairs and keeps a box when its FP64 area
// is below the float `best` of the boxes kept so far. An edge's box is the same for both
// directions of the edge (every term only changes sign, exactly), so it is evaluated once per
// hull edge j (P[j] -> P[j+1]): ea[j] = FP32 area, within e = 1e-4 R^2 of the FP64 area (the
// rounding of the float frame, direction and extents stays below 6e-6 R^2, R = largest
// |P - P[0]|). Edges with ea[j] <= T are the contenders, with T grown from the smallest ea until
// no other edge lies within G = 2e + 1e-6 (T + 2e) above it. Every other edge then has a float
// area above every contender's FP64 area and above the float of the smallest area, so (i) the
// last box the reference keeps is a contender's and (ii) replaying the reference's walk over the
// contenders alone, with their FP64 areas, keeps the same boxes among them. Each contender's FP64
// extents are kept by one lane; the winner's corners come from them, negated for the reverse
// direction (exact), so they are the reference's. The skip test (edge length < 1e-6) is screened
// in FP32 too (|float len^2 - len^2| < 2^-21 len^2) and evaluated in FP64 only near 1e-12.
// Only the edges the walk visits take part (an unvisited edge's area is +inf): a pair walk that
// misses a vertex never looks at its edges, and a contender set made only of unvisited edges
// would leave no box where the reference keeps one.
// Up to 32 contenders (one per lane) are handled; more fall back to calipers_warp.
__device__ void calipers_fast(const double2* P, const float2* Pf, int n, const int2* pairs, int npairs, float* ea,
                              float r2, lp_bounding_box* out)
{
    const uint32_t lane = lane_id();
    lp_bounding_box box;
    for (int k = 0; k < 4; ++k)
        box.corners[k][0] = box.corners[k][1] = 0.0;
    box.area = 0.0f;
    box.angle_rad = 0.0f;
    box.is_valid = 0;
    if (n < 3)
    {
        if (lane == 0)
            *out = box;
        return;
    }
    const float ox = Pf[0].x, oy = Pf[0].y;
    const float e = 1e-4f * r2 + 1e-30f;
    // Only edges the walk visits can hold the reference's box: on a near-degenerate hull the pair
    // walk can miss a vertex, and with it an edge that may have the smallest area. Mark the
    // visited edges (ea[j] = 0, the edge mapping of `visit` below) before choosing contenders.
    for (int j = static_cast<int>(lane); j < n; j += 32)
        ea[j] = -1.0f;
    __syncwarp();
    for (int v = static_cast<int>(lane); v < 4 * npairs; v += 32)
    {
        const int2 pr = pairs[v >> 2];
        const int index = ((v >> 1) & 1) ? pr.y : pr.x;
        ea[(v & 1) ? index : ((index == 0) ? n - 1 : index - 1)] = 0.0f; // offset +1: edge index; -1: index - 1
    }
    __syncwarp();
    float amin = INFINITY;
    for (int j = static_cast<int>(lane); j < n; j += 32)
    {
        const int j1 = (j + 1 == n) ? 0 : j + 1;
        const float fx = Pf[j1].x - Pf[j].x, fy = Pf[j1].y - Pf[j].y;
        const float fl2 = fx * fx + fy * fy;
        bool skip = fl2 < 0.9999e-12f || ea[j] != 0.0f; // unvisited edges never compete
        if (!skip && !(fl2 > 1.0001e-12f))
        {
            const double dx = P[j1].x - P[j].x, dy = P[j1].y - P[j].y;
            skip = sqrt(dx * dx + dy * dy) < 1.0e-6;
        }
        float a = INFINITY; // edges the reference skips never compete
        if (!skip)
        {
            const float fl = sqrtf(fl2);
            const float ux = fx / fl, uy = fy / fl;
            float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
            for (int k = 0; k < n; ++k)
            {
                const float tx = Pf[k].x - ox, ty = Pf[k].y - oy;
                const float rx = tx * ux + ty * uy;
                const float ry = -tx * uy + ty * ux;
                mnx = fminf(mnx, rx);
                mxx = fmaxf(mxx, rx);
                mny = fminf(mny, ry);
                mxy = fmaxf(mxy, ry);
            }
            a = (mxx - mnx) * (mxy - mny);
        }
        ea[j] = a;
        amin = fminf(amin, a);
    }
    amin = warp_min_f(amin);
    __syncwarp();
    if (amin == INFINITY)
    {
        if (lane == 0)
            *out = box; // every edge is skipped: no box, as in the reference
        return;
    }
    float T = amin;
    for (int it = 0; it <= n; ++it)
    {
        const float G = 2.0f * e + 1e-6f * (T + 2.0f * e);
        float nt = T;
        for (int j = static_cast<int>(lane); j < n; j += 32)
            if (ea[j] > T && ea[j] <= T + G)
                nt = fmaxf(nt, ea[j]);
        nt = warp_max_f(nt);
        if (nt == T)
            break;
        T = nt;
    }
    // FP64 centroid of the hull vertices, as the reference's loop sums them
    double sx, sy;
    sum_xy_fp64(P, n, sx, sy);
    const double cq = ((lane & 1u) ? sy : sx) / static_cast<double>(n);
    const double cx = __shfl_sync(0xffffffffu, cq, 0), cy = __shfl_sync(0xffffffffu, cq, 1);
    // contender c (in edge order) is held by lane c: its edge, direction, FP64 extents and area
    int my_j = -1;
    int ncont = 0;
    for (int base = 0; base < n; base += 32)
    {
        const int j = base + static_cast<int>(lane);
        const uint32_t mask = __ballot_sync(0xffffffffu, j < n && ea[j] <= T);
        for (uint32_t mm = mask; mm != 0u; mm &= mm - 1u, ++ncont)
            if (static_cast<int>(lane) == ncont) // contender ncont goes to lane ncont
                my_j = base + __ffs(mm) - 1;
        if (ncont > 32)
            break;
    }
    if (ncont > 32)
    {
        calipers_warp(P, n, pairs, npairs, out);
        return;
    }
    // each contender's unit direction on its own lane (one square root and division sequence)
    double my_ux = 0.0, my_uy = 0.0, my_mnx = 0.0, my_mxx = 0.0, my_mny = 0.0, my_mxy = 0.0, my_area = 0.0;
    if (my_j >= 0)
    {
        const int j1 = (my_j + 1 == n) ? 0 : my_j + 1;
        const double ex = P[j1].x - P[my_j].x, ey = P[j1].y - P[my_j].y;
        const double len = sqrt(ex * ex + ey * ey);
        my_ux = ex / len;
        my_uy = ey / len;
    }
    // FP32 projection error bound of extents_screened: the float centroid is within 2^-24 (|cx| +
    // |cy|) of the FP64 one, the float direction within 2^-24 per component, and every difference,
    // product and sum rounds by 2^-24 relative to |P - c|_1 <= 3 sqrt(r2); the window takes 4x
    // (centroid) and 8x (rounding) those sums as tol / 2.
    const float cxf = __double2float_rn(cx), cyf = __double2float_rn(cy);
    const float tol = 2.0f * ((fabsf(cxf) + fabsf(cyf)) * 2.384185791015625e-7f + 3.0f * sqrtf(r2) * 1.9073486328125e-6f) + 1e-30f;
    for (int c = 0; c < ncont; ++c)
    {
        const double ux = __shfl_sync(0xffffffffu, my_ux, c), uy = __shfl_sync(0xffffffffu, my_uy, c);
        double mnx, mxx, mny, mxy;
        if (n <= 32)
            extents_screened(P, Pf, n, cx, cy, ux, uy, cxf, cyf, tol, mnx, mxx, mny, mxy);
        else
            extents_fp64(P, n, cx, cy, ux, uy, mnx, mxx, mny, mxy);
        if (static_cast<int>(lane) == c)
        {
            my_mnx = mnx;
            my_mxx = mxx;
            my_mny = mny;
            my_mxy = mxy;
            my_area = (mxx - mnx) * (mxy - mny);
        }
    }
    // The reference's walk over the contenders. Its float `best` only ever takes contenders' float
    // areas F = fl32(A), and rounding is monotone, so a visit's test A < (double)best is F < best,
    // or at F == best the contender's bit `below` = (A < (double)F). The final best is therefore
    // the smallest F of all visits, and the kept box is the last visit with that F which passes:
    // the first one (it meets a larger best; at F = +inf only with `below`) and every later one
    // with `below`. Each lane takes every 32nd visit (pair pi, side e2, neighbour o).
    float my_f = INFINITY;
    int my_below = 0;
    if (my_j >= 0)
    {
        my_f = __double2float_rn(my_area);
        my_below = my_area < static_cast<double>(my_f);
    }
    const int nvis = 4 * npairs;
    auto visit = [&](int v, int& j, bool& rev, float& f, int& below) {
        const int2 pr = pairs[v >> 2];
        const int index = ((v >> 1) & 1) ? pr.y : pr.x;
        const int o = v & 1;
        int nb = index + (o == 0 ? -1 : 1);
        if (nb < 0)
            nb += n;
        else if (nb >= n)
            nb -= n;
        j = (o == 1) ? index : nb; // hull edge j joins P[j] and P[j+1]
        rev = (o == 0);            // walked from P[j+1] to P[j]
        const bool cont = ea[j] <= T;
        f = INFINITY;
        below = 0;
        for (int c = 0; c < ncont; ++c)
        {
            const int jc = __shfl_sync(0xffffffffu, my_j, c);
            const float fc = __shfl_sync(0xffffffffu, my_f, c);
            const int bc = __shfl_sync(0xffffffffu, my_below, c);
            if (cont && j == jc)
            {
                f = fc;
                below = bc;
            }
        }
        return cont;
    };
    float fmin = INFINITY;
    bool any = false;
    for (int v0 = 0; v0 < nvis; v0 += 32)
    {
        const int v = v0 + static_cast<int>(lane);
        int j, below;
        bool rev;
        float f;
        const bool cont = visit(min(v, nvis - 1), j, rev, f, below) && v < nvis;
        if (cont)
            fmin = fminf(fmin, f);
        any |= cont;
    }
    fmin = warp_min_f(fmin);
    any = __any_sync(0xffffffffu, any);
    int first = INT32_MAX, lastb = -1;
    for (int v0 = 0; any && v0 < nvis; v0 += 32)
    {
        const int v = v0 + static_cast<int>(lane);
        int j, below;
        bool rev;
        float f;
        const bool cont = visit(min(v, nvis - 1), j, rev, f, below) && v < nvis;
        if (cont && f == fmin)
        {
            first = min(first, v);
            if (below)
                lastb = max(lastb, v);
        }
    }
    first = static_cast<int>(__reduce_min_sync(0xffffffffu, static_cast<unsigned>(first)));
    lastb = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(lastb + 1))) - 1;
    const int win = (lastb >= 0) ? lastb : ((any && fmin < INFINITY) ? first : -1);
    float best = __double2float_rn(DBL_MAX);
    int wj = -1;
    bool wrev = false;
    if (win >= 0)
    {
        int below;
        float f;
        visit(win, wj, wrev, f, below);
        best = fmin;
    }
    if (wj >= 0)
    {
        const int src = __ffs(__ballot_sync(0xffffffffu, my_j == wj)) - 1;
        double ux = __shfl_sync(0xffffffffu, my_ux, src), uy = __shfl_sync(0xffffffffu, my_uy, src);
        double mnx = __shfl_sync(0xffffffffu, my_mnx, src), mxx = __shfl_sync(0xffffffffu, my_mxx, src);
        double mny = __shfl_sync(0xffffffffu, my_mny, src), mxy = __shfl_sync(0xffffffffu, my_mxy, src);
        if (wrev)
        {
            // reverse direction: u and every projection change sign exactly
            ux = -ux;
            uy = -uy;
            const double a0 = mnx, a1 = mny;
            mnx = -mxx;
            mxx = -a0;
            mny = -mxy;
            mxy = -a1;
        }
        box.area = best;
        box.corners[0][0] = mnx * ux - mny * uy + cx;
        box.corners[0][1] = mnx * uy + mny * ux + cy;
        box.corners[1][0] = mxx * ux - mny * uy + cx;
        box.corners[1][1] = mxx * uy + mny * ux + cy;
        box.corners[2][0] = mxx * ux - mxy * uy + cx;
        box.corners[2][1] = mxx * uy + mxy * ux + cy;
        box.corners[3][0] = mnx * ux - mxy * uy + cx;
        box.corners[3][1] = mnx * uy + mxy * ux + cy;
        box.angle_rad = lpm::atan2_approx(__double2float_rn(uy), __double2float_rn(ux));
        box.is_valid = 1;
    }
    if (lane == 0)
        *out = box;
}

// Antipodal pairs and the rotating-calipers box of hull P (h vertices) by one warp. With float
// copies Pf and h floats of scratch ea the comparisons are screened in FP32; without them
// (Pf == nullptr) everything runs in FP64.
__device__ void calipers_box(ScanState* st, const double2* P, const float2* Pf, float* ea, int h, int2* pairs,
                             lp_bounding_box* out)
{
    const uint32_t lane = lane_id();
    const int cap = 4 * h + 16;
    int npairs = 0;
    if (Pf != nullptr)
    {
        const float ox = Pf[0].x, oy = Pf[0].y;
        float r2 = 0.0f, mabs = 0.0f;
        for (int k = static_cast<int>(lane); k < h; k += 32)
        {
            const float lx = Pf[k].x - ox, ly = Pf[k].y - oy;
            r2 = fmaxf(r2, lx * lx + ly * ly);
            mabs = fmaxf(mabs, fmaxf(fabsf(Pf[k].x), fabsf(Pf[k].y)));
        }
        r2 = warp_max_f(r2) * 1.001f;
        mabs = warp_max_f(mabs);
        const AreaCmpFiltered cmp{P, Pf, ox, oy, 2.0f * (4e-6f * r2 + 1e-13f * mabs * sqrtf(r2)) + 1e-30f};
        if (lane == 0)
            npairs = antipodal_pairs(cmp, h, pairs, cap);
        npairs = __shfl_sync(0xffffffffu, npairs, 0);
        if (npairs > cap)
        {
            if (lane == 0)
                raise_err(st, ERR_INTERNAL);
            npairs = cap;
        }
        __syncwarp();
        calipers_fast(P, Pf, h, pairs, npairs, ea, r2, out);
    }
    else
    {
        if (lane == 0)
            npairs = antipodal_pairs(AreaCmpFp64{P}, h, pairs, cap);
        npairs = __shfl_sync(0xffffffffu, npairs, 0);
        if (npairs > cap)
        {
            if (lane == 0)
                raise_err(st, ERR_INTERNAL);
            npairs = cap;
        }
        __syncwarp();
        calipers_warp(P, h, pairs, npairs, out);
    }
}

// Orientation test of the monotone chain for float points: decided in FP32 when the float
// determinant exceeds 2^-21 (|t1| + |t2|) in magnitude (its rounding error stays below
// 6 * 2^-24 of that sum, the FP64 form's below 3 * 2^-53), else evaluated in FP64 as written.
// b - a is exact in binary32 (Knuth's TwoSum of b and -a leaves no error).
__device__ __forceinline__ bool diff_exact(float b, float a, float s)
{
    const float a1 = s - b;
    const float b1 = s - a1;
    return ((-a) - a1) + (b - b1) == 0.0f;
}

// u * v has an exact binary32 error term (no underflow in the product).
__device__ __forceinline__ bool prod_err_exact(float u, float v, float t)
{
    return fabsf(t) >= 1e-30f || u == 0.0f || v == 0.0f;
}

__device__ __forceinline__ bool ccw_or_colinear_f(float ax, float ay, float bx, float by, float cx, float cy)
{
    const float u = bx - ax, v = cy - ay, w = by - ay, z = cx - ax;
    const float t1 = u * v;
    const float t2 = w * z;
    const float d = t1 - t2;
    const float bound = (fabsf(t1) + fabsf(t2)) * 4.76837158203125e-7f + 1e-30f;
    if (d > bound)
        return false;
    if (d < -bound)
        return true;
    // Near-tie. When the four differences are exact binary32 values, each product of two of them
    // is exact in binary64 (48 significant bits), so the binary64 expression above has the sign
    // of u v - w z exactly. Rounding to binary32 is monotone, so t1 < t2 implies u v < w z (and
    // t1 > t2 the converse); at t1 == t2 the difference is e1 - e2, the exact product errors.
    if (diff_exact(bx, ax, u) && diff_exact(cy, ay, v) && diff_exact(by, ay, w) && diff_exact(cx, ax, z) &&
        prod_err_exact(u, v, t1) && prod_err_exact(w, z, t2))
    {
        if (t1 != t2)
            return t1 < t2;
        return __fmaf_rn(u, v, -t1) <= __fmaf_rn(w, z, -t2);
    }
    return ccw_or_colinear(ax, ay, bx, by, cx, cy);
}

__device__ __forceinline__ bool chain_pops(const HPt<float>& a, const HPt<float>& b, const HPt<float>& c)
{
    return ccw_or_colinear_f(a.x, a.y, b.x, b.y, c.x, c.y);
}
__device__ __forceinline__ bool chain_pops(const HPt<double>& a, const HPt<double>& b, const HPt<double>& c)
{
    return ccw_or_colinear(a.x, a.y, b.x, b.y, c.x, c.y);
}

// One half of the monotone chain over sorted candidates C[0..m) (polygonizer.cpp:62-88) by one
// thread: the lower half walks C forwards, the upper half backwards from C[m - 1]. The reference's
// second loop continues on the stack of the first but never pops below C[m - 1] (its k >= t
// test), so the upper half is the same walk on its own stack starting from that point. The two
// points below the top stay in registers. Writes the stack to S, returns its size.
template <typename T>
__device__ int chain_half(const HPt<T>* C, int m, int* S, bool upper)
{
    int k = 0;
    HPt<T> a{}, b{};
    for (int j = 0; j < m; ++j)
    {
        const int i = upper ? m - 1 - j : j;
        const HPt<T> c = C[i];
        while (k > 1 && chain_pops(a, b, c))
        {
            --k;
            b = a;
            if (k > 1)
                a = C[S[k - 2]];
        }
        a = b;
        b = c;
        S[k++] = i;
    }
    return k;
}

// The whole chain by one thread: hull positions into H (capacity 2m), returns the hull size
// (the reference's k - 1: the last point repeats the first).
template <typename T>
__device__ int monotone_chain(const HPt<T>* C, int m, int* H)
{
    if (m == 0)
        return -1;
    const int kl = chain_half(C, m, H, false);
    const int ku = chain_half(C, m, H + kl - 1, true); // its first entry is H[kl - 1] = m - 1 again
    return kl + ku - 2;
}

// Strictly left of a -> b by a relative margin of 1e-5: the float cross product errs by less
// than 2.4e-7 (|ex| + |ey|)(|qx| + |qy|), so a point passing is strictly left in exact arithmetic.
__device__ __forceinline__ bool left_strict_f(float ax, float ay, float bx, float by, float px, float py)
{
    const float ex = bx - ax, ey = by - ay, qx = px - ax, qy = py - ay;
    const float cr = ex * qy - ey * qx;
    const float scale = (fabsf(ex) + fabsf(ey)) * (fabsf(qx) + fabsf(qy));
    return cr > 1e-5f * scale + 1e-30f;
}

// Bitonic sort of n candidates (capacity next_pow2(n)) in global memory by one block.
template <typename T>
__device__ void block_sort_global(HPt<T>* a, uint32_t n)
{
    const uint32_t np2 = next_pow2(n);
    for (uint32_t k = n + threadIdx.x; k < np2; k += blockDim.x)
        a[k] = HPt<T>{static_cast<T>(INFINITY), static_cast<T>(INFINITY), 0xffffffffu};
    __syncthreads();
    for (uint32_t k = 2; k <= np2; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
            for (uint32_t i = threadIdx.x; i < np2; i += blockDim.x)
            {
                const uint32_t ixj = i ^ j;
                if (ixj > i)
                {
                    const bool up = ((i & k) == 0);
                    const HPt<T> x = a[i], y = a[ixj];
                    if (up ? hpt_less(y, x) : hpt_less(x, y))
                    {
                        a[i] = y;
                        a[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
}

constexpr int kDirs = 16;         // extreme-point directions of the initial polygon
constexpr int kPolyCap = 256;     // refined polygon capacity
constexpr int kRefineRounds = 12; // farthest-point insertion rounds
constexpr uint32_t kBigCluster = 512; // larger clusters take a whole CTA; smaller ones one warp

struct HullSmem
{
    HPt<float> cand[kHullSmem];
    int stack[2 * kHullSmem + 2];
    double2 hp[kHullSmem];
    float2 pf[kHullSmem];     // hull vertices as floats
    uint32_t hkey[kHullSmem]; // hull vertex member keys, sorted
    int32_t diff[kHullSmem + 1];
    float2 poly[kPolyCap];
    float2 poly2[kPolyCap];
    float4 erec[kPolyCap]; // refinement edge e: start point and direction
    float2 emar[kPolyCap]; // its inside and outside margins per unit of |q|_1
    unsigned long long pkey[kPolyCap];
    unsigned long long ext[kDirs][kHullThreads / 32];
    float2 dirs[kDirs];
    int npoly;
    int grew;
    int ncand;
    int nhull;
    uint32_t work;
};

__device__ __forceinline__ unsigned long long fkey_payload(float v, uint32_t i)
{
    return (static_cast<unsigned long long>(ford(v)) << 32) | i;
}

// A cluster's z range from the ordered keys the cluster scatter accumulates (max of ~ord(z), max
// of ord(z)).
__device__ __forceinline__ float zkey_unord(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ float zkey_min(uint32_t k)
{
    return zkey_unord(~k);
}
__device__ __forceinline__ float zkey_max(uint32_t k)
{
    return zkey_unord(k);
}

// Members extreme in the kDirs = 16 directions 2 pi d / 16 (counter-clockwise). Directions d and
// d + 8 are opposite, so eight projections give both: the largest along d, and for d + 8 the
// smallest along d. Any extreme member serves (the polygon only has to consist of members); ties
// keep the first member a thread sees and, across threads, the larger member position.
struct Extremes16
{
    float hi[8], lo[8];
    uint32_t ih[8], il[8];
    __device__ __forceinline__ void init()
    {
#pragma unroll
        for (int d = 0; d < 8; ++d)
        {
            hi[d] = -INFINITY;
            lo[d] = INFINITY;
            ih[d] = il[d] = 0u;
        }
    }
    __device__ __forceinline__ void add(const float2* dirs, float x, float y, uint32_t i)
    {
#pragma unroll
        for (int d = 0; d < 8; ++d)
        {
            const float v = x * dirs[d].x + y * dirs[d].y;
            if (v > hi[d])
            {
                hi[d] = v;
                ih[d] = i;
            }
            if (v < lo[d])
            {
                lo[d] = v;
                il[d] = i;
            }
        }
    }
    __device__ __forceinline__ unsigned long long key(int d) const
    {
        return d < 8 ? fkey_payload(hi[d], ih[d]) : fkey_payload(-lo[d - 8], il[d - 8]);
    }
};

// Large clusters: the two passes over every member (the 16 direction extremes, the first
// refinement round against the polygon they span) run grid-wide before the hull kernel, in
// (cluster, chunk of kPreChunk members) items, so the cluster's CTA starts at the second round.
// Both reduce exactly (packed-key maxima; the survivors are a set, listed in any order), with
// the hull kernel's expressions, so the hull kernel continues from the same state.
constexpr uint32_t kPreMin = 8192;
constexpr uint32_t kPreChunk = 4096;

__device__ __forceinline__ void hull_dirs(float2* dirs)
{
    if (threadIdx.x < kDirs)
    {
        const float a = 6.28318530717958647692f * static_cast<float>(threadIdx.x) / kDirs;
        dirs[threadIdx.x] = make_float2(cosf(a), sinf(a));
    }
}

// The first polygon from the extremes' packed keys: extreme members in direction order (counter-
// clockwise), repeats dropped. Thread 0.
__device__ int first_polygon(const float2* xy, uint32_t n, const unsigned long long* best, float2* poly)
{
    int np = 0;
    uint32_t prev = 0xffffffffu;
    for (int d = 0; d < kDirs; ++d)
    {
        const uint32_t i = static_cast<uint32_t>(best[d] & 0xffffffffull);
        if (n > 0 && i != prev)
        {
            poly[np++] = xy[i];
            prev = i;
        }
    }
    if (np > 1 && poly[np - 1].x == poly[0].x && poly[np - 1].y == poly[0].y)
        --np;
    return np;
}

__global__ void __launch_bounds__(256) k_hull_pre_ext(BatchDev b)
{
    __shared__ float2 dirs[kDirs];
    __shared__ unsigned long long ext[kDirs][8];
    hull_dirs(dirs);
    __syncthreads();
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t nitems = b.queue[6];
    for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
    {
        const uint2 w = b.pre_items[it];
        const uint32_t g = w.x, start = b.cl_start[g], n = b.cl_cnt[g];
        const uint32_t i0 = w.y * kPreChunk, i1 = min(n, i0 + kPreChunk);
        const float2* xy = b.mxy + start;
        Extremes16 ex;
        ex.init();
        for (uint32_t i = i0 + threadIdx.x; i < i1; i += blockDim.x)
        {
            const float2 q = xy[i];
            ex.add(dirs, q.x, q.y, i);
        }
#pragma unroll
        for (int d = 0; d < kDirs; ++d)
        {
            const unsigned long long v = warp_max64(ex.key(d));
            if (lane == 0)
                ext[d][warp] = v;
        }
        __syncthreads();
        if (threadIdx.x < kDirs)
        {
            unsigned long long best = ext[threadIdx.x][0];
            for (uint32_t k = 1; k < (blockDim.x >> 5); ++k)
                best = ext[threadIdx.x][k] > best ? ext[threadIdx.x][k] : best;
            atomicMax(&b.pre_ext[16ull * g + threadIdx.x], best);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_hull_pre_ref(BatchDev b)
{
    __shared__ float2 poly[kDirs];
    __shared__ float4 erec[kDirs];
    __shared__ float2 emar[kDirs];
    __shared__ unsigned long long pkey[kDirs];
    __shared__ int npoly;
    const uint32_t lane = lane_id();
    const uint32_t nitems = b.queue[6];
    for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x)
    {
        const uint2 w = b.pre_items[it];
        const uint32_t g = w.x, start = b.cl_start[g], n = b.cl_cnt[g];
        const uint32_t i0 = w.y * kPreChunk, i1 = min(n, i0 + kPreChunk);
        const float2* xy = b.mxy + start;
        if (threadIdx.x == 0)
            npoly = first_polygon(xy, n, b.pre_ext + 16ull * g, poly);
        __syncthreads();
        const int np = npoly;
        if (np >= 3)
        {
            for (int e = threadIdx.x; e < np; e += blockDim.x)
            {
                pkey[e] = 0ull;
                const float2 a = poly[e], c = poly[(e + 1 == np) ? 0 : e + 1];
                const float ex = c.x - a.x, ey = c.y - a.y;
                const float l1 = fabsf(ex) + fabsf(ey);
                erec[e] = make_float4(a.x, a.y, ex, ey);
                emar[e] = make_float2(1e-5f * l1, 1e-6f * l1);
            }
            __syncthreads();
            uint32_t* act0 = reinterpret_cast<uint32_t*>(b.hs_stack + 2ull * start + 2ull * g);
            for (uint32_t base = i0; base < i1; base += blockDim.x)
            {
                const uint32_t i = base + threadIdx.x;
                bool keep = false;
                if (i < i1)
                {
                    // the hull kernel's round-0 test: strictly inside every edge by the margin, and
                    // the farthest member outside each edge
                    const float2 q = xy[i];
                    bool in = true;
                    for (int e = 0; e < np; ++e)
                    {
                        const float4 r = erec[e];
                        const float2 mg = emar[e];
                        const float qx = q.x - r.x, qy = q.y - r.y;
                        const float cr = r.z * qy - r.w * qx;
                        const float aq = fabsf(qx) + fabsf(qy);
                        if (!(cr > mg.x * aq))
                            in = false;
                        if (cr < -(mg.y * aq))
                        {
                            const unsigned long long key = fkey_payload(-cr, i);
                            if (key > pkey[e])
                                atomicMax(&pkey[e], key);
                        }
                    }
                    keep = !in;
                }
                const uint32_t mask = __ballot_sync(0xffffffffu, keep);
                uint32_t at = 0;
                if (lane == 0 && mask)
                    at = atomicAdd(&b.pre_nact[g], static_cast<uint32_t>(__popc(mask)));
                at = __shfl_sync(0xffffffffu, at, 0);
                if (keep)
                    act0[at + static_cast<uint32_t>(__popc(mask & ((1u << lane) - 1u)))] = i;
            }
            __syncthreads();
            if (threadIdx.x < static_cast<uint32_t>(np) && pkey[threadIdx.x] != 0ull)
                atomicMax(&b.pre_pk[16ull * g + threadIdx.x], pkey[threadIdx.x]);
        }
        __syncthreads();
    }
}

// Cluster g of scan s: z range, hull (local indices into hull_tmp at cl_start), boxes.
__device__ void hull_one(const BatchDev& b, HullSmem& sm, uint32_t g, int s, int compute_obb)
{
    ScanState* st = &b.state[s];
    const uint32_t n = b.cl_cnt[g];
    const uint32_t start = b.cl_start[g];
    const uint32_t* mem = b.members + start;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0)
        sm.ncand = 0;

    // 1. the extreme member in each of kDirs directions (float projections: any member is a valid
    //    polygon vertex, exactness is not needed here), from the members' x, y stored contiguously
    //    by the cluster scatter; the z range is already known. The members are read as aligned
    //    pairs (slot v: members 2v - a and 2v - a + 1, a = start mod 2), four 16-byte loads in
    //    flight per thread; the halves outside [0, n) are skipped (the loads stay inside the
    //    allocation: it starts at or before member start - a and has 16 bytes after its end).
    const float2* xy = b.mxy + start;
    HPt<float>* gs = reinterpret_cast<HPt<float>*>(b.hs_cand) + 2ull * start; // capacity 2n >= next_pow2(n)
    const int32_t a2 = static_cast<int32_t>(start & 1u);
    const float4* xv = reinterpret_cast<const float4*>(b.mxy + (start - static_cast<uint32_t>(a2)));
    const uint32_t npair = (n + static_cast<uint32_t>(a2) + 1u) / 2u;
    const bool pre = n > kPreMin; // extremes and round 0 came from the grid-wide passes
    Extremes16 ex;
    ex.init();
    for (uint32_t v0 = threadIdx.x; !pre && v0 < npair; v0 += 4u * blockDim.x)
    {
        float4 q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const uint32_t v = v0 + static_cast<uint32_t>(u) * blockDim.x;
            q[u] = (v < npair) ? xv[v] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const int32_t i = 2 * static_cast<int32_t>(v0 + static_cast<uint32_t>(u) * blockDim.x) - a2;
            if (i >= 0 && i < static_cast<int32_t>(n))
                ex.add(sm.dirs, q[u].x, q[u].y, static_cast<uint32_t>(i));
            if (i + 1 >= 0 && i + 1 < static_cast<int32_t>(n))
                ex.add(sm.dirs, q[u].z, q[u].w, static_cast<uint32_t>(i + 1));
        }
    }
    if (!pre)
    {
        unsigned long long ext[kDirs];
#pragma unroll
        for (int d = 0; d < kDirs; ++d)
            ext[d] = warp_max64(ex.key(d));
        if (lane == 0)
        {
#pragma unroll
            for (int d = 0; d < kDirs; ++d)
                sm.ext[d][warp] = ext[d];
        }
    }
    else if (threadIdx.x < kDirs * (kHullThreads / 32))
    {
        const uint32_t d = threadIdx.x / (kHullThreads / 32), w = threadIdx.x % (kHullThreads / 32);
        sm.ext[d][w] = (w == 0) ? b.pre_ext[16ull * g + d] : 0ull;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        b.cl_zmin[g] = zkey_min(b.cl_zkey[2u * g]);
        b.cl_zmax[g] = zkey_max(b.cl_zkey[2u * g + 1u]);
        // initial polygon: extreme members in direction order (counter-clockwise), repeats dropped
        int np = 0;
        uint32_t prev = 0xffffffffu;
        for (int d = 0; d < kDirs; ++d)
        {
            unsigned long long best = sm.ext[d][0];
            for (int w = 1; w < kHullThreads / 32; ++w)
                best = sm.ext[d][w] > best ? sm.ext[d][w] : best;
            const uint32_t i = static_cast<uint32_t>(best & 0xffffffffull);
            if (n > 0 && i != prev)
            {
                sm.poly[np++] = xy[i];
                prev = i;
            }
        }
        if (np > 1 && sm.poly[np - 1].x == sm.poly[0].x && sm.poly[np - 1].y == sm.poly[0].y)
            --np;
        sm.npoly = np;
    }
    __syncthreads();

    int32_t* hull_dst = b.hull_tmp + start;
    if (n < 3)
    {
        // convexHull with fewer than 3 points returns 0..n-1 (polygonizer.cpp:36-41)
        if (threadIdx.x == 0)
        {
            for (uint32_t i = 0; i < n; ++i)
                hull_dst[i] = static_cast<int32_t>(i);
            b.hull_cnt[g] = n;
            if (compute_obb)
            {
                lp_bounding_box z;
                memset(&z, 0, sizeof(z));
                b.obb_c[g] = z;
                b.obb_p[g] = z;
            }
        }
        __syncthreads();
        return;
    }

    // 2. refine the polygon: insert the member farthest outside each edge (Quickhull step),
    //    while it grows and fits. Every vertex is a member, so the polygon stays inside the hull.
    //    Members proven strictly inside the current polygon leave the active set: the float test
    //    keeps a 1e-5 relative margin, far above its rounding error, so no hull vertex is dropped.
    uint32_t* act[2] = {reinterpret_cast<uint32_t*>(b.hs_stack + 2ull * start + 2ull * g), nullptr};
    act[1] = act[0] + n; // two member lists of n entries in the chain-stack scratch (2n + 2)
    int cur = -1;        // -1: the active set is all members
    uint32_t nact = n;
    for (int round = 0; round < kRefineRounds; ++round)
    {
        const int np = sm.npoly;
        if (np < 3)
            break;
        for (int e = threadIdx.x; e < np; e += blockDim.x)
        {
            sm.pkey[e] = 0ull;
            const float2 a = sm.poly[e], c = sm.poly[(e + 1 == np) ? 0 : e + 1];
            const float ex = c.x - a.x, ey = c.y - a.y;
            const float l1 = fabsf(ex) + fabsf(ey);
            sm.erec[e] = make_float4(a.x, a.y, ex, ey);
            sm.emar[e] = make_float2(1e-5f * l1, 1e-6f * l1);
        }
        if (threadIdx.x == 0)
            sm.ncand = 0;
        __syncthreads();
        const int nxt = (cur == 0) ? 1 : 0;
        // two members per thread and edge load; q = p - a, cr < 0: right of the edge, outside
        auto edge = [&](const float4& r, const float2& mg, int e, float px, float py, uint32_t i, bool& in) {
            const float qx = px - r.x, qy = py - r.y;
            const float cr = r.z * qy - r.w * qx;
            const float aq = fabsf(qx) + fabsf(qy);
            if (!(cr > mg.x * aq))
                in = false;
            if (cr < -(mg.y * aq))
            {
                const unsigned long long key = fkey_payload(-cr, i);
                if (key > sm.pkey[e])
                    atomicMax(&sm.pkey[e], key);
            }
        };
        // members ok0 / ok1 (at least one): a missing one repeats the other and is not listed
        auto test2 = [&](float2 p0, uint32_t i0, bool ok0, float2 p1, uint32_t i1, bool ok1) {
            if (!ok0)
            {
                p0 = p1;
                i0 = i1;
            }
            if (!ok1)
            {
                p1 = p0;
                i1 = i0;
            }
            bool in0 = true, in1 = true;
            for (int e = 0; e < np; ++e)
            {
                const float4 r = sm.erec[e];
                const float2 mg = sm.emar[e];
                edge(r, mg, e, p0.x, p0.y, i0, in0);
                edge(r, mg, e, p1.x, p1.y, i1, in1);
            }
            if (ok0 && !in0)
                act[nxt][atomicAdd(&sm.ncand, 1)] = i0;
            if (ok1 && !in1)
                act[nxt][atomicAdd(&sm.ncand, 1)] = i1;
        };
        if (cur < 0 && pre)
        {
            // round 0 ran grid-wide against this polygon: its survivors are in act[0], and the
            // farthest member outside each edge is in the pass's record
            for (int e = threadIdx.x; e < np; e += blockDim.x)
                sm.pkey[e] = b.pre_pk[16ull * g + e];
            if (threadIdx.x == 0)
                sm.ncand = static_cast<int>(b.pre_nact[g]);
        }
        else if (cur < 0)
        {
            // all members: the aligned pairs of step 1, one 16-byte load each
            for (uint32_t v = threadIdx.x; v < npair; v += blockDim.x)
            {
                const float4 q = xv[v];
                const int32_t i = 2 * static_cast<int32_t>(v) - a2;
                test2(make_float2(q.x, q.y), static_cast<uint32_t>(max(i, 0)), i >= 0,
                      make_float2(q.z, q.w), static_cast<uint32_t>(i + 1), i + 1 < static_cast<int32_t>(n));
            }
        }
        else
        {
            for (uint32_t t = threadIdx.x; t < nact; t += 2u * blockDim.x)
            {
                const uint32_t t1 = t + blockDim.x;
                const bool two = t1 < nact;
                const uint32_t i0 = act[cur][t];
                const uint32_t i1 = two ? act[cur][t1] : i0;
                test2(xy[i0], i0, true, xy[i1], i1, two);
            }
        }
        __syncthreads();
        cur = nxt;
        nact = static_cast<uint32_t>(sm.ncand);
        if (threadIdx.x == 0)
        {
            int add = 0;
            for (int e = 0; e < np; ++e)
                add += (sm.pkey[e] != 0ull);
            sm.grew = 0;
            if (add > 0 && np + add <= kPolyCap)
            {
                int w = 0;
                for (int e = 0; e < np; ++e)
                {
                    sm.poly2[w++] = sm.poly[e];
                    if (sm.pkey[e] != 0ull)
                    {
                        const uint32_t i = static_cast<uint32_t>(sm.pkey[e] & 0xffffffffull);
                        sm.poly2[w++] = xy[i];
                    }
                }
                for (int e = 0; e < w; ++e)
                    sm.poly[e] = sm.poly2[e];
                sm.npoly = w;
                sm.grew = 1;
            }
        }
        __syncthreads();
        if (!sm.grew)
            break;
    }

    // 3. candidates: active members not strictly inside the polygon by a relative margin far
    //    above float rounding (a hull vertex is never strictly inside a polygon of members)
    const int npf = sm.npoly;
    auto inside = [&](float px, float py) {
        if (npf < 3)
            return false;
        for (int d = 0; d < npf; ++d)
        {
            const float2 a = sm.poly[d], c = sm.poly[(d + 1 == npf) ? 0 : d + 1];
            if (!left_strict_f(a.x, a.y, c.x, c.y, px, py))
                return false;
        }
        return true;
    };
    if (threadIdx.x == 0)
        sm.ncand = 0;
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < nact; t += blockDim.x)
    {
        const uint32_t i = (cur < 0) ? t : act[cur][t];
        const uint32_t o = mem[i];
        const float2 p = xy[i];
        if (!inside(p.x, p.y))
        {
            const int pos = atomicAdd(&sm.ncand, 1);
            if (pos < kHullSmem)
                sm.cand[pos] = HPt<float>{p.x, p.y, o};
            gs[pos] = HPt<float>{p.x, p.y, o};
        }
    }
    __syncthreads();
    const int m = sm.ncand;
    const bool small = m <= kHullSmem;

    // 4. sort by (x, y, input order) and the monotone chain
    const HPt<float>* C;
    int* H;
    if (small)
    {
        const uint32_t np2 = next_pow2(static_cast<uint32_t>(m));
        for (uint32_t i = m + threadIdx.x; i < np2; i += blockDim.x)
            sm.cand[i] = HPt<float>{INFINITY, INFINITY, 0xffffffffu};
        __syncthreads();
        block_bitonic_sort(sm.cand, np2, [](const HPt<float>& a, const HPt<float>& c) { return hpt_less(a, c); });
        C = sm.cand;
        H = sm.stack;
    }
    else
    {
        block_sort_global(gs, static_cast<uint32_t>(m));
        C = gs;
        H = b.hs_stack + 2ull * start + 2ull * g; // capacity 2n + 2 >= 2m + 2
    }
    __syncthreads();
    // lower half on thread 0, upper half on thread 32 (another warp) into H + m + 1; then the
    // upper half moves down behind the lower one (forwards: the source lies above the target)
    if (threadIdx.x == 0)
        sm.nhull = chain_half(C, m, H, false);
    else if (threadIdx.x == 32)
        sm.grew = chain_half(C, m, H + m + 1, true);
    __syncthreads();
    if (threadIdx.x == 0)
    {
        const int kl = sm.nhull, ku = sm.grew;
        for (int j = 1; j < ku - 1; ++j)
            H[kl - 1 + j] = H[m + 1 + j];
        sm.nhull = (m == 0) ? -1 : kl + ku - 2;
    }
    __syncthreads();
    const int h = sm.nhull;
    {
        // a hull vertex with an identical candidate next to it: the reference's pick among them
        // follows std::sort's order (k_hull_ties replays it)
        bool tie = false;
        for (int j = threadIdx.x; j < h; j += blockDim.x)
        {
            const int q = H[j];
            const HPt<float> c = C[q];
            tie |= (q > 0 && C[q - 1].x == c.x && C[q - 1].y == c.y) ||
                   (q + 1 < static_cast<int>(m) && C[q + 1].x == c.x && C[q + 1].y == c.y);
        }
        if (__syncthreads_or(tie) && threadIdx.x == 0)
            b.tie_list[atomicAdd(&b.queue[5], 1u)] = g;
    }

    // 5 + 6. Local index of each hull vertex (the number of members before it in input order) and
    //        the boxes. They only read the hull: warps 0 and 1 compute the calipers and PCA boxes
    //        while the other warps count (all warps count when no boxes are asked for).
    const bool fast = h <= kHullSmem;
    double2* P = fast ? sm.hp : (b.hs_pts + start);
    if (compute_obb)
        for (int j = threadIdx.x; j < h; j += blockDim.x)
        {
            const HPt<float> c = C[H[j]];
            P[j] = make_double2(static_cast<double>(c.x), static_cast<double>(c.y));
            if (fast)
                sm.pf[j] = make_float2(c.x, c.y);
        }
    const uint32_t np2 = next_pow2(static_cast<uint32_t>(h));
    if (fast)
    {
        for (int j = threadIdx.x; j < h; j += blockDim.x)
            sm.hkey[j] = C[H[j]].key;
        for (uint32_t j = h + threadIdx.x; j < np2; j += blockDim.x)
            sm.hkey[j] = 0xffffffffu;
        for (int j = threadIdx.x; j <= h; j += blockDim.x)
            sm.diff[j] = 0;
    }
    __syncthreads();
    if (fast)
        block_bitonic_sort(sm.hkey, np2, [](uint32_t a, uint32_t c) { return a < c; });
    const uint32_t ix0 = compute_obb ? 64u : 0u; // first counting thread
    const uint32_t ncount = blockDim.x - ix0;
    if (compute_obb && warp < 2)
    {
        // the refinement's edge records are free: float scratch of the calipers screen
        if (warp == 0)
            calipers_box(st, P, fast ? sm.pf : nullptr, reinterpret_cast<float*>(sm.erec), h,
                         b.hs_pairs + 4ull * start + 16ull * g, &b.obb_c[g]);
        else
            pca_box_warp(P, h, &b.obb_p[g]);
    }
    else if (fast)
    {
        // member o adds 1 to every hull vertex with a larger key: diff[upper_bound(o)] += 1. Each
        // thread walks a contiguous chunk of the member list as aligned quadruples (slot v:
        // members 4v - a .. 4v - a + 3, a = start mod 4; entries outside [0, n) skipped, the loads
        // stay inside the allocation). Members come in ascending index runs, so consecutive
        // members mostly fall into the same bin: a member inside the current bin's key interval
        // skips the search, and a bin's count is added once when the bin changes.
        const uint32_t a4 = start & 3u;
        const uint4* mv = reinterpret_cast<const uint4*>(b.members + (start - a4));
        const uint32_t nq = (n + a4 + 3u) / 4u;
        const uint32_t per = (nq + ncount - 1u) / ncount;
        const uint32_t q0 = (threadIdx.x - ix0) * per, q1 = min(nq, q0 + per);
        int cb = h, cc = 0;               // current bin and its pending count
        uint32_t blo = 1u, bhi = 0u;      // its key interval [blo, bhi) (empty: no bin yet)
        auto member = [&](uint32_t o) {
            if (o >= blo && o < bhi)
            {
                ++cc;
                return;
            }
            int l = 0, hi = h;
            while (l < hi)
            {
                const int mid = (l + hi) >> 1;
                if (sm.hkey[mid] > o)
                    hi = mid;
                else
                    l = mid + 1;
            }
            if (l != cb)
            {
                if (cc > 0 && cb < h)
                    atomicAdd(&sm.diff[cb], cc);
                cb = l;
                cc = 0;
            }
            ++cc;
            blo = (l > 0) ? sm.hkey[l - 1] : 0u;
            bhi = (l < h) ? sm.hkey[l] : 0xffffffffu;
        };
        for (uint32_t v0 = q0; v0 < q1; v0 += 4u)
        {
            uint4 q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                q[u] = (v0 + u < q1) ? mv[v0 + u] : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                const int32_t i = 4 * static_cast<int32_t>(v0 + u) - static_cast<int32_t>(a4);
                const uint32_t oo[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (v0 + u < q1 && i + c >= 0 && i + c < static_cast<int32_t>(n))
                        member(oo[c]);
            }
        }
        if (cc > 0 && cb < h)
            atomicAdd(&sm.diff[cb], cc);
    }
    else
    {
        for (int j = static_cast<int>(warp - ix0 / 32u); j < h; j += static_cast<int>(ncount / 32u))
        {
            const uint32_t key = C[H[j]].key;
            uint32_t cnt = 0;
            for (uint32_t base = 0; base < n; base += 32)
            {
                const uint32_t i = base + lane;
                const bool lt = (i < n) && (mem[i] < key);
                cnt += __popc(__ballot_sync(0xffffffffu, lt));
            }
            if (lane == 0)
                hull_dst[j] = static_cast<int32_t>(cnt);
        }
    }
    __syncthreads();
    if (fast)
    {
        if (threadIdx.x == 0)
        {
            int run = 0;
            for (int t = 0; t < h; ++t)
            {
                run += sm.diff[t];
                sm.diff[t] = run; // members with a smaller key than hkey[t]
            }
        }
        __syncthreads();
        for (int j = threadIdx.x; j < h; j += blockDim.x)
        {
            const uint32_t key = C[H[j]].key;
            int lo = 0, hi = h - 1;
            while (lo < hi)
            {
                const int mid = (lo + hi) >> 1;
                if (sm.hkey[mid] < key)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            hull_dst[j] = sm.diff[lo];
        }
    }
    if (threadIdx.x == 0)
        b.hull_cnt[g] = static_cast<uint32_t>(h);
    __syncthreads();
}

// ---------------------------------------------------------------------------------------------
// Warp path for clusters of at most kBigCluster members: the same steps as hull_one without CTA
// barriers (the 16-direction polygon is the prefilter; candidates rarely exceed a warp's buffer,
// and then the sort and the chain stack move to global scratch).
// ---------------------------------------------------------------------------------------------
constexpr int kWarpCand = 256;
constexpr uint32_t kWarpRefineMin = 48; // more candidates than this: refine the polygon first
constexpr int kWarpPoly = 64;           // refined polygon capacity of the warp path

struct WarpSmem
{
    HPt<float> cand[kWarpCand];
    int stack[2 * kWarpCand + 2];
    double2 hp[kWarpCand];
    float2 pf[kWarpCand];
    float2 poly[kDirs];
    int npoly;
};

// Scratch of the warp path's polygon refinement (inside WarpSmem::hp, unused until the boxes).
struct WarpRefine
{
    float2 rp[kWarpPoly], rp2[kWarpPoly];
    float4 erec[kWarpPoly];
    float2 emar[kWarpPoly];
    unsigned long long pkey[kWarpPoly];
};
static_assert(sizeof(WarpRefine) <= sizeof(double2) * kWarpCand, "refinement scratch exceeds the box scratch");

// Quickhull rounds over the candidates C[0..m) (at most 16 per lane), starting from the warp's
// 16-direction polygon: each round tests every candidate against the polygon's edges (keeping
// the farthest candidate outside each edge), compacts away the candidates strictly inside, and
// inserts the farthest ones. Returns the number of candidates left in C.
__device__ uint32_t warp_refine(WarpSmem& ws, HPt<float>* C, uint32_t m, int np)
{
    WarpRefine& wr = *reinterpret_cast<WarpRefine*>(ws.hp);
    const uint32_t lane = lane_id();
    for (int e = static_cast<int>(lane); e < np; e += 32)
        wr.rp[e] = ws.poly[e];
    __syncwarp();
    for (int round = 0; round < 4 && m > kWarpRefineMin; ++round)
    {
        for (int e = static_cast<int>(lane); e < np; e += 32)
        {
            const float2 a = wr.rp[e], c = wr.rp[(e + 1 == np) ? 0 : e + 1];
            const float ex = c.x - a.x, ey = c.y - a.y;
            const float l1 = fabsf(ex) + fabsf(ey);
            wr.erec[e] = make_float4(a.x, a.y, ex, ey);
            wr.emar[e] = make_float2(1e-5f * l1, 1e-6f * l1);
            wr.pkey[e] = 0ull;
        }
        __syncwarp();
        uint32_t inbits = 0u;
        for (uint32_t base = 0, q = 0; base < m; base += 32, ++q)
        {
            const uint32_t k = base + lane;
            bool in = false;
            if (k < m)
            {
                const HPt<float> c = C[k];
                in = true;
                for (int e = 0; e < np; ++e)
                {
                    const float4 r = wr.erec[e];
                    const float2 mg = wr.emar[e];
                    const float qx = c.x - r.x, qy = c.y - r.y;
                    const float cr = r.z * qy - r.w * qx; // < 0: right of the edge, outside
                    const float aq = fabsf(qx) + fabsf(qy);
                    if (!(cr > mg.x * aq))
                        in = false;
                    if (cr < -(mg.y * aq))
                    {
                        const unsigned long long key = fkey_payload(-cr, k);
                        if (key > wr.pkey[e])
                            atomicMax(&wr.pkey[e], key);
                    }
                }
            }
            inbits |= (in ? 1u : 0u) << q;
        }
        __syncwarp();
        // lane 0 inserts each edge's farthest outside candidate (positions before compaction)
        int grew = 0, nnew = np;
        if (lane == 0)
        {
            int add = 0;
            for (int e = 0; e < np; ++e)
                add += (wr.pkey[e] != 0ull);
            if (add > 0 && np + add <= kWarpPoly)
            {
                int w = 0;
                for (int e = 0; e < np; ++e)
                {
                    wr.rp2[w++] = wr.rp[e];
                    if (wr.pkey[e] != 0ull)
                    {
                        const HPt<float> c = C[static_cast<uint32_t>(wr.pkey[e] & 0xffffffffull)];
                        wr.rp2[w++] = make_float2(c.x, c.y);
                    }
                }
                for (int e = 0; e < w; ++e)
                    wr.rp[e] = wr.rp2[e];
                nnew = w;
                grew = 1;
            }
        }
        __syncwarp();
        grew = __shfl_sync(0xffffffffu, grew, 0);
        np = __shfl_sync(0xffffffffu, nnew, 0);
        // compact in place (every chunk is read before any of its positions is written)
        uint32_t wpos = 0;
        for (uint32_t base = 0, q = 0; base < m; base += 32, ++q)
        {
            const uint32_t k = base + lane;
            const bool keep = k < m && !((inbits >> q) & 1u);
            HPt<float> c{0.0f, 0.0f, 0u};
            if (keep)
                c = C[k];
            const uint32_t mask = __ballot_sync(0xffffffffu, keep);
            __syncwarp();
            if (keep)
                C[wpos + __popc(mask & ((1u << lane) - 1u))] = c;
            wpos += __popc(mask);
        }
        m = wpos;
        __syncwarp();
        if (!grew)
            break;
    }
    return m;
}

__device__ void hull_one_warp(const BatchDev& b, WarpSmem& ws, const float2* dirs, uint32_t g, int s, int compute_obb)
{
    ScanState* st = &b.state[s];
    const uint32_t n = b.cl_cnt[g];
    const uint32_t start = b.cl_start[g];
    const uint32_t* mem = b.members + start;
    const uint32_t lane = lane_id();
    const float2* xy = b.mxy + start;
    Extremes16 ex;
    ex.init();
    for (uint32_t i = lane; i < n; i += 32)
    {
        const float2 p = xy[i];
        ex.add(dirs, p.x, p.y, i);
    }
    unsigned long long ext[kDirs];
#pragma unroll
    for (int d = 0; d < kDirs; ++d)
        ext[d] = warp_max64(ex.key(d));
    if (lane == 0)
    {
        b.cl_zmin[g] = zkey_min(b.cl_zkey[2u * g]);
        b.cl_zmax[g] = zkey_max(b.cl_zkey[2u * g + 1u]);
        int np = 0;
        uint32_t prev = 0xffffffffu;
        for (int d = 0; d < kDirs; ++d)
        {
            const uint32_t i = static_cast<uint32_t>(ext[d] & 0xffffffffull);
            if (n > 0 && i != prev)
            {
                ws.poly[np++] = xy[i];
                prev = i;
            }
        }
        if (np > 1 && ws.poly[np - 1].x == ws.poly[0].x && ws.poly[np - 1].y == ws.poly[0].y)
            --np;
        ws.npoly = np;
    }
    __syncwarp();
    int32_t* hull_dst = b.hull_tmp + start;
    if (n < 3)
    {
        if (lane == 0)
        {
            for (uint32_t i = 0; i < n; ++i)
                hull_dst[i] = static_cast<int32_t>(i);
            b.hull_cnt[g] = n;
            if (compute_obb)
            {
                lp_bounding_box z;
                memset(&z, 0, sizeof(z));
                b.obb_c[g] = z;
                b.obb_p[g] = z;
            }
        }
        __syncwarp();
        return;
    }
    const int npf = ws.npoly;
    auto inside = [&](float px, float py) {
        if (npf < 3)
            return false;
        for (int d = 0; d < npf; ++d)
        {
            const float2 a = ws.poly[d], c = ws.poly[(d + 1 == npf) ? 0 : d + 1];
            if (!left_strict_f(a.x, a.y, c.x, c.y, px, py))
                return false;
        }
        return true;
    };
    HPt<float>* gs = reinterpret_cast<HPt<float>*>(b.hs_cand) + 2ull * start; // capacity 2n >= next_pow2(n)
    uint32_t m = 0;
    for (uint32_t base = 0; base < n; base += 32)
    {
        const uint32_t i = base + lane;
        bool keep = false;
        HPt<float> c{0.0f, 0.0f, 0u};
        if (i < n)
        {
            const uint32_t o = mem[i];
            const float2 p = xy[i];
            keep = !inside(p.x, p.y);
            c = HPt<float>{p.x, p.y, o};
        }
        const uint32_t mask = __ballot_sync(0xffffffffu, keep);
        if (keep)
        {
            const uint32_t pos = m + __popc(mask & ((1u << lane) - 1u));
            if (pos < static_cast<uint32_t>(kWarpCand))
                ws.cand[pos] = c;
            gs[pos] = c;
        }
        m += __popc(mask);
    }
    __syncwarp();
    // Many candidates (members spread along the boundary, e.g. an arc): refine the polygon as the
    // CTA path does (insert the candidate farthest outside each edge, drop the candidates proven
    // strictly inside by the 1e-5 relative margin), a few rounds, in the box scratch (ws.hp).
    HPt<float>* C0 = (m <= static_cast<uint32_t>(kWarpCand)) ? ws.cand : gs;
    if (m > kWarpRefineMin && npf >= 3)
        m = warp_refine(ws, C0, m, npf);
    const bool small = m <= static_cast<uint32_t>(kWarpCand);
    if (small && C0 == gs)
    {
        for (uint32_t k = lane; k < m; k += 32)
            ws.cand[k] = gs[k];
        __syncwarp();
    }
    HPt<float>* C = small ? ws.cand : gs;
    int* H = small ? ws.stack : (b.hs_stack + 2ull * start + 2ull * g);
    if (m <= 32u)
    {
        // one candidate per lane, sorted in registers (hpt_less is a total order: any sort agrees)
        HPt<float> v = (lane < m) ? C[lane] : HPt<float>{INFINITY, INFINITY, 0xffffffffu};
#pragma unroll
        for (uint32_t k = 2; k <= 32; k <<= 1)
        {
#pragma unroll
            for (uint32_t j = k >> 1; j > 0; j >>= 1)
            {
                HPt<float> o;
                o.x = __shfl_xor_sync(0xffffffffu, v.x, j);
                o.y = __shfl_xor_sync(0xffffffffu, v.y, j);
                o.key = __shfl_xor_sync(0xffffffffu, v.key, j);
                const bool up = ((lane & k) == 0), lower = ((lane & j) == 0);
                if ((lower == up) ? hpt_less(o, v) : hpt_less(v, o))
                    v = o;
            }
        }
        __syncwarp();
        if (lane < m)
            C[lane] = v;
    }
    else
    {
        const uint32_t np2 = next_pow2(m);
        for (uint32_t i = m + lane; i < np2; i += 32)
            C[i] = HPt<float>{INFINITY, INFINITY, 0xffffffffu};
        __syncwarp();
        warp_bitonic_smem(C, np2, [](const HPt<float>& x, const HPt<float>& y) { return hpt_less(x, y); });
    }
    int h = 0;
    if (lane == 0)
        h = monotone_chain(C, static_cast<int>(m), H);
    h = __shfl_sync(0xffffffffu, h, 0);
    __syncwarp();
    {
        bool tie = false;
        for (int j = static_cast<int>(lane); j < h; j += 32)
        {
            const int q = H[j];
            const HPt<float> c = C[q];
            tie |= (q > 0 && C[q - 1].x == c.x && C[q - 1].y == c.y) ||
                   (q + 1 < static_cast<int>(m) && C[q + 1].x == c.x && C[q + 1].y == c.y);
        }
        if (__any_sync(0xffffffffu, tie) && lane == 0)
            b.tie_list[atomicAdd(&b.queue[5], 1u)] = g;
    }
    for (int j = 0; j < h; ++j)
    {
        const uint32_t key = C[H[j]].key;
        uint32_t cnt = 0;
        for (uint32_t base = 0; base < n; base += 32)
        {
            const uint32_t i = base + lane;
            cnt += __popc(__ballot_sync(0xffffffffu, (i < n) && (mem[i] < key)));
        }
        if (lane == 0)
            hull_dst[j] = static_cast<int32_t>(cnt);
    }
    if (lane == 0)
        b.hull_cnt[g] = static_cast<uint32_t>(h);
    if (compute_obb)
    {
        const bool fast = h <= kWarpCand;
        double2* P = fast ? ws.hp : (b.hs_pts + start);
        for (int j = static_cast<int>(lane); j < h; j += 32)
        {
            const HPt<float> c = C[H[j]];
            P[j] = make_double2(static_cast<double>(c.x), static_cast<double>(c.y));
            if (fast)
                ws.pf[j] = make_float2(c.x, c.y);
        }
        __syncwarp();
        // the chain stack is free again: float scratch of the calipers screen
        calipers_box(st, P, fast ? ws.pf : nullptr, reinterpret_cast<float*>(ws.stack), h,
                     b.hs_pairs + 4ull * start + 16ull * g, &b.obb_c[g]);
        pca_box_warp(P, h, &b.obb_p[g]);
    }
    __syncwarp();
}

// Work items: every cluster of the batch. queue[2] counts clusters of more than kBigCluster
// members (listed from the front of `work`, taken by whole CTAs first), queue[3] the others
// (listed from the back, taken one warp each).
__global__ void k_hull_worklist(BatchDev b, uint32_t* work)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= b.ncl)
        return;
    const int s = find_scan(b.nscan, g, [&](int q) { return b.scans[q].cl_off; });
    if (g - b.scans[s].cl_off >= b.state[s].n_clusters)
        return;
    const uint32_t n = b.cl_cnt[g];
    if (n > b.hull_cta_min) // hull_cta_min <= kBigCluster: the warp path's limit
        work[atomicAdd(&b.queue[2], 1u)] = g;
    else
        work[b.ncl - 1u - atomicAdd(&b.queue[3], 1u)] = g;
    if (n > kPreMin)
    {
        // the grid-wide member passes: records cleared, one item per kPreChunk members (queue[6])
        for (int d = 0; d < 16; ++d)
        {
            b.pre_ext[16ull * g + d] = 0ull;
            b.pre_pk[16ull * g + d] = 0ull;
        }
        b.pre_nact[g] = 0u;
        const uint32_t nch = (n + kPreChunk - 1u) / kPreChunk;
        const uint32_t at = atomicAdd(&b.queue[6], nch);
        for (uint32_t c = 0; c < nch; ++c)
            b.pre_items[at + c] = make_uint2(g, c);
    }
}

__device__ __forceinline__ uint32_t work_item(const BatchDev& b, const uint32_t* work, uint32_t w)
{
    const uint32_t nbig = b.queue[2];
    return (w < nbig) ? work[w] : work[b.ncl - 1u - (w - nbig)];
}

constexpr size_t kHullDynSmem = sizeof(HullSmem) > (kHullThreads / 32) * sizeof(WarpSmem)
                                    ? sizeof(HullSmem)
                                    : (kHullThreads / 32) * sizeof(WarpSmem);

// Persistent CTAs: first every large cluster (one CTA each, queue[1] is the head), then every
// small cluster (one warp each, queue[4] is the head).
__global__ void __launch_bounds__(kHullThreads) k_hull(BatchDev b, int compute_obb, const uint32_t* work)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ float2 dirs[kDirs];
    HullSmem& sm = *reinterpret_cast<HullSmem*>(smraw);
    if (threadIdx.x < kDirs)
    {
        const float a = 6.28318530717958647692f * static_cast<float>(threadIdx.x) / kDirs;
        dirs[threadIdx.x] = make_float2(cosf(a), sinf(a));
        sm.dirs[threadIdx.x] = dirs[threadIdx.x];
    }
    const uint32_t nbig = b.queue[2];
    const uint32_t nsmall = b.queue[3];
    for (;;)
    {
        __syncthreads();
        if (threadIdx.x == 0)
            sm.work = atomicAdd(&b.queue[1], 1u);
        __syncthreads();
        const uint32_t w = sm.work;
        if (w >= nbig)
            break;
        const uint32_t g = work[w];
        const int s = find_scan(b.nscan, g, [&](int q) { return b.scans[q].cl_off; });
        hull_one(b, sm, g, s, compute_obb);
    }
    __syncthreads(); // the CTA's shared memory now becomes eight per-warp regions
    WarpSmem& ws = reinterpret_cast<WarpSmem*>(smraw)[threadIdx.x >> 5];
    for (;;)
    {
        uint32_t w = 0;
        if (lane_id() == 0)
            w = atomicAdd(&b.queue[4], 1u);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= nsmall)
            break;
        const uint32_t g = work[b.ncl - 1u - w];
        const int s = find_scan(b.nscan, g, [&](int q) { return b.scans[q].cl_off; });
        hull_one_warp(b, ws, dirs, g, s, compute_obb);
    }
}

// Dense hull output: hull_cnt holds the exclusive scan (hull offsets over the batch).
// ---------------------------------------------------------------------------------------------
// The reference's order among identical points (Polygonizer::convexHull, polygonizer.cpp:51-59):
// std::sort orders the point indices by x, then (|dx| < DBL_EPSILON) y, and leaves points that
// compare equal in whatever order its introsort produced. The monotone chain keeps, of a run of
// identical points, the first in that order at the leftmost vertex and on the upper chain, and
// the last on the lower chain up to the rightmost vertex. The hull kernels order ties by input
// index; where a hull vertex has an identical point, the whole cluster's std::sort is replayed
// (lp_introsort.cuh) and each vertex re-picked from its run.
// ---------------------------------------------------------------------------------------------
template <typename T>
struct HRec
{
    T x, y;
    uint32_t idx;
};

template <typename T>
struct HullLess // the reference's sort comparator on its binary64 PointXY
{
    __device__ __forceinline__ bool operator()(const HRec<T>& a, const HRec<T>& b) const
    {
        const double ax = static_cast<double>(a.x), bx = static_cast<double>(b.x);
        return ax < bx || (fabs(ax - bx) < DBL_EPSILON && static_cast<double>(a.y) < static_cast<double>(b.y));
    }
};

// The same comparator on binary32 coordinates widened to binary64, decided in binary32 where that
// is exact: equal finite x compare by y (|dx| = 0; infinite x give inf - inf = NaN, not below
// DBL_EPSILON); distinct x of which one is at least 2^-20 in magnitude differ by at least 2^-44, so
// only x both below 2^-20 need the binary64 difference.
template <>
struct HullLess<float>
{
    __device__ __forceinline__ bool operator()(const HRec<float>& a, const HRec<float>& b) const
    {
        if (a.x < b.x)
            return true;
        if (a.x == b.x)
            return fabsf(a.x) < INFINITY && a.y < b.y;
        if (fabsf(a.x) < 0x1p-20f && fabsf(b.x) < 0x1p-20f)
            return fabs(static_cast<double>(a.x) - static_cast<double>(b.x)) < DBL_EPSILON && a.y < b.y;
        return false;
    }
};

template <typename T>
struct IdxLess
{
    __device__ __forceinline__ bool operator()(const HRec<T>& a, const HRec<T>& b) const { return a.idx < b.idx; }
};

// rec: the n points in input order (idx = position). hull (h local indices, in input-order ties)
// is rewritten with the reference's picks; vxy(j): the coordinates of hull vertex j (read before
// hull[j] is rewritten); ge/le: n entries each.
template <typename T, class VertexXY>
__device__ void hull_repair_ties(HRec<T>* rec, uint32_t n, int32_t* hull, int h, VertexXY vxy, uint32_t* ge,
                                 uint32_t* le, isort::SortShared& ss)
{
    __shared__ int s_jr;
    isort::cta_sort(rec, n, HullLess<T>{}, ge, le, ss);
    if (threadIdx.x == 0)
    {
        // the rightmost vertex ends the lower chain: the lexicographic maximum, its last occurrence
        // (a cloud of identical points has the hull [first, last] of one coordinate)
        int jr = 0;
        double2 best = vxy(0);
        for (int j = 1; j < h; ++j)
        {
            const double2 v = vxy(j);
            if (v.x > best.x || (v.x == best.x && v.y >= best.y))
            {
                jr = j;
                best = v;
            }
        }
        s_jr = jr;
    }
    __syncthreads();
    const int jr = s_jr;
    const HullLess<T> less{};
    for (int j = threadIdx.x; j < h; j += blockDim.x)
    {
        const double2 v = vxy(j);
        const HRec<T> t{static_cast<T>(v.x), static_cast<T>(v.y), 0u};
        // equal range of the vertex's point in the sorted records
        uint32_t lo = 0, hi = n;
        while (lo < hi)
        {
            const uint32_t mid = (lo + hi) / 2;
            if (less(rec[mid], t))
                lo = mid + 1;
            else
                hi = mid;
        }
        uint32_t lo2 = lo, hi2 = n;
        while (lo2 < hi2)
        {
            const uint32_t mid = (lo2 + hi2) / 2;
            if (!less(t, rec[mid]))
                lo2 = mid + 1;
            else
                hi2 = mid;
        }
        if (lo2 > lo)
            hull[j] = static_cast<int32_t>(rec[(j == 0 || j > jr) ? lo : lo2 - 1].idx);
    }
    __syncthreads();
}

// Clusters listed by k_hull (a hull vertex with an identical candidate): the members' records in
// input order (sorted by member key), then the repair. The sorts are chains of dependent accesses,
// so clusters of at most kTieSmemRecs members are sorted in shared memory (records, then the ge / le
// lists); larger ones use the cluster's scratch: the candidate area (records), the chain stack
// area (ge / le). The vertices' coordinates go to the FP64 hull area.
constexpr uint32_t kTieSmemRecs = 4096;
constexpr size_t kTieDynSmem = static_cast<size_t>(kTieSmemRecs) * (sizeof(HRec<float>) + 8);

__global__ void __launch_bounds__(kHullThreads) k_hull_ties(BatchDev b)
{
    __shared__ isort::SortShared ss;
    extern __shared__ __align__(16) unsigned char tsm[];
    const uint32_t ntie = b.queue[5]; // the tie count (queue[4] is the small-cluster head)
    for (uint32_t t = blockIdx.x; t < ntie; t += gridDim.x)
    {
        const uint32_t g = b.tie_list[t];
        const uint32_t start = b.cl_start[g], n = b.cl_cnt[g];
        const int h = static_cast<int>(b.hull_cnt[g + 1] - b.hull_cnt[g]); // scanned: offsets
        const bool local = n <= kTieSmemRecs;
        HRec<float>* rec = local ? reinterpret_cast<HRec<float>*>(tsm)
                                 : reinterpret_cast<HRec<float>*>(reinterpret_cast<HPt<float>*>(b.hs_cand) + 2ull * start);
        uint32_t* ge = local ? reinterpret_cast<uint32_t*>(tsm + kTieSmemRecs * sizeof(HRec<float>))
                             : reinterpret_cast<uint32_t*>(b.hs_stack + 2ull * start + 2ull * g);
        uint32_t* le = ge + (local ? kTieSmemRecs : n);
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        {
            const float2 p = b.mxy[start + k];
            rec[k] = HRec<float>{p.x, p.y, b.members[start + k]};
        }
        __syncthreads();
        isort::cta_sort(rec, n, IdxLess<float>{}, ge, le, ss);
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x)
            rec[k].idx = k; // local index: position in input order
        __syncthreads();
        int32_t* hull = b.hull_tmp + start;
        double2* hv = b.hs_pts + start; // the vertices' coordinates, kept before the records re-sort
        for (int j = threadIdx.x; j < h; j += blockDim.x)
            hv[j] = make_double2(static_cast<double>(rec[hull[j]].x), static_cast<double>(rec[hull[j]].y));
        __syncthreads();
        hull_repair_ties(rec, n, hull, h, [=](int j) { return hv[j]; }, ge, le, ss);
    }
}

__global__ void k_hull_compact(BatchDev b, const uint32_t* work)
{
    const uint32_t total = b.queue[2] + b.queue[3];
    for (uint32_t w = blockIdx.x; w < total; w += gridDim.x)
    {
        const uint32_t g = work_item(b, work, w);
        const uint32_t off = b.hull_cnt[g];
        const uint32_t cnt = b.hull_cnt[g + 1] - off;
        for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x)
            b.hull_out[off + i] = b.hull_tmp[b.cl_start[g] + i];
    }
}

// ---------------------------------------------------------------------------------------------
// Standalone single-polygon entry points (double inputs): one CTA.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kHullThreads) k_hull_single(const double2* pts, uint32_t n, HPt<double>* scratch,
                                                            int* stack, int32_t* out, uint32_t* n_out)
{
    // the sort runs in global scratch (capacity next_pow2(n)); no prefilter (the polygon is
    // the caller's whole input)
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        scratch[i] = HPt<double>{pts[i].x, pts[i].y, i};
    __syncthreads();
    block_sort_global(scratch, n);
    __syncthreads();
    __shared__ int hn;
    __shared__ isort::SortShared ss;
    if (threadIdx.x == 0)
        hn = monotone_chain(scratch, static_cast<int>(n), stack);
    __syncthreads();
    bool tie = false;
    for (int j = threadIdx.x; j < hn; j += blockDim.x)
    {
        const int q = stack[j];
        const HPt<double> c = scratch[q];
        out[j] = static_cast<int32_t>(c.key);
        tie |= (q > 0 && scratch[q - 1].x == c.x && scratch[q - 1].y == c.y) ||
               (q + 1 < static_cast<int>(n) && scratch[q + 1].x == c.x && scratch[q + 1].y == c.y);
    }
    if (threadIdx.x == 0)
        *n_out = static_cast<uint32_t>(hn);
    if (__syncthreads_or(tie))
    {
        // a vertex with an identical point: the reference's std::sort order decides which one. The
        // sort buffer takes the records (24 bytes each, as its entries) and the chain stack (2n + 8
        // ints, free now) the partition lists; the vertices' coordinates are read from the input.
        auto* rec = reinterpret_cast<HRec<double>*>(scratch);
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
            rec[i] = HRec<double>{pts[i].x, pts[i].y, i};
        __syncthreads();
        uint32_t* ge = reinterpret_cast<uint32_t*>(stack);
        hull_repair_ties(rec, n, out, hn, [=](int j) { return pts[out[j]]; }, ge, ge + n, ss);
    }
}

__global__ void k_boxes_single(const double2* P, uint32_t n, int2* pairs, int cap, int kind, lp_bounding_box* out,
                               int* npairs_out)
{
    if (threadIdx.x >= 32)
        return;
    const uint32_t lane = lane_id();
    int np = 0;
    if (lane == 0)
        np = antipodal_pairs(AreaCmpFp64{P}, static_cast<int>(n), pairs, cap);
    np = __shfl_sync(0xffffffffu, np, 0);
    if (lane == 0 && npairs_out)
        *npairs_out = np;
    if (np > cap)
        np = cap;
    __syncwarp();
    if (kind == 0)
        calipers_warp(P, static_cast<int>(n), pairs, np, out);
    else if (kind == 1 && lane == 0)
        pca_box(P, static_cast<int>(n), out);
}
} // namespace

namespace
{
// The vehicle gates (processor.cpp:679-755), one warp per cluster. Lane 0 checks the hull size, the
// point count, the height against the table's limits and the volume of the hull area (polygonArea,
// polygonizer.hpp:186-198, binary64 in hull order); a cluster that passes is boxed by rotating
// calipers over all its points in input order, which is what the reference passes
// (polygonizer_points_), with the same routine the hulls' boxes use; lane 0 then checks the hull's
// share of the box (> 0.4) and the box's edges against the vehicle types in order.
__global__ void k_obj_gate(ObjDev o, VehicleTableDev vt, int enabled, double2* P, float2* Pf, float* ea, int2* pairs,
                           ScanState* st)
{
    const uint32_t l = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u;
    if (l >= o.K)
        return;
    const uint32_t lane = lane_id();
    const uint32_t off = o.cl_off[l], nc = o.cl_off[l + 1] - off;
    const uint32_t h0 = o.hull_off[l], h = o.hull_off[l + 1] - h0;
    const double height = static_cast<double>(o.zmax[l]) - static_cast<double>(o.zmin[l]);
    double area = 0.0, volume = 0.0;
    int pass = 0;
    if (lane == 0)
    {
        lp_bounding_box none;
        for (int k = 0; k < 4; ++k)
            none.corners[k][0] = none.corners[k][1] = 0.0;
        none.area = 0.0f;
        none.angle_rad = 0.0f;
        none.is_valid = 0;
        o.boxes[l] = none;
        o.cls[l] = -1;
        if (enabled && h >= 3 && nc > 150 && height > vt.min_h && height < vt.max_h)
        {
            auto vx = [&](uint32_t k) { return static_cast<double>(o.cloud[off + static_cast<uint32_t>(o.hull_idx[h0 + k])].x); };
            auto vy = [&](uint32_t k) { return static_cast<double>(o.cloud[off + static_cast<uint32_t>(o.hull_idx[h0 + k])].y); };
            double a = 0.0;
            for (uint32_t k = 0; k + 1 < h; ++k)
                a += (vx(k) * vy(k + 1)) - (vx(k + 1) * vy(k));
            a += (vx(h - 1) * vy(0)) - (vx(0) * vy(h - 1));
            area = fabs(a) * 0.5;
            volume = area * height;
            pass = (volume > vt.min_v && volume < vt.max_v) ? 1 : 0;
        }
    }
    pass = __shfl_sync(0xffffffffu, pass, 0);
    if (!pass)
        return;
    area = __shfl_sync(0xffffffffu, area, 0);
    volume = __shfl_sync(0xffffffffu, volume, 0);
    for (uint32_t k = lane; k < nc; k += 32)
    {
        const lp_xyzrgb& p = o.cloud[off + k];
        P[off + k] = make_double2(static_cast<double>(p.x), static_cast<double>(p.y));
        Pf[off + k] = make_float2(p.x, p.y);
    }
    __syncwarp();
    calipers_box(st, P + off, Pf + off, ea + off, static_cast<int>(nc), pairs + 4ull * off + 16ull * l, &o.boxes[l]);
    __syncwarp();
    if (lane != 0)
        return;
    const lp_bounding_box box = o.boxes[l];
    if (!box.is_valid || !(area / static_cast<double>(box.area) > 0.4))
        return;
    auto dist = [&](int a, int c) {
        const double dx = box.corners[a][0] - box.corners[c][0];
        const double dy = box.corners[a][1] - box.corners[c][1];
        return sqrt(dx * dx + dy * dy);
    };
    const double e1 = dist(0, 1), e2 = dist(1, 2);
    const double len = fmax(e1, e2), wid = fmin(e1, e2);
    for (int v = 0; v < 5; ++v)
    {
        const double* d = vt.dims[v];
        const double* bb = vt.bounds[v];
        if (len > d[0] && len < d[1] && wid > d[2] && wid < d[3] && height > d[4] && height < d[5] && volume > bb[0] &&
            volume < bb[1] && area > bb[2] && area < bb[3])
        {
            o.cls[l] = v;
            break;
        }
    }
}
} // namespace

void launch_objects_gates(cudaStream_t st, const ObjDev& o, const VehicleTableDev& vt, int enabled, double2* P,
                          float2* Pf, float* ea, int2* pairs, ScanState* state, uint64_t& launches)
{
    if (o.K == 0)
        return;
    k_obj_gate<<<div_up(o.K, 4u), 128, 0, st>>>(o, vt, enabled, P, Pf, ea, pairs, state);
    launches += 1;
}

void launch_polygons(Launcher& L, const BatchDev& b, const BatchHost& hb, int compute_obb)
{
    (void)hb;
    // the work list reuses the cluster fill counters' scratch (cl_fill, ncl + 1 entries)
    uint32_t* work = b.cl_fill;
    LP_LAUNCH(L, k_hull_worklist, div_up(b.ncl, 256u), 256, b, work);
    LP_LAUNCH(L, k_hull_pre_ext, static_cast<uint32_t>(sm_count()) * 4u, 256, b);
    LP_LAUNCH(L, k_hull_pre_ref, static_cast<uint32_t>(sm_count()) * 4u, 256, b);
    const int sms = sm_count();
    LP_LAUNCH_SMEM(L, k_hull, static_cast<uint32_t>(sms) * hb.hull_ctas_per_sm, kHullThreads, kHullDynSmem, b, compute_obb,
                   static_cast<const uint32_t*>(work));
    L.scan(b.hull_cnt, b.hull_cnt, b.ncl + 1);
    LP_LAUNCH_SMEM(L, k_hull_ties, static_cast<uint32_t>(sms), kHullThreads, kTieDynSmem, b);
    LP_LAUNCH(L, k_hull_compact, static_cast<uint32_t>(sms * 8), 128, b, static_cast<const uint32_t*>(work));
}

void init_kernel_attributes()
{
    init_kdtree_attributes();
    cudaFuncSetAttribute(k_hull, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kHullDynSmem));
    cudaFuncSetAttribute(k_hull_ties, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTieDynSmem));
}

int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

void launch_hull_single(Launcher& L, const double2* pts, uint32_t n, void* scratch, int* stack, int32_t* out,
                        uint32_t* n_out)
{
    LP_LAUNCH(L, k_hull_single, 1, kHullThreads, pts, n, reinterpret_cast<HPt<double>*>(scratch), stack, out, n_out);
}

void launch_boxes_single(Launcher& L, const double2* P, uint32_t n, int2* pairs, int cap, int kind, lp_bounding_box* out,
                         int* npairs_out)
{
    LP_LAUNCH(L, k_boxes_single, 1, 32, P, n, pairs, cap, kind, out, npairs_out);
}
} // namespace lpg

// =============================================================================================
// Convex hull without any allocation (lp_convex_hull_noalloc, lidar_gb300.h).
//
// For callers that must not allocate device memory: code that runs inside a real-time loop
// whose memory is reserved up front (cudaMalloc can synchronise the device and stall other
// work), plugin hosts whose allocator policy forbids it, or code paths where an allocation
// failure cannot be handled. The caller passes device buffers for the input and the output; the
// kernel's working memory is the file-scope array below, which every GPU that loads this library
// holds (2.1 MiB) until the process exits.
// =============================================================================================
namespace
{
constexpr uint32_t kNoallocMaxPoints = LP_NOALLOC_HULL_MAX_POINTS;
// sort buffer: next_pow2(n) points of 24 bytes; chain stack: 2n + 8 ints
constexpr size_t kNoallocSortBytes = static_cast<size_t>(kNoallocMaxPoints) * 24;
constexpr size_t kNoallocStackBytes = (2 * static_cast<size_t>(kNoallocMaxPoints) + 8) * 4;

static __device__ __align__(256) unsigned char g_noalloc_hull_scratch[kNoallocSortBytes + kNoallocStackBytes];

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kNoallocMaxDevices] = {};

__global__ void k_hull_noalloc_small(uint32_t n, int32_t* out, uint32_t* n_out)
{
    // fewer than 3 points: indices 0..n-1 (polygonizer.cpp:36-41)
    if (threadIdx.x < n)
        out[threadIdx.x] = static_cast<int32_t>(threadIdx.x);
    if (threadIdx.x == 0)
        *n_out = n;
}
} // namespace

extern "C" lp_status lp_convex_hull_noalloc(const double* d_xy, uint32_t n, int32_t* d_indices_out, uint32_t* d_n_out,
                                            void* stream)
{
    if (!d_n_out || (n && (!d_xy || !d_indices_out)))
        return LP_ERR_BAD_ARG;
    if (n > kNoallocMaxPoints)
        return LP_ERR_CAPACITY; // more points than the static working array holds
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoallocMaxDevices)
    {
        cudaGetLastError();
        return LP_ERR_NO_DEVICE;
    }
    void* scratch = nullptr;
    {
        // once per device, with that device current: the device address of the static array
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev])
        {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_hull_scratch);
            if (e != cudaSuccess || !p)
            {
                cudaGetLastError();
                return LP_ERR_CUDA;
            }
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the status is this launch's own (cudaLaunchKernel's return value), so an error left behind
    // by some other code in the process is neither reported as this call's nor cleared
    cudaError_t e;
    if (n < 3)
    {
        void* args[] = {&n, &d_indices_out, &d_n_out};
        e = cudaLaunchKernel(reinterpret_cast<const void*>(&k_hull_noalloc_small), dim3(1), dim3(32), args, 0, st);
    }
    else
    {
        // every scratch element the kernel reads is written earlier in the same launch, so the
        // previous call's contents never leak into this one
        auto* sort_buf = reinterpret_cast<lpg::HPt<double>*>(scratch);
        int* stack = reinterpret_cast<int*>(static_cast<unsigned char*>(scratch) + kNoallocSortBytes);
        const double2* xy = reinterpret_cast<const double2*>(d_xy);
        void* args[] = {&xy, &n, &sort_buf, &stack, &d_indices_out, &d_n_out};
        e = cudaLaunchKernel(reinterpret_cast<const void*>(&lpg::k_hull_single), dim3(1), dim3(lpg::kHullThreads), args,
                             0, st);
    }
    return e == cudaSuccess ? LP_OK : LP_ERR_CUDA;
}
