// eigen_svd2.h — Eigen 3.4.0's JacobiSVD restated for a square real 2x2 matrix (V only).
//
// TEST INFRASTRUCTURE ONLY: used by the oracle's PCA box (lp_oracle.cpp) and by the Eigen
// stand-in (shim/Eigen/Dense) that the reference's polygonizer.cpp:323-336 is compiled against.
// Eigen is not installed here; this follows its published algorithm (Eigen/src/SVD/JacobiSVD.h,
// Eigen/src/SVD/RealSvd2x2.h, Eigen/src/Jacobi/Jacobi.h of release 3.4.0, the version Ubuntu
// 22.04 / ROS 2 Humble ships) in the same binary64 operation order:
//   1. scale = max |a_ij| (1 if zero; a non-finite coefficient is an error), W = A / scale, V = I;
//   2. sweep while |W10| or |W01| exceeds max(DBL_MIN, 2 eps max(|W00|, |W11|)) (the maximum
//      grows with the diagonal after each sweep): a left rotation makes the (1, 0) block
//      symmetric, makeJacobi's rotation diagonalises it; W is rotated on both sides, V on the right;
//   3. singular values |W_ii| · scale, sorted descending by a strict comparison (equal values keep
//      their columns): column 1 of V becomes column 0 only when its value is larger.
// Below the threshold no rotation is applied, so a near-diagonal covariance keeps V = I where a
// closed-form angle would turn the axes by up to 45 degrees on a near-isotropic matrix.
// Eigen loops until the threshold test passes; the sweeps here stop after kMaxSweeps, which the
// 2x2 case never reaches (one or two sweeps in practice).
#pragma once
#include <algorithm>
#include <cmath>
#include <limits>

namespace eigen_svd2
{
constexpr int kMaxSweeps = 64;

struct Rot // Eigen's JacobiRotation<double>: (c, s)
{
    double c, s;
};

// apply_rotation_in_the_plane for a pair of 2-vectors x, y: x' = c x + s y, y' = -s x + c y;
// the identity rotation leaves them untouched.
inline void rotate(double& x0, double& x1, double& y0, double& y1, Rot r)
{
    if (r.c == 1.0 && r.s == 0.0)
        return;
    const double a0 = x0, a1 = x1, b0 = y0, b1 = y1;
    x0 = r.c * a0 + r.s * b0;
    x1 = r.c * a1 + r.s * b1;
    y0 = -r.s * a0 + r.c * b0;
    y1 = -r.s * a1 + r.c * b1;
}

// JacobiRotation::makeJacobi(x, y, z): the rotation diagonalising [[x, y], [y, z]].
inline Rot make_jacobi(double x, double y, double z)
{
    const double deno = 2.0 * std::fabs(y);
    if (deno < std::numeric_limits<double>::min())
        return {1.0, 0.0};
    const double tau = (x - z) / deno;
    const double w = std::sqrt(tau * tau + 1.0);
    const double t = tau > 0.0 ? 1.0 / (tau + w) : 1.0 / (tau - w);
    const double sign_t = t > 0.0 ? 1.0 : -1.0;
    const double n = 1.0 / std::sqrt(t * t + 1.0);
    return {n, -sign_t * (y / std::fabs(y)) * std::fabs(t) * n};
}

// V of the SVD of [[a00, a01], [a10, a11]], row-major into v[4]. False for a non-finite input
// (Eigen's InvalidInput), with v untouched.
inline bool jacobi_svd2_v(double a00, double a01, double a10, double a11, double v[4])
{
    if (!(std::isfinite(a00) && std::isfinite(a01) && std::isfinite(a10) && std::isfinite(a11)))
        return false;
    double scale = std::max(std::max(std::fabs(a00), std::fabs(a01)), std::max(std::fabs(a10), std::fabs(a11)));
    if (scale == 0.0)
        scale = 1.0;
    double w00 = a00 / scale, w01 = a01 / scale, w10 = a10 / scale, w11 = a11 / scale;
    double v00 = 1.0, v01 = 0.0, v10 = 0.0, v11 = 1.0;
    const double precision = 2.0 * std::numeric_limits<double>::epsilon();
    const double tiny = std::numeric_limits<double>::min();
    double max_diag = std::max(std::fabs(w00), std::fabs(w11));
    for (int sweep = 0; sweep < kMaxSweeps; ++sweep)
    {
        const double threshold = std::max(tiny, precision * max_diag);
        if (!(std::fabs(w10) > threshold || std::fabs(w01) > threshold))
            break;
        // real_2x2_jacobi_svd on the pair (p, q) = (1, 0): m = [[W11, W10], [W01, W00]]
        double m00 = w11, m01 = w10, m10 = w01, m11 = w00;
        Rot r1{1.0, 0.0};
        const double t = m00 + m11, d = m10 - m01;
        if (!(std::fabs(d) < tiny))
        {
            const double u = t / d;
            const double tmp = std::sqrt(1.0 + u * u);
            r1 = {u / tmp, 1.0 / tmp};
        }
        rotate(m00, m01, m10, m11, r1);
        const Rot rr = make_jacobi(m00, m01, m11);
        const Rot rl{r1.c * rr.c - r1.s * -rr.s, r1.c * -rr.s + r1.s * rr.c}; // r1 * rr^T
        const Rot rt{rr.c, -rr.s};                                           // rr^T (right side)
        rotate(w10, w11, w00, w01, rl); // rows 1 and 0 of W
        rotate(w01, w11, w00, w10, rt); // columns 1 and 0 of W
        rotate(v01, v11, v00, v10, rt); // columns 1 and 0 of V
        max_diag = std::max(max_diag, std::max(std::fabs(w11), std::fabs(w00)));
    }
    if (std::fabs(w11) * scale > std::fabs(w00) * scale)
    {
        std::swap(v00, v01);
        std::swap(v10, v11);
    }
    v[0] = v00;
    v[1] = v01;
    v[2] = v10;
    v[3] = v11;
    return true;
}
} // namespace eigen_svd2
