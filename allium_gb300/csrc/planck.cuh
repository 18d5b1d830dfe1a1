// Normalised Planck and Rosseland integrals over [0, x], x = E / T:
//   b(x) = 15/pi^4 int_0^x t^3 / (e^t - 1) dt,
//   r(x) = b(x) - 15/(4 pi^4) x^4 / (e^x - 1)   (the derivative-weighted form),
// evaluated as allium does (src/planck.hpp:157-186): the smaller of the Taylor
// series through x^21 and the polylogarithm form with nine terms per Li_k
// (B. A. Clark, J. Comput. Phys. 70 (1987) 311-329).
//
// Taylor: x^3/(e^x - 1) = x^2 sum_n B_n x^n / n!, so int_0^x = sum_n B_n x^{n+3} / (n! (n+3))
// with the Bernoulli numbers B_0 = 1, B_1 = -1/2, B_2 = 1/6, B_4 = -1/30, ...
// Polylogarithm: b(x) = 1 - 15/pi^4 (6 Li_4 + 6 x Li_3 + 3 x^2 Li_2 + x^3 Li_1)(e^{-x}).
#pragma once

#include <cmath>

namespace allium {

constexpr double kPlanckPi = 3.14159265358979323846;
constexpr double kPlanckNorm = 15.0 / (kPlanckPi * kPlanckPi * kPlanckPi * kPlanckPi);
constexpr double kRosselandMax = 1.1579208923731619e77;   // x^4 overflows beyond (DBL_MAX)^(1/4)

// B_n / (n! (n + 3)) for the nonzero Bernoulli numbers up to B_18
constexpr double planck_taylor_coef(double bn, double nfact, int n) { return bn / (nfact * (n + 3)); }

__host__ __device__ inline double planck_taylor(double x) {
    constexpr double c3 = planck_taylor_coef(1.0, 1.0, 0);
    constexpr double c4 = planck_taylor_coef(-0.5, 1.0, 1);
    constexpr double c5 = planck_taylor_coef(1.0 / 6.0, 2.0, 2);
    constexpr double c7 = planck_taylor_coef(-1.0 / 30.0, 24.0, 4);
    constexpr double c9 = planck_taylor_coef(1.0 / 42.0, 720.0, 6);
    constexpr double c11 = planck_taylor_coef(-1.0 / 30.0, 40320.0, 8);
    constexpr double c13 = planck_taylor_coef(5.0 / 66.0, 3628800.0, 10);
    constexpr double c15 = planck_taylor_coef(-691.0 / 2730.0, 479001600.0, 12);
    constexpr double c17 = planck_taylor_coef(7.0 / 6.0, 87178291200.0, 14);
    constexpr double c19 = planck_taylor_coef(-3617.0 / 510.0, 20922789888000.0, 16);
    constexpr double c21 = planck_taylor_coef(43867.0 / 798.0, 6402373705728000.0, 18);
    const double y = x * x;
    double s = c21;
    s = s * y + c19;
    s = s * y + c17;
    s = s * y + c15;
    s = s * y + c13;
    s = s * y + c11;
    s = s * y + c9;
    s = s * y + c7;
    s = s * y + c5;                       // c5 + c7 x^2 + ... + c21 x^16
    return kPlanckNorm * (x * y) * (c3 + x * (c4 + x * s));
}

__host__ __device__ inline double planck_polylog(double x) {
    const double q = exp(-x);
    double ql = 1.0, li1 = 0.0, li2 = 0.0, li3 = 0.0, li4 = 0.0;
    for (int l = 1; l <= 9; ++l) {
        ql *= q;
        const double r = 1.0 / l;
        double t = ql * r;
        li1 += t;
        t *= r;
        li2 += t;
        t *= r;
        li3 += t;
        t *= r;
        li4 += t;
    }
    return 1.0 - kPlanckNorm * (6.0 * li4 + x * (6.0 * li3 + x * (3.0 * li2 + x * li1)));
}

// b(x); x >= 0
__host__ __device__ inline double planck_fraction(double x) {
    if (x > 1e100) return 1.0;
    if (x == 0.0) return 0.0;
    const double t = planck_taylor(x), p = planck_polylog(x);
    return (p < t) ? p : t;
}

// r(x) from b(x)
__host__ __device__ inline double rosseland_from_planck(double x, double b) {
    if (x > kRosselandMax) return b;
    return b - 0.25 * kPlanckNorm * (x * x) * (x * x) / expm1(x);
}

}  // namespace allium
