// Bessel functions J0 and Y0 of a positive argument in FP64, on the host and
// on the device, for the 2D Hankel kernel i H0^(1)(R) / 4 = (-Y0(R) + i J0(R)) / 4
// (2D/codes/integral2d.hpp:16-57, where the reference takes them from Boost).
//
//  x <= 4       the power series (Abramowitz & Stegun 9.1.10, 9.1.13; t = x^2/4)
//                 J0(x) = sum_k (-t)^k / (k!)^2
//                 Y0(x) = (2/pi) [(ln(x/2) + gamma) J0(x) + sum_{k>=1} (-1)^(k+1) H_k t^k / (k!)^2]
//               in double arithmetic (terms below 7 in magnitude: a few ulps absolute)
//  4 < x <= 24  the same sums with terms and running sums as double-double pairs
//               (Dekker's product through fma, Knuth's two-sum), which keeps the
//               cancellation among terms up to 3e8 below double rounding
//  x > 24       Hankel's asymptotic expansion (A&S 9.2.5, 9.2.9, 9.2.10, order 0):
//                 J0 = sqrt(2/(pi x)) (P cos c - Q sin c), Y0 = sqrt(2/(pi x)) (P sin c + Q cos c),
//                 c = x - pi/4, P = sum_k (-1)^k a_2k / x^2k, Q = sum_k (-1)^k a_(2k+1) / x^(2k+1),
//                 a_k = prod_{j<=k} (-(2j-1)^2) / (k! 8^k), summed until the terms stop shrinking
#pragma once
#include <cmath>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#define __device__
#endif
#endif

namespace h2w {
namespace bessel {

constexpr double kGamma = 0.57721566490153286061;  // Euler's constant
constexpr double kTwoOverPi = 0.63661977236758134308;
constexpr double kPi4 = 0.78539816339744830962;

struct dd {
    double hi, lo;
};
__host__ __device__ inline dd dd_two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__host__ __device__ inline dd dd_add(dd a, dd b) {
    dd s = dd_two_sum(a.hi, b.hi);
    double e = s.lo + a.lo + b.lo;
    return dd_two_sum(s.hi, e);
}
__host__ __device__ inline dd dd_mul(dd a, dd b) {
    double p = a.hi * b.hi;
    double e = fma(a.hi, b.hi, -p);
    e = fma(a.hi, b.lo, fma(a.lo, b.hi, e));
    return dd_two_sum(p, e);
}
__host__ __device__ inline dd dd_div_d(dd a, double b) {
    double q = a.hi / b;
    // remainder a - q b exactly (q b as a pair), then one correction
    double p = q * b;
    double pe = fma(q, b, -p);
    double r = ((a.hi - p) - pe) + a.lo;
    double q2 = r / b;
    return dd_two_sum(q, q2);
}

// J0 and the series part S of Y0 (Y0 = (2/pi)((ln(x/2) + gamma) J0 + S)) for x <= 24
__host__ __device__ inline void series(double x, double &j0, double &s) {
    if (x <= 4.0) {
        const double t = 0.25 * x * x;
        double term = 1.0, sj = 1.0, sy = 0.0, hk = 0.0;
        for (int k = 1; k < 40; ++k) {
            term = term * (-t) / ((double)k * (double)k);
            hk += 1.0 / (double)k;
            sj += term;
            sy -= hk * term;  // (-1)^(k+1) H_k t^k / (k!)^2 = -H_k term
            if (fabs(term) * (hk + 1.0) < 1e-20) break;
        }
        j0 = sj;
        s = sy;
        return;
    }
    dd xx = {x * x, fma(x, x, -(x * x))};
    dd t = {0.25 * xx.hi, 0.25 * xx.lo};
    dd term = {1.0, 0.0}, sj = {1.0, 0.0}, sy = {0.0, 0.0}, hk = {0.0, 0.0};
    for (int k = 1; k < 90; ++k) {
        term = dd_mul(term, dd{-t.hi, -t.lo});
        term = dd_div_d(term, (double)k * (double)k);
        hk = dd_add(hk, dd_div_d(dd{1.0, 0.0}, (double)k));
        sj = dd_add(sj, term);
        dd ht = dd_mul(hk, term);
        sy = dd_add(sy, dd{-ht.hi, -ht.lo});
        if (k > 2 * x && fabs(term.hi) * hk.hi < 1e-34) break;
    }
    j0 = sj.hi + sj.lo;
    s = sy.hi + sy.lo;
}

__host__ __device__ inline void asymptotic(double x, double &j0, double &y0) {
    // a_k / x^k with a_k = prod_{j<=k} (-(2j-1)^2) / (k! 8^k); P from even k, Q from odd k
    double p = 1.0, q = 0.0, term = 1.0, last = 1e300;
    for (int k = 1; k < 80; ++k) {
        const double m = (2.0 * k - 1.0);
        term = term * (-(m * m)) / (8.0 * k * x);
        if (fabs(term) >= last) break;
        last = fabs(term);
        // (-1)^(k/2) sign pattern of P and Q
        if (k % 2 == 0) p += ((k / 2) % 2 ? -term : term);
        else q += (((k - 1) / 2) % 2 ? -term : term);
        if (fabs(term) < 1e-18) break;
    }
    const double c = x - kPi4;
    const double f = sqrt(kTwoOverPi / x);
    const double sc = sin(c), cc = cos(c);
    j0 = f * (p * cc - q * sc);
    y0 = f * (p * sc + q * cc);
}

// J0(x), Y0(x) for x > 0
__host__ __device__ inline void j0y0(double x, double &j0, double &y0) {
    if (x > 24.0) {
        asymptotic(x, j0, y0);
        return;
    }
    double s;
    series(x, j0, s);
    y0 = kTwoOverPi * ((log(0.5 * x) + kGamma) * j0 + s);
}

}  // namespace bessel
}  // namespace h2w
