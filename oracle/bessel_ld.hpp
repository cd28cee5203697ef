// J0 and Y0 of the 2D Hankel kernel i H0^(1)(R) / 4 = (-Y0(R) + i J0(R)) / 4,
// where the reference calls Boost (2D/codes/integral2d.hpp:16-50).
//
// Test infrastructure only: shared by the CPU oracle (h2w_oracle.cpp) and by
// the Boost stand-in the reference's 2D Hankel build is compiled against
// (boost_shim/), so both evaluate the same values. The power series
// (Abramowitz & Stegun 9.1.10, 9.1.13; t = x^2/4)
//     J0(x) = sum_k (-t)^k / (k!)^2
//     Y0(x) = (2/pi) [(ln(x/2) + gamma) J0(x) + sum_{k>=1} (-1)^(k+1) H_k t^k / (k!)^2]
// summed in long double, for 0 < x <= 8 (pair distances of points in a square
// of semi-length up to 2.8); other arguments give NaN, since the oracle is
// only run on such sets.
#pragma once
#include <cmath>

namespace h2wo_bessel {

inline void j0y0_series(double xd, double &j0, double &y0) {
    if (!(xd > 0.0) || xd > 8.0) {
        j0 = y0 = std::nan("");
        return;
    }
    const long double x = xd, t = 0.25L * x * x;
    long double term = 1.0L, sj = 1.0L, sy = 0.0L, hk = 0.0L;
    for (int k = 1; k < 200; ++k) {
        term = term * (-t) / ((long double)k * (long double)k);
        hk += 1.0L / (long double)k;
        sj += term;
        sy -= hk * term;
        if (fabsl(term) * (hk + 1.0L) < 1e-30L) break;
    }
    const long double gamma = 0.577215664901532860606512090082402431L;
    const long double two_over_pi = 0.636619772367581343075535053490057448L;
    j0 = (double)sj;
    y0 = (double)(two_over_pi * ((logl(0.5L * x) + gamma) * sj + sy));
}

}  // namespace h2wo_bessel
