// Stand-in for the two Boost.Math functions the reference's 2D Hankel build
// calls (besselJ / besselY, 2D/codes/integral2d.hpp:16-50, always at order 0),
// so that the reference's own 2D Hankel code can be compiled and run here
// without Boost. Test infrastructure only (oracle/Makefile's ref2d_*_hankel
// targets). Order 0 is computed by the oracle's own long-double series
// (bessel_ld.hpp), whose values are checked against scipy separately; any
// other order stops the program.
#pragma once
#include <cstdio>
#include <cstdlib>

#include "bessel_ld.hpp"

namespace boost {
namespace math {

inline double cyl_bessel_j(double v, double x) {
    if (v != 0.0) {
        std::fprintf(stderr, "boost_shim: cyl_bessel_j of order %g is not provided\n", v);
        std::abort();
    }
    double j0, y0;
    h2wo_bessel::j0y0_series(x, j0, y0);
    return j0;
}

inline double cyl_neumann(double v, double x) {
    if (v != 0.0) {
        std::fprintf(stderr, "boost_shim: cyl_neumann of order %g is not provided\n", v);
        std::abort();
    }
    double j0, y0;
    h2wo_bessel::j0y0_series(x, j0, y0);
    return y0;
}

}  // namespace math
}  // namespace boost
