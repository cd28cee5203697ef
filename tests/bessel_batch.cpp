// Host build of the library's J0/Y0 (h2weak_gb300/csrc/bessel.cuh) for the CPU
// test against an independent implementation (tests/test_bessel.py).
#include <cstdint>

#include "../h2weak_gb300/csrc/bessel.cuh"

extern "C" void j0y0_batch(const double *x, int64_t n, double *j0, double *y0) {
    for (int64_t i = 0; i < n; ++i) h2w::bessel::j0y0(x[i], j0[i], y0[i]);
}
