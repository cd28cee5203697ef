// Kernel-matrix entries on the device, shared by the assembly and the
// learned-proposal kernels.
#pragma once
#include "kernels.cuh"

namespace h2w {

// ------------------------------------------------------------ entries ---
// The entry between two distinct points given by their coordinates a, b
// (getMatrixEntry off the diagonal, in the reference's operation order).
static __device__ __forceinline__ double kentry_ab(const KParams &k, const double *a, const double *b) {
    if (k.dim == 1) {
        double R = fabs(__dsub_rn(a[0], b[0]));
        if (k.choice == 0) return log(R);
        const double aa = 0.0001;
        return R < aa ? __ddiv_rn(R, aa) : __ddiv_rn(aa, R);
    }
    double dx = __dsub_rn(a[0], b[0]), dy = __dsub_rn(a[1], b[1]);
    if (k.dim == 2) {
        double R2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        if (k.choice == 0) return __dmul_rn(k.c2d, log(R2));
        double R = __dsqrt_rn(R2);
        const double aa = 0.0001;
        return R < aa ? __ddiv_rn(R, aa) : __ddiv_rn(aa, R);
    }
    double dz = __dsub_rn(a[2], b[2]);
    double R2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    double R = __dsqrt_rn(R2);
    if (k.choice == 0) return __ddiv_rn(1.0, __dmul_rn(k.four_pi, R));
    const double aa = 0.0001;
    if (R < aa) return __ddiv_rn(__dsub_rn(__dmul_rn(R, log(R)), 1.0), k.den_small);
    return __ddiv_rn(log(R), k.loga);
}

static __device__ __forceinline__ double kentry(const KParams &k, int i, int j) {
    if (i == j) return k.diag;
    return kentry_ab(k, k.pts + (size_t)i * k.dim, k.pts + (size_t)j * k.dim);
}

}  // namespace h2w
