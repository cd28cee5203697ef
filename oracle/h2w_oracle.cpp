// CPU restatement of H2weak's nested H2*, semi-nested (H2+H)* and non-nested
// H* HODLRdD operators (tree build, NCA/ACA compression, matvec passes,
// GMRES) in 1D/2D/3D: real FP64 kernels choice 0 and 1, and the complex
// Helmholtz kernel choice 2 of the reference's USE_Helm build (3D), the
// operator templated on its scalar.
//
// TEST INFRASTRUCTURE ONLY (the oracle): tests, smoke() and bench.py's CPU
// baseline call it as the checker; the GPU library never links it.
//
// Every routine cites the reference routine it restates (paths relative to
// the reference project). Arithmetic is done operation by operation in the
// reference's order with separately rounded multiplies and adds (built with
// -ffp-contract=off); reductions that the reference delegates to Eigen
// (dot, norm, gemv, triangular solves) sum in ascending index order, the
// order of the Eigen-subset shim the reference is compiled against for the
// golden dumps, so this restatement and that build agree bit for bit.
#include "h2w_oracle.h"
#include "bessel_ld.hpp"
#include "gmres_ref.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <type_traits>
#include <vector>
#include <omp.h>

namespace {

const double PI = 4.0 * std::atan(1.0);  // */codes/headers.hpp:18

// Scalars: double (the reference's real build) or std::complex<double> (its
// complex Helmholtz build, 3D/codes/headers.hpp:35-40); abs, conj and |.|^2
// as the C++ runtime and Eigen evaluate them (gmres_ref.hpp).
using h2w_ref::abs_;
using h2w_ref::abs2_;
using h2w_ref::conj_;
using cplx = std::complex<double>;

template <class S> struct MatT {  // column-major dense block
    int r = 0, c = 0;
    std::vector<S> a;
    MatT() {}
    MatT(int rr, int cc) : r(rr), c(cc), a((size_t)rr * cc, S(0.0)) {}
    S &operator()(int i, int j) { return a[(size_t)i + (size_t)j * r]; }
    S operator()(int i, int j) const { return a[(size_t)i + (size_t)j * r]; }
    long size() const { return (long)r * c; }
};
template <class S> using VecT = std::vector<S>;

// Order of the sums in gemv / gemvT: ascending (the shim's, so results are
// the reference build's bit for bit) or, set through h2wo_set_sum_order for a
// test of how much a product depends on its summation order, descending.
int g_sum_reverse = 0;

// y = A x, every row summed from 0 in ascending column order. The block is
// swept column by column: each y[i] still takes exactly the row's sequence of
// rounded products and sums, while the column-major block streams
// contiguously and the rows vectorise.
template <class S> VecT<S> gemv(const MatT<S> &A, const VecT<S> &x) {
    VecT<S> y((size_t)A.r, S(0.0));
    S *yp = y.data();
    const int r = A.r;
    for (int jj = 0; jj < A.c; ++jj) {
        const int j = g_sum_reverse ? A.c - 1 - jj : jj;
        const S xj = x[(size_t)j];
        const S *col = A.a.data() + (size_t)j * (size_t)r;
        for (int i = 0; i < r; ++i) {
            S p = col[i] * xj;
            yp[i] = yp[i] + p;
        }
    }
    return y;
}
// y = A^T x (a transpose: no conjugation), every column summed from 0 in
// ascending row order; four columns at a time, each with its own running sum,
// so that four independent chains of adds overlap.
template <bool Rev, class S> void gemvT_cols(const MatT<S> &A, const S *xp, S *y) {
    const int r = A.r;
    int j = 0;
    for (; j + 4 <= A.c; j += 4) {
        const S *c0 = A.a.data() + (size_t)j * (size_t)r;
        const S *c1 = c0 + r, *c2 = c1 + r, *c3 = c2 + r;
        S s0 = S(0.0), s1 = S(0.0), s2 = S(0.0), s3 = S(0.0);
        for (int ii = 0; ii < r; ++ii) {
            const int i = Rev ? r - 1 - ii : ii;
            const S xi = xp[i];
            S p0 = c0[i] * xi, p1 = c1[i] * xi, p2 = c2[i] * xi, p3 = c3[i] * xi;
            s0 = s0 + p0;
            s1 = s1 + p1;
            s2 = s2 + p2;
            s3 = s3 + p3;
        }
        y[j] = s0;
        y[j + 1] = s1;
        y[j + 2] = s2;
        y[j + 3] = s3;
    }
    for (; j < A.c; ++j) {
        const S *cj = A.a.data() + (size_t)j * (size_t)r;
        S s = S(0.0);
        for (int ii = 0; ii < r; ++ii) {
            const int i = Rev ? r - 1 - ii : ii;
            S p = cj[i] * xp[i];
            s = s + p;
        }
        y[j] = s;
    }
}
template <class S> VecT<S> gemvT(const MatT<S> &A, const VecT<S> &x) {
    VecT<S> y((size_t)A.c, S(0.0));
    if (g_sum_reverse) gemvT_cols<true>(A, x.data(), y.data());
    else gemvT_cols<false>(A, x.data(), y.data());
    return y;
}
template <class S> void addto(VecT<S> &y, const VecT<S> &x) { for (size_t i = 0; i < y.size(); ++i) y[i] += x[i]; }
// Eigen's a.dot(b) (conjugate-first) and norm()
template <class S> S dot(const VecT<S> &a, const VecT<S> &b) { return h2w_ref::dot(a, b); }
template <class S> double nrm(const VecT<S> &a) { return h2w_ref::nrm(a); }

// Triangular solves with the semantics of Eigen's triangularView::solve.
// Lower, on the left, column by column: T X = B.
template <class S> void trsv_lower(const MatT<S> &T, bool transposed, S *x, int n) {
    // T lower (or T^T lower when transposed=true, i.e. T upper read as T(q,i))
    for (int i = 0; i < n; ++i) {
        S s = x[i];
        for (int q = 0; q < i; ++q) {
            S t = transposed ? T(q, i) : T(i, q);
            S p = t * x[q];
            s = s - p;
        }
        x[i] = s / (transposed ? T(i, i) : T(i, i));
    }
}
template <class S> void trsv_upper(const MatT<S> &T, bool transposed, S *x, int n) {
    for (int i = n - 1; i >= 0; --i) {
        S s = x[i];
        for (int q = i + 1; q < n; ++q) {
            S t = transposed ? T(q, i) : T(i, q);
            S p = t * x[q];
            s = s - p;
        }
        x[i] = s / T(i, i);
    }
}
// X T = B with T upper: row by row forward substitution.
template <class S> MatT<S> solve_right_upper(const MatT<S> &T, const MatT<S> &B) {
    MatT<S> X = B;
    int n = T.r;
    std::vector<S> x((size_t)n);
    for (int rr = 0; rr < B.r; ++rr) {
        for (int j = 0; j < n; ++j) x[(size_t)j] = B(rr, j);
        for (int j = 0; j < n; ++j) {
            S s = x[(size_t)j];
            for (int q = 0; q < j; ++q) { S p = x[(size_t)q] * T(q, j); s = s - p; }
            x[(size_t)j] = s / T(j, j);
        }
        for (int j = 0; j < n; ++j) X(rr, j) = x[(size_t)j];
    }
    return X;
}
// X T = B with T lower: row by row backward substitution.
template <class S> MatT<S> solve_right_lower(const MatT<S> &T, const MatT<S> &B) {
    MatT<S> X = B;
    int n = T.r;
    std::vector<S> x((size_t)n);
    for (int rr = 0; rr < B.r; ++rr) {
        for (int j = 0; j < n; ++j) x[(size_t)j] = B(rr, j);
        for (int j = n - 1; j >= 0; --j) {
            S s = x[(size_t)j];
            for (int q = j + 1; q < n; ++q) { S p = x[(size_t)q] * T(q, j); s = s - p; }
            x[(size_t)j] = s / T(j, j);
        }
        for (int j = 0; j < n; ++j) X(rr, j) = x[(size_t)j];
    }
    return X;
}

// J0 and Y0 of the 2D Hankel kernel: the long-double series of bessel_ld.hpp
using h2wo_bessel::j0y0_series;

// Gauss-Legendre nodes and weights on [-1,1] by Newton iteration on the
// Legendre recurrence in long double, ordered as the reference's table
// (*/codes/Gauss_Legendre_Nodes_and_Weights.hpp:17): by increasing |x|,
// negative node first.
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    std::vector<long double> xs, ws;
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int i = 1; i <= n; ++i) {
        long double z = cosl(pi * (i - 0.25L) / (n + 0.5L));
        long double pp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p1 = 1, p2 = 0;
            for (int k = 1; k <= n; ++k) {
                long double p3 = p2;
                p2 = p1;
                p1 = ((2.0L * k - 1.0L) * z * p2 - (k - 1.0L) * p3) / k;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0L);
            long double dz = p1 / pp;
            z -= dz;
            if (fabsl(dz) < 1e-30L) break;
        }
        xs.push_back(z);
        ws.push_back(2.0L / ((1.0L - z * z) * pp * pp));
    }
    // xs are descending positive..negative; collect by |x| ascending, negative first
    std::vector<std::pair<long double, long double>> pr;
    for (int i = 0; i < n; ++i) pr.push_back({xs[(size_t)i], ws[(size_t)i]});
    std::sort(pr.begin(), pr.end(), [](const std::pair<long double, long double> &a,
                                        const std::pair<long double, long double> &b) {
        long double fa = fabsl(a.first), fb = fabsl(b.first);
        if (fa != fb) return fa < fb;
        return a.first < b.first;
    });
    x.clear();
    w.clear();
    for (auto &p : pr) { x.push_back((double)p.first); w.push_back((double)p.second); }
}

template <class S> struct BoxT {
    using Mat = MatT<S>;
    using Vec = VecT<S>;
    std::vector<int> pts;            // chargeLocations
    int nb[26];                      // neighborNumbers
    std::vector<int> il;             // interactionList
    std::vector<char> ilv;           // isVertex per interaction-list slot
    int ic[3] = {0, 0, 0};           // integer coordinates at the box's level
    // far field (2D/3D)
    std::vector<int> chk, chg;       // incoming_checkPoints / incoming_chargePoints
    Mat L2P;
    // vertex / 1D nested
    std::vector<int> chkv, chgv;     // *_ver (1D: incoming_* of the nested basis)
    Mat Lv, Rv;
    Mat M2M[8];
    std::vector<Mat> m2l;            // per interaction-list slot (1D: per neighbour slot)
    Mat dense[27];
    // semi-nested pairs per interaction-list slot (1D: per neighbour slot)
    std::vector<std::vector<int>> rowb, colb;
    std::vector<Mat> Lc, Rc, Ac, Ar;  // 2D/3D CUR; 1D: Ac=U, Ar=V^T
    // matvec work
    Vec q, out, in, inv, pot, potv;
};

template <class S> struct OracleT {
    using Mat = MatT<S>;
    using Vec = VecT<S>;
    using Box = BoxT<S>;
    int dim, form, nL, tol_pow, choice;
    int64_t N;
    std::vector<double> P;  // n*dim
    int64_t kernel_n, diag_n;
    double Kii = 0.0, hd = 1.0;
    cplx Kii_c = 0.0;  // the 2D Hankel kernel's complex self term
    S diag_val = S(1.0);
    int nch, nnb;
    std::vector<std::vector<Box>> T;

    // ---- kernel entries: 1D/codes/kernel.hpp:108-185, 2D/codes/kernel.hpp:118-124,197-228,298-318,
    //      3D/codes/kernel.hpp:123-129,146-170,172-193
    S entry(int i, int j) const {
        if constexpr (std::is_same<S, double>::value) return entry_real(i, j);
        else return dim == 2 ? entry_hankel(i, j) : entry_helm(i, j);
    }
    // IE_2D_Helm / Helmholtz2D (2D/codes/kernel.hpp:126-144, choice 10), the
    // reference's expression I * (J0(R) + I * Y0(R)) / 4.0 with R2 = X + Y;
    // diagonal (1 + 15 ln N + Kii) / h^2
    cplx entry_hankel(int i, int j) const {
        if (i == j) return diag_val;
        const double *a = &P[(size_t)i * dim], *b = &P[(size_t)j * dim];
        double R2 = (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]);
        double R = std::sqrt(R2);
        double j0, y0;
        j0y0_series(R, j0, y0);
        const cplx I(0.0, 1.0);
        return I * (j0 + I * y0) / 4.0;
    }
    // Helmholtz3D (3D/codes/kernel.hpp:133-144, choice 2), the reference's expression:
    // exp(I R) / (4 PI) off the diagonal, 500 sqrt(N) on it
    cplx entry_helm(int i, int j) const {
        const double *a = &P[(size_t)i * dim], *b = &P[(size_t)j * dim];
        double R2 = (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]);
        double R = std::sqrt(R2);
        if (i == j) return 500 * std::sqrt(double(diag_n));
        const cplx I(0.0, 1.0);
        return (std::exp(I * R)) / (4.0 * PI);
    }
    double entry_real(int i, int j) const {
        if (i == j) return h2w_ref::real_(diag_val);
        const double *a = &P[(size_t)i * dim], *b = &P[(size_t)j * dim];
        if (dim == 1) {
            double R = std::fabs(a[0] - b[0]);
            if (choice == 0) return std::log(R);
            double aa = 0.0001;
            if (R < aa) return R / aa;
            return aa / R;
        }
        double dx = a[0] - b[0], dy = a[1] - b[1];
        double R2;
        if (dim == 2) {
            double X = dx * dx, Y = dy * dy;
            R2 = X + Y;
            if (choice == 0) {
                double c = -1.0 / (2 * PI);
                double c5 = c * 0.5;
                return c5 * std::log(R2);
            }
            double R = std::sqrt(R2);
            double aa = 0.0001;
            if (R < aa) return R / aa;
            return aa / R;
        }
        double dz = a[2] - b[2];
        double X = dx * dx, Y = dy * dy, Z = dz * dz;
        R2 = (X + Y) + Z;
        double R = std::sqrt(R2);
        if (choice == 0) {
            double f = 4.0 * PI;
            double den = f * R;
            return 1.0 / den;
        }
        double aa = 0.0001;
        if (R < aa) {
            double num = R * std::log(R) - 1.0;
            double den = aa * std::log(aa) - 1.0;
            return num / den;
        }
        double num = 1.0 * std::log(R);
        return num / std::log(aa);
    }
    Mat block(const std::vector<int> &I, const std::vector<int> &J) const {
        Mat M((int)I.size(), (int)J.size());
        for (int j = 0; j < M.c; ++j)
            for (int i = 0; i < M.r; ++i) M(i, j) = entry(I[(size_t)i], J[(size_t)j]);
        return M;
    }

    // ---- self term, 1D/codes/integral1d.hpp:17-39, 2D/codes/integral2d.hpp:60-90, 3D/codes/integral3d.hpp:13-50
    void setup_kernel() {
        if (choice == 0) {
            double h;
            if (dim == 1) h = 1.0 / double(kernel_n);
            else if (dim == 2) h = 1.0 / std::sqrt(double(kernel_n));
            else h = 1.0 / std::cbrt(double(kernel_n));
            std::vector<double> x, w;
            gauss_legendre(16, x, w);
            double lo = 0.0, hi = h * 0.5;
            double cx = 0.5 * (hi - lo), Lx = 0.5 * (hi + lo);
            double res = 0.0;
            if (dim == 1) {
                for (int i = 0; i < 16; ++i) {
                    double tx = cx * x[(size_t)i] + Lx;
                    res += w[(size_t)i] * std::log(std::fabs(1.0 * tx));
                }
                res *= cx;
                res *= 2;
                Kii = res;
                hd = h;
            } else if (dim == 2) {
                double c = -1.0 / (2 * PI);
                for (int i = 0; i < 16; ++i) {
                    double tx = cx * x[(size_t)i] + Lx;
                    for (int j = 0; j < 16; ++j) {
                        double ty = cx * x[(size_t)j] + Lx;
                        double v = c * 0.5 * std::log(tx * tx + ty * ty);
                        res += w[(size_t)i] * w[(size_t)j] * v;
                    }
                }
                res *= (cx * cx);
                res *= 4;
                Kii = res;
                hd = std::pow(h, 2.0);
            } else {
                for (int i = 0; i < 16; ++i) {
                    double tx = cx * x[(size_t)i] + Lx;
                    for (int j = 0; j < 16; ++j) {
                        double ty = cx * x[(size_t)j] + Lx;
                        for (int k = 0; k < 16; ++k) {
                            double tz = cx * x[(size_t)k] + Lx;
                            double v = 1.0 / ((4 * PI) * std::sqrt(tx * tx + ty * ty + tz * tz));
                            res += (w[(size_t)i] * w[(size_t)j] * w[(size_t)k] * v);
                        }
                    }
                }
                res *= (cx * cx * cx);
                res *= 8;
                Kii = res;
                hd = std::pow(h, 3.0);
            }
            diag_val = (1.0 + Kii) / hd;
        } else if (choice == 10) {
            // userkernel constructor (2D/codes/kernel.hpp:101-114): the complex self
            // term by double_integral (2D/codes/integral2d.hpp:59-90) over [0, h/2]^2
            double h = 1.0 / std::sqrt(double(kernel_n));
            std::vector<double> x, w;
            gauss_legendre(16, x, w);
            double lo = 0.0, hi = h * 0.5;
            double cx = 0.5 * (hi - lo), Lx = 0.5 * (hi + lo);
            cplx res = 0.0;
            const cplx I(0.0, 1.0);
            for (int i = 0; i < 16; ++i) {
                double tx = cx * x[(size_t)i] + Lx;
                for (int j = 0; j < 16; ++j) {
                    double ty = cx * x[(size_t)j] + Lx;
                    double j0, y0;
                    j0y0_series(std::sqrt(tx * tx + ty * ty), j0, y0);
                    res += w[(size_t)i] * w[(size_t)j] * (I * (j0 + I * y0) / 4.0);
                }
            }
            res *= (cx * cx);
            res *= 4;
            Kii_c = res;
            Kii = res.real();
            hd = std::pow(h, 2.0);
            if constexpr (!std::is_same<S, double>::value)
                diag_val = (1.0 + 15 * std::log(double(diag_n)) + res) / hd;
        } else {
            if (dim == 1) diag_val = std::sqrt((double)diag_n);
            else if (dim == 2) diag_val = 1.0;
            else diag_val = std::sqrt((double)diag_n);
        }
    }

    // ---- tree build ----------------------------------------------------
    // Child c of box k is box 2^d k + c (createTree, 1D/codes/HODLR1Dtree.hpp:79-113,
    // 2D/codes/HODLR2Dtree.hpp:104-140, 3D/codes/HODLR3Dtree.hpp:116-152). Child
    // positions (assign_center_location 2D :426-449, 3D :1700-1741):
    //   2D 0(-,-) 1(+,-) 2(+,+) 3(-,+); 3D the same at z-, then 4..7 at z+.
    int cbit(int c, int axis) const {
        static const int o2[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        static const int o3[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
        if (dim == 1) return c;
        if (dim == 2) return o2[c][axis];
        return o3[c][axis];
    }
    // Neighbour slot of an adjacent (face/edge) offset, or -1.
    // 2D slots (2D/codes/HODLR2Dtree.hpp:142-407): 0 y-, 1 x+, 2 y+, 3 x-.
    // 3D slots (3D/codes/HODLR3Dtree.hpp:155-1666): lexicographic 3x3x3 offset,
    // z slowest, x fastest, self removed; corner offsets never used.
    int nslot(const int *o) const {
        if (dim == 2) {
            if (o[0] == 0 && o[1] == -1) return 0;
            if (o[0] == 1 && o[1] == 0) return 1;
            if (o[0] == 0 && o[1] == 1) return 2;
            if (o[0] == -1 && o[1] == 0) return 3;
            return -1;
        }
        int nz = (o[0] != 0) + (o[1] != 0) + (o[2] != 0);
        if (nz == 0 || nz == 3) return -1;
        int s = (o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1);
        return s > 13 ? s - 1 : s;
    }

    void build_tree() {
        nch = 1 << dim;
        nnb = dim == 1 ? 2 : (dim == 2 ? 4 : 26);
        T.assign((size_t)nL + 1, {});
        for (int j = 0; j <= nL; ++j) {
            size_t nb = (size_t)1 << (dim * j);
            T[(size_t)j].resize(nb);
            for (size_t k = 0; k < nb; ++k) {
                Box &b = T[(size_t)j][k];
                for (int s = 0; s < 26; ++s) b.nb[s] = -1;
                if (j > 0) {
                    const Box &p = T[(size_t)j - 1][k / (size_t)nch];
                    int c = (int)(k % (size_t)nch);
                    for (int a = 0; a < dim; ++a) b.ic[a] = 2 * p.ic[a] + cbit(c, a);
                }
            }
        }
        // Neighbours and ordered interaction lists of the children of each box,
        // level by level (assign_Child*_Interaction).
        for (int j = 0; j < nL; ++j) {
            for (size_t k = 0; k < T[(size_t)j].size(); ++k) {
                for (int c = 0; c < nch; ++c) {
                    size_t kc = (size_t)nch * k + (size_t)c;
                    Box &b = T[(size_t)j + 1][kc];
                    if (dim == 1) {
                        // 1D/codes/HODLR1Dtree.hpp:116-133: siblings only
                        if (c == 0) b.nb[1] = (int)kc + 1;
                        else b.nb[0] = (int)kc - 1;
                        continue;
                    }
                    // groups: the parent itself (siblings), then the parent's
                    // neighbours in slot order
                    std::vector<int> groups;
                    groups.push_back((int)k);
                    for (int s = 0; s < nnb; ++s)
                        if (T[(size_t)j][k].nb[s] != -1) groups.push_back(T[(size_t)j][k].nb[s]);
                    for (size_t g = 0; g < groups.size(); ++g) {
                        int q = groups[g];
                        std::vector<int> vert, far;
                        int nnear = 0;
                        for (int e = 0; e < nch; ++e) {
                            int kk = nch * q + e;
                            if ((size_t)kk == kc) continue;
                            const Box &o = T[(size_t)j + 1][(size_t)kk];
                            int off[3] = {0, 0, 0}, m = 0, nz = 0;
                            for (int a = 0; a < dim; ++a) {
                                off[a] = o.ic[a] - b.ic[a];
                                m = std::max(m, std::abs(off[a]));
                                nz += off[a] != 0;
                            }
                            if (m >= 2) far.push_back(kk);
                            else if (nz == dim) vert.push_back(kk);
                            else { b.nb[nslot(off)] = kk; ++nnear; }
                        }
                        std::vector<int> order;
                        if (dim == 3 && nnear > 0) {
                            // 3D tables push the corner-sharing child first
                            order = vert;
                            order.insert(order.end(), far.begin(), far.end());
                        } else {
                            order = vert;
                            order.insert(order.end(), far.begin(), far.end());
                            std::sort(order.begin(), order.end());
                        }
                        for (int x : order) {
                            b.il.push_back(x);
                            // separate_vertex_interaction (2D :452-475, 3D :1744-1767):
                            // corner-sharing boxes are "vertex"
                            bool isv = std::find(vert.begin(), vert.end(), x) != vert.end();
                            b.ilv.push_back((char)isv);
                        }
                    }
                }
            }
        }
        // assignChargeLocations: 1D/codes/HODLR1Dtree.hpp:168-196, 2D :478-519, 3D :1769-1837.
        // Split on coord <= centre; 3D tests z, then x, then y; 2D x then y.
        T[0][0].pts.resize((size_t)N);
        for (int64_t i = 0; i < N; ++i) T[0][0].pts[(size_t)i] = (int)i;
        // centres: root 0, child = parent +- 0.5*radius(parent level), radius halves per level
        std::vector<std::vector<double>> cen((size_t)nL + 1);
        cen[0].assign((size_t)dim, 0.0);
        std::vector<double> rad((size_t)nL + 1);
        rad[0] = 1.0;
        for (int j = 1; j <= nL; ++j) rad[(size_t)j] = 0.5 * rad[(size_t)j - 1];
        for (int j = 1; j <= nL; ++j) {
            size_t nb = T[(size_t)j].size();
            cen[(size_t)j].resize(nb * (size_t)dim);
            double shift = 0.5 * rad[(size_t)j - 1];
            for (size_t k = 0; k < nb; ++k) {
                size_t p = k / (size_t)nch;
                int c = (int)(k % (size_t)nch);
                for (int a = 0; a < dim; ++a) {
                    double pc = cen[(size_t)j - 1][p * (size_t)dim + (size_t)a];
                    cen[(size_t)j][k * (size_t)dim + (size_t)a] = cbit(c, a) ? pc + shift : pc - shift;
                }
            }
        }
        for (int j = 0; j < nL; ++j) {
            for (size_t k = 0; k < T[(size_t)j].size(); ++k) {
                const double *cc = &cen[(size_t)j][k * (size_t)dim];
                for (int idx : T[(size_t)j][k].pts) {
                    const double *p = &P[(size_t)idx * (size_t)dim];
                    int child;
                    if (dim == 1) child = p[0] <= cc[0] ? 0 : 1;
                    else if (dim == 2) {
                        if (p[0] <= cc[0]) child = p[1] <= cc[1] ? 0 : 3;
                        else child = p[1] <= cc[1] ? 1 : 2;
                    } else {
                        int lo;
                        if (p[0] <= cc[0]) lo = p[1] <= cc[1] ? 0 : 3;
                        else lo = p[1] <= cc[1] ? 1 : 2;
                        child = p[2] <= cc[2] ? lo : lo + 4;
                    }
                    T[(size_t)j + 1][(size_t)nch * k + (size_t)child].pts.push_back(idx);
                }
            }
        }
        // assignNonLeafChargeLocations: concatenation of the children.
        for (int j = nL - 1; j > 0; --j)
            for (size_t k = 0; k < T[(size_t)j].size(); ++k) {
                Box &b = T[(size_t)j][k];
                b.pts.clear();
                for (int c = 0; c < nch; ++c) {
                    const auto &cp = T[(size_t)j + 1][(size_t)nch * k + (size_t)c].pts;
                    b.pts.insert(b.pts.end(), cp.begin(), cp.end());
                }
            }
    }

    // ---- ACA / NCA: 1D/codes/aca.hpp:296-446 (ACA_only_nodes), 2D/codes/aca.hpp:158-294
    // (ACA_only_nodesCUR, same pivoting), 1D/codes/aca.hpp:40-156 (ACA_only_nodesUV).
    struct ACA {
        int rank = 0;
        std::vector<int> rows, cols;  // local pivot indices in pivot order
        Mat Ac, L, R, U, Vt;
    };
    // maxAbsVector (1D/codes/aca.hpp:23-38): first allowed index, strict '>'.
    static int max_abs(const Vec &v, const std::vector<char> &allowed) {
        int index = -1;
        double mx = 0.0;
        for (size_t i = 0; i < v.size(); ++i) {
            if (!allowed[i]) continue;
            if (index < 0) { index = (int)i; mx = abs_(v[i]); continue; }
            if (abs_(v[i]) > std::fabs(mx)) { index = (int)i; mx = abs_(v[i]); }
        }
        return index;
    }
    ACA aca(const std::vector<int> &I, const std::vector<int> &J, bool want_ac, bool want_uv) const {
        ACA res;
        int N1 = (int)I.size(), N2 = (int)J.size();
        int mn = N1 > N2 ? N2 : N1;
        double tol = std::pow(10, -1.0 * tol_pow);
        double tiny = std::pow(10, -36);
        std::vector<char> rrow((size_t)N1, 1), rcol((size_t)N2, 1);
        std::vector<Vec> Uv, Vv, AcV;
        Vec row((size_t)N2), col((size_t)N1);
        auto get_row = [&](int ri, Vec &out) {
            for (int s = 0; s < N2; ++s) out[(size_t)s] = entry(I[(size_t)ri], J[(size_t)s]);
        };
        auto get_col = [&](int ci, Vec &out) {
            for (int s = 0; s < N1; ++s) out[(size_t)s] = entry(I[(size_t)s], J[(size_t)ci]);
        };
        int row_index = 0, col_index = 0, l_local;
        for (l_local = 0; l_local < N1; ++l_local) {
            row_index = l_local;
            get_row(row_index, row);
            col_index = max_abs(row, rcol);
            if (col_index >= 0 && abs_(row[(size_t)col_index]) > tiny) break;
        }
        if (l_local == N1) return res;
        Vec v = row;
        res.rows.push_back(row_index);
        res.cols.push_back(col_index);
        get_col(col_index, col);
        Vec u((size_t)N1);
        S piv = row[(size_t)col_index];
        for (int s = 0; s < N1; ++s) u[(size_t)s] = col[(size_t)s] / piv;
        Uv.push_back(u);
        Vv.push_back(v);
        if (want_ac) AcV.push_back(col);
        rcol[(size_t)col_index] = 0;
        rrow[(size_t)row_index] = 0;
        res.rank = 1;
        double normS = 0.0;
        row_index = max_abs(col, rrow);
        while (nrm(u) * nrm(v) > tol * normS && res.rank < mn) {
            res.rows.push_back(row_index);
            get_row(row_index, row);
            Vec row_temp = row;
            for (int l = 0; l < res.rank; ++l) {
                S ul = Uv[(size_t)l][(size_t)row_index];
                const Vec &Vl = Vv[(size_t)l];
                for (int s = 0; s < N2; ++s) { S p = ul * Vl[(size_t)s]; row[(size_t)s] -= p; }
            }
            col_index = max_abs(row, rcol);
            res.cols.push_back(col_index);
            v = row;
            get_col(col_index, col);
            Vec col_temp = col;
            for (int l = 0; l < res.rank; ++l) {
                S vl = Vv[(size_t)l][(size_t)col_index];
                const Vec &Ul = Uv[(size_t)l];
                for (int s = 0; s < N1; ++s) { S p = vl * Ul[(size_t)s]; col[(size_t)s] -= p; }
            }
            piv = row[(size_t)col_index];
            for (int s = 0; s < N1; ++s) u[(size_t)s] = col[(size_t)s] / piv;
            if (nrm(u) < 1e-36 || nrm(v) < 1e-36) {
                res.rows.pop_back();
                res.cols.pop_back();
                break;
            }
            Uv.push_back(u);
            Vv.push_back(v);
            if (want_ac) AcV.push_back(col_temp);
            ++res.rank;
            rcol[(size_t)col_index] = 0;
            rrow[(size_t)row_index] = 0;
            double uv = nrm(u) * nrm(v);
            normS = normS * normS + uv * uv;
            for (int l = 0; l < res.rank; ++l) {
                S du = dot(Uv[(size_t)l], u), dv = dot(Vv[(size_t)l], v);
                S t = du * dv;
                normS += 2 * abs_(t);
            }
            normS = std::sqrt(normS);
            row_index = max_abs(col, rrow);
        }
        int r = res.rank;
        if (want_ac) {
            res.Ac = Mat(N1, r);
            for (int i = 0; i < r; ++i)
                for (int s = 0; s < N1; ++s) res.Ac(s, i) = AcV[(size_t)i][(size_t)s];
        }
        if (want_uv) {
            res.U = Mat(N1, r);
            res.Vt = Mat(r, N2);
            for (int i = 0; i < r; ++i) {
                for (int s = 0; s < N1; ++s) res.U(s, i) = Uv[(size_t)i][(size_t)s];
                for (int s = 0; s < N2; ++s) res.Vt(i, s) = Vv[(size_t)i][(size_t)s];
            }
        }
        res.L = Mat(r, r);
        res.R = Mat(r, r);
        for (int i = 0; i < r; ++i) {
            res.L(i, i) = 1.0;
            for (int j = 0; j < i; ++j) res.L(i, j) = Uv[(size_t)j][(size_t)res.rows[(size_t)i]];
        }
        for (int i = 0; i < r; ++i) {
            res.R(i, i) = Vv[(size_t)i][(size_t)res.cols[(size_t)i]];
            for (int j = 0; j < i; ++j) res.R(j, i) = Vv[(size_t)j][(size_t)res.cols[(size_t)i]];
        }
        return res;
    }

    // (L^T)^-1 (R^T)^-1 B, column by column (assemble_M2M_ver, 2D :790-813; 1D assemble_M2M :279-302)
    Mat lr_t_solve(const Mat &L, const Mat &R, Mat B) const {
        int n = L.r;
        for (int c = 0; c < B.c; ++c) {
            S *x = &B.a[(size_t)c * (size_t)B.r];
            trsv_lower(R, true, x, n);  // R^T is lower
            trsv_upper(L, true, x, n);  // L^T is upper
        }
        return B;
    }

    std::vector<int> children_concat(int j, int k, bool far_check) const {
        // pivot_selection_bottom_up (2D :537-550) / getParticlesFromChildren_incoming (3D :1880-1894)
        std::vector<int> out;
        if (j == nL) return T[(size_t)j][(size_t)k].pts;
        for (int c = 0; c < nch; ++c) {
            const Box &ch = T[(size_t)j + 1][(size_t)nch * (size_t)k + (size_t)c];
            const auto &v = far_check ? ch.chk : ch.chkv;
            out.insert(out.end(), v.begin(), v.end());
        }
        return out;
    }

    // ---- assembly -------------------------------------------------------
    void assemble_1d() {
        for (int j = 1; j <= nL; ++j)
            for (auto &b : T[(size_t)j]) { b.m2l.assign(2, Mat()); b.Lc.assign(2, Mat()); b.Ac.assign(2, Mat()); b.Ar.assign(2, Mat()); }
        if (form == 0) {
            // getNodes / getNodes_incoming_box: 1D/codes/HODLR1Dtree.hpp:231-276 (top-down)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 1)
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    std::vector<int> cols;
                    for (int nn = 0; nn < 2; ++nn)
                        if (b.nb[nn] != -1) {
                            const auto &pp = lv[(size_t)b.nb[nn]].pts;
                            cols.insert(cols.end(), pp.begin(), pp.end());
                        }
                    if (j > 1) {
                        const auto &pc = T[(size_t)j - 1][(size_t)k / 2].chgv;
                        cols.insert(cols.end(), pc.begin(), pc.end());
                    }
                    ACA a = aca(b.pts, cols, false, false);
                    b.Lv = a.L;
                    b.Rv = a.R;
                    for (int r : a.rows) b.chkv.push_back(b.pts[(size_t)r]);
                    for (int c : a.cols) b.chgv.push_back(cols[(size_t)c]);
                }
            }
            // assemble_M2M :279-302
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 4)
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    if (j == nL) b.M2M[0] = lr_t_solve(b.Lv, b.Rv, block(b.chgv, b.pts));
                    else
                        for (int c = 0; c < 2; ++c)
                            b.M2M[c] = lr_t_solve(b.Lv, b.Rv, block(b.chgv, T[(size_t)j + 1][(size_t)(2 * k + c)].chkv));
                }
            }
            // assemble_M2L :346-365 (sibling; the partner's block is the transpose)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k)
                    for (int nn = 0; nn < 2; ++nn)
                        if (lv[(size_t)k].nb[nn] != -1)
                            lv[(size_t)k].m2l[(size_t)nn] = block(lv[(size_t)k].chkv, lv[(size_t)lv[(size_t)k].nb[nn]].chkv);
            }
        } else {
            // getUVtTree_nn / getUVtInstance :418-443 (ACA_only_nodesUV)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 1)
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    b.rowb.assign(2, {});
                    b.colb.assign(2, {});
                    for (int nn = 0; nn < 2; ++nn) {
                        int q = b.nb[nn];
                        if (q == -1) continue;
                        ACA a = aca(b.pts, lv[(size_t)q].pts, false, true);
                        b.Ac[(size_t)nn] = a.U;
                        b.Ar[(size_t)nn] = a.Vt;
                        for (int r : a.rows) b.rowb[(size_t)nn].push_back(b.pts[(size_t)r]);
                        for (int c : a.cols) b.colb[(size_t)nn].push_back(lv[(size_t)q].pts[(size_t)c]);
                    }
                }
            }
        }
        // assemble_NearField :466-474 (self block only)
        auto &lf = T[(size_t)nL];
#pragma omp parallel for
        for (long k = 0; k < (long)lf.size(); ++k) lf[(size_t)k].dense[0] = block(lf[(size_t)k].pts, lf[(size_t)k].pts);
    }

    void assemble_nd() {
        for (int j = 1; j <= nL; ++j)
            for (auto &b : T[(size_t)j]) {
                size_t n = b.il.size();
                b.m2l.assign(n, Mat());
                b.rowb.assign(n, {});
                b.colb.assign(n, {});
                b.Lc.assign(n, Mat());
                b.Rc.assign(n, Mat());
                b.Ac.assign(n, Mat());
                b.Ar.assign(n, Mat());
            }
        // far field, bottom-up NCA: getNodes + getNodes_incoming_box (2D :552-597, 3D :1872-1939);
        // H* (form 2) has no nested far field (2D/codes/matvec.hpp:136-160)
        for (int j = nL; j >= 2 && form != 2; --j) {
            auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 1)
            for (long k = 0; k < (long)lv.size(); ++k) {
                Box &b = lv[(size_t)k];
                std::vector<int> rows = children_concat(j, (int)k, true), cols;
                for (size_t in = 0; in < b.il.size(); ++in)
                    if (!b.ilv[in]) {
                        std::vector<int> c2 = children_concat(j, b.il[in], true);
                        cols.insert(cols.end(), c2.begin(), c2.end());
                    }
                ACA a = aca(rows, cols, true, false);
                if (a.rank > 0) {
                    for (int r : a.rows) b.chk.push_back(rows[(size_t)r]);
                    for (int c : a.cols) b.chg.push_back(cols[(size_t)c]);
                    Mat t = solve_right_upper(a.R, a.Ac);
                    b.L2P = solve_right_lower(a.L, t);
                } else {
                    b.L2P = Mat((int)rows.size(), 0);
                }
            }
        }
        // M2L far: assemble_M2L_far (2D :655-675, 3D :1978-1998)
        for (int j = 2; j <= nL && form != 2; ++j) {
            auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 4)
            for (long k = 0; k < (long)lv.size(); ++k) {
                Box &b = lv[(size_t)k];
                for (size_t in = 0; in < b.il.size(); ++in)
                    if (!b.ilv[in]) b.m2l[in] = block(b.chk, lv[(size_t)b.il[in]].chk);
            }
        }
        if (form == 0) {
            // vertex, top-down NCA: getNodes_ver + getNodes_incoming_box_vertex (2D :741-786, 3D :2062-2107)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 1)
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    std::vector<int> cols;
                    for (size_t i = 0; i < b.il.size(); ++i)
                        if (b.ilv[i]) {
                            const auto &pp = lv[(size_t)b.il[i]].pts;
                            cols.insert(cols.end(), pp.begin(), pp.end());
                        }
                    if (j > 1) {
                        const auto &pc = T[(size_t)j - 1][(size_t)k / (size_t)nch].chgv;
                        cols.insert(cols.end(), pc.begin(), pc.end());
                    }
                    ACA a = aca(b.pts, cols, false, false);
                    b.Lv = a.L;
                    b.Rv = a.R;
                    for (int r : a.rows) b.chkv.push_back(b.pts[(size_t)r]);
                    for (int c : a.cols) b.chgv.push_back(cols[(size_t)c]);
                }
            }
            // assemble_M2L_ver (2D :859-880, 3D :2164-2185), assemble_M2M_ver (2D :790-813, 3D :2110-2133)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 4)
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    for (size_t in = 0; in < b.il.size(); ++in)
                        if (b.ilv[in]) b.m2l[in] = block(b.chkv, lv[(size_t)b.il[in]].chkv);
                    if (j == nL) b.M2M[0] = lr_t_solve(b.Lv, b.Rv, block(b.chgv, b.pts));
                    else
                        for (int c = 0; c < nch; ++c)
                            b.M2M[c] = lr_t_solve(b.Lv, b.Rv,
                                                  block(b.chgv, T[(size_t)j + 1][(size_t)nch * (size_t)k + (size_t)c].chkv));
                }
            }
        } else {
            // semi-nested vertex pairs: getUVtTree_sn + assembleAcAr_sn (2D :953-1005, 3D :2250-2321);
            // H*: every interaction-list pair, getUVtTree_nn + assembleAcAr_nn (2D :971-1021, 3D :2239-2321)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 1)
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    for (size_t i = 0; i < b.il.size(); ++i) {
                        if (!b.ilv[i] && form == 1) continue;
                        const auto &qp = lv[(size_t)b.il[i]].pts;
                        ACA a = aca(b.pts, qp, false, false);
                        b.Lc[i] = a.L;
                        b.Rc[i] = a.R;
                        for (int r = 0; r < a.rank; ++r) b.rowb[i].push_back(b.pts[(size_t)a.rows[(size_t)r]]);
                        for (int c = 0; c < a.rank; ++c) b.colb[i].push_back(qp[(size_t)a.cols[(size_t)c]]);
                        if (!b.colb[i].empty()) {
                            b.Ac[i] = block(b.pts, b.colb[i]);
                            b.Ar[i] = block(b.rowb[i], qp);
                        }
                    }
                }
            }
        }
        // near field: assemble_NearField (2D :1075-1090, 3D :2375-2390); slot nnb = self
        auto &lf = T[(size_t)nL];
#pragma omp parallel for schedule(dynamic, 4)
        for (long k = 0; k < (long)lf.size(); ++k) {
            Box &b = lf[(size_t)k];
            for (int n = 0; n < nnb; ++n)
                if (b.nb[n] != -1) b.dense[n] = block(b.pts, lf[(size_t)b.nb[n]].pts);
            b.dense[nnb] = block(b.pts, b.pts);
        }
    }

    // ---- matvec ---------------------------------------------------------
    void assign_charges(const S *x) {  // assignCharges (1D :215-229, 3D :1854-1868)
        for (int j = 1; j <= nL; ++j)
            for (auto &b : T[(size_t)j]) {
                b.q.resize(b.pts.size());
                for (size_t i = 0; i < b.pts.size(); ++i) b.q[i] = x[b.pts[i]];
            }
    }
    void reorder(const Vec &yp, S *y) {  // reorder (1D :519-533, 3D :2489-2503)
        size_t cnt = 0;
        for (auto &b : T[(size_t)nL])
            for (int idx : b.pts) y[idx] = yp[cnt++];
    }

    void matvec_1d(const S *x, S *y) {
        assign_charges(x);
        Vec yp((size_t)N, 0.0);
        if (form == 0) {
            // evaluate_M2M (1D :304-344)
            for (int j = nL; j >= 1; --j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    if (j == nL) b.out = gemv(b.M2M[0], b.q);
                    else {
                        b.out.assign(b.chkv.size(), 0.0);
                        for (int c = 0; c < 2; ++c) addto(b.out, gemv(b.M2M[c], T[(size_t)j + 1][(size_t)(2 * k + c)].out));
                    }
                }
            }
            // evaluate_M2L (1D :367-388)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    b.in.assign(b.chkv.size(), 0.0);
                    for (int nn = 0; nn < 2; ++nn)
                        if (b.nb[nn] != -1) addto(b.in, gemv(b.m2l[(size_t)nn], lv[(size_t)b.nb[nn]].out));
                }
            }
            // evaluate_L2L (1D :390-416)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    if (j != nL)
                        for (int c = 0; c < 2; ++c) addto(T[(size_t)j + 1][(size_t)(2 * k + c)].in, gemvT(b.M2M[c], b.in));
                    else b.pot = gemvT(b.M2M[0], b.in);
                }
            }
            // evaluate_NearField (1D :476-485)
            auto &lf = T[(size_t)nL];
#pragma omp parallel for
            for (long k = 0; k < (long)lf.size(); ++k) addto(lf[(size_t)k].pot, gemv(lf[(size_t)k].dense[0], lf[(size_t)k].q));
            // collect_all_potentials (1D :487-501)
            size_t cnt = 0;
            for (auto &b : lf)
                for (S v : b.pot) { yp[cnt] = 0.0 + v; ++cnt; }
        } else {
            // fast_multiplication_nn (1D :445-464)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    b.pot.assign(b.q.size(), 0.0);
                    for (int nn = 0; nn < 2; ++nn)
                        if (b.nb[nn] != -1) addto(b.pot, gemv(b.Ac[(size_t)nn], gemv(b.Ar[(size_t)nn], lv[(size_t)b.nb[nn]].q)));
                }
            }
            auto &lf = T[(size_t)nL];
#pragma omp parallel for
            for (long k = 0; k < (long)lf.size(); ++k) addto(lf[(size_t)k].pot, gemv(lf[(size_t)k].dense[0], lf[(size_t)k].q));
            // collect_all_potential_nn (1D :503-517)
            for (int j = 1; j <= nL; ++j) {
                size_t cnt = 0;
                for (auto &b : T[(size_t)j])
                    for (S v : b.pot) { yp[cnt] += v; ++cnt; }
            }
        }
        reorder(yp, y);
    }

    // H* (USE_HODLRdD): evaluateFarField_nn (2D :1053-1071, 3D :2353-2373) sets every
    // box's potential from its pairs, evaluate_NearField adds the leaf blocks,
    // collect_all_potentials_nn (2D :1175-1189, 3D :2473-2487) sums the levels.
    void matvec_nn(const S *x, S *y) {
        assign_charges(x);
        for (int j = 1; j <= nL; ++j) {
            auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 4)
            for (long k = 0; k < (long)lv.size(); ++k) {
                Box &b = lv[(size_t)k];
                b.pot.assign(b.q.size(), 0.0);
                for (size_t i = 0; i < b.il.size(); ++i) {
                    if (b.colb[i].empty()) continue;
                    Vec t = gemv(b.Ar[i], lv[(size_t)b.il[i]].q);
                    int r = b.Lc[i].r;
                    trsv_lower(b.Lc[i], false, t.data(), r);
                    trsv_upper(b.Rc[i], false, t.data(), r);
                    addto(b.pot, gemv(b.Ac[i], t));
                }
            }
        }
        auto &lf = T[(size_t)nL];
#pragma omp parallel for
        for (long k = 0; k < (long)lf.size(); ++k) {
            Box &b = lf[(size_t)k];
            for (int n = 0; n < nnb; ++n)
                if (b.nb[n] != -1) addto(b.pot, gemv(b.dense[n], lf[(size_t)b.nb[n]].q));
            addto(b.pot, gemv(b.dense[nnb], b.q));
        }
        Vec yp((size_t)N, 0.0);
        for (int j = 1; j <= nL; ++j) {
            size_t cnt = 0;
            for (auto &b : T[(size_t)j])
                for (S v : b.pot) { yp[cnt] += v; ++cnt; }
        }
        reorder(yp, y);
    }

    void matvec_nd(const S *x, S *y) {
        if (form == 2) {
            matvec_nn(x, y);
            return;
        }
        assign_charges(x);
        // evaluate_M2M_far (2D :617-653, 3D :1941-1976)
        for (int j = nL; j >= 2; --j) {
            auto &lv = T[(size_t)j];
#pragma omp parallel for
            for (long k = 0; k < (long)lv.size(); ++k) {
                Box &b = lv[(size_t)k];
                Vec src;
                if (j == nL) src = b.q;
                else
                    for (int c = 0; c < nch; ++c) {
                        const Vec &o = T[(size_t)j + 1][(size_t)nch * (size_t)k + (size_t)c].out;
                        src.insert(src.end(), o.begin(), o.end());
                    }
                b.out = gemvT(b.L2P, src);
            }
        }
        // evaluate_M2L_far (2D :678-699, 3D :2000-2021)
        for (int j = 2; j <= nL; ++j) {
            auto &lv = T[(size_t)j];
#pragma omp parallel for
            for (long k = 0; k < (long)lv.size(); ++k) {
                Box &b = lv[(size_t)k];
                b.in.assign(b.chk.size(), 0.0);
                for (size_t in = 0; in < b.il.size(); ++in)
                    if (!b.ilv[in]) addto(b.in, gemv(b.m2l[in], lv[(size_t)b.il[in]].out));
            }
        }
        // evaluate_L2L_far (2D :702-734, 3D :2023-2055)
        for (int j = 2; j <= nL; ++j) {
            auto &lv = T[(size_t)j];
#pragma omp parallel for
            for (long k = 0; k < (long)lv.size(); ++k) {
                Box &b = lv[(size_t)k];
                if (j != nL) {
                    Vec t = gemv(b.L2P, b.in);
                    size_t ind = 0;
                    for (int c = 0; c < nch; ++c) {
                        Box &ch = T[(size_t)j + 1][(size_t)nch * (size_t)k + (size_t)c];
                        for (size_t i = 0; i < ch.chk.size(); ++i) ch.in[i] += t[ind + i];
                        ind += ch.chk.size();
                    }
                } else b.pot = gemv(b.L2P, b.in);
            }
        }
        auto &lf = T[(size_t)nL];
        if (form == 0) {
            // evaluate_M2M_ver (2D :815-856, 3D :2135-2162)
            for (int j = nL; j >= 1; --j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    if (j == nL) b.out = gemv(b.M2M[0], b.q);
                    else {
                        b.out.assign(b.chkv.size(), 0.0);
                        for (int c = 0; c < nch; ++c)
                            addto(b.out, gemv(b.M2M[c], T[(size_t)j + 1][(size_t)nch * (size_t)k + (size_t)c].out));
                    }
                }
            }
            // evaluate_M2L_ver (2D :882-903, 3D :2187-2208)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    b.inv.assign(b.chkv.size(), 0.0);
                    for (size_t in = 0; in < b.il.size(); ++in)
                        if (b.ilv[in]) addto(b.inv, gemv(b.m2l[in], lv[(size_t)b.il[in]].out));
                }
            }
            // evaluate_L2L_ver (2D :906-932, 3D :2210-2237)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    if (j != nL)
                        for (int c = 0; c < nch; ++c)
                            addto(T[(size_t)j + 1][(size_t)nch * (size_t)k + (size_t)c].inv, gemvT(b.M2M[c], b.inv));
                    else b.potv = gemvT(b.M2M[0], b.inv);
                }
            }
        }
        // evaluate_NearField (2D :1093-1125, 3D :2392-2423)
        if (nL < 2)
            for (auto &b : lf) b.pot.assign(b.q.size(), 0.0);
#pragma omp parallel for
        for (long k = 0; k < (long)lf.size(); ++k) {
            Box &b = lf[(size_t)k];
            for (int n = 0; n < nnb; ++n)
                if (b.nb[n] != -1) addto(b.pot, gemv(b.dense[n], lf[(size_t)b.nb[n]].q));
            addto(b.pot, gemv(b.dense[nnb], b.q));
        }
        Vec yp((size_t)N, 0.0);
        if (form == 0) {
            // collect_all_potentials_n (2D :1128-1142, 3D :2426-2440)
            size_t cnt = 0;
            for (auto &b : lf)
                for (size_t i = 0; i < b.pot.size(); ++i) {
                    S pv = b.pot[i] + b.potv[i];
                    yp[cnt] = 0.0 + pv;
                    ++cnt;
                }
        } else {
            // evaluateFarField_sn (2D :1023-1051, 3D :2323-2351)
            for (int j = 1; j <= nL; ++j) {
                auto &lv = T[(size_t)j];
#pragma omp parallel for schedule(dynamic, 4)
                for (long k = 0; k < (long)lv.size(); ++k) {
                    Box &b = lv[(size_t)k];
                    b.potv.assign(b.q.size(), 0.0);
                    for (size_t i = 0; i < b.il.size(); ++i) {
                        if (b.colb[i].empty() || !b.ilv[i]) continue;
                        Vec t = gemv(b.Ar[i], lv[(size_t)b.il[i]].q);
                        int r = b.Lc[i].r;
                        trsv_lower(b.Lc[i], false, t.data(), r);
                        trsv_upper(b.Rc[i], false, t.data(), r);
                        addto(b.potv, gemv(b.Ac[i], t));
                    }
                }
            }
            // collect_all_potentials_semi_1 / _semi_2 (2D :1144-1173, 3D :2442-2471)
            size_t cnt = 0;
            for (auto &b : lf)
                for (S v : b.pot) { yp[cnt] = 0.0 + v; ++cnt; }
            for (int j = 1; j <= nL; ++j) {
                cnt = 0;
                for (auto &b : T[(size_t)j])
                    for (S v : b.potv) { yp[cnt] += v; ++cnt; }
            }
        }
        reorder(yp, y);
    }

    // ---- storage: findMemory_n / _sn / _nn (1D :535-588, 2D :1207-1328, 3D :2505-2628)
    double memory() const {
        double mem = 0.0;
        if (dim == 1) {
            for (int j = 1; j <= nL; ++j)
                for (const auto &b : T[(size_t)j]) {
                    for (int nn = 0; nn < 2; ++nn) {
                        if (b.nb[nn] == -1) continue;
                        if (form == 0) mem += (double)b.m2l[(size_t)nn].size();
                        else mem += (double)(b.Ac[(size_t)nn].size() + b.Ar[(size_t)nn].size());
                    }
                    if (form == 0) {
                        if (j == nL) mem += 2.0 * (double)b.M2M[0].size();
                        else for (int c = 0; c < 2; ++c) mem += 2.0 * (double)b.M2M[c].size();
                    }
                }
            if (form == 0)
                for (const auto &b : T[(size_t)nL]) mem += (double)b.dense[0].size();
            return mem;
        }
        for (int j = 2; j <= nL; ++j)
            for (const auto &b : T[(size_t)j]) {
                mem += 2.0 * (double)b.L2P.size();
                for (size_t i = 0; i < b.il.size(); ++i)
                    if (!b.ilv[i]) mem += (double)b.m2l[i].size();
            }
        for (int j = 1; j <= nL; ++j)
            for (const auto &b : T[(size_t)j]) {
                if (form == 0) {
                    if (j == nL) mem += 2.0 * (double)b.M2M[0].size();
                    else for (int c = 0; c < nch; ++c) mem += 2.0 * (double)b.M2M[c].size();
                }
                for (size_t i = 0; i < b.il.size(); ++i) {
                    if (!b.ilv[i] && form != 2) continue;  // findMemory_nn counts every pair
                    if (form == 0) mem += (double)b.m2l[i].size();
                    else mem += (double)(b.Lc[i].size() + b.Rc[i].size() + b.Ac[i].size() + b.Ar[i].size());
                }
            }
        for (const auto &b : T[(size_t)nL]) {
            mem += (double)(b.pts.size() * b.pts.size());
            for (int n = 0; n < nnb; ++n)
                if (b.nb[n] != -1) mem += (double)(b.pts.size() * T[(size_t)nL][(size_t)b.nb[n]].pts.size());
        }
        return mem;
    }

    void matvec(const S *x, S *y) {
        if (dim == 1) matvec_1d(x, y);
        else matvec_nd(x, y);
    }

    // ---- GMRES: */codes/gmres.hpp:30-200 (oracle/gmres_ref.hpp) ------------
    int gmres(const S *bb, S *x, int max_iter, int tol_pow, int *iters, double *resid) {
        return h2w_ref::gmres([this](const S *in, S *out) { matvec(in, out); }, (size_t)N, bb, x, max_iter,
                              tol_pow, iters, resid);
    }
};

}  // namespace

// One oracle handle: the real operator, or the complex Helmholtz one (choice 2,
// 3D); complex vectors cross the C API as interleaved (re, im) doubles.
struct h2wo {
    OracleT<double> *r = nullptr;
    OracleT<cplx> *c = nullptr;
    ~h2wo() {
        delete r;
        delete c;
    }
};

// run f on the handle's operator with its scalar pointer type
template <class F> auto on(h2wo *h, F &&f) {
    if (h->c) return f(*h->c, (cplx *)nullptr);
    return f(*h->r, (double *)nullptr);
}

template <class S> void init_oracle(OracleT<S> &o, int dim, int form, int64_t n, const double *pts, int nlevels,
                                    int tol_pow, int choice, int64_t kernel_n, int64_t diag_n) {
    o.dim = dim;
    o.form = form;
    o.N = n;
    o.P.assign(pts, pts + (size_t)n * (size_t)dim);
    o.nL = nlevels;
    o.tol_pow = tol_pow;
    o.choice = choice;
    o.kernel_n = kernel_n;
    o.diag_n = diag_n;
    o.setup_kernel();
    o.build_tree();
}

template <class S>
static void list_of(const OracleT<S> &o, int which, std::vector<int64_t> &ptr, std::vector<int32_t> &val) {
    ptr.assign(1, 0);
    val.clear();
    auto add = [&](const std::vector<int> &v) {
        for (int x : v) val.push_back(x);
        ptr.push_back((int64_t)val.size());
    };
    for (int j = 0; j <= o.nL; ++j)
        for (const auto &b : o.T[(size_t)j]) {
            switch (which) {
            case 0: add(b.pts); break;
            case 1: add(std::vector<int>(b.nb, b.nb + o.nnb)); break;
            case 2: add(b.il); break;
            case 3: { std::vector<int> f(b.ilv.begin(), b.ilv.end()); add(f); break; }
            case 4: add(o.dim == 1 ? b.chkv : b.chk); break;
            case 5: add(o.dim == 1 ? b.chgv : b.chg); break;
            case 6: add(o.dim == 1 ? std::vector<int>() : b.chkv); break;
            case 7: add(o.dim == 1 ? std::vector<int>() : b.chgv); break;
            case 8:
            case 9:
                if (o.dim == 1) {
                    if (j == 0) break;
                    for (int nn = 0; nn < 2; ++nn) {
                        if (b.rowb.size() == 2) add(which == 8 ? b.rowb[(size_t)nn] : b.colb[(size_t)nn]);
                        else add({});
                    }
                } else {
                    for (size_t i = 0; i < b.il.size(); ++i) {
                        if (b.rowb.size() == b.il.size()) add(which == 8 ? b.rowb[i] : b.colb[i]);
                        else add({});
                    }
                }
                break;
            case 10:
                if (j == 0) break;
                {
                    std::vector<int> rk;
                    for (int nn = 0; nn < 2; ++nn)
                        rk.push_back(b.nb[nn] == -1 ? -1 : (b.Ac.size() == 2 ? b.Ac[(size_t)nn].c : 0));
                    add(rk);
                }
                break;
            default: break;
            }
        }
}


extern "C" {

h2wo *h2wo_create(int dim, int form, int64_t n, const double *pts, int nlevels, int tol_pow, int choice,
                  int64_t kernel_n, int64_t diag_n) {
    if (dim < 1 || dim > 3 || n < 1 || nlevels < 1 || (form != 0 && form != 1 && form != 2) || (form == 2 && dim == 1) ||
        (choice != 0 && choice != 1 && choice != 2 && choice != 10) || (choice == 2 && dim != 3) ||
        (choice == 10 && dim != 2))
        return nullptr;
    h2wo *h = new h2wo;
    if (choice == 2 || choice == 10) {
        h->c = new OracleT<cplx>;
        init_oracle(*h->c, dim, form, n, pts, nlevels, tol_pow, choice, kernel_n, diag_n);
    } else {
        h->r = new OracleT<double>;
        init_oracle(*h->r, dim, form, n, pts, nlevels, tol_pow, choice, kernel_n, diag_n);
    }
    return h;
}

void h2wo_destroy(h2wo *o) { delete o; }

int h2wo_assemble(h2wo *h) {
    return on(h, [](auto &o, auto *) {
        if (o.dim == 1) o.assemble_1d();
        else o.assemble_nd();
        return 0;
    });
}

int h2wo_matvec(h2wo *h, const double *x, double *y) {
    return on(h, [&](auto &o, auto *t) {
        using S = std::remove_pointer_t<decltype(t)>;
        o.matvec(reinterpret_cast<const S *>(x), reinterpret_cast<S *>(y));
        return 0;
    });
}

int h2wo_dense_matvec(h2wo *h, const double *x, double *y) {
    // getTruePoten (1D :590-604, 2D :1333-1346, 3D :2630-2643)
    return on(h, [&](auto &o, auto *t) {
        using S = std::remove_pointer_t<decltype(t)>;
        const S *xs = reinterpret_cast<const S *>(x);
        S *ys = reinterpret_cast<S *>(y);
#pragma omp parallel for schedule(dynamic, 64)
        for (long i = 0; i < (long)o.N; ++i) {
            S s = S(0.0);
            for (long j = 0; j < (long)o.N; ++j) { S p = o.entry((int)i, (int)j) * xs[j]; s = s + p; }
            ys[i] = s;
        }
        return 0;
    });
}

int h2wo_gmres(h2wo *h, const double *b, double *x, int max_iter, int tol_pow, int *iters, double *resid) {
    return on(h, [&](auto &o, auto *t) {
        using S = std::remove_pointer_t<decltype(t)>;
        return o.gmres(reinterpret_cast<const S *>(b), reinterpret_cast<S *>(x), max_iter, tol_pow, iters, resid);
    });
}

double h2wo_memory(h2wo *h) {
    return on(h, [](auto &o, auto *) { return o.memory(); });
}
double h2wo_kii(h2wo *h) {
    return on(h, [](auto &o, auto *) { return o.Kii; });
}

/* entries K(rows[i], cols[j]); complex kernels write (re, im) pairs */
int h2wo_entries(h2wo *h, const int32_t *rows, int64_t nr, const int32_t *cols, int64_t nc, double *out) {
    return on(h, [&](auto &o, auto *t) {
        using S = std::remove_pointer_t<decltype(t)>;
        S *os = reinterpret_cast<S *>(out);
        for (int64_t i = 0; i < nr; ++i)
            for (int64_t j = 0; j < nc; ++j) os[i * nc + j] = o.entry(rows[i], cols[j]);
        return 0;
    });
}

int h2wo_is_complex(h2wo *h) { return h->c ? 1 : 0; }

void h2wo_set_sum_order(int reverse) { g_sum_reverse = reverse ? 1 : 0; }

int64_t h2wo_list(h2wo *h, int which, int64_t *ptr, int32_t *val) {
    std::vector<int64_t> p;
    std::vector<int32_t> v;
    on(h, [&](auto &o, auto *) { list_of(o, which, p, v); return 0; });
    if (ptr) std::memcpy(ptr, p.data(), p.size() * sizeof(int64_t));
    if (val && !v.empty()) std::memcpy(val, v.data(), v.size() * sizeof(int32_t));
    return (int64_t)v.size();
}

int64_t h2wo_list_nptr(h2wo *h, int which) {
    std::vector<int64_t> p;
    std::vector<int32_t> v;
    on(h, [&](auto &o, auto *) { list_of(o, which, p, v); return 0; });
    return (int64_t)p.size();
}

}  // extern "C"
