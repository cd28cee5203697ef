// The reference's unrestarted GMRES (iterative_solver::GMRES,
// 1D/codes/gmres.hpp:30-200; 2D and 3D copies alike) restated as a template
// over the operator and its scalar: `matvec(const S *x, S *y)` computes y = A x
// (S = double, or std::complex<double> for the complex Helmholtz builds).
//
// TEST INFRASTRUCTURE ONLY: used by the CPU oracle (oracle/h2w_oracle.cpp)
// and by the adapter test program (tests/adapter_gmres.cpp), which drives the
// GPU operator through include/h2w_adapter.hpp exactly as the reference's
// GMRES<T> drives its operator. Every multiply and add is separately rounded
// (built with -ffp-contract=off), sums run in ascending index order (the
// Eigen-subset shim's order).
#ifndef H2W_GMRES_REF_HPP
#define H2W_GMRES_REF_HPP
#include <cmath>
#include <complex>
#include <cstddef>
#include <vector>

namespace h2w_ref {

using Vec = std::vector<double>;
using cplx = std::complex<double>;

// Scalars: the reference's real build (dtype = double) and its complex
// Helmholtz builds (dtype = std::complex<double>, 3D/codes/headers.hpp:35-40).
inline double conj_(double a) { return a; }
inline cplx conj_(const cplx &a) { return std::conj(a); }
inline double abs_(double a) { return std::fabs(a); }
inline double abs_(const cplx &a) { return std::abs(a); }
inline double abs2_(double a) { return a * a; }
inline double real_(double a) { return a; }
inline double real_(const cplx &a) { return a.real(); }
inline double abs2_(const cplx &a) {
    double r = a.real() * a.real(), i = a.imag() * a.imag();
    return r + i;
}

// Eigen's a.dot(b): sum of conj(a_i) b_i, ascending
template <class S>
S dot(const std::vector<S> &a, const std::vector<S> &b) {
    S s = S(0.0);
    for (size_t i = 0; i < a.size(); ++i) { S p = conj_(a[i]) * b[i]; s = s + p; }
    return s;
}
// Eigen's norm(): sqrt of the sum of |a_i|^2
template <class S>
double nrm(const std::vector<S> &a) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) { double p = abs2_(a[i]); s = s + p; }
    return std::sqrt(s);
}

// GeneratePlaneRotation / ApplyPlaneRotation (1D/codes/gmres.hpp:30-62)
inline void gen_rot(double dx, double dy, double &cs, double &sn) {
    if (dy == 0.0) { cs = 1.0; sn = 0.0; }
    else if (std::fabs(dy) > std::fabs(dx)) {
        double temp = dx / dy;
        sn = 1.0 / std::sqrt(1.0 + temp * temp);
        cs = temp * sn;
    } else {
        double temp = dy / dx;
        cs = 1.0 / std::sqrt(1.0 + temp * temp);
        sn = temp * cs;
    }
}
inline void app_rot(double &dx, double &dy, double cs, double sn) {
    double a = cs * dx, b = sn * dy;
    double temp = a + b;
    double c = -sn * dx, d = cs * dy;
    dy = c + d;
    dx = temp;
}
// the complex builds' forms (3D/codes/gmres.hpp:52-75, 2D/codes/gmres.hpp:52-75)
inline void gen_rot(const cplx &dx, const cplx &dy, cplx &cs, cplx &sn) {
    if (dx == cplx(0)) {
        cs = cplx(0);
        sn = cplx(1);
    } else {
        double scale = std::abs(dx) + std::abs(dy);
        double norm = scale * std::sqrt(std::abs(dx / scale) * std::abs(dx / scale) +
                                        std::abs(dy / scale) * std::abs(dy / scale));
        cplx alpha = dx / std::abs(dx);
        cs = std::abs(dx) / norm;
        sn = alpha * std::conj(dy) / norm;
    }
}
inline void app_rot(cplx &dx, cplx &dy, const cplx &cs, const cplx &sn) {
    cplx temp = cs * dx + sn * dy;
    dy = -sn * dx + cs * dy;
    dx = temp;
}

// Update (1D/codes/gmres.hpp:64-90): back substitution, x += V y
template <class S, class HF>
void update(S *x, size_t n, int k, HF &h, const std::vector<S> &s, const std::vector<std::vector<S>> &v) {
    std::vector<S> y = s;
    for (int i = k; i >= 0; --i) {
        y[(size_t)i] /= h(i, i);
        for (int jj = i - 1; jj >= 0; --jj) { S p = h(jj, i) * y[(size_t)i]; y[(size_t)jj] -= p; }
    }
    for (int jj = 0; jj <= k; ++jj)
        for (size_t t = 0; t < n; ++t) { S p = v[(size_t)jj][t] * y[(size_t)jj]; x[t] += p; }
}

// GMRES (1D/codes/gmres.hpp:92-200): x0 = x on entry, restart = max_iter,
// stop when |s(i+1)| / ||b|| < 10^-tol_pow. Returns 0 when converged.
// S = double, or std::complex<double> for the complex builds (whose
// Gram-Schmidt coefficient is w.dot(v_k), Eigen's conjugate-first dot).
template <class S, class MV>
int gmres(MV &&matvec, size_t n, const S *bb, S *x, int max_iter, int tol_pow, int *iters, double *resid) {
    using V = std::vector<S>;
    int m = max_iter;
    double gtol = std::pow(10, -1.0 * tol_pow);
    std::vector<S> H((size_t)(m + 1) * (size_t)m, S(0.0));  // column-major (m+1) x m
    auto h = [&](int r, int c) -> S & { return H[(size_t)r + (size_t)c * (size_t)(m + 1)]; };
    V s((size_t)m + 1, S(0.0)), cs((size_t)m + 1, S(0.0)), sn((size_t)m + 1, S(0.0));
    V b(bb, bb + n);
    double normb = nrm(b);
    V out(n);
    matvec(x, out.data());
    V r(n);
    for (size_t i = 0; i < n; ++i) r[i] = b[i] - out[i];
    double beta = nrm(r);
    if (normb == 0.0) normb = 1;
    *resid = beta / normb;
    if (*resid <= gtol) { *iters = 0; return 0; }
    std::vector<V> v((size_t)m + 1);
    int j = 1;
    while (j <= max_iter) {
        double ib = 1.0 / beta;
        v[0].resize(n);
        for (size_t i = 0; i < n; ++i) v[0][i] = r[i] * ib;
        s.assign((size_t)m + 1, S(0.0));
        s[0] = beta;
        for (int i = 0; i < m && j <= max_iter; ++i, ++j) {
            V w(n);
            matvec(v[(size_t)i].data(), w.data());
            for (int k = 0; k <= i; ++k) {
                h(k, i) = dot(w, v[(size_t)k]);
                S hk = h(k, i);
                for (size_t t = 0; t < n; ++t) { S p = hk * v[(size_t)k][t]; w[t] -= p; }
            }
            h(i + 1, i) = nrm(w);
            S ih = S(1.0) / h(i + 1, i);
            v[(size_t)i + 1].resize(n);
            for (size_t t = 0; t < n; ++t) v[(size_t)i + 1][t] = ih * w[t];
            for (int k = 0; k < i; ++k) app_rot(h(k, i), h(k + 1, i), cs[(size_t)k], sn[(size_t)k]);
            gen_rot(h(i, i), h(i + 1, i), cs[(size_t)i], sn[(size_t)i]);
            app_rot(h(i, i), h(i + 1, i), cs[(size_t)i], sn[(size_t)i]);
            app_rot(s[(size_t)i], s[(size_t)i + 1], cs[(size_t)i], sn[(size_t)i]);
            *resid = abs_(s[(size_t)i + 1]) / normb;
            if (*resid < gtol) {
                update(x, n, i, h, s, v);
                *iters = j;
                return 0;
            }
        }
        update(x, n, m - 1, h, s, v);
        matvec(x, out.data());
        for (size_t t = 0; t < n; ++t) r[t] = b[t] - out[t];
        beta = nrm(r);
        *resid = beta / normb;
        if (*resid < gtol) { *iters = j; return 0; }
    }
    *iters = j - 1;
    return 1;
}

}  // namespace h2w_ref
#endif
