// The reference's unrestarted GMRES (iterative_solver::GMRES,
// 1D/codes/gmres.hpp:30-200; 2D and 3D copies alike) restated as a template
// over the operator: `matvec(const double *x, double *y)` computes y = A x.
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
#include <cstddef>
#include <vector>

namespace h2w_ref {

using Vec = std::vector<double>;

inline double dot(const Vec &a, const Vec &b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) { double p = a[i] * b[i]; s = s + p; }
    return s;
}
inline double nrm(const Vec &a) { return std::sqrt(dot(a, a)); }

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

// Update (1D/codes/gmres.hpp:64-90): back substitution, x += V y
template <class HF>
void update(double *x, size_t n, int k, HF &h, const Vec &s, const std::vector<Vec> &v) {
    Vec y = s;
    for (int i = k; i >= 0; --i) {
        y[(size_t)i] /= h(i, i);
        for (int jj = i - 1; jj >= 0; --jj) { double p = h(jj, i) * y[(size_t)i]; y[(size_t)jj] -= p; }
    }
    for (int jj = 0; jj <= k; ++jj)
        for (size_t t = 0; t < n; ++t) { double p = v[(size_t)jj][t] * y[(size_t)jj]; x[t] += p; }
}

// GMRES (1D/codes/gmres.hpp:92-200): x0 = x on entry, restart = max_iter,
// stop when |s(i+1)| / ||b|| < 10^-tol_pow. Returns 0 when converged.
template <class MV>
int gmres(MV &&matvec, size_t n, const double *bb, double *x, int max_iter, int tol_pow, int *iters, double *resid) {
    int m = max_iter;
    double gtol = std::pow(10, -1.0 * tol_pow);
    std::vector<double> H((size_t)(m + 1) * (size_t)m, 0.0);  // column-major (m+1) x m
    auto h = [&](int r, int c) -> double & { return H[(size_t)r + (size_t)c * (size_t)(m + 1)]; };
    Vec s((size_t)m + 1, 0.0), cs((size_t)m + 1, 0.0), sn((size_t)m + 1, 0.0);
    Vec b(bb, bb + n);
    double normb = nrm(b);
    Vec out(n);
    matvec(x, out.data());
    Vec r(n);
    for (size_t i = 0; i < n; ++i) r[i] = b[i] - out[i];
    double beta = nrm(r);
    if (normb == 0.0) normb = 1;
    *resid = beta / normb;
    if (*resid <= gtol) { *iters = 0; return 0; }
    std::vector<Vec> v((size_t)m + 1);
    int j = 1;
    while (j <= max_iter) {
        double ib = 1.0 / beta;
        v[0].resize(n);
        for (size_t i = 0; i < n; ++i) v[0][i] = r[i] * ib;
        s.assign((size_t)m + 1, 0.0);
        s[0] = beta;
        for (int i = 0; i < m && j <= max_iter; ++i, ++j) {
            Vec w(n);
            matvec(v[(size_t)i].data(), w.data());
            for (int k = 0; k <= i; ++k) {
                h(k, i) = dot(w, v[(size_t)k]);
                double hk = h(k, i);
                for (size_t t = 0; t < n; ++t) { double p = hk * v[(size_t)k][t]; w[t] -= p; }
            }
            h(i + 1, i) = nrm(w);
            double ih = 1.0 / h(i + 1, i);
            v[(size_t)i + 1].resize(n);
            for (size_t t = 0; t < n; ++t) v[(size_t)i + 1][t] = ih * w[t];
            for (int k = 0; k < i; ++k) app_rot(h(k, i), h(k + 1, i), cs[(size_t)k], sn[(size_t)k]);
            gen_rot(h(i, i), h(i + 1, i), cs[(size_t)i], sn[(size_t)i]);
            app_rot(h(i, i), h(i + 1, i), cs[(size_t)i], sn[(size_t)i]);
            app_rot(s[(size_t)i], s[(size_t)i + 1], cs[(size_t)i], sn[(size_t)i]);
            *resid = std::fabs(s[(size_t)i + 1]) / normb;
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
