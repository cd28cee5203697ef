// The drop-in path end to end: the reference's GMRES (restated in
// oracle/gmres_ref.hpp, 1D/codes/gmres.hpp:92-200) drives the GPU operator
// through the C++ adapter with the reference's member names
// (include/h2w_adapter.hpp: tree_initialisation, mat_vec_prod), as a
// reference driver would after swapping its operator class
// (2D/codes/main.cpp:19-34). Prints one line: "iters resid err N".
//
// usage: adapter_gmres <dim> <form> <n_param> <nLevels> <tol_pow> <choice> <gmres_tol_pow> <x_true file>
#include <Eigen/Dense>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gmres_ref.hpp"
#include "h2w_adapter.hpp"

int main(int argc, char **argv) {
    if (argc < 9) return 2;
    const int dim = atoi(argv[1]), form = atoi(argv[2]), n = atoi(argv[3]), nl = atoi(argv[4]);
    const int tol = atoi(argv[5]), choice = atoi(argv[6]), gtol = atoi(argv[7]);
    using Vec = Eigen::VectorXd;
    auto *p = new h2w_initialisation<Vec>(dim, form, n, nl, tol, choice);
    p->tree_initialisation();
    const int64_t N = p->N();
    std::vector<double> xt((size_t)N);
    FILE *f = fopen(argv[8], "rb");
    if (!f || fread(xt.data(), 8, (size_t)N, f) != (size_t)N) return 3;
    fclose(f);
    // right-hand side with the exact dense product on the GPU (getTruePoten)
    std::vector<double> b((size_t)N);
    if (h2w_dense_matvec(p->h, xt.data(), b.data(), 0, N, H2W_HOST) != H2W_OK) return 4;
    std::vector<double> x((size_t)N, 1.0);
    int iters = 0;
    double resid = 0.0;
    auto mv = [&](const double *in, double *out) {
        Vec charge((int)N), output;
        for (int64_t i = 0; i < N; ++i) charge(i) = in[i];
        p->mat_vec_prod(charge, output);
        for (int64_t i = 0; i < N; ++i) out[i] = output(i);
    };
    h2w_ref::gmres(mv, (size_t)N, b.data(), x.data(), 500, gtol, &iters, &resid);
    double e2 = 0.0, t2 = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        e2 += (x[(size_t)i] - xt[(size_t)i]) * (x[(size_t)i] - xt[(size_t)i]);
        t2 += xt[(size_t)i] * xt[(size_t)i];
    }
    printf("%d %.17g %.17g %lld\n", iters, resid, std::sqrt(e2 / t2), (long long)N);
    delete p;
    return 0;
}
