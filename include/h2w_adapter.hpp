/* h2w_adapter.hpp — header-only C++ adapter with the member names of the
 * reference's operator facade (class initialisation, 1D/codes/matvec.hpp:73-181,
 * 2D/codes/matvec.hpp:106-173, 3D/codes/matvec.hpp:6-180), so that the
 * reference's own iterative_solver::GMRES<T>(T*&, Vec&, Vec&) template
 * ({1D,2D,3D}/codes/gmres.hpp:92-200) drives the GB300 operator unchanged.
 *
 * Vec is any vector type with size(), data() and resize(n) over double
 * (Eigen::VectorXd in the reference). The compression form and dimension,
 * which the reference selects with -DUSE_* flags, are constructor arguments.
 */
#ifndef H2W_ADAPTER_HPP
#define H2W_ADAPTER_HPP
#include <cmath>
#include <stdexcept>
#include <string>

#include "h2w.h"

template <class Vec>
class h2w_initialisation {
public:
    /* n_param: N (1D), sqrt(N) (2D) or cbrt(N) (3D), as the reference's drivers take it;
     * the reference's unused semi-length L is fixed to 1. */
    h2w_initialisation(int dim, int form, int n_param, int nLevels, int TOL_POW, int Kernel_Choice, int device = 0)
        : dim_(dim), n_param_(n_param) {
        h2w_config c{};
        c.dim = dim;
        c.form = form;
        c.choice = Kernel_Choice;
        c.tol_pow = TOL_POW;
        c.nlevels = nLevels;
        c.rank_cap = 0;
        int64_t N = dim == 1 ? n_param : (dim == 2 ? (int64_t)n_param * n_param : (int64_t)n_param * n_param * n_param);
        c.kernel_n = N;
        c.diag_n = dim == 1 ? 2 * N : N; /* 1D drivers push the grid twice */
        c.device = device;
        check(h2w_create(&c, &h), "h2w_create");
        N_ = N;
    }
    ~h2w_initialisation() { h2w_destroy(h); }
    h2w_initialisation(const h2w_initialisation &) = delete;
    h2w_initialisation &operator=(const h2w_initialisation &) = delete;

    /* set_Uniform_Nodes + tree build + NCA compression on the GPU */
    void tree_initialisation() {
        check(h2w_gen_grid(h, n_param_), "h2w_gen_grid");
        check(h2w_build_tree(h), "h2w_build_tree");
        check(h2w_assemble(h, H2W_ASSEMBLE_NCA), "h2w_assemble");
    }

    /* output = A charge, both in original point order; output is resized to N */
    void mat_vec_prod(Vec &charge, Vec &output) {
        if ((int64_t)charge.size() != N_) throw std::invalid_argument("charge has the wrong length");
        output.resize(N_);
        check(h2w_matvec(h, charge.data(), output.data(), 1, H2W_PREC_FP64, H2W_HOST, nullptr), "h2w_matvec");
    }

    /* findMemory_n / findMemory_sn */
    double memory() {
        double e = 0;
        check(h2w_storage_entries(h, &e), "h2w_storage_entries");
        return e;
    }

    int64_t N() const { return N_; }
    h2w_handle *h = nullptr;

private:
    void check(int rc, const char *what) {
        if (rc != H2W_OK)
            throw std::runtime_error(std::string(what) + " failed: " + (h ? h2w_last_error(h) : "no handle"));
    }
    int dim_;
    int n_param_;
    int64_t N_ = 0;
};

#endif
