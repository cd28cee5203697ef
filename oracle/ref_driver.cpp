// Driver that runs the H2weak reference headers, unmodified, for one
// (dimension, form) pair and dumps everything the parity tests need.
//
// Test infrastructure only. Built by oracle/Makefile into oracle/_ref/ from
// the reference sources where they lie (one binary per dimension and form,
// because the reference's class names collide across dimensions). Compiled
// with -ffp-contract=off so that the scalar arithmetic of the reference is
// not contracted into fused multiply-adds on hosts whose baseline ISA has FMA.
//
// It follows the reference's own call sequences:
//   tree_initialisation   1D/codes/matvec.hpp:97-119 (nested), :142-161 (semi-nested)
//                         2D/codes/matvec.hpp:133-162, :185-210
//                         3D/codes/matvec.hpp:33-61,   :86-113
//   mat_vec_prod          1D/codes/matvec.hpp:121-138, :163-178; 2D :163-182, :212-233; 3D :63-83, :115-136
//   GMRES                 */codes/gmres.hpp:92-200
//   getTruePoten          1D/codes/HODLR1Dtree.hpp:590-604 (2D/3D alike)
//   findMemory_n/_sn      1D/codes/HODLR1Dtree.hpp:535-588, 2D/codes/HODLR2Dtree.hpp:1207-1305,
//                         3D/codes/HODLR3Dtree.hpp:2505-2628
//
// Complex builds (-DUSE_Helm, 3D Helmholtz, choice 2; -DUSE_Hankel, 2D Hankel,
// choice 10): every vector in and out is N interleaved (re, im) pairs of doubles.
//
// Usage: refXd_F <n_param> <nLevels> <leaf_param> <L> <tol_pow> <choice>
//                <in.bin> <out.bin> <gmres_maxiter> <gmres_tolpow>
// n_param is N (1D), sqrt(N) (2D) or cbrt(N) (3D); leaf_param is nmax (1D)
// or the per-axis leaf count (2D/3D), exactly as the reference main() takes
// them. in.bin: int64 npts (0 = the reference's uniform grid), npts*d
// doubles, int64 nvec, nvec*N doubles (matvec inputs), int64 do_gmres,
// N doubles (manufactured solution), int64 do_dense.
#include "gmres.hpp"
#include <cstdint>
#include <cstdio>
#include <chrono>

#ifndef H2W_DIM
#error "H2W_DIM must be 1, 2 or 3"
#endif

static FILE *g_out = nullptr;

static void put_rec(const char *name, int code, const void *data, int64_t count, size_t elem) {
    char nm[32];
    memset(nm, 0, sizeof(nm));
    strncpy(nm, name, 31);
    fwrite(nm, 1, 32, g_out);
    int32_t c = code;
    fwrite(&c, 4, 1, g_out);
    fwrite(&count, 8, 1, g_out);
    if (count) fwrite(data, elem, (size_t)count, g_out);
}
static void put_i32(const char *n, const std::vector<int32_t> &v) { put_rec(n, 1, v.data(), (int64_t)v.size(), 4); }
static void put_i64(const char *n, const std::vector<int64_t> &v) { put_rec(n, 2, v.data(), (int64_t)v.size(), 8); }
static void put_f64(const char *n, const std::vector<double> &v) { put_rec(n, 3, v.data(), (int64_t)v.size(), 8); }
static void put_f64p(const char *n, const double *p, int64_t c) { put_rec(n, 3, p, c, 8); }

struct CSR {
    std::vector<int64_t> ptr{0};
    std::vector<int32_t> val;
    void add(const std::vector<int> &v) {
        for (int x : v) val.push_back(x);
        ptr.push_back((int64_t)val.size());
    }
    void put(const std::string &name) {
        put_i64((name + ".ptr").c_str(), ptr);
        put_i32((name + ".val").c_str(), val);
    }
};

static std::vector<double> read_f64(FILE *f, int64_t n) {
    std::vector<double> v((size_t)n);
    if (n && fread(v.data(), 8, (size_t)n, f) != (size_t)n) { fprintf(stderr, "short read\n"); exit(2); }
    return v;
}
static int64_t read_i64(FILE *f) {
    int64_t x;
    if (fread(&x, 8, 1, f) != 1) { fprintf(stderr, "short read\n"); exit(2); }
    return x;
}

#if H2W_DIM == 1
using PtT = double;
static const int NCHILD = 2;
static const int NNB = 2;
#define NBOXES(K, j) ((K)->nNodesPerLevel[j])
#elif H2W_DIM == 2
using PtT = pts2D;
static const int NCHILD = 4;
static const int NNB = 4;
#define NBOXES(K, j) ((K)->nBoxesPerLevel[j])
#else
using PtT = pts3D;
static const int NCHILD = 8;
static const int NNB = 26;
#define NBOXES(K, j) ((K)->nBoxesPerLevel[j])
#endif

// Scalars on the wire: one double (real kernels) or an interleaved (re, im)
// pair (the complex builds: -DUSE_Helm, 3D/codes/headers.hpp:35-40; -DUSE_Hankel,
// 2D/codes/headers.hpp:34-40).
#if defined(USE_Helm) || defined(USE_Hankel)
static const int CW = 2;
static dtype scal_in(const double *p) { return dtype(p[0], p[1]); }
static void scal_out(std::vector<double> &o, const dtype &v) {
    o.push_back(v.real());
    o.push_back(v.imag());
}
#else
static const int CW = 1;
static dtype scal_in(const double *p) { return p[0]; }
static void scal_out(std::vector<double> &o, const dtype &v) { o.push_back(v); }
#endif
static void put_vec(const char *n, const Vec &v) {
    std::vector<double> o;
    for (long i = 0; i < v.size(); ++i) scal_out(o, v(i));
    put_f64(n, o);
}

static void pt_to_doubles(const PtT &p, double *o) {
#if H2W_DIM == 1
    o[0] = p;
#elif H2W_DIM == 2
    o[0] = p.x; o[1] = p.y;
#else
    o[0] = p.x; o[1] = p.y; o[2] = p.z;
#endif
}
static PtT doubles_to_pt(const double *o) {
    PtT p;
#if H2W_DIM == 1
    p = o[0];
#elif H2W_DIM == 2
    p.x = o[0]; p.y = o[1];
#else
    p.x = o[0]; p.y = o[1]; p.z = o[2];
#endif
    return p;
}

int main(int argc, char **argv) {
    if (argc < 11) { fprintf(stderr, "usage: see header\n"); return 2; }
    int n_param = atoi(argv[1]);
    int nLevels = atoi(argv[2]);
    int leaf_param = atoi(argv[3]);
    int Lh = atoi(argv[4]);
    int tol_pow = atoi(argv[5]);
    int choice = atoi(argv[6]);
    const char *in_path = argv[7];
    const char *out_path = argv[8];
    int gm_maxiter = atoi(argv[9]);
    int gm_tolpow = atoi(argv[10]);

    FILE *fi = fopen(in_path, "rb");
    if (!fi) { fprintf(stderr, "cannot open %s\n", in_path); return 2; }
    int64_t npts = read_i64(fi);
    std::vector<double> pts_in = read_f64(fi, npts * H2W_DIM);

    auto t0 = std::chrono::steady_clock::now();
    initialisation *p = new initialisation(n_param, nLevels, leaf_param, Lh, tol_pow, choice);
    if (npts == 0) {
        p->tree_initialisation();
    } else {
#if H2W_DIM == 1
        fprintf(stderr, "point injection is not supported in 1D\n");
        return 2;
#else
        // Same sequence as tree_initialisation, with the grid replaced by the
        // caller's points (the tree constructors fix N = n^d, so N is reset).
        userkernel *mykernel = new userkernel(p->particles, choice);
#if H2W_DIM == 2
        p->K = new HODLR2DTree<userkernel>(mykernel, n_param, nLevels, leaf_param, Lh, tol_pow);
#else
        p->K = new HODLR3DTree<userkernel>(mykernel, n_param, nLevels, leaf_param, Lh, tol_pow);
#endif
        p->particles.clear();
        for (int64_t i = 0; i < npts; ++i) p->particles.push_back(doubles_to_pt(&pts_in[(size_t)(i * H2W_DIM)]));
        p->K->N = (int)npts;
        p->K->K = new userkernel(p->particles, choice);
        auto *K = p->K;
        K->createTree();
#if H2W_DIM == 2
        K->assign_all_interaction();
        K->assign_center_location();
#else
        K->assign_Tree_Interactions();
        K->assign_Center_Location();
#endif
        K->separate_vertex_interaction();
        K->assignChargeLocations();
        K->assignNonLeafChargeLocations();
#ifdef USE_nHODLRdD
        K->getNodes();
        K->getNodes_ver();
        K->assemble_M2L_far();
        K->assemble_M2L_ver();
        K->assemble_M2M_ver();
        K->assemble_NearField();
#elif defined(USE_HODLRdD)
        K->getUVtTree_nn();
        K->assembleAcAr_nn();
        K->assemble_NearField();
#else
        K->getNodes();
        K->assemble_M2L_far();
        K->assemble_NearField();
        K->getUVtTree_sn();
        K->assembleAcAr_sn();
#endif
#endif
    }
    auto t1 = std::chrono::steady_clock::now();
    auto *K = p->K;
    const int N = K->N;
    const int nL = K->nLevels;

    int64_t nvec = read_i64(fi);
    std::vector<double> vecs = read_f64(fi, nvec * N * CW);
    int64_t do_gmres = read_i64(fi);
    std::vector<double> xtrue;
    if (do_gmres) xtrue = read_f64(fi, (int64_t)N * CW);
    int64_t do_dense = read_i64(fi);
    fclose(fi);

    g_out = fopen(out_path, "wb");
    if (!g_out) { fprintf(stderr, "cannot open %s\n", out_path); return 2; }
    put_i64("meta", {H2W_DIM, N, nL, tol_pow, choice,
#if defined(USE_nHODLRdD)
                     0
#elif defined(USE_HODLRdD)
                     2
#else
                     1
#endif
                    });
    std::vector<double> pts((size_t)N * H2W_DIM);
    for (int i = 0; i < N; ++i) pt_to_doubles(K->K->particles[(size_t)i], &pts[(size_t)i * H2W_DIM]);
    put_f64("points", pts);

    // Per (level, box) lists, levels 0..nL, boxes in numbering order.
    CSR charge, nbr, il, isv, chk, chg, chkv, chgv, rowb, colb;
    for (int j = 0; j <= nL; ++j) {
        for (int k = 0; k < NBOXES(K, j); ++k) {
            auto *b = K->tree[(size_t)j][(size_t)k];
            charge.add(b->chargeLocations);
            std::vector<int> nb(b->neighborNumbers, b->neighborNumbers + NNB);
            nbr.add(nb);
#if H2W_DIM == 1
            il.add({});
            isv.add({});
            chk.add(b->incoming_checkPoints);
            chg.add(b->incoming_chargePoints);
            chkv.add({});
            chgv.add({});
#else
            il.add(b->interactionList);
            std::vector<int> fl;
            for (int q : b->interactionList) fl.push_back(b->isVertex.count(q) ? (int)b->isVertex[q] : -1);
            isv.add(fl);
            chk.add(b->incoming_checkPoints);
            chg.add(b->incoming_chargePoints);
            chkv.add(b->incoming_checkPoints_ver);
            chgv.add(b->incoming_chargePoints_ver);
            for (size_t i = 0; i < b->interactionList.size(); ++i) {
#if defined(USE_snHODLRdD) || defined(USE_HODLRdD)
                rowb.add(b->row_basis[i]);
                colb.add(b->col_basis[i]);
#else
                rowb.add({});
                colb.add({});
#endif
            }
#endif
        }
    }
    charge.put("charge");
    nbr.put("nbr");
    il.put("il");
    isv.put("isvertex");
    chk.put("far_check");
    chg.put("far_charge");
    chkv.put("ver_check");
    chgv.put("ver_charge");
    rowb.put("sn_row");
    colb.put("sn_col");
#if H2W_DIM == 1 && defined(USE_snHODLRdD)
    // 1D semi-nested: per (level, box, sibling slot) ranks of U V^T.
    std::vector<int32_t> uvr;
    for (int j = 1; j <= nL; ++j)
        for (int k = 0; k < NBOXES(K, j); ++k)
            for (int nn = 0; nn < 2; ++nn) {
                int q = K->tree[(size_t)j][(size_t)k]->neighborNumbers[nn];
                uvr.push_back(q == -1 ? -1 : (int)K->tree[(size_t)j][(size_t)k]->U[q].cols());
            }
    put_i32("uv_rank", uvr);
#endif

#if defined(USE_nHODLRdD)
    K->findMemory_n();
#elif defined(USE_HODLRdD)
    K->findMemory_nn();
#else
    K->findMemory_sn();
#endif
    put_f64("memory", {K->memory});

    auto t2 = std::chrono::steady_clock::now();
    std::vector<double> ys;
    for (int64_t v = 0; v < nvec; ++v) {
        Vec x(N), y;
        for (int i = 0; i < N; ++i) x(i) = scal_in(&vecs[(size_t)((v * N + i) * CW)]);
        p->mat_vec_prod(x, y);
        for (int i = 0; i < N; ++i) scal_out(ys, y(i));
    }
    auto t3 = std::chrono::steady_clock::now();
    put_f64("matvec", ys);

    if (do_dense && nvec > 0) {
        Vec x(N);
        for (int i = 0; i < N; ++i) x(i) = scal_in(&vecs[(size_t)i * CW]);
        Vec yd = K->getTruePoten(x);
        put_vec("dense_matvec", yd);
    }
    double t_gmres = 0.0;
    if (do_gmres) {
        Vec b(N);
        for (int i = 0; i < N; ++i) b(i) = scal_in(&xtrue[(size_t)i * CW]);
        Vec rhs = K->getTruePoten(b);
        Vec x = Vec::Ones(N);
        auto g0 = std::chrono::steady_clock::now();
        iterative_solver *its = new iterative_solver(gm_maxiter, gm_tolpow);
        its->GMRES<initialisation>(p, x, rhs);
        auto g1 = std::chrono::steady_clock::now();
        t_gmres = std::chrono::duration<double>(g1 - g0).count();
        put_vec("gmres_rhs", rhs);
        put_vec("gmres_x", x);
        put_f64("gmres_stats", {(double)its->max_iter, its->resid, (x - b).norm() / b.norm()});
    }
    put_f64("timing", {std::chrono::duration<double>(t1 - t0).count(),
                       nvec ? std::chrono::duration<double>(t3 - t2).count() / (double)nvec : 0.0, t_gmres,
                       (double)omp_get_max_threads()});
    fclose(g_out);
    printf("N=%d nLevels=%d memory=%.0f storageGB=%g ratio=%g assembly_s=%g\n", N, nL, K->memory,
           K->memory * 8 * pow(10.0, -9), K->memory / (1.0 * N * N), std::chrono::duration<double>(t1 - t0).count());
    return 0;
}
