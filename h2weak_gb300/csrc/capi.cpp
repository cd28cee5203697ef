#include <type_traits>
// C ABI of the GB300 H2* / (H2+H)* library: handle, tree, GPU assembly,
// packed-operator plan, matvec launches and device-resident GMRES.
#include <algorithm>
#include <chrono>
#include <atomic>
#include <climits>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "bessel.cuh"
#include "h2w_internal.h"
#include "kernels.cuh"

using namespace h2w;

namespace {

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string &s) : std::runtime_error(s) {}
};
struct ApiError : std::runtime_error {
    int code;
    ApiError(int c, const std::string &s) : std::runtime_error(s), code(c) {}
};

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));                    \
    } while (0)

// Bumped by every device (re)allocation: a captured graph holds raw device
// pointers and is rebuilt when the generation moved.
std::atomic<uint64_t> g_alloc_gen{0};

template <class T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() {}
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { reset(); }
    void reset() {
        if (p) {
            cudaFree(p);
            g_alloc_gen.fetch_add(1);
        }
        p = nullptr;
        n = 0;
    }
    void alloc(size_t cnt) {
        reset();
        if (cnt == 0) cnt = 1;
        g_alloc_gen.fetch_add(1);
        cudaError_t e = cudaMalloc(&p, cnt * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw ApiError(H2W_ERR_NOMEM, "cudaMalloc of " + std::to_string(cnt * sizeof(T)) + " bytes failed");
        }
        n = cnt;
    }
    void upload(const std::vector<T> &v, cudaStream_t st = 0) {
        alloc(v.size());
        if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    }
};

// Device state of the lockstep GMRES for one Krylov-vector type T
template <class T> struct GmbStore {
    DBuf<T> V, w, vcur;
    DBuf<double> H, cs, sn, s, part, hsum, normb, resid, y, z, tol;
    DBuf<int32_t> conv, iter;
    int m = -1, rp = 0;
    int jres = -1;  // the last solve from x0 = 0: largest Arnoldi index + 1 (its residual is V z), else -1
};

inline int64_t pad4(int64_t x) { return (x + 3) & ~int64_t(3); }

constexpr int XW_CAP = 4096;          // gathered source width per target (elements)
constexpr int64_t ROW_SPLIT = 16384;  // rows * width above which a target is split (load balance)
constexpr int64_t MR_ROWS = 64;      // rows per target of the multi-vector stream (its result tile)
constexpr int64_t MR_XW_DEFAULT = 1024;  // gathered columns per multi-vector target before a column split

}  // namespace

namespace {
struct PlanBuilder;
}

struct h2w_handle {
    h2w_config cfg{};
    std::string err;
    std::vector<double> pts;
    Tree tree;
    bool has_tree = false, has_op = false;
    // skeletons: far[j] (2D/3D, j>=2), ver[j] (nested 2D/3D and 1D nested, j>=1), pairs[j]
    std::vector<Skel> far, ver;
    std::vector<Pairs> pairs;
    bool imp[10] = {false};
    std::vector<std::vector<int64_t>> imp_ptr;
    std::vector<std::vector<int32_t>> imp_val;
    // kernel parameters
    double diag = 0, c2d = 0, four_pi = 0, loga = 0, den_small = 0, kii = 0;
    // complex kernel (choice H2W_KERNEL_HELMHOLTZ): complex entries, the operator
    // stored realified (every complex block as [[Re, -Im], [Im, Re]] with rows and
    // columns interleaved), vectors as interleaved (re, im) doubles
    bool cplx = false;
    bool cgm_hermitian = false;  // H2W_OPT_COMPLEX_ARNOLDI
    double diag_im = 0;
    DBuf<double2> c_V, c_w, c_r, c_ax, c_part, c_h, c_y;  // complex GMRES state
    int64_t nv() const { return cplx ? 2 * tree.N : tree.N; }  // doubles per vector
    // device state
    DBuf<double> d_pts;
    DBuf<int32_t> d_perm;
    DBuf<double> d_op;
    DBuf<float> d_op32;
    DBuf<int64_t> d_roff, d_blob;  // packed target records of the matvec
    DBuf<int64_t> d_roff_m, d_blob_m, d_pstart_m;  // the multi-vector stream (64-row targets)
    // the warp-specialised FP32 product's operator copy: every (target, panel)
    // slice contiguous at its padded height, records pointing into it, and the
    // slices to copy (6 words each: source offset, lda, rows, width, offset, lda)
    DBuf<float> d_op32m;
    DBuf<int64_t> d_blob_mw, d_mslices;
    int64_t op32m_n = 0;
    // the same for the single-vector stream's FP32 products: each (target, panel)
    // slice of the FP32 operator contiguous at its padded height, so that a row
    // chunk of a block streams whole sectors (made on the first FP32 product)
    DBuf<float> d_op32s;
    DBuf<int64_t> d_blob_s, d_sslices;
    int64_t op32s_n = 0;
    bool op32s_ready = false;
    bool op32m_ready = false;
    DBuf<int32_t> d_mctr;                           // its per-phase target counters
    std::vector<Phase> mphases;
    DBuf<double> d_ws, d_x, d_y;
    DBuf<int32_t> d_ctr, d_err;
    DBuf<int64_t> d_pstart;
    DBuf<unsigned> d_bar;
    bool coop = true;  // one cooperative launch per matvec (else one launch per phase)
    int64_t spin_limit = 0;  // polls per grid-barrier wait of the single-vector cooperative launch (0: built-in)
    bool nca_df = true;      // group NCA of log kernels in double-FP32 arithmetic (H2W_OPT_NCA_DF)
    // far-field M2L evaluated during each single-vector product instead of stored
    // (H2W_OPT_FAR_ON_THE_FLY, applies at assembly): work items, row / column
    // point ids, source workspace rows, claim counter, FP32 coordinates, and the
    // phase at which the product's stored stream is split around the kernel
    bool far_fly = false, fly_active = false;
    DBuf<FlyItem> d_fly_items;
    DBuf<int32_t> d_fly_rowpid, d_fly_cpid, d_fly_cws;
    DBuf<unsigned long long> d_fly_ctr;
    DBuf<float> d_pts4;
    DBuf<float> d_ptsdf, d_logtab;  // (hi, lo) points and the log table of the double-FP32 form
    DBuf<float> d_nca_logtab;       // the log table of the double-FP32 pivot search
    int fly_split = 0;
    int64_t fly_entries = 0;  // kernel entries one product evaluates
    std::vector<std::pair<int64_t, int64_t>> fly_rows;  // workspace rows the kernel writes
    FlyK32 k32{};
    DBuf<float> d_ws32;
    std::vector<Phase> phases;
    std::vector<int64_t> ph_op, ph_vec;   // per phase: operator and vector elements moved
    // launch profiling of the block-row GEMV (events bracket every phase launch)
    bool prof = false;
    struct ProfRec { cudaEvent_t a, b; int prec, phase; int rp = 1; };  // prec + 2: multi-vector launch
    std::vector<ProfRec> prof_recs;
    std::vector<cudaEvent_t> ev_pool;
    bool fused_scatter = true, fused_scatter_m = true;  // per target stream
    std::shared_ptr<PlanBuilder> plan;                  // logical targets (re-cut by the autotuner)
    int nph_total = 0;
    int64_t mr_xw = MR_XW_DEFAULT;                      // column cap of the multi-vector stream
    int64_t row_split = ROW_SPLIT;                      // row split of the single-vector stream
    int64_t ws_n = 0, yperm_off = 0, op_n = 0;
    double storage = 0;
    int64_t op_bytes_read = 0;  // elements of operator data one matvec reads
    // GMRES state
    DBuf<double> g_V, g_w, g_vcur, g_H, g_cs, g_sn, g_s, g_part, g_scal, g_tmp, g_b, g_r, g_npart;
    DBuf<int32_t> g_iter;
    int g_m = -1;
    DBuf<double> s_b, s_x, s_r, s_d;   // solver vectors in leaf order (kept between calls)
    // multiple right-hand sides: interleaved workspaces (ws_n x rp), staging, batched GMRES
    DBuf<double> m_wsd, m_xi, m_yi, m_ri, m_di, m_bi, m_stage_x, m_stage_y, m_onorm, m_ores;
    DBuf<float> m_wsf, m_xf;
    DBuf<double> d_opdf, m_xdf;  // (hi, lo) FP32 pairs (8 bytes each) of the operator and of an input block
    std::vector<int64_t> ph_t0, ph_t1;   // phase target ranges (per-phase launches)
    GmbStore<double> gbd;  // FP64 Krylov vectors (FP64 solves)
    GmbStore<float> gbf;   // FP32 Krylov vectors (inner solves of the refinement, H2W_OPT_F32_BASIS)
    bool f32_basis = true;
    // dataflow launch of the multi-vector stream (H2W_OPT_DATAFLOW): producer counts
    // (initial and working copy) and consumer lists
    bool dataflow = true;
    bool producer_warp = true;  // the FP32 dataflow product's warp-specialised form (H2W_OPT_PRODUCER_WARP)
    DBuf<int32_t> d_mdep0, d_mdep, d_mcidx;
    DBuf<int64_t> d_mcoff;
    DBuf<int32_t> d_sdep0, d_sdep, d_scidx, d_sctr;  // the same for the single-vector stream
    DBuf<int64_t> d_scoff;
    int64_t mflow_edges = 0;
    // multi-vector plan: targets, panels, operator entries per column, entries
    // the kernel multiplies (rows to warp granularity, each panel's columns to
    // chunks), atomically accumulated targets, entries spanned by the row tiles
    int64_t mstats[6] = {0, 0, 0, 0, 0, 0};
    // graph-captured Arnoldi loops (a while node whose body is one step)
    struct LoopGraph {
        int kind, prec, m, rp, nrhs;
        uint64_t gen;
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        int64_t kernels_per_step;
    };
    std::vector<LoopGraph> loops;
    bool use_graphs = true, graph_failed = false;
    int ir_resid_prec = H2W_PREC_FP64;   // refinement residuals after the first (batched IR)
    // refinement residual updating r <- r - A32 d (H2W_OPT_IR_UPDATE) and the calibrated
    // error of the FP32 products per unit input norm (< 0: not measured for this operator)
    bool ir_update = true;
    bool tensor = false;  // FP32 multi-vector products on the tensor cores (H2W_OPT_TENSOR)
    double eta_multi = -1.0, eta_single = -1.0;
    DBuf<double> m_ti, m_dn, s_t;
    // learned NCA proposals: model, assembly switch, training-data recorder, statistics
    DBuf<float> d_mlp;
    float mlp_calib = 1.f;
    int mlp_margin = 2;
    bool learned = false, learn_rec = false;
    std::vector<float> rec_X;
    std::vector<uint8_t> rec_y;
    int64_t learn_blocks = 0, learn_accepted = 0;
    int64_t learn_reject[3] = {0, 0, 0};  // no usable pivots, non-finite, stopping test failed
    double learn_rhat = 0.0, learn_r1 = 0.0;
    double learn_ms = 0.0;
    cudaStream_t stream = nullptr;

    KParams kparams() const {
        KParams k;
        k.pts = d_pts.p;
        k.dim = cfg.dim;
        k.choice = cfg.choice;
        k.diag = diag;
        k.c2d = c2d;
        k.four_pi = four_pi;
        k.loga = loga;
        k.den_small = den_small;
        k.diag_im = diag_im;
        return k;
    }
};

namespace {

// ------------------------------------------------------ kernel set-up ---
// Gauss-Legendre 16-point self term, as the reference integrates it
// (1D/codes/integral1d.hpp:17-39, 2D/codes/integral2d.hpp:60-90,
// 3D/codes/integral3d.hpp:13-50); nodes by Newton iteration on the Legendre
// recurrence, ordered by |x| with the negative node first.
void gl16(std::vector<double> &x, std::vector<double> &w) {
    const int n = 16;
    std::vector<std::pair<long double, long double>> pr;
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int i = 1; i <= n; ++i) {
        long double z = cosl(pi * (i - 0.25L) / (n + 0.5L)), pp = 0;
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
        pr.push_back({z, 2.0L / ((1.0L - z * z) * pp * pp)});
    }
    std::sort(pr.begin(), pr.end(), [](auto &a, auto &b) {
        long double fa = fabsl(a.first), fb = fabsl(b.first);
        return fa != fb ? fa < fb : a.first < b.first;
    });
    x.clear();
    w.clear();
    for (auto &p : pr) {
        x.push_back((double)p.first);
        w.push_back((double)p.second);
    }
}

void setup_kernel(h2w_handle *h) {
    const double PI = 4.0 * std::atan(1.0);
    const int dim = h->cfg.dim;
    const int64_t N = h->tree.N;
    const int64_t kn = h->cfg.kernel_n > 0 ? h->cfg.kernel_n : N;
    const int64_t dn = h->cfg.diag_n > 0 ? h->cfg.diag_n : N;
    h->c2d = (-1.0 / (2 * PI)) * 0.5;
    h->four_pi = 4.0 * PI;
    const double a = 0.0001;
    h->loga = std::log(a);
    h->den_small = a * std::log(a) - 1.0;
    if (h->cfg.choice == 0) {
        double hh = dim == 1 ? 1.0 / double(kn) : (dim == 2 ? 1.0 / std::sqrt(double(kn)) : 1.0 / std::cbrt(double(kn)));
        std::vector<double> x, w;
        gl16(x, w);
        double lo = 0.0, hi = hh * 0.5, cx = 0.5 * (hi - lo), Lx = 0.5 * (hi + lo), res = 0.0, hd;
        if (dim == 1) {
            for (int i = 0; i < 16; ++i) res += w[i] * std::log(std::fabs(1.0 * (cx * x[i] + Lx)));
            res *= cx;
            res *= 2;
            hd = hh;
        } else if (dim == 2) {
            const double c = -1.0 / (2 * PI);
            for (int i = 0; i < 16; ++i) {
                double tx = cx * x[i] + Lx;
                for (int j = 0; j < 16; ++j) {
                    double ty = cx * x[j] + Lx;
                    res += w[i] * w[j] * (c * 0.5 * std::log(tx * tx + ty * ty));
                }
            }
            res *= (cx * cx);
            res *= 4;
            hd = std::pow(hh, 2.0);
        } else {
            for (int i = 0; i < 16; ++i) {
                double tx = cx * x[i] + Lx;
                for (int j = 0; j < 16; ++j) {
                    double ty = cx * x[j] + Lx;
                    for (int k = 0; k < 16; ++k) {
                        double tz = cx * x[k] + Lx;
                        res += (w[i] * w[j] * w[k] * (1.0 / ((4 * PI) * std::sqrt(tx * tx + ty * ty + tz * tz))));
                    }
                }
            }
            res *= (cx * cx * cx);
            res *= 8;
            hd = std::pow(hh, 3.0);
        }
        h->kii = res;
        h->diag = (1.0 + res) / hd;
    } else if (h->cfg.choice == H2W_KERNEL_HELMHOLTZ && dim == 3) {
        // Helmholtz3D diagonal, 3D/codes/kernel.hpp:140-141
        h->diag = 500 * std::sqrt(double(dn));
        h->diag_im = 0.0;
    } else if (h->cfg.choice == H2W_KERNEL_HANKEL) {
        // IE_2D_Helm diagonal (1 + 15 ln N + Kii) / h^2 (2D/codes/kernel.hpp:128-132); Kii the
        // 16 x 16 Gauss-Legendre integral of i H0^(1)(R) / 4 over [0, h/2]^2, times 4
        // (the userkernel constructor, 2D/codes/kernel.hpp:101-114; double_integral,
        // 2D/codes/integral2d.hpp:59-90)
        const double hh = 1.0 / std::sqrt(double(kn));
        std::vector<double> x, w;
        gl16(x, w);
        const double lo = 0.0, hi = hh * 0.5, cx = 0.5 * (hi - lo), Lx = 0.5 * (hi + lo);
        std::complex<double> res = 0.0;
        for (int i = 0; i < 16; ++i) {
            const double tx = cx * x[i] + Lx;
            for (int j = 0; j < 16; ++j) {
                const double ty = cx * x[j] + Lx;
                double j0, y0;
                bessel::j0y0(std::sqrt(tx * tx + ty * ty), j0, y0);
                const std::complex<double> f(-y0 / 4.0, j0 / 4.0);
                res += w[i] * w[j] * f;
            }
        }
        res *= (cx * cx);
        res *= 4;
        const double h2 = std::pow(hh, 2.0);
        const std::complex<double> d = (1.0 + 15 * std::log(double(dn)) + res) / h2;
        h->kii = res.real();
        h->diag = d.real();
        h->diag_im = d.imag();
    } else {
        h->diag = dim == 2 ? 1.0 : std::sqrt((double)dn);
    }
}

// ------------------------------------------------------------- helpers ---
std::vector<int32_t> box_pts(const Tree &t, int j, int64_t k) {
    return std::vector<int32_t>(t.perm.begin() + t.off[j][k], t.perm.begin() + t.off[j][k + 1]);
}
void append(std::vector<int32_t> &a, const int32_t *b, int64_t n) { a.insert(a.end(), b, b + n); }

// ------------------------------------------------------------ NCA runs ---
// Run the batched NCA on problems (R[p], C[p]); returns local pivots.
void record_blocks(h2w_handle *h, const std::vector<NcaProb> &probs, const DBuf<int32_t> &di,
                   const std::vector<std::vector<int32_t>> &prow, const std::vector<std::vector<int32_t>> &pcol,
                   size_t p0);
void record_lists(h2w_handle *h, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
                  const std::vector<std::vector<int32_t>> &prow, const std::vector<std::vector<int32_t>> &pcol);
void run_nca_small(h2w_handle *h, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
                   std::vector<std::vector<int32_t>> &prow, std::vector<std::vector<int32_t>> &pcol,
                   std::vector<size_t> &over);

constexpr int64_t NCA_BIG = 8192;  // rows + columns from which a block gets a group of CTAs
constexpr int64_t NCA_MED = 2048;  // ... and from which it does when one CTA per block would leave SMs idle
constexpr int NCA_SMALL_CAP = 512;   // pivots one CTA per block holds; larger blocks move to the groups

// Scratch bytes a batch of NCA blocks may take: most of the free device
// memory (nothing else of the operator is resident while pivots are searched).
size_t nca_budget() {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return (size_t)8 << 30;
    }
    const size_t keep = (size_t)4 << 30;
    return fr > keep + ((size_t)2 << 30) ? (fr - keep) * 3 / 4 : (size_t)1 << 30;
}

// Large blocks: groups of CTAs of one cooperative launch per block
// (ncabig.cu), in batches within the scratch budget. There is no built-in
// rank limit (the reference's loop bound is min(rows, columns),
// 1D/codes/aca.hpp:363): each block starts with scratch for `start` pivots
// (at most min(rows, columns)), and a block that fills it runs again with
// twice as much until it fits; only an explicit rank_cap stops it
// (H2W_ERR_RANK).
void run_nca_big(h2w_handle *h, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
                 const std::vector<size_t> &big, std::vector<std::vector<int32_t>> &prow,
                 std::vector<std::vector<int32_t>> &pcol, int start = 1024) {
    const double tol = std::pow(10, -1.0 * h->cfg.tol_pow);
    const int cap = h->cfg.rank_cap > 0 ? h->cfg.rank_cap : INT32_MAX;
    KParams kp = h->kparams();
    cudaStream_t st = h->stream;
    std::vector<std::pair<size_t, int>> pend;  // (problem, scratch pivots)
    for (size_t p : big) {
        const int mn = (int)std::min(R[p].size(), C[p].size());
        pend.push_back({p, std::min(std::min(mn, cap), std::max(start, 1))});
    }
    while (!pend.empty()) {
        const size_t budget = nca_budget();
        std::vector<std::pair<size_t, int>> again;
        size_t q0 = 0;
        while (q0 < pend.size()) {
            std::vector<NcaProb> probs;
            std::vector<int64_t> moff;
            std::vector<int32_t> idx;
            size_t scr = 0;
            int64_t piv = 0, mw = 0;
            int dcap = 1;
            size_t q = q0;
            for (; q < pend.size(); ++q) {
                const size_t p = pend[q].first;
                const int n1 = (int)R[p].size(), n2 = (int)C[p].size();
                const int rc = pend[q].second;
                const size_t need = (size_t)rc * (size_t)(n1 + n2);
                if (!probs.empty() && (scr + need) * 8 > budget) break;
                NcaProb pb{};
                pb.ri = (int64_t)idx.size();
                append(idx, R[p].data(), n1);
                pb.ci = (int64_t)idx.size();
                append(idx, C[p].data(), n2);
                pb.u = (int64_t)scr;
                pb.v = (int64_t)(scr + (size_t)rc * n1);
                scr += need;
                pb.piv = piv;
                piv += rc;
                pb.n1 = n1;
                pb.n2 = n2;
                pb.rcap = rc;
                probs.push_back(pb);
                moff.push_back(mw);
                mw += (n1 + 31) / 32 + (n2 + 31) / 32;
                dcap = std::max(dcap, rc);
            }
            // kernels built on log: residuals in double-FP32 arithmetic on the FP32 pipes
            const bool df = h->nca_df && ((h->cfg.dim < 3 && h->cfg.choice == 0) || (h->cfg.dim == 3 && h->cfg.choice == 1));
            const int grid = nca_group_grid(dcap, df);
            if (df && !h->d_nca_logtab.p) {  // the pair logarithm's table
                std::vector<float> lt(128 * 8);
                fly_df_logtab(lt.data());
                h->d_nca_logtab.upload(lt, st);
            }
            if (grid <= 0) throw ApiError(H2W_ERR_CUDA, "NCA group kernel: no co-resident grid");
            const int nb = (int)probs.size();
            // groups sized to the widest block (about four residual entries per
            // thread and pass, at least two CTAs, at most 32), as many groups
            // as blocks while the grid allows
            int64_t wmax = 0;
            for (const NcaProb &pb : probs) wmax = std::max<int64_t>(wmax, (int64_t)pb.n1 + pb.n2);
            const int smin = (int)std::min<int64_t>(32, std::max<int64_t>(2, (wmax + 2047) / 2048));
            const int G = std::max(1, std::min(nb, grid / smin));
            DBuf<NcaProb> dp;
            DBuf<int64_t> dm;
            DBuf<int32_t> di, drank, dpr, dpc, dst, derr;
            DBuf<uint32_t> dmask;
            DBuf<unsigned> dbar;
            DBuf<double> dscr, ddots;
            DBuf<char> dpartr, dpartc;
            dp.upload(probs, st);
            dm.upload(moff, st);
            di.upload(idx, st);
            dscr.alloc(scr);
            dmask.alloc((size_t)mw);
            drank.alloc((size_t)nb);
            dpr.alloc((size_t)piv);
            dpc.alloc((size_t)piv);
            dst.alloc(1);
            derr.alloc(1);
            dbar.alloc((size_t)2 * G);
            dpartr.alloc(nca_group_part_bytes() * (size_t)grid);
            dpartc.alloc(nca_group_part_bytes() * (size_t)grid);
            ddots.alloc((size_t)grid * 2 * dcap + (size_t)G * dcap);
            CK(cudaMemsetAsync(dst.p, 0, 4, st));
            CK(cudaMemsetAsync(derr.p, 0, 4, st));
            CK(cudaMemsetAsync(dbar.p, 0, (size_t)2 * G * sizeof(unsigned), st));
            CK(launch_nca_group(dp.p, dm.p, nb, G, grid, di.p, kp, tol, dscr.p, dmask.p, drank.p, dpr.p, dpc.p, dst.p,
                                dbar.p, derr.p, dpartr.p, dpartc.p, ddots.p, dcap, df, df ? h->d_nca_logtab.p : nullptr,
                                st));
            std::vector<int32_t> rk((size_t)nb), hpr((size_t)piv), hpc((size_t)piv);
            int32_t status = 0, errf = 0;
            CK(cudaMemcpyAsync(rk.data(), drank.p, rk.size() * 4, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(hpr.data(), dpr.p, hpr.size() * 4, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(hpc.data(), dpc.p, hpc.size() * 4, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(&status, dst.p, 4, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(&errf, derr.p, 4, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (errf) throw ApiError(H2W_ERR_CUDA, "NCA group kernel: a group-barrier wait ran out");
            if (status & 2) throw ApiError(H2W_ERR_ARG, "non-finite kernel entries (coincident points?) in an NCA block");
            for (int k = 0; k < nb; ++k) {
                const auto &pq = pend[q0 + (size_t)k];
                const size_t p = pq.first;
                if (rk[(size_t)k] < 0) {  // scratch full: again with twice the pivots
                    const int mn = (int)std::min(R[p].size(), C[p].size());
                    const int lim = std::min(mn, cap);
                    if (pq.second >= lim)
                        throw ApiError(H2W_ERR_RANK, "an NCA block needed more than rank_cap = " +
                                                         std::to_string(h->cfg.rank_cap) + " pivots");
                    again.push_back({p, (int)std::min<int64_t>((int64_t)pq.second * 2, lim)});
                    continue;
                }
                prow[p].assign(hpr.begin() + probs[(size_t)k].piv, hpr.begin() + probs[(size_t)k].piv + rk[(size_t)k]);
                pcol[p].assign(hpc.begin() + probs[(size_t)k].piv, hpc.begin() + probs[(size_t)k].piv + rk[(size_t)k]);
            }
            q0 = q;
        }
        pend.swap(again);
    }
}

// The NCA pivot search: one CTA per block (nca_kernel) in batches that fit
// the scratch budget; blocks of NCA_BIG or more rows + columns, and blocks
// whose rank outgrows one CTA's scratch, get groups of CTAs (run_nca_big).
// Blocks of NCA_MED or more rows + columns get groups too when there are no
// more of them than SMs (one CTA each would leave SMs idle), and always for
// the kernels whose group search runs in double-FP32 arithmetic.
// H2W_NCA_BIG=0 keeps every block that fits on one CTA.
void run_nca_plain(h2w_handle *h, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
                   std::vector<std::vector<int32_t>> &prow, std::vector<std::vector<int32_t>> &pcol) {
    prow.assign(R.size(), {});
    pcol.assign(R.size(), {});
    std::vector<size_t> big, med, small;
    const char *eb = getenv("H2W_NCA_BIG");
    const bool use_big = !(eb && std::string(eb) == "0");
    for (size_t p = 0; p < R.size(); ++p) {
        const int64_t w = (int64_t)(R[p].size() + C[p].size());
        (use_big && w >= NCA_BIG ? big : use_big && w >= NCA_MED ? med : small).push_back(p);
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, std::max(0, h->cfg.device)) != cudaSuccess) {
        cudaGetLastError();
        sms = 0;
    }
    // kernels built on log search in double-FP32 arithmetic on the groups,
    // faster than one CTA's FP64 whatever the count
    const bool df = h->nca_df && ((h->cfg.dim < 3 && h->cfg.choice == 0) || (h->cfg.dim == 3 && h->cfg.choice == 1));
    if (!df && (int64_t)med.size() > (int64_t)sms) small.insert(small.end(), med.begin(), med.end()), med.clear();
    std::sort(small.begin(), small.end());
    // H2W_TIMING=1: the time of each part of the search on stderr (diagnostic)
    static const bool timing = getenv("H2W_TIMING") && std::string(getenv("H2W_TIMING")) == "1";
    auto now = [] { return std::chrono::steady_clock::now(); };
    auto t0 = now();
    if (!big.empty()) run_nca_big(h, R, C, big, prow, pcol);
    auto tm = now();
    if (!med.empty()) run_nca_big(h, R, C, med, prow, pcol, NCA_SMALL_CAP);
    auto t1 = now();
    std::vector<size_t> over;
    if (!small.empty()) {
        std::vector<std::vector<int32_t>> Rs, Cs, prs, pcs;
        const bool all_small = small.size() == R.size();
        if (!all_small)
            for (size_t p : small) {
                Rs.push_back(R[p]);
                Cs.push_back(C[p]);
            }
        const std::vector<std::vector<int32_t>> &RR = all_small ? R : Rs, &CC = all_small ? C : Cs;
        std::vector<std::vector<int32_t>> &PR = all_small ? prow : prs, &PC = all_small ? pcol : pcs;
        std::vector<size_t> ov;
        run_nca_small(h, RR, CC, PR, PC, ov);
        for (size_t k : ov) over.push_back(all_small ? k : small[k]);
        if (!all_small)
            for (size_t k = 0; k < small.size(); ++k) {
                prow[small[k]] = std::move(prs[k]);
                pcol[small[k]] = std::move(pcs[k]);
            }
        auto t2 = now();
        // blocks whose rank outgrew one CTA: the group search from twice that scratch
        if (!over.empty()) run_nca_big(h, R, C, over, prow, pcol, 2 * NCA_SMALL_CAP);
        if (timing) {
            int64_t rb = 0, rs = 0;
            for (size_t p : big) rb += (int64_t)prow[p].size();
            for (size_t p : small) rs += (int64_t)prow[p].size();
            int64_t rm = 0;
            for (size_t p : med) rm += (int64_t)prow[p].size();
            fprintf(stderr, "h2w nca: %zu group blocks %.3f s (pivots %lld); %zu medium blocks on groups %.3f s (pivots "
                            "%lld); %zu one-CTA blocks %.3f s (pivots %lld); %zu outgrew one CTA %.3f s\n", big.size(),
                    std::chrono::duration<double>(tm - t0).count(), (long long)rb, med.size(),
                    std::chrono::duration<double>(t1 - tm).count(), (long long)rm, small.size(),
                    std::chrono::duration<double>(t2 - t1).count(), (long long)rs, over.size(),
                    std::chrono::duration<double>(now() - t2).count());
        }
    } else if (timing) {
        fprintf(stderr, "h2w nca: %zu group blocks %.3f s, %zu medium blocks on groups %.3f s\n", big.size(),
                std::chrono::duration<double>(tm - t0).count(), med.size(), std::chrono::duration<double>(t1 - tm).count());
    }
    if (h->learn_rec) {  // training data of the large blocks: recorded through the small path's recorder
        std::vector<size_t> rec = big;
        rec.insert(rec.end(), med.begin(), med.end());
        rec.insert(rec.end(), over.begin(), over.end());
        if (!rec.empty()) {
            std::vector<std::vector<int32_t>> R2, C2, pr2, pc2;
            for (size_t p : rec) {
                R2.push_back(R[p]);
                C2.push_back(C[p]);
                pr2.push_back(prow[p]);
                pc2.push_back(pcol[p]);
            }
            record_lists(h, R2, C2, pr2, pc2);
        }
    }
}

// One CTA per block. over: blocks whose rank outgrew the CTA's scratch
// (NCA_SMALL_CAP pivots, or rank_cap when smaller); their pivots are left
// empty for the caller to search with groups of CTAs.
void run_nca_small(h2w_handle *h, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
                   std::vector<std::vector<int32_t>> &prow, std::vector<std::vector<int32_t>> &pcol,
                   std::vector<size_t> &over) {
    const size_t np = R.size();
    prow.assign(np, {});
    pcol.assign(np, {});
    over.clear();
    const double tol = std::pow(10, -1.0 * h->cfg.tol_pow);
    const int cap = h->cfg.rank_cap > 0 ? std::min(h->cfg.rank_cap, NCA_SMALL_CAP) : NCA_SMALL_CAP;
    const size_t budget = (size_t)3 << 30;  // scratch bytes per batch
    KParams kp = h->kparams();
    size_t p0 = 0;
    while (p0 < np) {
        std::vector<NcaProb> probs;
        std::vector<int32_t> idx;
        size_t scr = 0;
        int64_t piv = 0;
        int mx1 = 1, mx2 = 1, mxr = 1;
        size_t p = p0;
        for (; p < np; ++p) {
            int n1 = (int)R[p].size(), n2 = (int)C[p].size();
            int rc = std::min(std::min(n1, n2), cap);
            size_t need = (size_t)rc * (size_t)(n1 + n2);
            if (!probs.empty() && (scr + need) * 8 > budget) break;
            NcaProb pb{};
            pb.ri = (int64_t)idx.size();
            append(idx, R[p].data(), n1);
            pb.ci = (int64_t)idx.size();
            append(idx, C[p].data(), n2);
            pb.u = (int64_t)scr;
            pb.v = (int64_t)(scr + (size_t)rc * n1);
            scr += need;
            pb.piv = piv;
            piv += rc;
            pb.n1 = n1;
            pb.n2 = n2;
            pb.rcap = rc;
            probs.push_back(pb);
            mx1 = std::max(mx1, n1);
            mx2 = std::max(mx2, n2);
            mxr = std::max(mxr, rc);
        }
        DBuf<NcaProb> dp;
        DBuf<int32_t> di, drank, dpr, dpc, dst;
        DBuf<double> dscr;
        dp.upload(probs, h->stream);
        di.upload(idx, h->stream);
        dscr.alloc(scr);
        drank.alloc(probs.size());
        dpr.alloc((size_t)piv);
        dpc.alloc((size_t)piv);
        dst.alloc(1);
        CK(cudaMemsetAsync(dst.p, 0, 4, h->stream));
        CK(launch_nca(dp.p, (int)probs.size(), di.p, kp, tol, dscr.p, drank.p, dpr.p, dpc.p, dst.p, mx1, mx2, mxr,
                      h->stream));
        std::vector<int32_t> rk(probs.size()), hpr((size_t)piv), hpc((size_t)piv);
        int32_t status = 0;
        CK(cudaMemcpyAsync(rk.data(), drank.p, rk.size() * 4, cudaMemcpyDeviceToHost, h->stream));
        if (piv) {
            CK(cudaMemcpyAsync(hpr.data(), dpr.p, hpr.size() * 4, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(hpc.data(), dpc.p, hpc.size() * 4, cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaMemcpyAsync(&status, dst.p, 4, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (status & 2) throw ApiError(H2W_ERR_ARG, "non-finite kernel entries (coincident points?) in an NCA block");
        bool any_over = false;
        for (size_t q = 0; q < probs.size(); ++q) {
            const NcaProb &pb = probs[q];
            if (rk[q] < 0) {
                if (h->cfg.rank_cap > 0 && h->cfg.rank_cap <= NCA_SMALL_CAP)
                    throw ApiError(H2W_ERR_RANK, "an NCA block needed more than rank_cap = " +
                                                     std::to_string(h->cfg.rank_cap) + " pivots");
                over.push_back(p0 + q);
                any_over = true;
                continue;
            }
            prow[p0 + q].assign(hpr.begin() + pb.piv, hpr.begin() + pb.piv + rk[q]);
            pcol[p0 + q].assign(hpc.begin() + pb.piv, hpc.begin() + pb.piv + rk[q]);
        }
        if (h->learn_rec && !any_over) record_blocks(h, probs, di, prow, pcol, p0);
        else if (h->learn_rec) {  // the finished blocks only (the others are recorded after the group search)
            std::vector<std::vector<int32_t>> R2, C2, pr2, pc2;
            for (size_t q = 0; q < probs.size(); ++q)
                if (rk[q] >= 0) {
                    R2.push_back(R[p0 + q]);
                    C2.push_back(C[p0 + q]);
                    pr2.push_back(prow[p0 + q]);
                    pc2.push_back(pcol[p0 + q]);
                }
            if (!R2.empty()) record_lists(h, R2, C2, pr2, pc2);
        }
        p0 = p;
    }
}

// Training data: the learned model's features of every candidate point of
// these blocks, labelled 1 where the NCA chose the point as a pivot.
void record_blocks(h2w_handle *h, const std::vector<NcaProb> &probs, const DBuf<int32_t> &di,
                   const std::vector<std::vector<int32_t>> &prow, const std::vector<std::vector<int32_t>> &pcol,
                   size_t p0) {
    std::vector<LearnProb> lp(probs.size());
    int64_t xo = 0;
    for (size_t q = 0; q < probs.size(); ++q) {
        LearnProb &l = lp[q];
        std::memset(&l, 0, sizeof(l));
        l.ri = probs[q].ri;
        l.ci = probs[q].ci;
        l.n1 = probs[q].n1;
        l.n2 = probs[q].n2;
        l.xo = xo;
        xo += l.n1 + l.n2;
    }
    DBuf<LearnProb> dl;
    DBuf<float> dx;
    dl.upload(lp, h->stream);
    dx.alloc((size_t)xo * LRN_F);
    CK(launch_learn_features(dl.p, (int)lp.size(), di.p, h->kparams(), h->cfg.tol_pow, dx.p, 0, h->stream));
    const size_t base = h->rec_y.size();
    h->rec_X.resize((base + (size_t)xo) * LRN_F);
    h->rec_y.resize(base + (size_t)xo, 0);
    CK(cudaMemcpyAsync(h->rec_X.data() + base * LRN_F, dx.p, (size_t)xo * LRN_F * 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t q = 0; q < lp.size(); ++q) {
        for (int32_t i : prow[p0 + q]) h->rec_y[base + (size_t)lp[q].xo + (size_t)i] = 1;
        for (int32_t j : pcol[p0 + q]) h->rec_y[base + (size_t)lp[q].xo + (size_t)lp[q].n1 + (size_t)j] = 1;
    }
}

// Training data of blocks given as lists (the large-block path).
void record_lists(h2w_handle *h, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
                  const std::vector<std::vector<int32_t>> &prow, const std::vector<std::vector<int32_t>> &pcol) {
    std::vector<NcaProb> probs(R.size());
    std::vector<int32_t> idx;
    for (size_t q = 0; q < R.size(); ++q) {
        probs[q].ri = (int64_t)idx.size();
        append(idx, R[q].data(), (int64_t)R[q].size());
        probs[q].ci = (int64_t)idx.size();
        append(idx, C[q].data(), (int64_t)C[q].size());
        probs[q].n1 = (int32_t)R[q].size();
        probs[q].n2 = (int32_t)C[q].size();
    }
    DBuf<int32_t> di;
    di.upload(idx, h->stream);
    record_blocks(h, probs, di, prow, pcol, 0);
}

// Learned proposals for every block (see learn.cu); blocks the NCA stopping
// test rejects go to the plain search.
void run_nca_learned(h2w_handle *h, const std::vector<std::vector<int32_t>> &R,
                     const std::vector<std::vector<int32_t>> &C, std::vector<std::vector<int32_t>> &prow,
                     std::vector<std::vector<int32_t>> &pcol) {
    const size_t np = R.size();
    prow.assign(np, {});
    pcol.assign(np, {});
    const double tol = std::pow(10, -1.0 * h->cfg.tol_pow);
    const size_t budget = (size_t)3 << 30;
    KParams kp = h->kparams();
    cudaStream_t st = h->stream;
    std::vector<size_t> rejected;
    size_t p0 = 0;
    while (p0 < np) {
        std::vector<LearnProb> probs;
        std::vector<int32_t> idx;
        std::vector<LearnTile> tiles;
        int64_t scr = 0, xo = 0, piv = 0;
        int mw1 = 1, mw2 = 1, mw3 = 1;
        size_t p = p0;
        for (; p < np; ++p) {
            const int n1 = (int)R[p].size(), n2 = (int)C[p].size();
            const int cap = std::min(std::min(n1, n2), LRN_CAP);
            const int64_t need = 2 * (int64_t)cap * (n1 + n2) + 3 * (int64_t)cap * cap;
            if (!probs.empty() && (size_t)(scr + need) * 8 + (size_t)(xo + n1) * (LRN_F + 1) * 4 > budget) break;
            LearnProb l;
            std::memset(&l, 0, sizeof(l));
            l.ri = (int64_t)idx.size();
            append(idx, R[p].data(), n1);
            l.ci = (int64_t)idx.size();
            append(idx, C[p].data(), n2);
            l.xo = xo;
            xo += n1;  // rows only are scored
            l.ac = scr; scr += (int64_t)cap * n1;
            l.ar = scr; scr += (int64_t)cap * n2;
            l.uu = scr; scr += (int64_t)cap * n1;
            l.vv = scr; scr += (int64_t)cap * n2;
            l.ff = scr; scr += (int64_t)cap * cap;
            l.gu = scr; scr += (int64_t)cap * cap;
            l.gv = scr; scr += (int64_t)cap * cap;
            l.piv = piv;
            piv += cap + 1;
            l.n1 = n1;
            l.n2 = n2;
            l.cap = cap;
            const int b = (int)probs.size();
            for (int64_t e = 0; e < (int64_t)n1 * cap; e += 8192)
                tiles.push_back({b, 0, (int32_t)e, (int32_t)std::min<int64_t>(8192, (int64_t)n1 * cap - e)});
            for (int64_t e = 0; e < (int64_t)n2 * cap; e += 8192)
                tiles.push_back({b, 1, (int32_t)e, (int32_t)std::min<int64_t>(8192, (int64_t)n2 * cap - e)});
            for (int e = 0; e < n1; e += 64) tiles.push_back({b, 2, e, std::min(64, n1 - e)});
            for (int e = 0; e < n2; e += 64) tiles.push_back({b, 3, e, std::min(64, n2 - e)});
            mw1 = std::max(mw1, (std::max(n1, n2) + 31) / 32);
            mw2 = std::max(mw2, (n1 + 31) / 32 + (n2 + 31) / 32);
            mw3 = std::max(mw3, (n2 + 31) / 32);
            probs.push_back(l);
        }
        const int nb = (int)probs.size();
        DBuf<LearnProb> dp;
        DBuf<LearnTile> dt;
        DBuf<int32_t> di, dpr, dpc, doi, doj, dor, doc;
        DBuf<LearnState> dls;
        DBuf<double> dscr;
        DBuf<float> dx, dz;
        dp.upload(probs, st);
        dt.upload(tiles, st);
        di.upload(idx, st);
        for (DBuf<int32_t> *v : {&dpr, &dpc, &doi, &doj, &dor, &doc}) v->alloc((size_t)piv);
        dls.alloc((size_t)nb);
        dscr.alloc((size_t)scr);
        CK(cudaMemsetAsync(dscr.p, 0, (size_t)scr * 8, st));
        dx.alloc((size_t)xo * LRN_F);
        dz.alloc((size_t)xo);
        CK(launch_learn_features(dp.p, nb, di.p, kp, h->cfg.tol_pow, dx.p, 1, st));
        CK(launch_mlp_forward(h->d_mlp.p, dx.p, xo, dz.p, st));
        CK(launch_learn_propose(dp.p, nb, dz.p, h->mlp_calib, h->mlp_margin, dpr.p, dpc.p, dls.p, mw1, st));
        CK(launch_learn_fill(dt.p, (int)tiles.size(), dp.p, di.p, kp, dpr.p, doj.p, dls.p, dscr.p, 1, st));
        CK(launch_learn_aca(dp.p, nb, tol, dscr.p, doi.p, doj.p, dls.p, mw3, st));
        CK(launch_learn_fill(dt.p, (int)tiles.size(), dp.p, di.p, kp, dpr.p, doj.p, dls.p, dscr.p, 0, st));
        CK(launch_learn_solve(dt.p, (int)tiles.size(), dp.p, doi.p, doj.p, dls.p, dscr.p, st));
        CK(launch_learn_gram(dt.p, (int)tiles.size(), dp.p, dls.p, dscr.p, st));
        CK(launch_learn_test(dp.p, nb, di.p, kp, tol, dpr.p, dpc.p, doi.p, doj.p, dls.p, dscr.p, dor.p, doc.p, mw2, st));
        std::vector<LearnState> ls((size_t)nb);
        std::vector<int32_t> hr((size_t)piv), hc((size_t)piv);
        CK(cudaMemcpyAsync(ls.data(), dls.p, (size_t)nb * sizeof(LearnState), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hr.data(), dor.p, (size_t)piv * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hc.data(), doc.p, (size_t)piv * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int q = 0; q < nb; ++q) {
            const LearnState &s = ls[(size_t)q];
            h->learn_rhat += s.rhat;
            h->learn_r1 += s.r1;
            if (!s.accept) ++h->learn_reject[s.rank == -1 ? 0 : (s.rank == -2 ? 1 : 2)];
            if (s.accept && s.rank > 0) {
                prow[p0 + q].assign(hr.begin() + probs[(size_t)q].piv, hr.begin() + probs[(size_t)q].piv + s.rank);
                pcol[p0 + q].assign(hc.begin() + probs[(size_t)q].piv, hc.begin() + probs[(size_t)q].piv + s.rank);
                ++h->learn_accepted;
            } else {
                rejected.push_back(p0 + q);
            }
        }
        h->learn_blocks += nb;
        p0 = p;
    }
    if (!rejected.empty()) {
        std::vector<std::vector<int32_t>> R2, C2, pr2, pc2;
        for (size_t q : rejected) {
            R2.push_back(R[q]);
            C2.push_back(C[q]);
        }
        run_nca_plain(h, R2, C2, pr2, pc2);
        for (size_t k = 0; k < rejected.size(); ++k) {
            prow[rejected[k]] = std::move(pr2[k]);
            pcol[rejected[k]] = std::move(pc2[k]);
        }
    }
}

// Complex kernel: one CTA per block (nca_c_kernel). Each block starts with
// scratch for 128 pivots (at most min(rows, columns)); blocks that fill it run
// again with twice as many, up to what one CTA's shared memory holds (the
// reference's own bound, min(rows, columns), otherwise; an explicit rank_cap
// stops earlier with H2W_ERR_RANK).
void run_nca_complex(h2w_handle *h, const std::vector<std::vector<int32_t>> &R,
                     const std::vector<std::vector<int32_t>> &C, std::vector<std::vector<int32_t>> &prow,
                     std::vector<std::vector<int32_t>> &pcol) {
    const size_t np = R.size();
    prow.assign(np, {});
    pcol.assign(np, {});
    const double tol = std::pow(10, -1.0 * h->cfg.tol_pow);
    const int cap = h->cfg.rank_cap > 0 ? h->cfg.rank_cap : INT32_MAX;
    int smem_max = 0;
    CK(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->cfg.device));
    KParams kp = h->kparams();
    std::vector<std::pair<size_t, int>> pend;
    for (size_t p = 0; p < np; ++p) {
        const int mn = (int)std::min(R[p].size(), C[p].size());
        pend.push_back({p, std::min(std::min(mn, cap), 128)});
    }
    const size_t budget = (size_t)2 << 30;  // scratch bytes per batch
    while (!pend.empty()) {
        std::vector<std::pair<size_t, int>> again;
        size_t q0 = 0;
        while (q0 < pend.size()) {
            std::vector<NcaProb> probs;
            std::vector<int32_t> idx;
            size_t scr = 0;
            int64_t piv = 0;
            int mx1 = 1, mx2 = 1, mxr = 1;
            size_t q = q0;
            for (; q < pend.size(); ++q) {
                const size_t p = pend[q].first;
                const int n1 = (int)R[p].size(), n2 = (int)C[p].size(), rc = pend[q].second;
                const size_t need = (size_t)rc * (size_t)(n1 + n2);
                if (!probs.empty() && (scr + need) * 16 > budget) break;
                if (nca_c_smem(std::max(mx1, n1), std::max(mx2, n2), std::max(mxr, rc)) > (size_t)smem_max) {
                    if (probs.empty())
                        throw ApiError(H2W_ERR_RANK, "a complex NCA block needs more pivots than one CTA holds (" +
                                                         std::to_string(rc) + ")");
                    break;
                }
                NcaProb pb{};
                pb.ri = (int64_t)idx.size();
                append(idx, R[p].data(), n1);
                pb.ci = (int64_t)idx.size();
                append(idx, C[p].data(), n2);
                pb.u = (int64_t)scr;
                pb.v = (int64_t)(scr + (size_t)rc * n1);
                scr += need;
                pb.piv = piv;
                piv += rc;
                pb.n1 = n1;
                pb.n2 = n2;
                pb.rcap = rc;
                probs.push_back(pb);
                mx1 = std::max(mx1, n1);
                mx2 = std::max(mx2, n2);
                mxr = std::max(mxr, rc);
            }
            DBuf<NcaProb> dp;
            DBuf<int32_t> di, drank, dpr, dpc, dst;
            DBuf<double2> dscr;
            dp.upload(probs, h->stream);
            di.upload(idx, h->stream);
            dscr.alloc(std::max<size_t>(scr, 1));
            drank.alloc(probs.size());
            dpr.alloc((size_t)std::max<int64_t>(piv, 1));
            dpc.alloc((size_t)std::max<int64_t>(piv, 1));
            dst.alloc(1);
            CK(cudaMemsetAsync(dst.p, 0, 4, h->stream));
            CK(launch_nca_c(dp.p, (int)probs.size(), di.p, kp, tol, dscr.p, drank.p, dpr.p, dpc.p, dst.p, mx1, mx2,
                            mxr, h->stream));
            std::vector<int32_t> rk(probs.size()), hpr((size_t)piv), hpc((size_t)piv);
            int32_t status = 0;
            CK(cudaMemcpyAsync(rk.data(), drank.p, rk.size() * 4, cudaMemcpyDeviceToHost, h->stream));
            if (piv) {
                CK(cudaMemcpyAsync(hpr.data(), dpr.p, hpr.size() * 4, cudaMemcpyDeviceToHost, h->stream));
                CK(cudaMemcpyAsync(hpc.data(), dpc.p, hpc.size() * 4, cudaMemcpyDeviceToHost, h->stream));
            }
            CK(cudaMemcpyAsync(&status, dst.p, 4, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (status & 2) throw ApiError(H2W_ERR_ARG, "non-finite kernel entries (coincident points?) in an NCA block");
            for (size_t k = 0; k < probs.size(); ++k) {
                const auto &pq = pend[q0 + k];
                const size_t p = pq.first;
                if (rk[k] < 0) {
                    const int mn = (int)std::min(R[p].size(), C[p].size());
                    const int lim = std::min(mn, cap);
                    if (pq.second >= lim)
                        throw ApiError(H2W_ERR_RANK, "an NCA block needed more than rank_cap = " +
                                                         std::to_string(h->cfg.rank_cap) + " pivots");
                    again.push_back({p, std::min(lim, 2 * pq.second)});
                    continue;
                }
                const NcaProb &pb = probs[k];
                prow[p].assign(hpr.begin() + pb.piv, hpr.begin() + pb.piv + rk[k]);
                pcol[p].assign(hpc.begin() + pb.piv, hpc.begin() + pb.piv + rk[k]);
            }
            q0 = q;
        }
        pend.swap(again);
    }
}

void run_nca(h2w_handle *h, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
             std::vector<std::vector<int32_t>> &prow, std::vector<std::vector<int32_t>> &pcol) {
    if (h->cplx) run_nca_complex(h, R, C, prow, pcol);
    else if (h->learned) run_nca_learned(h, R, C, prow, pcol);
    else run_nca_plain(h, R, C, prow, pcol);
}

void skel_from_pivots(Skel &s, const std::vector<std::vector<int32_t>> &R, const std::vector<std::vector<int32_t>> &C,
                      const std::vector<std::vector<int32_t>> &pr, const std::vector<std::vector<int32_t>> &pc) {
    s.ptr.assign(R.size() + 1, 0);
    s.chk.clear();
    s.chg.clear();
    for (size_t k = 0; k < R.size(); ++k) {
        for (size_t i = 0; i < pr[k].size(); ++i) {
            s.chk.push_back(R[k][(size_t)pr[k][i]]);
            s.chg.push_back(C[k][(size_t)pc[k][i]]);
        }
        s.ptr[k + 1] = (int64_t)s.chk.size();
    }
}

// rows of the far NCA / far transfer of box (j,k): leaf points or the
// children's far check points (pivot_selection_bottom_up, 2D :537-550)
std::vector<int32_t> far_rows(const h2w_handle *h, int j, int64_t k) {
    const Tree &t = h->tree;
    if (j == t.nL) return box_pts(t, j, k);
    std::vector<int32_t> r;
    const Skel &s = h->far[(size_t)j + 1];
    for (int c = 0; c < t.nch; ++c) {
        int64_t q = k * t.nch + c;
        append(r, s.chk.data() + s.ptr[q], s.rank(q));
    }
    return r;
}
// rows of a vertex / 1D nested transfer: leaf points or children's check points
std::vector<int32_t> ver_rows(const h2w_handle *h, int j, int64_t k) {
    const Tree &t = h->tree;
    if (j == t.nL) return box_pts(t, j, k);
    std::vector<int32_t> r;
    const Skel &s = h->ver[(size_t)j + 1];
    for (int c = 0; c < t.nch; ++c) {
        int64_t q = k * t.nch + c;
        append(r, s.chk.data() + s.ptr[q], s.rank(q));
    }
    return r;
}

void nca_far(h2w_handle *h) {
    const Tree &t = h->tree;
    h->far.assign((size_t)t.nL + 1, Skel{});
    for (int j = 0; j <= t.nL; ++j) h->far[(size_t)j].ptr.assign((size_t)t.nbox[(size_t)j] + 1, 0);
    for (int j = t.nL; j >= 2; --j) {
        const int64_t nb = t.nbox[(size_t)j];
        std::vector<std::vector<int32_t>> R((size_t)nb), C((size_t)nb), pr, pc;
        for (int64_t k = 0; k < nb; ++k) {
            R[(size_t)k] = far_rows(h, j, k);
            for (int64_t e = t.ilp[(size_t)j][(size_t)k]; e < t.ilp[(size_t)j][(size_t)k + 1]; ++e) {
                if (t.ilv[(size_t)j][(size_t)e]) continue;
                std::vector<int32_t> c = far_rows(h, j, t.il[(size_t)j][(size_t)e]);
                append(C[(size_t)k], c.data(), (int64_t)c.size());
            }
        }
        run_nca(h, R, C, pr, pc);
        skel_from_pivots(h->far[(size_t)j], R, C, pr, pc);
    }
}

void nca_ver(h2w_handle *h) {
    const Tree &t = h->tree;
    h->ver.assign((size_t)t.nL + 1, Skel{});
    h->ver[0].ptr.assign(2, 0);
    for (int j = 1; j <= t.nL; ++j) {
        const int64_t nb = t.nbox[(size_t)j];
        std::vector<std::vector<int32_t>> R((size_t)nb), C((size_t)nb), pr, pc;
        for (int64_t k = 0; k < nb; ++k) {
            R[(size_t)k] = box_pts(t, j, k);
            auto &c = C[(size_t)k];
            if (t.dim == 1) {
                for (int s = 0; s < 2; ++s) {
                    int32_t q = t.nb[(size_t)j][(size_t)(k * 2 + s)];
                    if (q != -1) append(c, t.perm.data() + t.off[(size_t)j][(size_t)q], t.cnt(j, q));
                }
            } else {
                for (int64_t e = t.ilp[(size_t)j][(size_t)k]; e < t.ilp[(size_t)j][(size_t)k + 1]; ++e) {
                    if (!t.ilv[(size_t)j][(size_t)e]) continue;
                    int32_t q = t.il[(size_t)j][(size_t)e];
                    append(c, t.perm.data() + t.off[(size_t)j][(size_t)q], t.cnt(j, q));
                }
            }
            if (j > 1) {
                const Skel &ps = h->ver[(size_t)j - 1];
                int64_t par = k / t.nch;
                append(c, ps.chg.data() + ps.ptr[(size_t)par], ps.rank(par));
            }
        }
        run_nca(h, R, C, pr, pc);
        skel_from_pivots(h->ver[(size_t)j], R, C, pr, pc);
    }
}

// Pair lists: 2D/3D semi-nested vertex pairs, 1D sibling pairs.
void pair_layout(h2w_handle *h) {
    const Tree &t = h->tree;
    h->pairs.assign((size_t)t.nL + 1, Pairs{});
    for (int j = 1; j <= t.nL; ++j) {
        Pairs &P = h->pairs[(size_t)j];
        for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
            if (t.dim == 1) {
                for (int s = 0; s < 2; ++s) {
                    int32_t q = t.nb[(size_t)j][(size_t)(k * 2 + s)];
                    if (q == -1) continue;
                    P.box.push_back((int32_t)k);
                    P.slot.push_back(s);
                    P.other.push_back(q);
                }
            } else {
                for (int64_t e = t.ilp[(size_t)j][(size_t)k]; e < t.ilp[(size_t)j][(size_t)k + 1]; ++e) {
                    // (H2+H)*: vertex pairs (getUVtTree_sn); H*: every interaction-list
                    // pair (getUVtTree_nn, 2D/codes/HODLR2Dtree.hpp:971-980,
                    // 3D/codes/HODLR3Dtree.hpp:2239-2280)
                    if (!t.ilv[(size_t)j][(size_t)e] && h->cfg.form != H2W_FORM_NONNESTED) continue;
                    P.box.push_back((int32_t)k);
                    P.slot.push_back((int32_t)(e - t.ilp[(size_t)j][(size_t)k]));
                    P.other.push_back(t.il[(size_t)j][(size_t)e]);
                }
            }
        }
        P.ptr.assign(P.box.size() + 1, 0);
    }
}

void nca_pairs(h2w_handle *h) {
    const Tree &t = h->tree;
    std::vector<std::vector<int32_t>> R, C, pr, pc;
    for (int j = 1; j <= t.nL; ++j) {
        Pairs &P = h->pairs[(size_t)j];
        for (size_t p = 0; p < P.box.size(); ++p) {
            R.push_back(box_pts(t, j, P.box[p]));
            C.push_back(box_pts(t, j, P.other[p]));
        }
    }
    run_nca(h, R, C, pr, pc);
    size_t q = 0;
    for (int j = 1; j <= t.nL; ++j) {
        Pairs &P = h->pairs[(size_t)j];
        P.row.clear();
        P.col.clear();
        for (size_t p = 0; p < P.box.size(); ++p, ++q) {
            for (size_t i = 0; i < pr[q].size(); ++i) {
                P.row.push_back(R[q][(size_t)pr[q][i]]);
                P.col.push_back(C[q][(size_t)pc[q][i]]);
            }
            P.ptr[p + 1] = (int64_t)P.row.size();
        }
    }
}

// --------------------------------------------------------- list import ---
// Per-(level, box) CSR lists -> skeletons / pairs.
void import_skel(h2w_handle *h, int which_chk, int which_chg, std::vector<Skel> &S, int jmin) {
    const Tree &t = h->tree;
    const auto &p1 = h->imp_ptr[(size_t)which_chk];
    const auto &v1 = h->imp_val[(size_t)which_chk];
    const auto &v2 = h->imp_val[(size_t)which_chg];
    const auto &p2 = h->imp_ptr[(size_t)which_chg];
    S.assign((size_t)t.nL + 1, Skel{});
    int64_t base = 0;
    for (int j = 0; j <= t.nL; ++j) {
        Skel &s = S[(size_t)j];
        s.ptr.assign((size_t)t.nbox[(size_t)j] + 1, 0);
        for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
            int64_t b = base + k;
            int64_t a0 = p1[(size_t)b], a1 = p1[(size_t)b + 1];
            if (p2[(size_t)b + 1] - p2[(size_t)b] != a1 - a0) throw ApiError(H2W_ERR_ARG, "pivot lists differ in length");
            if (j >= jmin)
                for (int64_t i = a0; i < a1; ++i) {
                    s.chk.push_back(v1[(size_t)i]);
                    s.chg.push_back(v2[(size_t)(p2[(size_t)b] + i - a0)]);
                }
            s.ptr[(size_t)k + 1] = (int64_t)s.chk.size();
        }
        base += t.nbox[(size_t)j];
    }
}

void import_pairs(h2w_handle *h) {
    const Tree &t = h->tree;
    const auto &pr = h->imp_ptr[H2W_LIST_SN_ROW];
    const auto &vr = h->imp_val[H2W_LIST_SN_ROW];
    const auto &pcp = h->imp_ptr[H2W_LIST_SN_COL];
    const auto &vc = h->imp_val[H2W_LIST_SN_COL];
    // entry index of (j, k, slot) in the CSR
    int64_t e = 0;
    std::vector<std::vector<int64_t>> first((size_t)t.nL + 1);
    for (int j = 0; j <= t.nL; ++j) {
        first[(size_t)j].assign((size_t)t.nbox[(size_t)j] + 1, 0);
        for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
            first[(size_t)j][(size_t)k] = e;
            if (t.dim == 1) e += j >= 1 ? 2 : 0;
            else e += t.ilp[(size_t)j][(size_t)k + 1] - t.ilp[(size_t)j][(size_t)k];
        }
    }
    if ((int64_t)pr.size() != e + 1) throw ApiError(H2W_ERR_ARG, "pair list has the wrong number of entries");
    for (int j = 1; j <= t.nL; ++j) {
        Pairs &P = h->pairs[(size_t)j];
        P.row.clear();
        P.col.clear();
        for (size_t p = 0; p < P.box.size(); ++p) {
            int64_t q = first[(size_t)j][(size_t)P.box[p]] + P.slot[p];
            int64_t a0 = pr[(size_t)q], a1 = pr[(size_t)q + 1];
            int64_t b0 = pcp[(size_t)q], b1 = pcp[(size_t)q + 1];
            if (a1 - a0 != b1 - b0) throw ApiError(H2W_ERR_ARG, "pair pivot lists differ in length");
            P.row.insert(P.row.end(), vr.begin() + a0, vr.begin() + a1);
            P.col.insert(P.col.end(), vc.begin() + b0, vc.begin() + b1);
            P.ptr[p + 1] = (int64_t)P.row.size();
        }
    }
}

// ---------------------------------------------------------------- plan ---
struct PlanBuilder {
    h2w_handle *h;
    std::vector<Target> T;
    std::vector<Panel> P;
    std::vector<Seg> S;
    std::vector<int32_t> idx;
    std::vector<FillJob> fills;
    std::vector<FactorJob> factors;
    std::vector<XferJob> xfers;
    int64_t opn = 0, fn = 0;
    int max_xfer_n = 0;
    int64_t read_elems = 0;
    // phase window of the targets being emitted, and per target
    int lo = 0, hi = 0;
    std::vector<std::pair<int, int>> win;
    // split parameters of the stream being realised: targets are cut into
    // row chunks of max(min_rows, row_split / width) rows (multiples of 4)
    int64_t row_split = ROW_SPLIT;
    int64_t min_rows = 4;
    int64_t xw_cap = XW_CAP;  // gathered columns per target before a column split
    bool fused = true;        // no leaf (scatter) target was column-split

    // column-major block: element (i, c) at a + c*lda + i, lda = pad4(rows)
    std::vector<int64_t> blocks;  // (a, lda, cols) of every block, in allocation order
    int64_t alloc(int64_t rows, int64_t cols, int32_t &lda) {
        lda = (int32_t)pad4(rows);
        int64_t a = opn;
        opn += pad4((int64_t)lda * cols);
        blocks.push_back(a);
        blocks.push_back(lda);
        blocks.push_back(cols);
        return a;
    }
    // The logical targets of a complex operator rewritten for its realified
    // form: every row, column, workspace and vector position doubled (interleaved
    // (re, im)), every block address mapped to its real block (4a, lda 2 lda).
    void realify() {
        auto addr = [&](int64_t a) {
            // the block holding complex address a: element (i, c) at base + c lda + i
            size_t lo = 0, hi = blocks.size() / 3;
            while (hi - lo > 1) {
                size_t mid = (lo + hi) / 2;
                if (blocks[3 * mid] <= a) lo = mid;
                else hi = mid;
            }
            const int64_t base = blocks[3 * lo], ld = blocks[3 * lo + 1];
            const int64_t o = a - base, c = o / ld, i = o - c * ld;
            return 4 * base + 2 * c * (2 * ld) + 2 * i;
        };
        for (LTarget &l : logical) {
            l.dst *= 2;
            l.nrows *= 2;
            for (PanelSpec &p : l.panels) {
                p.a = addr(p.a);
                p.lda *= 2;
                p.w *= 2;
                for (Seg &g : p.segs) {
                    g.src *= 2;
                    g.len *= 2;
                    g.xoff *= 2;
                }
            }
        }
        opn *= 4;
        read_elems *= 4;
    }
    int64_t put_idx(const int32_t *v, int64_t n) {
        int64_t o = (int64_t)idx.size();
        append(idx, v, n);
        return o;
    }
    int64_t put_idx(const std::vector<int32_t> &v) { return put_idx(v.data(), (int64_t)v.size()); }

    struct PanelSpec {
        int64_t a;
        int32_t lda, w;
        std::vector<Seg> segs;  // xoff relative to panel
    };
    // A block-row product before any splitting; the same logical targets are
    // realised once per target stream (single-vector and multi-vector).
    struct LTarget {
        int64_t dst;
        int32_t nrows, flags;
        std::vector<PanelSpec> panels;
        int lo, hi;
    };
    std::vector<LTarget> logical;
    void emit(int64_t dst, int32_t nrows, int32_t flags, const std::vector<PanelSpec> &panels) {
        if (nrows <= 0) return;
        for (auto &p : panels) read_elems += (int64_t)nrows * p.w;
        logical.push_back({dst, nrows, flags, panels, lo, hi});
    }
    // Realise the logical targets with the given split parameters into T/P/S/win.
    void realize(int64_t rs, int64_t mr, int64_t cap) {
        T.clear();
        P.clear();
        S.clear();
        win.clear();
        row_split = rs;
        min_rows = mr;
        xw_cap = cap;
        fused = true;
        for (const LTarget &l : logical) {
            lo = l.lo;
            hi = l.hi;
            split(l.dst, l.nrows, l.flags, l.panels);
        }
    }
    // Cut a target into row chunks and, past xw_cap gathered columns, into
    // atomically accumulated column chunks.
    void split(int64_t dst, int32_t nrows, int32_t flags, const std::vector<PanelSpec> &panels) {
        if (nrows <= 0) return;
        int64_t xw = 0;
        for (auto &p : panels) xw += pad4(p.w);
        if (xw == 0) return;
        if (xw <= xw_cap) {
            // row chunks are multiples of 4 rows so the kernel's 16-byte column loads stay aligned
            int64_t rows_per =
                std::max<int64_t>(min_rows, (row_split / std::max<int64_t>(xw, 1)) & ~int64_t(3));
            rows_per = std::min<int64_t>(rows_per, nrows);
            for (int64_t r0 = 0; r0 < nrows; r0 += rows_per) {
                int32_t nr = (int32_t)std::min<int64_t>(rows_per, nrows - r0);
                Target tg{};
                tg.dst = dst + r0;
                tg.nrows = nr;
                tg.flags = flags;
                tg.p0 = (int32_t)P.size();
                int32_t xo = 0;
                for (auto &p : panels) {
                    Panel pn{};
                    pn.a = p.a + r0;
                    pn.lda = p.lda;
                    pn.w = p.w;
                    pn.xoff = xo;
                    pn.s0 = (int32_t)S.size();
                    for (auto s : p.segs) S.push_back(s);
                    pn.s1 = (int32_t)S.size();
                    P.push_back(pn);
                    xo += (int32_t)pad4(p.w);
                }
                tg.p1 = (int32_t)P.size();
                tg.xw = xo;
                tg.ldsum = 0;
                for (auto &p : panels) tg.ldsum += p.lda;
                tg.gsz = xo >= 256 ? 32 : (xo >= 128 ? 16 : (xo >= 48 ? 8 : 4));
                T.push_back(tg);
                win.push_back({lo, hi});
            }
            return;
        }
        // column split, atomically accumulated sub-targets: whole panels in
        // groups of <= xw_cap gathered columns (as many groups as the width
        // needs, filled evenly), panels wider than xw_cap in chunks of xw_cap
        if (flags & T_SCATTER) fused = false;
        int64_t narrow = 0;
        for (auto &p : panels)
            if (pad4(p.w) <= xw_cap) narrow += pad4(p.w);
        if (narrow > 0) {
            const int64_t ng = (narrow + xw_cap - 1) / xw_cap, share = (narrow + ng - 1) / ng;
            std::vector<PanelSpec> grp;
            int64_t gw = 0;
            for (auto &p : panels) {
                if (pad4(p.w) > xw_cap) continue;
                if (!grp.empty() && (gw + pad4(p.w) > xw_cap || gw >= share)) {
                    split(dst, nrows, T_ATOMIC, grp);
                    grp.clear();
                    gw = 0;
                }
                grp.push_back(p);
                gw += pad4(p.w);
            }
            if (!grp.empty()) split(dst, nrows, T_ATOMIC, grp);
        }
        for (auto &p : panels) {
            if (pad4(p.w) <= xw_cap) continue;
            for (int64_t c0 = 0; c0 < p.w; c0 += xw_cap) {
                int64_t c1 = std::min<int64_t>(p.w, c0 + xw_cap);
                PanelSpec q;
                q.a = p.a + c0 * p.lda;
                q.lda = p.lda;
                q.w = (int32_t)(c1 - c0);
                for (auto s : p.segs) {
                    int64_t s0 = s.xoff, s1 = s.xoff + s.len;
                    int64_t lo = std::max(s0, c0), hi = std::min(s1, c1);
                    if (lo >= hi) continue;
                    Seg ns = s;
                    ns.src = s.src + (lo - s0);
                    ns.len = (int32_t)(hi - lo);
                    ns.xoff = (int32_t)(lo - c0);
                    q.segs.push_back(ns);
                }
                split(dst, nrows, T_ATOMIC, {q});
            }
        }
    }
};

// Host-side bounds and alignment check of every work item before any of it
// reaches the GPU: an inconsistent plan becomes an error status, never an
// out-of-bounds access.
void validate_plan(const PlanBuilder &pb, const h2w_handle *h, const std::vector<Phase> &phases) {
    auto bad = [](const char *what) { throw ApiError(H2W_ERR_STATE, std::string("internal plan check failed: ") + what); };
    const int64_t N = h->tree.N, wsn = h->ws_n, opn = pb.opn, nidx = (int64_t)pb.idx.size();
    for (const Phase &ph : phases)
        if (ph.t0 < 0 || ph.t1 < ph.t0 || ph.t1 > (int64_t)pb.T.size() || ph.max_xw > pb.xw_cap) bad("phase");
    for (const Target &t : pb.T) {
        if (t.nrows < 1 || t.dst < 0 || t.dst + t.nrows > wsn) bad("target rows");
        if (t.p0 < 0 || t.p1 < t.p0 || t.p1 > (int32_t)pb.P.size() || t.p1 - t.p0 > BRG_MAX_PANELS) bad("target panels");
        if ((t.flags & T_SCATTER) && (t.dst < h->yperm_off || t.dst + t.nrows > h->yperm_off + h->nv())) bad("scatter rows");
        int64_t xw = 0;
        for (int32_t q = t.p0; q < t.p1; ++q) {
            const Panel &p = pb.P[(size_t)q];
            if (p.a < 0 || p.w < 1 || p.lda < 1) bad("panel layout");
            const bool vec = (p.a % 4 == 0) && (p.lda % 4 == 0);
            if (p.a + (int64_t)(p.w - 1) * p.lda + (vec ? pad4(t.nrows) : t.nrows) > opn) bad("panel extent");
            if (p.xoff % 4 || p.xoff != xw) bad("panel xoff");
            if (p.s0 < 0 || p.s1 < p.s0 || p.s1 > (int32_t)pb.S.size()) bad("panel segs");
            for (int32_t e = p.s0; e < p.s1; ++e) {
                const Seg &sg = pb.S[(size_t)e];
                if (sg.len < 0 || sg.xoff < 0 || sg.xoff + sg.len > p.w) bad("segment span");
                if (sg.flags & S_GATHER) {
                    if (sg.src < 0 || sg.src + sg.len > h->nv()) bad("gather segment");
                } else if (sg.src < 0 || sg.src + sg.len > wsn) bad("workspace segment");
            }
            xw += pad4(p.w);
        }
        if (xw != t.xw || xw > pb.xw_cap || xw > BRG_XS_ELEMS) bad("target width");
    }
    for (const FactorJob &f : pb.factors)
        if (f.r < 1 || f.f < 0 || f.f + (int64_t)f.r * f.r > pb.fn || f.ii < 0 || f.ii + f.r > nidx || f.jj < 0 ||
            f.jj + f.r > nidx)
            bad("factor job");
    for (const XferJob &x : pb.xfers) {
        if (x.r < 1 || x.n < 1 || x.n > pb.max_xfer_n || x.f < 0 || x.f + (int64_t)x.r * x.r > pb.fn) bad("xfer job");
        if (x.jj < 0 || x.jj + x.r > nidx || x.pi < 0 || x.pi + x.n > nidx) bad("xfer indices");
        bool row = x.mode == X_ROW_RL || x.mode == X_ROW_R;
        if (row) {
            if (x.ld1 < x.n || x.a1 < 0 || x.a1 + (int64_t)(x.r - 1) * x.ld1 + x.n > opn) bad("xfer rows");
            if (x.a2 >= 0 && (x.ld2 < x.r || x.a2 + (int64_t)(x.n - 1) * x.ld2 + x.r > opn)) bad("xfer transposed");
        } else if (x.ld1 < x.r || x.a1 < 0 || x.a1 + (int64_t)(x.n - 1) * x.ld1 + x.r > opn) {
            bad("xfer columns");
        }
    }
    for (const FillJob &f : pb.fills)
        if (f.nr < 1 || f.nc < 1 || f.lda < f.nr || f.a < 0 || f.a + (int64_t)(f.nc - 1) * f.lda + f.nr > opn ||
            f.ri < 0 || f.ri + f.nr > nidx || f.ci < 0 || f.ci + f.nc > nidx)
            bad("fill job");
    for (int32_t v : pb.idx)
        if (v < 0 || v >= N) bad("point index");
}

// Phase assignment of the realised targets: fixed targets at their phase,
// flexible ones (largest first) into the least-loaded phase of their window;
// targets sorted by phase, heaviest first within a phase.
void assign_phases(h2w_handle *h, PlanBuilder &pb, int NPH, std::vector<Phase> &phases, bool &fused) {
    const size_t nt = pb.T.size();
    std::vector<int> ph(nt, 0);
    std::vector<double> load((size_t)NPH, 0.0);
    std::vector<size_t> flex;
    auto elems = [&](size_t q) { return (double)pb.T[q].nrows * (double)pb.T[q].xw; };
    for (size_t q = 0; q < nt; ++q) {
        if (pb.win[q].first == pb.win[q].second) {
            ph[q] = pb.win[q].first;
            load[(size_t)ph[q]] += elems(q);
        } else {
            flex.push_back(q);
        }
    }
    std::stable_sort(flex.begin(), flex.end(), [&](size_t a, size_t b) { return elems(a) > elems(b); });
    for (size_t q : flex) {
        int best = pb.win[q].first;
        for (int p2 = pb.win[q].first; p2 <= pb.win[q].second; ++p2)
            if (load[(size_t)p2] < load[(size_t)best]) best = p2;
        ph[q] = best;
        load[(size_t)best] += elems(q);
    }
    std::vector<size_t> order(nt);
    for (size_t q = 0; q < nt; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        if (ph[a] != ph[b]) return ph[a] < ph[b];
        return elems(a) > elems(b);
    });
    std::vector<Target> T2(nt);
    for (size_t q = 0; q < nt; ++q) T2[q] = pb.T[order[q]];
    pb.T.swap(T2);
    phases.clear();
    size_t q = 0;
    for (int p2 = 0; p2 < NPH; ++p2) {
        size_t q0 = q;
        while (q < nt && ph[order[q]] == p2) ++q;
        if (q > q0) phases.push_back({(int64_t)q0, (int64_t)q, 0, p2});
    }
    // leaves without any far contribution would never be scattered by the
    // fused path; fall back to an explicit scatter then.
    int64_t covered = 0;
    const Phase &lp = phases.back();
    for (int64_t r = lp.t0; r < lp.t1; ++r)
        if (pb.T[(size_t)r].flags & T_SCATTER) covered += pb.T[(size_t)r].nrows;
    fused = pb.fused && covered == h->nv();
    if (!fused)
        for (int64_t r = lp.t0; r < lp.t1; ++r)
            if (pb.T[(size_t)r].flags & T_SCATTER) pb.T[(size_t)r].flags = T_ACCUM;
    for (Phase &p2 : phases) {
        int mx = 0;
        for (int64_t r = p2.t0; r < p2.t1; ++r) mx = std::max(mx, pb.T[(size_t)r].xw);
        p2.max_xw = mx;
    }
}

// Packed records: header, panels, segments (layout documented at brg_kernel),
// plus the phase starts.
void pack_records(const PlanBuilder &pb, const std::vector<Phase> &phases, std::vector<int64_t> &roff,
                  std::vector<int64_t> &blob, std::vector<int64_t> &pstart, size_t max_words = BRG_REC_WORDS) {
    roff.assign(1, 0);
    blob.clear();
    for (const Target &tg : pb.T) {
        const size_t base = blob.size();
        int ns = 0;
        for (int32_t q = tg.p0; q < tg.p1; ++q) ns += pb.P[(size_t)q].s1 - pb.P[(size_t)q].s0;
        blob.push_back(tg.dst);
        blob.push_back((int64_t)(uint32_t)tg.nrows | ((int64_t)tg.flags << 32));
        blob.push_back((int64_t)(uint32_t)(tg.p1 - tg.p0) | ((int64_t)ns << 32));
        for (int32_t q = tg.p0; q < tg.p1; ++q) {
            const Panel &pn = pb.P[(size_t)q];
            blob.push_back(pn.a);
            blob.push_back((int64_t)(uint32_t)pn.lda | ((int64_t)pn.w << 32));
            blob.push_back(pn.xoff);
        }
        for (int32_t q = tg.p0; q < tg.p1; ++q) {
            const Panel &pn = pb.P[(size_t)q];
            for (int32_t e = pn.s0; e < pn.s1; ++e) {
                const Seg &sg = pb.S[(size_t)e];
                const int64_t code = ((int64_t)(pn.xoff + sg.xoff) << 1) | (sg.flags & S_GATHER ? 1 : 0);
                blob.push_back(sg.src);
                blob.push_back((int64_t)(uint32_t)sg.len | (code << 32));
            }
        }
        if (blob.size() - base > max_words)
            throw ApiError(H2W_ERR_STATE, "internal: target record exceeds the shared-memory record size");
        roff.push_back((int64_t)blob.size());
    }
    pstart.clear();
    for (auto &ph : phases) pstart.push_back(ph.t0);
    pstart.push_back(phases.empty() ? 0 : phases.back().t1);
}

// An accumulating target that is the first (in stored order, the order of
// the dependencies and phases) to write its rows adds onto the zeroed
// workspace: it becomes an overwrite and its epilogue reads nothing. Scatter
// targets write the result, not the workspace; atomic parts of a
// column-split row keep their atomics.
void first_writers_overwrite(const std::vector<int64_t> &roff, std::vector<int64_t> &blob, int64_t ws_n,
                             const std::vector<std::pair<int64_t, int64_t>> *prewritten = nullptr) {
    std::vector<uint8_t> written((size_t)ws_n, 0);
    if (prewritten)  // rows written before the stream runs (the far M2L kernel)
        for (const auto &r : *prewritten)
            for (int64_t q = r.first; q < r.second; ++q) written[(size_t)q] = 1;
    for (size_t t = 0; t + 1 < roff.size(); ++t) {
        const size_t o = (size_t)roff[t];
        const int64_t dst = blob[o], nrows = blob[o + 1] & 0xffffffff;
        int64_t flags = blob[o + 1] >> 32;
        if ((flags & T_ACCUM) && !(flags & T_ATOMIC)) {
            bool any = false;
            for (int64_t r = dst; r < dst + nrows && !any; ++r) any = written[(size_t)r] != 0;
            if (!any) {
                flags &= ~(int64_t)T_ACCUM;
                blob[o + 1] = nrows | (flags << 32);
            }
        }
        if (!(flags & T_SCATTER))
            for (int64_t r = dst; r < dst + nrows; ++r) written[(size_t)r] = 1;
    }
}

// Within a phase (and in the dataflow launch, between targets with no
// dependency) targets run concurrently, so non-atomic writers of the same
// workspace rows in one phase would race, and one that first_writers_overwrite
// turned into an overwrite would drop the other's terms. The tree passes never
// produce such a pair; this check makes a plan that did fail loudly.
void check_phase_writers(const std::vector<int64_t> &roff, const std::vector<int64_t> &blob,
                         const std::vector<Phase> &phases) {
    std::vector<std::pair<int64_t, int64_t>> w;
    for (const Phase &ph : phases) {
        w.clear();
        for (int64_t t = ph.t0; t < ph.t1; ++t) {
            const size_t o = (size_t)roff[(size_t)t];
            const int64_t dst = blob[o], nrows = blob[o + 1] & 0xffffffff, flags = blob[o + 1] >> 32;
            if ((flags & T_ATOMIC) || (flags & T_SCATTER)) continue;
            w.push_back({dst, dst + nrows});
        }
        std::sort(w.begin(), w.end());
        for (size_t q = 1; q < w.size(); ++q)
            if (w[q].first < w[q - 1].second)
                throw ApiError(H2W_ERR_STATE, "internal: two non-atomic targets of one phase write the same rows");
    }
}

// (Re)cut the single-vector target stream: row chunks of max(4,
// row_split / width) rows, column splits past XW_CAP; per-phase byte counts
// Producer -> consumer dependencies between the targets of a stream, over the
// workspace rows they touch, for the dataflow launch (no grid barriers). In
// target order (the phase order, a topological order of the tree passes):
// a target that reads rows (gathered sources, or its destination when it
// accumulates) depends on the earlier writers of those rows since the last
// overwrite; a target that writes rows depends on the earlier writers (an
// atomic writer: only on the last non-atomic one, atomic additions commute)
// and on the earlier readers since the last overwrite. Output: cnt[t]
// producers, and the consumers of each target in CSR (coff, cidx). Every
// dependency points from a lower target index to a higher one.
void build_deps(const PlanBuilder &pb, int64_t ws_n, std::vector<int32_t> &cnt, std::vector<int64_t> &coff,
                std::vector<int32_t> &cidx) {
    const size_t nt = pb.T.size();
    std::vector<int32_t> last_nw((size_t)ws_n, -1);
    std::vector<std::vector<int32_t>> atom((size_t)ws_n), rd((size_t)ws_n);
    std::vector<std::vector<int32_t>> prod(nt);
    std::vector<int32_t> deps, rows_read;
    for (size_t t = 0; t < nt; ++t) {
        const Target &tg = pb.T[t];
        const bool scatter = tg.flags & T_SCATTER, atomic = tg.flags & T_ATOMIC, accum = tg.flags & T_ACCUM;
        deps.clear();
        rows_read.clear();
        auto read_row = [&](int64_t r) {
            if (last_nw[(size_t)r] >= 0) deps.push_back(last_nw[(size_t)r]);
            for (int32_t a : atom[(size_t)r]) deps.push_back(a);
            rows_read.push_back((int32_t)r);
        };
        for (int32_t q = tg.p0; q < tg.p1; ++q) {
            const Panel &pn = pb.P[(size_t)q];
            for (int32_t e = pn.s0; e < pn.s1; ++e) {
                const Seg &sg = pb.S[(size_t)e];
                if (sg.flags & S_GATHER) continue;  // the input vector: no producer
                for (int64_t r = sg.src; r < sg.src + sg.len; ++r) read_row(r);
            }
        }
        if (accum)
            for (int64_t r = tg.dst; r < tg.dst + tg.nrows; ++r) read_row(r);
        if (!scatter)
            for (int64_t r = tg.dst; r < tg.dst + tg.nrows; ++r) {
                if (last_nw[(size_t)r] >= 0) deps.push_back(last_nw[(size_t)r]);
                if (!atomic)
                    for (int32_t a : atom[(size_t)r]) deps.push_back(a);
                for (int32_t a : rd[(size_t)r]) deps.push_back(a);
            }
        std::sort(deps.begin(), deps.end());
        deps.erase(std::unique(deps.begin(), deps.end()), deps.end());
        deps.erase(std::remove(deps.begin(), deps.end(), (int32_t)t), deps.end());
        prod[t] = deps;
        for (int32_t r : rows_read) rd[(size_t)r].push_back((int32_t)t);
        if (!scatter)
            for (int64_t r = tg.dst; r < tg.dst + tg.nrows; ++r) {
                if (atomic) {
                    atom[(size_t)r].push_back((int32_t)t);
                } else {
                    last_nw[(size_t)r] = (int32_t)t;
                    atom[(size_t)r].clear();
                    rd[(size_t)r].clear();
                }
            }
    }
    cnt.assign(nt, 0);
    coff.assign(nt + 1, 0);
    for (size_t t = 0; t < nt; ++t) {
        cnt[t] = (int32_t)prod[t].size();
        for (int32_t u : prod[t]) {
            if (u < 0 || (size_t)u >= t) throw ApiError(H2W_ERR_STATE, "dataflow dependency against the target order");
            ++coff[(size_t)u + 1];
        }
    }
    for (size_t t = 0; t < nt; ++t) coff[t + 1] += coff[t];
    cidx.assign((size_t)coff[nt], 0);
    std::vector<int64_t> fill(coff.begin(), coff.end() - 1);
    for (size_t t = 0; t < nt; ++t)
        for (int32_t u : prod[t]) cidx[(size_t)fill[(size_t)u]++] = (int32_t)t;
}

// for the profiling statistics.
void realize_single(h2w_handle *h, int64_t row_split) {
    if (!h->plan) throw ApiError(H2W_ERR_STATE, "operator not assembled");
    h->eta_single = -1.0;  // new cuts, new rounding: calibrate again
    if (row_split < 256 || row_split > (int64_t(1) << 24)) throw ApiError(H2W_ERR_ARG, "row split out of range");
    PlanBuilder &pb = *h->plan;
    std::vector<int64_t> roff, blob, pstart;
    pb.realize(row_split, 4, XW_CAP);
    assign_phases(h, pb, h->nph_total, h->phases, h->fused_scatter);
    h->ph_op.assign(h->phases.size(), 0);
    h->ph_vec.assign(h->phases.size(), 0);
    for (size_t pi = 0; pi < h->phases.size(); ++pi) {
        const Phase &ph = h->phases[pi];
        for (int64_t q = ph.t0; q < ph.t1; ++q) {
            const Target &tg = pb.T[(size_t)q];
            h->ph_vec[pi] += (int64_t)tg.nrows * ((tg.flags & (T_ACCUM | T_ATOMIC)) ? 2 : 1);
            for (int32_t p = tg.p0; p < tg.p1; ++p) {
                const Panel &pn = pb.P[(size_t)p];
                h->ph_op[pi] += (int64_t)tg.nrows * pn.w;
                for (int32_t e = pn.s0; e < pn.s1; ++e) h->ph_vec[pi] += pb.S[(size_t)e].len;
            }
        }
    }
    validate_plan(pb, h, h->phases);
    pack_records(pb, h->phases, roff, blob, pstart);
    first_writers_overwrite(roff, blob, h->ws_n, h->fly_active ? &h->fly_rows : nullptr);
    check_phase_writers(roff, blob, h->phases);
    {
        // FP32 records on the slice-contiguous copy: panel q of target t reads its
        // rows from slice (a', pad4(nrows)) instead of (a, lda); slices 16-byte aligned
        std::vector<int64_t> bs(blob), sl;
        int64_t off = 0;
        for (size_t t = 0; t + 1 < roff.size(); ++t) {
            const int64_t o = roff[t];
            const int64_t nrows = bs[(size_t)o + 1] & 0xffffffff, np = bs[(size_t)o + 2] & 0xffffffff;
            const int64_t ld = pad4(nrows);
            for (int64_t q = 0; q < np; ++q) {
                const size_t wa = (size_t)(o + 3 + 3 * q), wl = wa + 1;
                const int64_t a = bs[wa], lda = bs[wl] & 0xffffffff, w = bs[wl] >> 32;
                sl.insert(sl.end(), {a, lda, nrows, w, off, ld});
                bs[wa] = off;
                bs[wl] = (int64_t)(uint32_t)ld | (w << 32);
                off += pad4(ld * w);
            }
        }
        h->d_blob_s.upload(bs, h->stream);
        h->d_sslices.upload(sl, h->stream);
        h->op32s_n = off;
        h->op32s_ready = false;
        h->d_op32s.reset();
    }
    // the far M2L kernel runs between the upward passes (logical phases <= L)
    // and the downward ones (>= L + 1)
    h->fly_split = (int)h->phases.size();
    for (size_t q = 0; q < h->phases.size(); ++q)
        if (h->phases[q].logical >= h->tree.nL + 1) {
            h->fly_split = (int)q;
            break;
        }
    {
        std::vector<int32_t> cnt, cidx;
        std::vector<int64_t> coff;
        build_deps(pb, h->ws_n, cnt, coff, cidx);
        h->d_sdep0.upload(cnt, h->stream);
        h->d_sdep.alloc(cnt.size());
        h->d_scoff.upload(coff, h->stream);
        h->d_scidx.upload(cidx, h->stream);
        if (!h->d_sctr.p) h->d_sctr.alloc(1);
    }
    cudaStream_t st = h->stream;
    h->d_roff.upload(roff, st);
    h->d_blob.upload(blob, st);
    h->d_pstart.upload(pstart, st);
    h->row_split = row_split;
    pb.T = std::vector<Target>();
    pb.P = std::vector<Panel>();
    pb.S = std::vector<Seg>();
    CK(cudaStreamSynchronize(st));
}

// (Re)cut the multi-vector target stream from the handle's logical targets:
// 64-row targets of at most `cap` gathered columns; records, phase starts and
// per-phase counters uploaded. Cheaper than a new assembly (host work and a
// few small uploads); the operator itself is untouched.
void realize_multi(h2w_handle *h, int64_t cap) {
    if (!h->plan) throw ApiError(H2W_ERR_STATE, "operator not assembled");
    h->eta_multi = -1.0;
    if (cap < 32 || cap > MR_XS_ELEMS || cap % 4) throw ApiError(H2W_ERR_ARG, "multi-vector column cap out of range");
    PlanBuilder &pb = *h->plan;
    std::vector<int64_t> roff, blob, pstart;
    pb.realize(0, MR_ROWS, cap);
    assign_phases(h, pb, h->nph_total, h->mphases, h->fused_scatter_m);
    validate_plan(pb, h, h->mphases);
    pack_records(pb, h->mphases, roff, blob, pstart);
    if (roff.size() != pb.T.size() + 1) throw ApiError(H2W_ERR_STATE, "internal: multi-vector records not packed");
    first_writers_overwrite(roff, blob, h->ws_n);
    check_phase_writers(roff, blob, h->mphases);
    {
        const int64_t mt = 64, kc = 32, wr = 8;  // the kernel's row tile, column chunk and rows per warp
        int64_t *ms = h->mstats;
        std::fill(ms, ms + 6, int64_t(0));
        ms[0] = (int64_t)pb.T.size();
        for (const Target &t : pb.T) {
            const int64_t rows = (int64_t)t.nrows / mt * mt + ((int64_t)t.nrows % mt + wr - 1) / wr * wr;
            int64_t w = 0, chunked = 0;
            for (int32_t q = t.p0; q < t.p1; ++q) {
                const Panel &p = pb.P[(size_t)q];
                w += p.w;
                chunked += ((int64_t)p.w + kc - 1) / kc * kc;
            }
            ms[1] += t.p1 - t.p0;
            ms[2] += (int64_t)t.nrows * w;
            ms[3] += rows * chunked;
            ms[4] += (t.flags & T_ATOMIC) ? 1 : 0;
            ms[5] += ((int64_t)t.nrows + mt - 1) / mt * mt * chunked;
        }
    }
    {
        std::vector<int32_t> cnt, cidx;
        std::vector<int64_t> coff;
        build_deps(pb, h->ws_n, cnt, coff, cidx);
        h->d_mdep0.upload(cnt, h->stream);
        h->d_mdep.alloc(cnt.size());
        h->d_mcoff.upload(coff, h->stream);
        h->d_mcidx.upload(cidx, h->stream);
        h->mflow_edges = (int64_t)cidx.size();
    }
    cudaStream_t st = h->stream;
    h->d_roff_m.upload(roff, st);
    h->d_blob_m.upload(blob, st);
    h->d_pstart_m.upload(pstart, st);
    {
        // slice-contiguous copy for the warp-specialised FP32 product: each
        // target's panel slice (its <= 64 rows of a stored block) moves to its
        // own column-major block at leading dimension pad4(rows), so a chunk of
        // 32 columns is one contiguous copy
        std::vector<int64_t> bw = blob, sl;
        int64_t off = 0;
        for (size_t t = 0; t + 1 < roff.size(); ++t) {
            const int64_t o = roff[t];
            const int64_t rows = blob[(size_t)o + 1] & 0xffffffff, np = blob[(size_t)o + 2] & 0xffffffff;
            const int64_t ld = pad4(rows);
            for (int64_t q = 0; q < np; ++q) {
                const size_t pw = (size_t)(o + 3 + 3 * q);
                const int64_t a = blob[pw], lda = blob[pw + 1] & 0xffffffff, w = blob[pw + 1] >> 32;
                sl.insert(sl.end(), {a, lda, rows, w, off, ld});
                bw[pw] = off;
                bw[pw + 1] = ld | (w << 32);
                off += ld * w;
            }
        }
        h->d_blob_mw.upload(bw, st);
        h->d_mslices.upload(sl, st);
        h->op32m_n = off;
        h->op32m_ready = false;
    }
    h->d_mctr.alloc(std::max<size_t>(h->mphases.size(), 1));
    h->ph_t0.clear();
    h->ph_t1.clear();
    for (const Phase &ph : h->mphases) {
        h->ph_t0.push_back(ph.t0);
        h->ph_t1.push_back(ph.t1);
    }
    h->mr_xw = cap;
    pb.T = std::vector<Target>();
    pb.P = std::vector<Panel>();
    pb.S = std::vector<Seg>();
    CK(cudaStreamSynchronize(st));
}

void build_plan(h2w_handle *h) {
    Tree &t = h->tree;
    const int L = t.nL, dim = t.dim;
    const bool nested = h->cfg.form == H2W_FORM_NESTED;
    // H* (non-nested) has no nested far field: every interaction-list pair is a pair
    const bool has_far = dim > 1 && h->cfg.form != H2W_FORM_NONNESTED;
    const bool has_ver = nested;
    const bool has_pairs = !nested;
    auto pbp = std::make_shared<PlanBuilder>();
    PlanBuilder &pb = *pbp;
    pb.h = h;
    h->fused_scatter = h->fused_scatter_m = true;

    // ---- workspace layout
    int64_t wsn = 0;
    h->yperm_off = wsn;
    wsn += t.N;
    std::vector<int64_t> fo((size_t)L + 2, 0), fi((size_t)L + 2, 0), vo((size_t)L + 2, 0), vi((size_t)L + 2, 0),
        to((size_t)L + 2, 0);
    std::vector<std::vector<int64_t>> poff((size_t)L + 1);
    for (int j = 1; j <= L; ++j) {
        if (has_far && j >= 2) {
            int64_t R = (int64_t)h->far[(size_t)j].chk.size();
            fo[(size_t)j] = wsn; wsn += R;
            fi[(size_t)j] = wsn; wsn += R;
        }
        if (has_ver) {
            int64_t R = (int64_t)h->ver[(size_t)j].chk.size();
            vo[(size_t)j] = wsn; wsn += R;
            vi[(size_t)j] = wsn; wsn += R;
        }
        if (has_pairs) {
            to[(size_t)j] = wsn;
            wsn += (int64_t)h->pairs[(size_t)j].row.size();
        }
    }
    h->ws_n = wsn;
    auto leaf_gather = [&](int j, int64_t q, int32_t xoff) {
        Seg s{};
        s.src = t.off[(size_t)j][(size_t)q];
        s.len = (int32_t)t.cnt(j, q);
        s.xoff = xoff;
        s.flags = S_GATHER;
        return s;
    };
    auto ws_seg = [&](int64_t src, int64_t len, int32_t xoff) {
        Seg s{};
        s.src = src;
        s.len = (int32_t)len;
        s.xoff = xoff;
        s.flags = S_WS;
        return s;
    };

    // ---- transfer matrices (far and vertex / 1D nested)
    struct Xfer { int64_t up = -1, dn = -1; int32_t ldu = 0, ldd = 0, rows = 0, r = 0; };
    std::vector<std::vector<Xfer>> fx((size_t)L + 1), vx((size_t)L + 1);
    auto make_xfer = [&](const Skel &s, int64_t k, const std::vector<int32_t> &rows, Xfer &x) {
        int32_t r = (int32_t)s.rank(k);
        x.r = r;
        x.rows = (int32_t)rows.size();
        if (r == 0 || rows.empty()) return;
        FactorJob fj{};
        fj.f = pb.fn;
        pb.fn += (int64_t)r * r;
        fj.ii = pb.put_idx(s.chk.data() + s.ptr[(size_t)k], r);
        fj.jj = pb.put_idx(s.chg.data() + s.ptr[(size_t)k], r);
        fj.r = r;
        pb.factors.push_back(fj);
        x.up = pb.alloc(r, x.rows, x.ldu);
        x.dn = pb.alloc(x.rows, r, x.ldd);
        XferJob xj{};
        xj.f = fj.f;
        xj.jj = fj.jj;
        xj.pi = pb.put_idx(rows);
        xj.a1 = x.dn;
        xj.ld1 = x.ldd;
        xj.a2 = x.up;
        xj.ld2 = x.ldu;
        xj.r = r;
        xj.n = x.rows;
        xj.mode = X_ROW_RL;
        pb.xfers.push_back(xj);
        pb.max_xfer_n = std::max(pb.max_xfer_n, x.rows);
    };
    for (int j = 1; j <= L; ++j) {
        const int64_t nb = t.nbox[(size_t)j];
        if (has_far && j >= 2) {
            fx[(size_t)j].resize((size_t)nb);
            for (int64_t k = 0; k < nb; ++k) make_xfer(h->far[(size_t)j], k, far_rows(h, j, k), fx[(size_t)j][(size_t)k]);
        }
        if (has_ver) {
            vx[(size_t)j].resize((size_t)nb);
            for (int64_t k = 0; k < nb; ++k) make_xfer(h->ver[(size_t)j], k, ver_rows(h, j, k), vx[(size_t)j][(size_t)k]);
        }
    }
    auto child_off = [&](const Skel &s, int64_t k) { return s.ptr[(size_t)(k * t.nch)]; };
    auto child_len = [&](const Skel &s, int64_t k) { return s.ptr[(size_t)((k + 1) * t.nch)] - s.ptr[(size_t)(k * t.nch)]; };

    // Phase windows (2L+1 phases): up_j at L-j; M2L_j within [L-j+1, L+j-2]
    // (level 1: L); down_j at L+j; leaf at 2L; near field and pair phase A
    // anywhere before the leaf phase. Flexible targets are spread later.
    const int NPH = 2 * L + 1;
    // ---- UP phases, levels L..1
    for (int j = L; j >= 1; --j) {
        pb.lo = pb.hi = L - j;
        for (int kind = 0; kind < 2; ++kind) {
            if (kind == 0 && !(has_far && j >= 2)) continue;
            if (kind == 1 && !has_ver) continue;
            const Skel &s = kind == 0 ? h->far[(size_t)j] : h->ver[(size_t)j];
            const auto &X = kind == 0 ? fx[(size_t)j] : vx[(size_t)j];
            const int64_t outb = kind == 0 ? fo[(size_t)j] : vo[(size_t)j];
            for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
                const Xfer &x = X[(size_t)k];
                if (x.up < 0) continue;
                PlanBuilder::PanelSpec ps;
                ps.a = x.up;
                ps.lda = x.ldu;
                ps.w = x.rows;
                if (j == L) ps.segs.push_back(leaf_gather(j, k, 0));
                else {
                    const Skel &cs = kind == 0 ? h->far[(size_t)j + 1] : h->ver[(size_t)j + 1];
                    const int64_t cb = kind == 0 ? fo[(size_t)j + 1] : vo[(size_t)j + 1];
                    ps.segs.push_back(ws_seg(cb + child_off(cs, k), child_len(cs, k), 0));
                }
                pb.emit(outb + s.ptr[(size_t)k], x.r, T_ACCUM, {ps});
            }
        }
    }

    // ---- coupling phase: M2L (far, vertex), near field, pair phase A
    std::vector<std::vector<int64_t>> pfac((size_t)L + 1);
    // far M2L on the fly: its work items instead of stored blocks
    const bool fly = h->far_fly && has_far && L >= 2 && !h->cplx;
    h->fly_active = fly;
    h->fly_rows.clear();
    h->fly_entries = 0;
    std::vector<FlyItem> fitems;
    std::vector<int32_t> frow, fcpid, fcws;
    if (fly) {
        for (int j = 2; j <= L; ++j) {
            const Skel &s = h->far[(size_t)j];
            for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
                const int32_t r = (int32_t)s.rank(k);
                if (r == 0) continue;
                const int64_t cbeg = (int64_t)fcpid.size();
                for (int64_t e = t.ilp[(size_t)j][(size_t)k]; e < t.ilp[(size_t)j][(size_t)k + 1]; ++e) {
                    if (t.ilv[(size_t)j][(size_t)e]) continue;
                    const int32_t q = t.il[(size_t)j][(size_t)e];
                    for (int64_t i = s.ptr[(size_t)q]; i < s.ptr[(size_t)q + 1]; ++i) {
                        fcpid.push_back(s.chk[(size_t)i]);
                        const int64_t w = fo[(size_t)j] + i;
                        if (w > INT32_MAX) throw ApiError(H2W_ERR_STATE, "workspace too large for the far M2L kernel");
                        fcws.push_back((int32_t)w);
                    }
                }
                const int64_t nc = (int64_t)fcpid.size() - cbeg;
                if (nc == 0) continue;
                if (nc > INT32_MAX) throw ApiError(H2W_ERR_STATE, "far M2L source set too large");
                const int64_t rbeg = (int64_t)frow.size();
                append(frow, s.chk.data() + s.ptr[(size_t)k], r);
                const int nb = (r + FLY_ROWS - 1) / FLY_ROWS, per = (r + nb - 1) / nb;
                for (int32_t r0 = 0; r0 < r; r0 += per) {
                    FlyItem it{};
                    it.dst = fi[(size_t)j] + s.ptr[(size_t)k] + r0;
                    it.rows = rbeg + r0;
                    it.cbeg = cbeg;
                    it.nrows = std::min(per, r - r0);
                    it.ncols = (int32_t)nc;
                    fitems.push_back(it);
                }
                h->fly_rows.push_back({fi[(size_t)j] + s.ptr[(size_t)k], fi[(size_t)j] + s.ptr[(size_t)k] + r});
                h->fly_entries += (int64_t)r * nc;
            }
        }
        // bounds of every item against its buffers before any upload
        for (const FlyItem &it : fitems) {
            if (it.nrows < 1 || it.nrows > FLY_ROWS || it.ncols < 1 || it.dst < 0 || it.dst + it.nrows > wsn ||
                it.rows < 0 || it.rows + it.nrows > (int64_t)frow.size() || it.cbeg < 0 ||
                it.cbeg + it.ncols > (int64_t)fcpid.size())
                throw ApiError(H2W_ERR_STATE, "internal: far M2L work item out of range");
        }
        for (int32_t v : frow)
            if (v < 0 || v >= t.N) throw ApiError(H2W_ERR_STATE, "internal: far M2L row point out of range");
        for (size_t i = 0; i < fcpid.size(); ++i)
            if (fcpid[i] < 0 || fcpid[i] >= t.N || fcws[i] < 0 || fcws[i] >= wsn)
                throw ApiError(H2W_ERR_STATE, "internal: far M2L source out of range");
        // largest first for the persistent grid
        std::stable_sort(fitems.begin(), fitems.end(), [](const FlyItem &a, const FlyItem &b) {
            return (int64_t)a.nrows * a.ncols > (int64_t)b.nrows * b.ncols;
        });
    }
    {
        for (int j = 1; j <= L; ++j) {
            pb.lo = L - j + 1;
            pb.hi = j == 1 ? L : L + j - 2;
            for (int kind = 0; kind < 2; ++kind) {
                if (kind == 0 && !(has_far && j >= 2)) continue;
                if (kind == 0 && fly) continue;  // evaluated by the far M2L kernel
                if (kind == 1 && !has_ver) continue;
                const Skel &s = kind == 0 ? h->far[(size_t)j] : h->ver[(size_t)j];
                const int64_t outb = kind == 0 ? fo[(size_t)j] : vo[(size_t)j];
                const int64_t inb = kind == 0 ? fi[(size_t)j] : vi[(size_t)j];
                for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
                    int32_t r = (int32_t)s.rank(k);
                    if (r == 0) continue;
                    std::vector<int32_t> srcs;
                    if (dim == 1) {
                        for (int sl = 0; sl < 2; ++sl) {
                            int32_t q = t.nb[(size_t)j][(size_t)(k * 2 + sl)];
                            if (q != -1) srcs.push_back(q);
                        }
                    } else {
                        for (int64_t e = t.ilp[(size_t)j][(size_t)k]; e < t.ilp[(size_t)j][(size_t)k + 1]; ++e)
                            if ((bool)t.ilv[(size_t)j][(size_t)e] == (kind == 1)) srcs.push_back(t.il[(size_t)j][(size_t)e]);
                    }
                    int64_t W = 0;
                    for (int32_t q : srcs) W += s.rank(q);
                    if (W == 0) continue;
                    PlanBuilder::PanelSpec ps;
                    ps.a = pb.alloc(r, W, ps.lda);
                    ps.w = (int32_t)W;
                    int64_t ri = pb.put_idx(s.chk.data() + s.ptr[(size_t)k], r);
                    int32_t co = 0;
                    for (int32_t q : srcs) {
                        int32_t rq = (int32_t)s.rank(q);
                        if (rq == 0) continue;
                        ps.segs.push_back(ws_seg(outb + s.ptr[(size_t)q], rq, co));
                        FillJob fj{};
                        fj.a = ps.a + (int64_t)co * ps.lda;
                        fj.ri = ri;
                        fj.ci = pb.put_idx(s.chk.data() + s.ptr[(size_t)q], rq);
                        fj.nr = r;
                        fj.nc = rq;
                        fj.lda = ps.lda;
                        pb.fills.push_back(fj);
                        co += rq;
                    }
                    pb.emit(inb + s.ptr[(size_t)k], r, T_ACCUM, {ps});
                }
            }
        }
        // near field: neighbour slots in order, then self (assemble_NearField)
        pb.lo = 0;
        pb.hi = NPH - 2;
        for (int64_t k = 0; k < t.nbox[(size_t)L]; ++k) {
            int32_t n = (int32_t)t.cnt(L, k);
            if (n == 0) continue;
            std::vector<int32_t> srcs;
            if (dim > 1)
                for (int sl = 0; sl < t.nnb; ++sl) {
                    int32_t q = t.nb[(size_t)L][(size_t)(k * t.nnb + sl)];
                    if (q != -1) srcs.push_back(q);
                }
            srcs.push_back((int32_t)k);
            int64_t W = 0;
            for (int32_t q : srcs) W += t.cnt(L, q);
            PlanBuilder::PanelSpec ps;
            ps.a = pb.alloc(n, W, ps.lda);
            ps.w = (int32_t)W;
            int64_t ri = pb.put_idx(t.perm.data() + t.off[(size_t)L][(size_t)k], n);
            int32_t co = 0;
            for (int32_t q : srcs) {
                int32_t nq = (int32_t)t.cnt(L, q);
                if (nq == 0) continue;
                ps.segs.push_back(leaf_gather(L, q, co));
                FillJob fj{};
                fj.a = ps.a + (int64_t)co * ps.lda;
                fj.ri = ri;
                fj.ci = pb.put_idx(t.perm.data() + t.off[(size_t)L][(size_t)q], nq);
                fj.nr = n;
                fj.nc = nq;
                fj.lda = ps.lda;
                pb.fills.push_back(fj);
                co += nq;
            }
            pb.emit(h->yperm_off + t.off[(size_t)L][(size_t)k], n, T_ACCUM, {ps});
        }
        // pair phase A: t_p = G_p x_q with G = R^-1 L^-1 K(I, q) (2D/3D) or V^T = L^-1 K(I, q) (1D)
        if (has_pairs)
            for (int j = 1; j <= L; ++j) {
                Pairs &Pp = h->pairs[(size_t)j];
                pfac[(size_t)j].assign(Pp.box.size(), -1);
                for (size_t p = 0; p < Pp.box.size(); ++p) {
                    int32_t r = (int32_t)(Pp.ptr[p + 1] - Pp.ptr[p]);
                    int32_t q = Pp.other[p];
                    int32_t nq = (int32_t)t.cnt(j, q);
                    if (r == 0 || nq == 0) continue;
                    FactorJob fj{};
                    fj.f = pb.fn;
                    pb.fn += (int64_t)r * r;
                    fj.ii = pb.put_idx(Pp.row.data() + Pp.ptr[p], r);
                    fj.jj = pb.put_idx(Pp.col.data() + Pp.ptr[p], r);
                    fj.r = r;
                    pb.factors.push_back(fj);
                    pfac[(size_t)j][p] = fj.f;
                    PlanBuilder::PanelSpec ps;
                    ps.a = pb.alloc(r, nq, ps.lda);
                    ps.w = nq;
                    ps.segs.push_back(leaf_gather(j, q, 0));
                    XferJob xj{};
                    xj.f = fj.f;
                    xj.jj = fj.ii;  // column modes read K(I, p)
                    xj.pi = pb.put_idx(t.perm.data() + t.off[(size_t)j][(size_t)q], nq);
                    xj.a1 = ps.a;
                    xj.ld1 = ps.lda;
                    xj.a2 = -1;
                    xj.r = r;
                    xj.n = nq;
                    xj.mode = dim == 1 ? X_COL_L : X_COL_LR;
                    pb.xfers.push_back(xj);
                    pb.max_xfer_n = std::max(pb.max_xfer_n, nq);
                    pb.emit(to[(size_t)j] + Pp.ptr[p], r, T_ACCUM, {ps});
                }
            }
    }

    // ---- pair phase B matrices per box: [Ac_p1 | Ac_p2 | ...] (n_box x sum r_p)
    struct BMat { int64_t a = -1; int32_t lda = 0, w = 0; std::vector<Seg> segs; };
    std::vector<std::vector<BMat>> bm((size_t)L + 1);
    if (has_pairs)
        for (int j = 1; j <= L; ++j) {
            bm[(size_t)j].resize((size_t)t.nbox[(size_t)j]);
            Pairs &Pp = h->pairs[(size_t)j];
            // pairs are grouped by box in ascending box order
            size_t p = 0;
            while (p < Pp.box.size()) {
                int32_t k = Pp.box[p];
                size_t p1 = p;
                int64_t W = 0;
                while (p1 < Pp.box.size() && Pp.box[p1] == k) { W += Pp.ptr[p1 + 1] - Pp.ptr[p1]; ++p1; }
                int32_t n = (int32_t)t.cnt(j, k);
                BMat &B = bm[(size_t)j][(size_t)k];
                if (W > 0 && n > 0) {
                    B.a = pb.alloc(n, W, B.lda);
                    B.w = (int32_t)W;
                    int64_t ri = pb.put_idx(t.perm.data() + t.off[(size_t)j][(size_t)k], n);
                    int32_t co = 0;
                    for (size_t q = p; q < p1; ++q) {
                        int32_t r = (int32_t)(Pp.ptr[q + 1] - Pp.ptr[q]);
                        if (r == 0) continue;
                        B.segs.push_back(ws_seg(to[(size_t)j] + Pp.ptr[q], r, co));
                        if (dim == 1) {
                            // U = K(box, J) R^-1 with the pair's factors (1D ACA_only_nodesUV)
                            XferJob xj{};
                            xj.f = pfac[(size_t)j][q];
                            xj.jj = pb.put_idx(Pp.col.data() + Pp.ptr[q], r);
                            xj.pi = ri;
                            xj.a1 = B.a + (int64_t)co * B.lda;
                            xj.ld1 = B.lda;
                            xj.a2 = -1;
                            xj.r = r;
                            xj.n = n;
                            xj.mode = X_ROW_R;
                            if (xj.f >= 0) pb.xfers.push_back(xj);
                            pb.max_xfer_n = std::max(pb.max_xfer_n, n);
                        } else {
                            FillJob fj{};
                            fj.a = B.a + (int64_t)co * B.lda;
                            fj.ri = ri;
                            fj.ci = pb.put_idx(Pp.col.data() + Pp.ptr[q], r);
                            fj.nr = n;
                            fj.nc = r;
                            fj.lda = B.lda;
                            pb.fills.push_back(fj);
                        }
                        co += r;
                    }
                }
                p = p1;
            }
        }
    // ---- DOWN phases, levels 1..L-1, then the leaf phase
    for (int j = 1; j < L; ++j) {
        pb.lo = pb.hi = L + j;
        for (int kind = 0; kind < 2; ++kind) {
            if (kind == 0 && !(has_far && j >= 2)) continue;
            if (kind == 1 && !has_ver) continue;
            const Skel &s = kind == 0 ? h->far[(size_t)j] : h->ver[(size_t)j];
            const Skel &cs = kind == 0 ? h->far[(size_t)j + 1] : h->ver[(size_t)j + 1];
            const auto &X = kind == 0 ? fx[(size_t)j] : vx[(size_t)j];
            const int64_t inb = kind == 0 ? fi[(size_t)j] : vi[(size_t)j];
            const int64_t cinb = kind == 0 ? fi[(size_t)j + 1] : vi[(size_t)j + 1];
            for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
                const Xfer &x = X[(size_t)k];
                if (x.dn < 0) continue;
                PlanBuilder::PanelSpec ps;
                ps.a = x.dn;
                ps.lda = x.ldd;
                ps.w = x.r;
                ps.segs.push_back(ws_seg(inb + s.ptr[(size_t)k], x.r, 0));
                pb.emit(cinb + child_off(cs, k), x.rows, T_ACCUM, {ps});
            }
        }
    }
    {
        pb.lo = pb.hi = NPH - 1;
        for (int64_t k = 0; k < t.nbox[(size_t)L]; ++k) {
            int32_t n = (int32_t)t.cnt(L, k);
            if (n == 0) continue;
            std::vector<PlanBuilder::PanelSpec> pans;
            if (has_far && L >= 2 && fx[(size_t)L][(size_t)k].dn >= 0) {
                const Xfer &x = fx[(size_t)L][(size_t)k];
                PlanBuilder::PanelSpec ps;
                ps.a = x.dn;
                ps.lda = x.ldd;
                ps.w = x.r;
                ps.segs.push_back(ws_seg(fi[(size_t)L] + h->far[(size_t)L].ptr[(size_t)k], x.r, 0));
                pans.push_back(ps);
            }
            if (has_ver && vx[(size_t)L][(size_t)k].dn >= 0) {
                const Xfer &x = vx[(size_t)L][(size_t)k];
                PlanBuilder::PanelSpec ps;
                ps.a = x.dn;
                ps.lda = x.ldd;
                ps.w = x.r;
                ps.segs.push_back(ws_seg(vi[(size_t)L] + h->ver[(size_t)L].ptr[(size_t)k], x.r, 0));
                pans.push_back(ps);
            }
            if (has_pairs)
                for (int j = 1; j <= L; ++j) {
                    int64_t a = k >> (dim * (L - j));
                    const BMat &B = bm[(size_t)j][(size_t)a];
                    if (B.a < 0) continue;
                    PlanBuilder::PanelSpec ps;
                    ps.a = B.a + (t.off[(size_t)L][(size_t)k] - t.off[(size_t)j][(size_t)a]);
                    ps.lda = B.lda;
                    ps.w = B.w;
                    ps.segs = B.segs;
                    pans.push_back(ps);
                }
            pb.emit(h->yperm_off + t.off[(size_t)L][(size_t)k], n, T_ACCUM | T_SCATTER, pans);
        }
    }
    // ---- target streams. Single-vector: fine row chunks (load balance of a
    // GEMV); multi-vector: 64-row chunks, one result tile per target.
    h->nph_total = NPH;
    for (auto &x : pb.xfers)
        if (x.f < 0) throw ApiError(H2W_ERR_STATE, "internal: unresolved factor");
    validate_plan(pb, h, {});  // assembly jobs (no targets realised yet)

    // ---- device buffers and assembly kernels
    cudaStream_t st = h->stream;
    if (fly) {
        h->d_fly_items.upload(fitems, st);
        h->d_fly_rowpid.upload(frow, st);
        h->d_fly_cpid.upload(fcpid, st);
        h->d_fly_cws.upload(fcws, st);
        if (!h->d_fly_ctr.p) h->d_fly_ctr.alloc(1);
        h->d_pts4.alloc((size_t)t.N * 4);
        CK(launch_pts4(h->d_pts.p, dim, t.N, h->d_pts4.p, st));
        h->d_ptsdf.alloc((size_t)t.N * 8);
        CK(launch_ptsdf(h->d_pts.p, dim, t.N, h->d_ptsdf.p, st));
        std::vector<float> lt(128 * 8);
        fly_df_logtab(lt.data());
        h->d_logtab.upload(lt, st);
        CK(cudaStreamSynchronize(st));
        const double a = 0.0001;
        h->k32.c2d = (float)h->c2d;
        h->k32.inv4pi = (float)(1.0 / h->four_pi);
        h->k32.inv_loga = (float)(1.0 / h->loga);
        h->k32.inv_den = (float)(1.0 / h->den_small);
        h->k32.a = (float)a;
        h->k32.a2 = (float)(a * a);
        h->k32.inv_a = (float)(1.0 / a);
        // far boxes are not adjacent: their points are at least the deepest box width apart
        h->k32.sep = 2.0 / std::ldexp(1.0, L) > 2.0 * a ? 1 : 0;
    } else {
        h->d_fly_items.reset();
        h->d_fly_rowpid.reset();
        h->d_fly_cpid.reset();
        h->d_fly_cws.reset();
        h->d_pts4.reset();
        h->d_ptsdf.reset();
        h->d_logtab.reset();
    }
    if (h->cplx) {
        // complex operator image from the same jobs (complex units), then its
        // realified form; the real FP64 product kernels apply it
        DBuf<int32_t> didx;
        DBuf<FillJob> dfill;
        DBuf<FactorJob> dfac;
        DBuf<XferJob> dxf;
        DBuf<double2> dF, opc;
        DBuf<int64_t> dblk;
        didx.upload(pb.idx, st);
        dfill.upload(pb.fills, st);
        dfac.upload(pb.factors, st);
        dxf.upload(pb.xfers, st);
        dF.alloc((size_t)std::max<int64_t>(pb.fn, 1));
        opc.alloc((size_t)std::max<int64_t>(pb.opn, 1));
        CK(cudaMemsetAsync(opc.p, 0, (size_t)std::max<int64_t>(pb.opn, 1) * 16, st));
        CK(launch_assemble_c(dfac.p, (int)pb.factors.size(), dxf.p, (int)pb.xfers.size(), pb.max_xfer_n, dfill.p,
                             (int)pb.fills.size(), didx.p, h->kparams(), dF.p, opc.p, st));
        pb.realify();
        h->ws_n *= 2;
        h->yperm_off *= 2;
        h->op_n = pb.opn;
        h->op_bytes_read = pb.read_elems;
        h->d_op.alloc((size_t)pb.opn);
        CK(cudaMemsetAsync(h->d_op.p, 0, (size_t)pb.opn * 8, st));
        dblk.upload(pb.blocks, st);
        CK(launch_realify(dblk.p, (int64_t)pb.blocks.size() / 3, opc.p, h->d_op.p, st));
        CK(cudaStreamSynchronize(st));
        pb.idx = std::vector<int32_t>();
        pb.fills = std::vector<FillJob>();
        pb.factors = std::vector<FactorJob>();
        pb.xfers = std::vector<XferJob>();
        pb.blocks = std::vector<int64_t>();
        h->plan = pbp;
        realize_single(h, h->row_split);
    } else {
        h->op_n = pb.opn;
        h->op_bytes_read = pb.read_elems;
        h->d_op.alloc((size_t)pb.opn);
        CK(cudaMemsetAsync(h->d_op.p, 0, (size_t)pb.opn * 8, st));
        DBuf<int32_t> didx;
        DBuf<FillJob> dfill;
        DBuf<FactorJob> dfac;
        DBuf<XferJob> dxf;
        DBuf<double> dF;
        didx.upload(pb.idx, st);
        dfill.upload(pb.fills, st);
        dfac.upload(pb.factors, st);
        dxf.upload(pb.xfers, st);
        dF.alloc((size_t)std::max<int64_t>(pb.fn, 1));
        KParams kp = h->kparams();
        CK(launch_factor(dfac.p, (int)pb.factors.size(), didx.p, kp, dF.p, st));
        CK(launch_xfer(dxf.p, (int)pb.xfers.size(), pb.max_xfer_n, didx.p, kp, dF.p, h->d_op.p, st));
        CK(launch_fill(dfill.p, (int)pb.fills.size(), didx.p, kp, h->d_op.p, st));
        // the assembly's index and job lists are not needed again
        pb.idx = std::vector<int32_t>();
        pb.fills = std::vector<FillJob>();
        pb.factors = std::vector<FactorJob>();
        pb.xfers = std::vector<XferJob>();
        h->plan = pbp;
        realize_single(h, h->row_split);
        realize_multi(h, h->mr_xw);
    }
    h->d_ws.alloc((size_t)h->ws_n);
    h->d_ctr.alloc(h->phases.size() + 1);
    h->d_err.alloc(1);
    CK(cudaMemsetAsync(h->d_err.p, 0, 4, st));
    h->d_bar.alloc(2);
    CK(cudaMemsetAsync(h->d_bar.p, 0, 8, st));
    {
        const char *m = getenv("H2W_MATVEC");
        h->coop = !(m && std::string(m) == "phased");
        const char *g = getenv("H2W_GRAPH");
        if (g && std::string(g) == "0") h->use_graphs = false;
    }
    CK(cudaStreamSynchronize(st));
    h->d_op32.reset();
    h->d_opdf.reset();
    h->d_ws32.reset();
    h->d_op32m.reset();
    h->op32m_ready = false;
    h->eta_multi = h->eta_single = -1.0;
}

// Stored-entry count of the reference (findMemory_n / findMemory_sn / findMemory_nn).
double storage_entries(h2w_handle *h) {
    const Tree &t = h->tree;
    const int L = t.nL, dim = t.dim;
    const bool sn = h->cfg.form != H2W_FORM_NESTED;  // per-pair factors: (H2+H)* and H*
    double mem = 0;
    auto nrank = [](const Skel &s, int64_t k) { return (double)s.rank(k); };
    if (dim == 1) {
        for (int j = 1; j <= L; ++j)
            for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
                if (!sn) {
                    const Skel &s = h->ver[(size_t)j];
                    double r = nrank(s, k);
                    if (j == L) mem += 2.0 * r * (double)t.cnt(j, k);
                    else for (int c = 0; c < 2; ++c) mem += 2.0 * r * nrank(h->ver[(size_t)j + 1], 2 * k + c);
                    for (int sl = 0; sl < 2; ++sl) {
                        int32_t q = t.nb[(size_t)j][(size_t)(k * 2 + sl)];
                        if (q != -1) mem += r * nrank(s, q);
                    }
                }
            }
        if (!sn)
            for (int64_t k = 0; k < t.nbox[(size_t)L]; ++k) mem += (double)t.cnt(L, k) * (double)t.cnt(L, k);
        else
            for (int j = 1; j <= L; ++j) {
                const Pairs &P = h->pairs[(size_t)j];
                for (size_t p = 0; p < P.box.size(); ++p) {
                    double r = (double)(P.ptr[p + 1] - P.ptr[p]);
                    mem += r * ((double)t.cnt(j, P.box[p]) + (double)t.cnt(j, P.other[p]));
                }
            }
        return mem;
    }
    // findMemory_nn (2D/codes/HODLR2Dtree.hpp:1307-1328, 3D/codes/HODLR3Dtree.hpp:2561-2583): pairs and near field only
    const bool nn = h->cfg.form == H2W_FORM_NONNESTED;
    for (int j = 2; j <= L && !nn; ++j)
        for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
            const Skel &s = h->far[(size_t)j];
            double r = nrank(s, k);
            if (r > 0) mem += 2.0 * r * (double)far_rows(h, j, k).size();
            for (int64_t e = t.ilp[(size_t)j][(size_t)k]; e < t.ilp[(size_t)j][(size_t)k + 1]; ++e)
                if (!t.ilv[(size_t)j][(size_t)e]) mem += r * nrank(s, t.il[(size_t)j][(size_t)e]);
        }
    if (!sn) {
        for (int j = 1; j <= L; ++j)
            for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
                const Skel &s = h->ver[(size_t)j];
                double r = nrank(s, k);
                if (j == L) mem += 2.0 * r * (double)t.cnt(j, k);
                else for (int c = 0; c < t.nch; ++c) mem += 2.0 * r * nrank(h->ver[(size_t)j + 1], k * t.nch + c);
                for (int64_t e = t.ilp[(size_t)j][(size_t)k]; e < t.ilp[(size_t)j][(size_t)k + 1]; ++e)
                    if (t.ilv[(size_t)j][(size_t)e]) mem += r * nrank(s, t.il[(size_t)j][(size_t)e]);
            }
    } else {
        for (int j = 1; j <= L; ++j) {
            const Pairs &P = h->pairs[(size_t)j];
            for (size_t p = 0; p < P.box.size(); ++p) {
                double r = (double)(P.ptr[p + 1] - P.ptr[p]);
                if (r == 0) continue;
                mem += 2.0 * r * r + r * (double)t.cnt(j, P.box[p]) + r * (double)t.cnt(j, P.other[p]);
            }
        }
    }
    for (int64_t k = 0; k < t.nbox[(size_t)L]; ++k) {
        double n = (double)t.cnt(L, k);
        mem += n * n;
        for (int sl = 0; sl < t.nnb; ++sl) {
            int32_t q = t.nb[(size_t)L][(size_t)(k * t.nnb + sl)];
            if (q != -1) mem += n * (double)t.cnt(L, q);
        }
    }
    return mem;
}

// ---------------------------------------------------------- matvec run ---
cudaEvent_t prof_event(h2w_handle *h) {
    cudaEvent_t e;
    if (!h->ev_pool.empty()) {
        e = h->ev_pool.back();
        h->ev_pool.pop_back();
    } else {
        CK(cudaEventCreate(&e));
    }
    return e;
}

// phase == number of phases: the whole matvec (cooperative launch);
// FLY_PHASE: the far-field M2L kernel of a product with the far field on the fly
constexpr int FLY_PHASE = 1 << 20;
template <class F>
void prof_launch(h2w_handle *h, int prec, int phase, cudaStream_t st, F &&launch) {
    const bool whole = phase >= (int)h->phases.size();
    if (!h->prof || (!whole && h->phases[(size_t)phase].t1 <= h->phases[(size_t)phase].t0)) {
        CK(launch());
        return;
    }
    h2w_handle::ProfRec r{prof_event(h), prof_event(h), prec, phase};
    CK(cudaEventRecord(r.a, st));
    CK(launch());
    CK(cudaEventRecord(r.b, st));
    h->prof_recs.push_back(r);
}

// y = A x. permuted: x and y in leaf order (GMRES works there: no gather or
// scatter per product); otherwise original point order.
// df: with the far field on the fly, its M2L in double-FP32 arithmetic
// (FP64-accurate on the FP32 pipes) where that form exists; the stored passes
// stay FP64.
void run_matvec_f64(h2w_handle *h, const double *dx, double *dy, cudaStream_t st, bool permuted = false,
                    bool df = false) {
    const int32_t *perm = permuted ? nullptr : h->d_perm.p;
    const int nph = (int)h->phases.size();
    CK(cudaMemsetAsync(h->d_ws.p, 0, (size_t)h->ws_n * 8, st));
    if (h->fly_active) {
        // stored passes up to the upward ones, the far M2L kernel, the rest
        auto stored = [&](int a, int b) {
            if (b <= a) return;
            if (h->coop) {
                prof_launch(h, H2W_PREC_FP64, nph, st, [&] {
                    return launch_coop_f64(h->d_roff.p, h->d_blob.p, h->d_pstart.p + a, b - a, h->d_op.p, h->d_ws.p,
                                           dx, dy, perm, h->d_bar.p, h->d_err.p, st, h->spin_limit);
                });
            } else {
                for (int q = a; q < b; ++q) {
                    const Phase &ph = h->phases[(size_t)q];
                    prof_launch(h, H2W_PREC_FP64, q, st, [&] {
                        return launch_brg_f64(h->d_roff.p, h->d_blob.p, ph.t0, ph.t1, h->d_op.p, h->d_ws.p, dx, dy,
                                              perm, st);
                    });
                }
            }
        };
        stored(0, h->fly_split);
        prof_launch(h, df ? H2W_PREC_DF64 : H2W_PREC_FP64, FLY_PHASE, st, [&] {
            if (df)
                return launch_fly_df64(h->d_fly_items.p, (int64_t)h->d_fly_items.n, h->d_fly_ctr.p, h->d_fly_rowpid.p,
                                       h->d_fly_cpid.p, h->d_fly_cws.p, h->d_ptsdf.p, h->d_logtab.p, h->d_ws.p,
                                       h->kparams(), h->k32, st);
            return launch_fly_f64(h->d_fly_items.p, (int64_t)h->d_fly_items.n, h->d_fly_ctr.p, h->d_fly_rowpid.p,
                                  h->d_fly_cpid.p, h->d_fly_cws.p, h->d_ws.p, h->kparams(), st);
        });
        stored(h->fly_split, nph);
    } else if (h->coop && h->dataflow) {
        CK(cudaMemcpyAsync(h->d_sdep.p, h->d_sdep0.p, h->d_sdep0.n * 4, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemsetAsync(h->d_sctr.p, 0, 4, st));
        prof_launch(h, H2W_PREC_FP64, nph, st, [&] {
            return launch_brg_flow_f64(h->d_roff.p, h->d_blob.p, 0, (int64_t)h->d_roff.n - 1, h->d_sctr.p, h->d_sdep.p,
                                       h->d_scoff.p, h->d_scidx.p, h->d_op.p, h->d_ws.p, dx, dy, perm, h->d_err.p, st);
        });
    } else if (h->coop) {
        prof_launch(h, H2W_PREC_FP64, nph, st, [&] {
            return launch_coop_f64(h->d_roff.p, h->d_blob.p, h->d_pstart.p, nph, h->d_op.p, h->d_ws.p, dx, dy, perm,
                                   h->d_bar.p, h->d_err.p, st, h->spin_limit);
        });
    } else {
        for (size_t q = 0; q < h->phases.size(); ++q) {
            const Phase &ph = h->phases[q];
            prof_launch(h, H2W_PREC_FP64, (int)q, st, [&] {
                return launch_brg_f64(h->d_roff.p, h->d_blob.p, ph.t0, ph.t1, h->d_op.p, h->d_ws.p, dx, dy, perm, st);
            });
        }
    }
    if (!h->fused_scatter) {
        if (permuted)
            CK(cudaMemcpyAsync(dy, h->d_ws.p + h->yperm_off, (size_t)h->nv() * 8, cudaMemcpyDeviceToDevice, st));
        else
            CK(launch_scatter_f64(h->d_ws.p + h->yperm_off, dy, h->d_perm.p, h->nv(), st));
    }
}

void ensure_f32(h2w_handle *h) {
    if (h->d_op32.p) return;
    h->d_op32.alloc((size_t)h->op_n);
    CK(launch_convert_f32(h->d_op.p, h->d_op32.p, h->op_n, h->stream));
    h->d_ws32.alloc((size_t)h->ws_n);
    CK(cudaStreamSynchronize(h->stream));
}

// the slice-contiguous FP32 operator of the warp-specialised product
void ensure_f32m(h2w_handle *h) {
    ensure_f32(h);
    if (h->op32m_ready) return;
    h->d_op32m.reset();
    h->d_op32m.alloc((size_t)std::max<int64_t>(h->op32m_n, 4));
    CK(launch_slice_copy_f32(h->d_op32.p, h->d_mslices.p, (int64_t)h->d_mslices.n / 6, h->d_op32m.p, h->stream));
    CK(cudaStreamSynchronize(h->stream));  // products may run on a caller's stream
    h->op32m_ready = true;
}

// the slice-contiguous FP32 operator of the single-vector stream
void ensure_f32s(h2w_handle *h) {
    ensure_f32(h);
    if (h->op32s_ready) return;
    h->d_op32s.reset();
    h->d_op32s.alloc((size_t)std::max<int64_t>(h->op32s_n, 4));
    CK(launch_slice_copy_f32(h->d_op32.p, h->d_sslices.p, (int64_t)h->d_sslices.n / 6, h->d_op32s.p, h->stream));
    CK(cudaStreamSynchronize(h->stream));  // products may run on a caller's stream
    h->op32s_ready = true;
}

// FP32 operator and workspace; x and y stay FP64 in original order (the
// conversions happen in the kernel's gather and scatter).
void run_matvec_f32(h2w_handle *h, const double *dx, double *dy, cudaStream_t st, bool permuted = false) {
    ensure_f32s(h);
    const int32_t *perm = permuted ? nullptr : h->d_perm.p;
    const int nph = (int)h->phases.size();
    CK(cudaMemsetAsync(h->d_ws32.p, 0, (size_t)h->ws_n * 4, st));
    if (h->fly_active) {
        auto stored = [&](int a, int b) {
            if (b <= a) return;
            if (h->coop) {
                prof_launch(h, H2W_PREC_FP32, nph, st, [&] {
                    return launch_coop_f32(h->d_roff.p, h->d_blob_s.p, h->d_pstart.p + a, b - a, h->d_op32s.p,
                                           h->d_ws32.p, dx, dy, perm, h->d_bar.p, h->d_err.p, st, h->spin_limit);
                });
            } else {
                for (int q = a; q < b; ++q) {
                    const Phase &ph = h->phases[(size_t)q];
                    prof_launch(h, H2W_PREC_FP32, q, st, [&] {
                        return launch_brg_f32(h->d_roff.p, h->d_blob_s.p, ph.t0, ph.t1, h->d_op32s.p, h->d_ws32.p, dx, dy,
                                              perm, st);
                    });
                }
            }
        };
        stored(0, h->fly_split);
        prof_launch(h, H2W_PREC_FP32, FLY_PHASE, st, [&] {
            return launch_fly_f32(h->d_fly_items.p, (int64_t)h->d_fly_items.n, h->d_fly_ctr.p, h->d_fly_rowpid.p,
                                  h->d_fly_cpid.p, h->d_fly_cws.p, h->d_pts4.p, h->d_ws32.p, h->kparams(), h->k32, st);
        });
        stored(h->fly_split, nph);
    } else if (h->coop && h->dataflow) {
        CK(cudaMemcpyAsync(h->d_sdep.p, h->d_sdep0.p, h->d_sdep0.n * 4, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemsetAsync(h->d_sctr.p, 0, 4, st));
        prof_launch(h, H2W_PREC_FP32, nph, st, [&] {
            return launch_brg_flow_f32(h->d_roff.p, h->d_blob_s.p, 0, (int64_t)h->d_roff.n - 1, h->d_sctr.p, h->d_sdep.p,
                                       h->d_scoff.p, h->d_scidx.p, h->d_op32s.p, h->d_ws32.p, dx, dy, perm, h->d_err.p,
                                       st);
        });
    } else if (h->coop) {
        prof_launch(h, H2W_PREC_FP32, nph, st, [&] {
            return launch_coop_f32(h->d_roff.p, h->d_blob_s.p, h->d_pstart.p, nph, h->d_op32s.p, h->d_ws32.p, dx, dy,
                                   perm, h->d_bar.p, h->d_err.p, st, h->spin_limit);
        });
    } else {
        for (size_t q = 0; q < h->phases.size(); ++q) {
            const Phase &ph = h->phases[q];
            prof_launch(h, H2W_PREC_FP32, (int)q, st, [&] {
                return launch_brg_f32(h->d_roff.p, h->d_blob_s.p, ph.t0, ph.t1, h->d_op32s.p, h->d_ws32.p, dx, dy, perm,
                                      st);
            });
        }
    }
    if (!h->fused_scatter) {
        if (permuted) CK(vec_f32_to_f64(h->d_ws32.p + h->yperm_off, dy, h->tree.N, st));
        else CK(launch_scatter_f32(h->d_ws32.p + h->yperm_off, dy, h->d_perm.p, h->tree.N, st));
    }
}

// ------------------------------------------------------- captured loops ---
// The Arnoldi step as the body of a conditional while node: body(s, cond)
// enqueues one step on s and ends with the kernel that sets cond. Cached per
// (kind, precision, m, rp, nrhs, tol) and rebuilt when any device buffer was
// reallocated since the capture. Returns nullptr when capture is unavailable
// (the caller then runs the host loop). kps: kernels one step launches.
// Whether loop_graph holds a valid captured step for this key (no capture needed).
bool loop_graph_cached(h2w_handle *h, int kind, int prec, int m, int rp, int nrhs) {
    if (!h->use_graphs || h->graph_failed || h->prof) return false;
    const uint64_t gen = g_alloc_gen.load();
    for (const h2w_handle::LoopGraph &L : h->loops)
        if (L.kind == kind && L.prec == prec && L.m == m && L.rp == rp && L.nrhs == nrhs) return L.gen == gen;
    return false;
}

template <class F>
cudaGraphExec_t loop_graph(h2w_handle *h, int kind, int prec, int m, int rp, int nrhs, int64_t &kps, F &&body) {
    if (!h->use_graphs || h->graph_failed || h->prof) return nullptr;
    const uint64_t gen = g_alloc_gen.load();
    for (size_t i = 0; i < h->loops.size(); ++i) {
        h2w_handle::LoopGraph &L = h->loops[i];
        if (L.kind == kind && L.prec == prec && L.m == m && L.rp == rp && L.nrhs == nrhs) {
            if (L.gen == gen) {
                kps = L.kernels_per_step;
                return L.exec;
            }
            cudaGraphExecDestroy(L.exec);
            cudaGraphDestroy(L.graph);
            h->loops.erase(h->loops.begin() + (long)i);
            break;
        }
    }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const int64_t c0 = launch_count();
    bool capturing = false;
    try {
        CK(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle cond;
        CK(cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault));
        // zero-initialised storage (the struct's union has no default constructor in C++)
        alignas(cudaGraphNodeParams) unsigned char npbuf[sizeof(cudaGraphNodeParams)] = {};
        cudaGraphNodeParams *np = reinterpret_cast<cudaGraphNodeParams *>(npbuf);
        np->type = cudaGraphNodeTypeConditional;
        np->conditional.handle = cond;
        np->conditional.type = cudaGraphCondTypeWhile;
        np->conditional.size = 1;
        cudaGraphNode_t node;
        CK(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, np));
        cudaGraph_t bodyg = np->conditional.phGraph_out[0];
        CK(cudaStreamBeginCaptureToGraph(h->stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        capturing = true;
        body(h->stream, cond);
        cudaGraph_t out = nullptr;
        capturing = false;
        CK(cudaStreamEndCapture(h->stream, &out));
        CK(cudaGraphInstantiate(&exec, graph, 0));
    } catch (const std::exception &) {
        if (capturing) {
            cudaGraph_t out = nullptr;
            cudaStreamEndCapture(h->stream, &out);
        }
        cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        count_launch(c0 - launch_count());
        h->graph_failed = true;
        return nullptr;
    }
    kps = launch_count() - c0;
    count_launch(-kps);  // the captured launches run when the graph does
    h->loops.push_back({kind, prec, m, rp, nrhs, gen, graph, exec, kps});
    return exec;
}

// ----------------------------------------------- multiple right-hand sides ---
// Interleaved block width for nrhs columns (the multi-vector kernel is
// compiled for 16, 32 and 64).
int rp_for(int nrhs) { return nrhs <= 16 ? 16 : (nrhs <= 32 ? 32 : 64); }
constexpr int MR_MAX = 64;

// A multi-vector launch, bracketed by events while profiling is on.
template <class F>
void mr_prof(h2w_handle *h, int prec, int rp, cudaStream_t st, F &&launch) {
    if (!h->prof) {
        CK(launch());
        return;
    }
    h2w_handle::ProfRec r{prof_event(h), prof_event(h), prec + 2, (int)h->mphases.size(), rp};
    CK(cudaEventRecord(r.a, st));
    CK(launch());
    CK(cudaEventRecord(r.b, st));
    h->prof_recs.push_back(r);
}

// Y = A X for an interleaved leaf-order block of rp vectors (xi, yi: N x rp).
void run_matvec_multi(h2w_handle *h, int prec, int rp, const double *xi, double *yi, cudaStream_t st) {
    if (h->fly_active)
        throw ApiError(H2W_ERR_STATE, "multi-vector products need the stored far field (H2W_OPT_FAR_ON_THE_FLY is on)");
    const int nph = (int)h->mphases.size();
    const size_t wsz = (size_t)h->ws_n * (size_t)rp;
    if (h->ws_n >= (int64_t)INT32_MAX - 2 || h->tree.N >= (int64_t)INT32_MAX - 2)
        throw ApiError(H2W_ERR_ARG, "workspace too large for the multi-vector kernel's source map");
    MrPhases ph{h->ph_t0.data(), h->ph_t1.data(), nph};
    CK(cudaMemsetAsync(h->d_mctr.p, 0, (size_t)std::max(nph, 1) * 4, st));
    const MrPhases *phased = h->coop ? nullptr : &ph;
    if (prec == H2W_PREC_FP32) {
        ensure_f32(h);
        if (h->m_wsf.n < wsz) h->m_wsf.alloc(wsz);
        CK(cudaMemsetAsync(h->m_wsf.p, 0, wsz * 4, st));
        const size_t nx = (size_t)h->tree.N * (size_t)rp;
        if (h->m_xf.n < nx) h->m_xf.alloc(nx);
        CK(vec_f64_to_f32(xi, h->m_xf.p, (int64_t)nx, st));
        const bool flow = h->dataflow && h->coop && !h->tensor;
        if (flow && h->producer_warp) ensure_f32m(h);
        if (flow) CK(cudaMemcpyAsync(h->d_mdep.p, h->d_mdep0.p, h->d_mdep0.n * 4, cudaMemcpyDeviceToDevice, st));
        mr_prof(h, prec, rp, st, [&] {
            if (flow && h->producer_warp)
                return launch_mw_f32_flow(rp, h->d_roff_m.p, h->d_blob_mw.p, (int64_t)h->d_roff_m.n - 1, h->d_mctr.p,
                                          h->d_mdep.p, h->d_mcoff.p, h->d_mcidx.p, h->d_op32m.p, h->m_wsf.p, h->m_xf.p,
                                          yi, h->d_err.p, st);
            if (flow)
                return launch_mr_f32_flow(rp, h->d_roff_m.p, h->d_blob_m.p, (int64_t)h->d_roff_m.n - 1, h->d_mctr.p,
                                          h->d_mdep.p, h->d_mcoff.p, h->d_mcidx.p, h->d_op32.p, h->m_wsf.p, h->m_xf.p,
                                          yi, h->d_err.p, st);
            if (h->tensor)
                return launch_mrt_f32(rp, h->d_roff_m.p, h->d_blob_m.p, h->d_pstart_m.p, nph, phased, h->d_mctr.p,
                                      h->d_op32.p, h->m_wsf.p, h->m_xf.p, yi, h->d_bar.p, h->d_err.p, st);
            return launch_mr_f32(rp, h->d_roff_m.p, h->d_blob_m.p, h->d_pstart_m.p, nph, phased, h->d_mctr.p, h->d_op32.p,
                                 h->m_wsf.p, h->m_xf.p, yi, h->d_bar.p, h->d_err.p, st);
        });
        if (!h->fused_scatter_m) CK(launch_mr_widen_f32(h->m_wsf.p + (size_t)h->yperm_off * rp, yi, h->tree.N * rp, st));
    } else {
        if (h->m_wsd.n < wsz) h->m_wsd.alloc(wsz);
        CK(cudaMemsetAsync(h->m_wsd.p, 0, wsz * 8, st));
        if (prec == H2W_PREC_DF64) {  // operator split once; the input block split per product
            if (!h->d_opdf.p) {
                h->d_opdf.alloc((size_t)h->op_n);
                CK(launch_mr_split(h->d_op.p, h->d_opdf.p, h->op_n, st));
            }
            const size_t nx = (size_t)h->tree.N * (size_t)rp;
            if (h->m_xdf.n < nx) h->m_xdf.alloc(nx);
            CK(launch_mr_split(xi, h->m_xdf.p, (int64_t)nx, st));
        }
        const bool flow = h->dataflow && h->coop;
        if (flow) CK(cudaMemcpyAsync(h->d_mdep.p, h->d_mdep0.p, h->d_mdep0.n * 4, cudaMemcpyDeviceToDevice, st));
        mr_prof(h, prec, rp, st, [&] {
            if (flow) {
                const bool df = prec == H2W_PREC_DF64;
                return launch_mr_f64_flow(rp, df, h->d_roff_m.p, h->d_blob_m.p, (int64_t)h->d_roff_m.n - 1,
                                          h->d_mctr.p, h->d_mdep.p, h->d_mcoff.p, h->d_mcidx.p,
                                          df ? h->d_opdf.p : h->d_op.p, h->m_wsd.p, df ? h->m_xdf.p : xi, yi,
                                          h->d_err.p, st);
            }
            if (prec == H2W_PREC_DF64)
                return launch_mr_df64(rp, h->d_roff_m.p, h->d_blob_m.p, h->d_pstart_m.p, nph, phased, h->d_mctr.p,
                                      h->d_opdf.p, h->m_wsd.p, h->m_xdf.p, yi, h->d_bar.p, h->d_err.p, st);
            return launch_mr_f64(rp, h->d_roff_m.p, h->d_blob_m.p, h->d_pstart_m.p, nph, phased, h->d_mctr.p, h->d_op.p,
                                 h->m_wsd.p, xi, yi, h->d_bar.p, h->d_err.p, st);
        });
        if (!h->fused_scatter_m) CK(launch_mr_widen_f64(h->m_wsd.p + (size_t)h->yperm_off * rp, yi, h->tree.N * rp, st));
    }
}

// y = A32 x for an FP32 interleaved block, FP32 result (no conversions)
void run_matvec_multi_f32io(h2w_handle *h, int rp, const float *xf, float *yf, cudaStream_t st) {
    if (h->fly_active)
        throw ApiError(H2W_ERR_STATE, "multi-vector products need the stored far field (H2W_OPT_FAR_ON_THE_FLY is on)");
    const int nph = (int)h->mphases.size();
    const size_t wsz = (size_t)h->ws_n * (size_t)rp;
    if (h->ws_n >= (int64_t)INT32_MAX - 2 || h->tree.N >= (int64_t)INT32_MAX - 2)
        throw ApiError(H2W_ERR_ARG, "workspace too large for the multi-vector kernel's source map");
    MrPhases ph{h->ph_t0.data(), h->ph_t1.data(), nph};
    CK(cudaMemsetAsync(h->d_mctr.p, 0, (size_t)std::max(nph, 1) * 4, st));
    const MrPhases *phased = h->coop ? nullptr : &ph;
    ensure_f32(h);
    if (h->m_wsf.n < wsz) h->m_wsf.alloc(wsz);
    CK(cudaMemsetAsync(h->m_wsf.p, 0, wsz * 4, st));
    const bool flow = h->dataflow && h->coop && !h->tensor;
    if (flow && h->producer_warp) ensure_f32m(h);
    if (flow) CK(cudaMemcpyAsync(h->d_mdep.p, h->d_mdep0.p, h->d_mdep0.n * 4, cudaMemcpyDeviceToDevice, st));
    mr_prof(h, H2W_PREC_FP32, rp, st, [&] {
        if (flow && h->producer_warp)
            return launch_mw_f32_flow(rp, h->d_roff_m.p, h->d_blob_mw.p, (int64_t)h->d_roff_m.n - 1, h->d_mctr.p,
                                      h->d_mdep.p, h->d_mcoff.p, h->d_mcidx.p, h->d_op32m.p, h->m_wsf.p, xf, yf,
                                      h->d_err.p, st);
        if (flow)
            return launch_mr_f32_flow(rp, h->d_roff_m.p, h->d_blob_m.p, (int64_t)h->d_roff_m.n - 1, h->d_mctr.p,
                                      h->d_mdep.p, h->d_mcoff.p, h->d_mcidx.p, h->d_op32.p, h->m_wsf.p, xf, yf, h->d_err.p,
                                      st);
        if (h->tensor)
            return launch_mrt_f32(rp, h->d_roff_m.p, h->d_blob_m.p, h->d_pstart_m.p, nph, phased, h->d_mctr.p,
                                  h->d_op32.p, h->m_wsf.p, xf, yf, h->d_bar.p, h->d_err.p, st);
        return launch_mr_f32(rp, h->d_roff_m.p, h->d_blob_m.p, h->d_pstart_m.p, nph, phased, h->d_mctr.p, h->d_op32.p,
                             h->m_wsf.p, xf, yf, h->d_bar.p, h->d_err.p, st);
    });
    if (!h->fused_scatter_m)
        CK(cudaMemcpyAsync(yf, h->m_wsf.p + (size_t)h->yperm_off * rp, (size_t)h->tree.N * rp * 4,
                           cudaMemcpyDeviceToDevice, st));
}

void ensure_multi_vectors(h2w_handle *h) {
    const size_t n = (size_t)h->tree.N * MR_MAX;
    if (h->m_xi.n < n) h->m_xi.alloc(n);
    if (h->m_yi.n < n) h->m_yi.alloc(n);
}

inline GmbStore<double> &gmb_store(h2w_handle *h, double *) { return h->gbd; }
inline GmbStore<float> &gmb_store(h2w_handle *h, float *) { return h->gbf; }

template <class T>
GmbT<T> gmb_state(h2w_handle *h, int m, int rp, int nrhs) {
    const int64_t N = h->tree.N;
    const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(3 * 152, (N + 127) / 128));
    GmbStore<T> &S = gmb_store(h, (T *)nullptr);
    if (S.m != m || S.rp != rp) {
        S.V.alloc((size_t)N * rp * (size_t)(m + 1));
        S.w.alloc((size_t)N * rp);
        S.vcur.alloc((size_t)N * rp);
        S.H.alloc((size_t)rp * (size_t)(m + 1) * (size_t)m);
        S.cs.alloc((size_t)rp * (m + 1));
        S.sn.alloc((size_t)rp * (m + 1));
        S.s.alloc((size_t)rp * (m + 1));
        S.part.alloc((size_t)nblk * (m + 1) * rp);
        S.hsum.alloc((size_t)(m + 1) * rp);
        S.normb.alloc((size_t)rp);
        S.resid.alloc((size_t)rp);
        S.y.alloc((size_t)(m + 1) * rp);
        S.z.alloc((size_t)(m + 2) * rp);
        S.conv.alloc((size_t)rp);
        S.tol.alloc(1);
        S.iter.alloc(2);
        S.m = m;
        S.rp = rp;
    }
    GmbT<T> g;
    g.V = S.V.p;
    g.w = S.w.p;
    g.vcur = S.vcur.p;
    g.H = S.H.p;
    g.cs = S.cs.p;
    g.sn = S.sn.p;
    g.s = S.s.p;
    g.part = S.part.p;
    g.hsum = S.hsum.p;
    g.normb = S.normb.p;
    g.resid = S.resid.p;
    g.y = S.y.p;
    g.z = S.z.p;
    g.conv = S.conv.p;
    g.tolp = S.tol.p;
    g.iter = S.iter.p;
    g.N = N;
    g.m = m;
    g.rp = rp;
    g.nrhs = nrhs;
    g.nblk = nblk;
    return g;
}

// Lockstep GMRES over the nrhs <= rp systems of an interleaved leaf-order
// block: bi right-hand sides, xi initial guesses (updated in place; x0_zero:
// skip the initial product). iters / resid per column (nrhs entries).
template <class T>
int gmres_batch_run_t(h2w_handle *h, const double *bi, double *xi, int rp, int nrhs, int max_iter, double tol,
                      int prec, bool x0_zero, int *iters, double *resid) {
    if (max_iter < 1 || max_iter > 400) throw ApiError(H2W_ERR_ARG, "batched GMRES: max_iter must be in 1..400");
    constexpr bool F32 = std::is_same<T, float>::value;
    GmbT<T> g = gmb_state<T>(h, max_iter, rp, nrhs);
    // w = A vcur: the FP32 basis feeds the FP32 product directly (no conversions)
    auto product = [&](cudaStream_t s) {
        if constexpr (F32) run_matvec_multi_f32io(h, rp, g.vcur, g.w, s);
        else run_matvec_multi(h, prec, rp, g.vcur, g.w, s);
    };
    const int kind = F32 ? 2 : 1;
    cudaStream_t st = h->stream;
    CK(cudaMemcpyAsync(g.tolp, &tol, 8, cudaMemcpyHostToDevice, st));  // read by the Givens step
    if (x0_zero) {
        CK(gmb_start(g, bi, nullptr, tol, st));  // also sets normb = ||bi||
    } else {
        if (F32) throw ApiError(H2W_ERR_ARG, "batched GMRES: the FP32 basis starts from x0 = 0");
        CK(gmb_norms(g, bi, g.normb, 1, st));
        if (h->m_ri.n < (size_t)h->tree.N * rp) h->m_ri.alloc((size_t)h->tree.N * MR_MAX);
        run_matvec_multi(h, prec, rp, xi, h->m_ri.p, st);
        CK(gmb_start(g, bi, h->m_ri.p, tol, st));
    }
    std::vector<int32_t> conv((size_t)rp);
    auto read_conv = [&] {
        CK(cudaMemcpyAsync(conv.data(), g.conv, (size_t)rp * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int c = 0; c < nrhs; ++c)
            if (conv[(size_t)c] == -1) return false;
        return true;
    };
    bool done = read_conv();
    int last = -1;
    bool looped = false;
    if (!done && h->use_graphs && !h->graph_failed && !h->prof) {
        // graph path: the batched Arnoldi steps as one while-loop graph launch
        // before a capture, one product outside it makes its buffers and launch attributes
        if (!loop_graph_cached(h, kind, prec, max_iter, rp, nrhs)) product(st);
        int64_t kps = 0;
        cudaGraphExec_t ex = loop_graph(h, kind, prec, max_iter, rp, nrhs, kps, [&](cudaStream_t s, cudaGraphConditionalHandle c) {
            product(s);
            CK(gmb_arnoldi(g, s));
            CK(gmb_loop(g, c, s));
        });
        if (ex) {
            CK(cudaGraphLaunch(ex, st));
            int32_t it2[2];
            CK(cudaMemcpyAsync(it2, g.iter, 8, cudaMemcpyDeviceToHost, st));
            read_conv();
            count_launch(kps * it2[1]);
            last = it2[1] - 1;
            looped = true;
        }
    }
    for (int i = 0; i < max_iter && !done && !looped; ++i) {
        product(st);
        CK(gmb_arnoldi(g, st));
        last = i;
        done = read_conv();
    }
    int kmax = -1;
    for (int c = 0; c < nrhs; ++c) {
        const int cv = conv[(size_t)c];
        kmax = std::max(kmax, cv >= 0 ? cv : (cv == -1 ? last : -1));
    }
    CK(gmb_finish(g, xi, last, kmax, st));
    // the solved system's residual bi - A d is V z (Arnoldi relation) from x0 = 0
    gmb_store(h, (T *)nullptr).jres = (x0_zero && kmax + 1 <= max_iter) ? kmax + 1 : -1;
    std::vector<double> rs((size_t)rp);
    CK(cudaMemcpyAsync(rs.data(), g.resid, (size_t)rp * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    bool all = true;
    for (int c = 0; c < nrhs; ++c) {
        const int cv = conv[(size_t)c];
        iters[c] = cv >= 0 ? cv + 1 : (cv == -2 ? 0 : last + 1);
        resid[c] = rs[(size_t)c];
        if (cv == -1) all = false;
    }
    return all ? H2W_OK : H2W_ERR_NOT_CONVERGED;
}

// FP32-operator solves from x0 = 0 run on the FP32 basis (H2W_OPT_F32_BASIS),
// everything else on the FP64 basis
int gmres_batch_run(h2w_handle *h, const double *bi, double *xi, int rp, int nrhs, int max_iter, double tol, int prec,
                    bool x0_zero, int *iters, double *resid) {
    if (prec == H2W_PREC_FP32 && x0_zero && h->f32_basis)
        return gmres_batch_run_t<float>(h, bi, xi, rp, nrhs, max_iter, tol, prec, x0_zero, iters, resid);
    return gmres_batch_run_t<double>(h, bi, xi, rp, nrhs, max_iter, tol, prec, x0_zero, iters, resid);
}

// --------------------------------------------------------------- GMRES ---
GmresDev gmres_state(h2w_handle *h, int m) {
    const int64_t N = h->tree.N;
    const int nblk = (int)std::max<int64_t>(1, std::min<int64_t>(2 * 152, (N + 1023) / 1024));
    if (h->g_m != m) {
        h->g_V.alloc((size_t)N * (size_t)(m + 1));
        h->g_w.alloc((size_t)N);
        h->g_vcur.alloc((size_t)N);
        h->g_H.alloc((size_t)(m + 1) * (size_t)m);
        h->g_cs.alloc((size_t)m + 1);
        h->g_sn.alloc((size_t)m + 1);
        h->g_s.alloc((size_t)m + 1);
        h->g_part.alloc((size_t)3 * nblk * (size_t)(m + 1));
        h->g_scal.alloc(8);
        h->g_iter.alloc(2);
        h->g_tmp.alloc((size_t)N);
        h->g_r.alloc((size_t)N);
        h->g_m = m;
    }
    GmresDev g;
    g.V = h->g_V.p;
    g.w = h->g_w.p;
    g.vcur = h->g_vcur.p;
    g.H = h->g_H.p;
    g.cs = h->g_cs.p;
    g.sn = h->g_sn.p;
    g.s = h->g_s.p;
    g.part = h->g_part.p;
    g.scal = h->g_scal.p;
    g.iter = h->g_iter.p;
    g.N = N;
    g.m = m;
    g.nblk = nblk;
    return g;
}

double dnorm(h2w_handle *h, const double *x) {
    if (!h->g_npart.p) h->g_npart.alloc(256);
    if (!h->g_scal.p) h->g_scal.alloc(8);
    CK(vec_norm(x, h->tree.N, h->g_npart.p, 256, h->g_scal.p + 4, h->stream));
    double v;
    CK(cudaMemcpyAsync(&v, h->g_scal.p + 4, 8, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return v;
}

// Refinement residual updating. After an accurate residual r_k = b - A x_k,
// the next one is r_{k+1} = r_k - A d_k in exact arithmetic; forming A d_k
// with the FP32 operator costs an error of about eta * ||d_k||, eta being the
// FP32 product's error per unit input norm. That update replaces the FP64
// (or double-FP32) product while the summed bound since the last accurate
// residual, IR_UPDATE_SAFETY * eta * ||d||, stays below IR_UPDATE_SHARE of
// the stopping tolerance times ||b||; the stopping test and the reported
// residual add that bound to ||r||, so they bound the true residual. Updates
// also need the accurate residual's own rounding error, estimated as
// IR_UPDATE_SAFETY * eta * 2^-29 * ||x|| (FP64 unit roundoff in place of
// FP32's), to be below IR_UPDATE_FLOOR of the tolerance times ||b||: near the
// FP64 floor an updated residual would keep falling while the true one
// cannot. eta is measured once per operator: max over calibration vectors z
// (pseudo-random and smooth) of ||A32 z - A z|| / ||z||.
constexpr double IR_UPDATE_SAFETY = 10.0, IR_UPDATE_SHARE = 0.25, IR_UPDATE_FLOOR = 0.01;
// The update may instead be read from the inner solve: with d = V y from
// GMRES on A32 d = r (r rounded to the basis precision, r_f), the Arnoldi
// relation gives r_f - A32 d = V_{k+1} (beta e1 - Hbar y), so
// r - A32 d = (r - r_f) + V_{k+1} z costs a basis combination, no product. Its
// error adds the rounding of the Arnoldi relation (each basis vector's
// product and the orthogonalisation) to that of the product; it is charged
// IR_UPDATE_ARNOLDI times the product's bound.
constexpr double IR_UPDATE_ARNOLDI = 4.0;
constexpr double IR_U64_OVER_U32 = 0x1.0p-29;

// Relative tolerance of a refinement step's inner solve: enough to bring the
// residual ||r|| to a tenth of the outer target tol * ||b||, within
// [1e-6, 0.1]; 1e-6 when ||r|| is not known (the first step).
double inner_tol(double tol, double nb, double nr) {
    if (!(nr > 0) || !(nb > 0)) return 1e-6;
    return std::min(0.1, std::max(1e-6, 0.1 * tol * nb / nr));
}

double fp32_error_single(h2w_handle *h, cudaStream_t st) {
    if (h->eta_single >= 0) return h->eta_single;
    const int64_t N = h->tree.N;
    for (DBuf<double> *v : {&h->s_d, &h->s_r, &h->s_t})
        if (v->n < (size_t)N) v->alloc((size_t)N);
    double eta = 0.0;
    for (int c = 0; c < 2; ++c) {
        CK(launch_calib_fill(h->s_d.p, N, 1, c, st));
        run_matvec_f32(h, h->s_d.p, h->s_r.p, st, true);
        run_matvec_f64(h, h->s_d.p, h->s_t.p, st, true, h->ir_resid_prec == H2W_PREC_DF64);
        CK(vec_axpby(1.0, h->s_r.p, -1.0, h->s_t.p, h->s_r.p, N, st));
        const double nz = dnorm(h, h->s_d.p);
        if (nz > 0) eta = std::max(eta, dnorm(h, h->s_r.p) / nz);
    }
    h->eta_single = eta;
    return eta;
}

// The same for the multi-vector product: rp calibration columns at once, the
// accurate product in the refinement's residual precision. Uses m_ri, m_di, m_ti.
template <class T>
double fp32_error_multi(h2w_handle *h, const GmbT<T> &g, int rp, cudaStream_t st) {
    if (h->eta_multi >= 0) return h->eta_multi;
    const int64_t N = h->tree.N;
    const size_t len = (size_t)N * rp;
    if (h->m_ti.n < (size_t)N * MR_MAX) h->m_ti.alloc((size_t)N * MR_MAX);
    if (h->m_dn.n < (size_t)2 * MR_MAX) h->m_dn.alloc((size_t)2 * MR_MAX);
    double *z = h->m_di.p, *y32 = h->m_ri.p, *y = h->m_ti.p;
    CK(launch_calib_fill(z, N, rp, 0, st));
    run_matvec_multi(h, H2W_PREC_FP32, rp, z, y32, st);
    run_matvec_multi(h, h->ir_resid_prec, rp, z, y, st);
    CK(vec_axpby(1.0, y32, -1.0, y, y32, (int64_t)len, st));
    CK(gmb_norms(g, y32, h->m_dn.p, 0, st));
    CK(gmb_norms(g, z, h->m_dn.p + MR_MAX, 0, st));
    std::vector<double> n((size_t)2 * MR_MAX);
    CK(cudaMemcpyAsync(n.data(), h->m_dn.p, n.size() * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double eta = 0.0;
    for (int c = 0; c < rp; ++c)
        if (n[(size_t)(MR_MAX + c)] > 0) eta = std::max(eta, n[(size_t)c] / n[(size_t)(MR_MAX + c)]);
    h->eta_multi = eta;
    return eta;
}

// Solve the upper-triangular least-squares system H(0:k,0:k) y = s(0:k) on
// the host, as Update does (*/codes/gmres.hpp:77-90), then x += V y.
void gmres_xupdate(h2w_handle *h, const GmresDev &g, double *dx, int k) {
    const int m = g.m;
    std::vector<double> H((size_t)(m + 1) * (size_t)(k + 1)), s((size_t)k + 1);
    CK(cudaMemcpyAsync(H.data(), g.H, H.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(s.data(), g.s, s.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    auto Hc = [&](int r, int c) { return H[(size_t)r + (size_t)c * (size_t)(m + 1)]; };
    std::vector<double> y = s;
    for (int i = k; i >= 0; --i) {
        y[(size_t)i] /= Hc(i, i);
        for (int j = i - 1; j >= 0; --j) y[(size_t)j] -= Hc(j, i) * y[(size_t)i];
    }
    CK(cudaMemcpyAsync(h->g_tmp.p, y.data(), y.size() * 8, cudaMemcpyHostToDevice, h->stream));
    CK(gmres_update(g, dx, h->g_tmp.p, k, h->stream));
}

// All max_iter steps taken without meeting the tolerance: x += V y over all
// columns, then the true relative residual.
int gmres_unconverged(h2w_handle *h, const GmresDev &g, const double *db, double *dx, int max_iter, double tol,
                      int prec, double normb, int *iters, double *resid) {
    cudaStream_t st = h->stream;
    gmres_xupdate(h, g, dx, max_iter - 1);
    if (prec == H2W_PREC_FP32) run_matvec_f32(h, dx, h->g_r.p, st, true);
    else run_matvec_f64(h, dx, h->g_r.p, st, true);
    CK(vec_axpby(1.0, db, -1.0, h->g_r.p, h->g_r.p, h->tree.N, st));
    *resid = dnorm(h, h->g_r.p) / normb;
    *iters = max_iter;
    return *resid < tol ? H2W_OK : H2W_ERR_NOT_CONVERGED;
}

// FP64 GMRES on device vectors in leaf order (the operator is applied as
// P A P^T, which leaves GMRES unchanged up to rounding); matvec precision
// chosen by prec.
int gmres_run(h2w_handle *h, const double *db, double *dx, int max_iter, double tol, int prec, int *iters,
              double *resid, bool x0_zero = false) {
    GmresDev g = gmres_state(h, max_iter);
    cudaStream_t st = h->stream;
    const int64_t N = h->tree.N;
    CK(cudaMemcpyAsync(g.scal + 6, &tol, 8, cudaMemcpyHostToDevice, st));  // read by the Givens step
    auto A = [&](const double *in, double *out) {
        if (prec == H2W_PREC_FP32) run_matvec_f32(h, in, out, st, true);
        else run_matvec_f64(h, in, out, st, true);
    };
    double normb = dnorm(h, db);
    if (normb == 0.0) normb = 1;
    if (x0_zero) {
        CK(gmres_start(g, db, nullptr, normb, st));
    } else {
        A(dx, h->g_r.p);
        CK(gmres_start(g, db, h->g_r.p, normb, st));
    }
    double sc[4];
    CK(cudaMemcpyAsync(sc, g.scal, 32, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *resid = sc[1];
    if (sc[1] <= tol) {
        *iters = 0;
        return H2W_OK;
    }
    // graph path: the Arnoldi steps as one while-loop graph launch
    if (h->use_graphs && !h->graph_failed && !h->prof) {
        if (prec == H2W_PREC_FP32) ensure_f32(h);
        gmres_prepare();
        // before a capture, one product outside it makes its buffers and launch
        // attributes (the step recomputes w)
        if (!loop_graph_cached(h, 0, prec, max_iter, 1, 1)) A(g.vcur, g.w);
        int64_t kps = 0;
        cudaGraphExec_t ex = loop_graph(h, 0, prec, max_iter, 1, 1, kps, [&](cudaStream_t s, cudaGraphConditionalHandle c) {
            if (prec == H2W_PREC_FP32) run_matvec_f32(h, g.vcur, g.w, s, true);
            else run_matvec_f64(h, g.vcur, g.w, s, true);
            CK(gmres_cgs2(g, s));
            CK(gmres_finish_iter(g, s));
            CK(gmres_loop_cond(g, c, s));
        });
        if (ex) {
            CK(cudaGraphLaunch(ex, st));
            int32_t it2[2];
            CK(cudaMemcpyAsync(sc, g.scal, 32, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(it2, g.iter, 8, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            count_launch(kps * it2[1]);
            *resid = sc[1];
            if (sc[2] != 0.0) {
                gmres_xupdate(h, g, dx, it2[0]);
                CK(cudaStreamSynchronize(st));
                *iters = it2[1];
                return H2W_OK;
            }
            return gmres_unconverged(h, g, db, dx, max_iter, tol, prec, normb, iters, resid);
        }
    }
    for (int i = 0; i < max_iter; ++i) {
        A(g.vcur, g.w);
        CK(gmres_cgs2(g, st));
        CK(gmres_finish_iter(g, st));
        CK(cudaMemcpyAsync(sc, g.scal, 32, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        *resid = sc[1];
        if (sc[2] != 0.0) {
            gmres_xupdate(h, g, dx, i);
            CK(cudaStreamSynchronize(st));
            *iters = i + 1;
            return H2W_OK;
        }
    }
    return gmres_unconverged(h, g, db, dx, max_iter, tol, prec, normb, iters, resid);
}

// Device-side failure flag of the cooperative matvec (a grid barrier whose
// bounded wait ran out).
void check_device_error(h2w_handle *h) {
    if (!h->d_err.p) return;
    int32_t e = 0;
    CK(cudaMemcpyAsync(&e, h->d_err.p, 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (e) {
        CK(cudaMemsetAsync(h->d_err.p, 0, 4, h->stream));
        CK(cudaMemsetAsync(h->d_bar.p, 0, 8, h->stream));
        static const char *what[] = {"", "a grid-barrier wait", "a tensor-pipeline wait", "a dependency wait",
                                     "a stage (mbarrier or counter) wait"};
        throw ApiError(H2W_ERR_CUDA, std::string("matvec: ") + (e >= 1 && e <= 4 ? what[e] : "a device wait") +
                                         " ran out (device error flag " + std::to_string(e) + ")");
    }
}

// ------------------------------------------------ many independent problems
}  // namespace

// A batch of assembled operators on one device, run together: one merged
// record stream (every problem's single-vector targets, phase-aligned at the
// leaf end, heaviest first within a merged phase) drives one cooperative
// launch per product; the solvers run every problem's GMRES in lockstep over
// concatenated vectors. The handles must outlive the batch and must not be
// re-assembled while it exists.
struct h2w_batch {
    std::vector<h2w_handle *> hs;
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    int64_t Ntot = 0;
    std::vector<int64_t> off, wsoff;        // P+1: vector and workspace offsets
    std::vector<int> unfused;               // problems whose leaf rows need an explicit scatter
    DBuf<int64_t> roff, blob, pstart;
    int nphase = 0;
    DBuf<BatchProb> tab64_orig, tab64_leaf, tab32_orig, tab32_leaf;
    DBuf<double> ws64;
    DBuf<float> ws32;
    DBuf<unsigned> bar;
    DBuf<int32_t> errf;
    DBuf<int64_t> perm_all;                 // global leaf position -> global original position
    DBuf<double> sx, sy, bl, xl, r, d;      // staging and solver vectors (Ntot each)
    // segmented GMRES state
    DBuf<double> V, w, vcur, H, cs, sn, s, part, hsum, normb, resid, y, onorm, ores;
    DBuf<int32_t> conv, iter, bprob, pblk;
    DBuf<int64_t> brow;
    int g_m = -1, nblk = 0;
};

namespace {

template <class F>
int bguarded(h2w_batch *b, F &&f) {
    if (!b) return H2W_ERR_ARG;
    try {
        if (cudaSetDevice(b->device) != cudaSuccess) {
            b->err = "cudaSetDevice failed";
            return H2W_ERR_CUDA;
        }
        return f();
    } catch (const ApiError &e) {
        b->err = e.what();
        return e.code;
    } catch (const CudaError &e) {
        b->err = e.what();
        return H2W_ERR_CUDA;
    } catch (const std::bad_alloc &) {
        b->err = "host allocation failed";
        return H2W_ERR_NOMEM;
    } catch (const std::exception &e) {
        b->err = e.what();
        return H2W_ERR_ARG;
    }
}

void batch_check_error(h2w_batch *b) {
    int32_t e = 0;
    CK(cudaMemcpyAsync(&e, b->errf.p, 4, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    if (e) {
        CK(cudaMemsetAsync(b->errf.p, 0, 4, b->stream));
        CK(cudaMemsetAsync(b->bar.p, 0, 8, b->stream));
        throw ApiError(H2W_ERR_CUDA, "batch matvec: a grid-barrier wait ran out (device error flag)");
    }
}

// y = A x for every problem: x, y concatenated, leaf order (leaf) or each
// problem's original point order.
void run_batch(h2w_batch *b, int prec, const double *x, double *y, bool leaf, const int32_t *active = nullptr) {
    cudaStream_t st = b->stream;
    const bool f32 = prec == H2W_PREC_FP32;
    const int P = (int)b->hs.size();
    if (f32 && !b->tab32_orig.p) {
        if (!b->ws32.p) b->ws32.alloc((size_t)b->wsoff[(size_t)P]);
        std::vector<BatchProb> to(P), tl(P);
        for (int p = 0; p < P; ++p) {
            ensure_f32(b->hs[(size_t)p]);
            to[(size_t)p] = {b->hs[(size_t)p]->d_op32.p, b->ws32.p + b->wsoff[(size_t)p], b->hs[(size_t)p]->d_perm.p,
                             b->off[(size_t)p]};
            tl[(size_t)p] = to[(size_t)p];
            tl[(size_t)p].perm = nullptr;
        }
        b->tab32_orig.upload(to, st);
        b->tab32_leaf.upload(tl, st);
    }
    const BatchProb *tab = f32 ? (leaf ? b->tab32_leaf.p : b->tab32_orig.p) : (leaf ? b->tab64_leaf.p : b->tab64_orig.p);
    if (f32) CK(cudaMemsetAsync(b->ws32.p, 0, (size_t)b->wsoff[(size_t)P] * 4, st));
    else CK(cudaMemsetAsync(b->ws64.p, 0, (size_t)b->wsoff[(size_t)P] * 8, st));
    if (f32)
        CK(launch_brgb_f32(b->roff.p, b->blob.p, b->pstart.p, b->nphase, tab, active, x, y, b->bar.p, b->errf.p, st));
    else
        CK(launch_brgb_f64(b->roff.p, b->blob.p, b->pstart.p, b->nphase, tab, active, x, y, b->bar.p, b->errf.p, st));
    for (int p : b->unfused) {
        h2w_handle *h = b->hs[(size_t)p];
        const int64_t N = h->tree.N, o = b->off[(size_t)p], w0 = b->wsoff[(size_t)p] + h->yperm_off;
        if (f32) {
            if (leaf) CK(vec_f32_to_f64(b->ws32.p + w0, y + o, N, st));
            else CK(launch_scatter_f32(b->ws32.p + w0, y + o, h->d_perm.p, N, st));
        } else {
            if (leaf) CK(cudaMemcpyAsync(y + o, b->ws64.p + w0, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
            else CK(launch_scatter_f64(b->ws64.p + w0, y + o, h->d_perm.p, N, st));
        }
    }
}

GmresSeg gms_state(h2w_batch *b, int m) {
    const int P = (int)b->hs.size();
    const int64_t N = b->Ntot;
    if (b->g_m != m) {
        b->V.alloc((size_t)N * (size_t)(m + 1));
        b->w.alloc((size_t)N);
        b->vcur.alloc((size_t)N);
        b->H.alloc((size_t)P * (size_t)(m + 1) * (size_t)m);
        b->cs.alloc((size_t)P * (m + 1));
        b->sn.alloc((size_t)P * (m + 1));
        b->s.alloc((size_t)P * (m + 1));
        b->part.alloc((size_t)b->nblk * (m + 1));
        b->hsum.alloc((size_t)P * (m + 1));
        b->y.alloc((size_t)P * (m + 1));
        b->g_m = m;
    }
    GmresSeg g;
    g.V = b->V.p;
    g.w = b->w.p;
    g.vcur = b->vcur.p;
    g.H = b->H.p;
    g.cs = b->cs.p;
    g.sn = b->sn.p;
    g.s = b->s.p;
    g.part = b->part.p;
    g.hsum = b->hsum.p;
    g.normb = b->normb.p;
    g.resid = b->resid.p;
    g.y = b->y.p;
    g.conv = b->conv.p;
    g.iter = b->iter.p;
    g.bprob = b->bprob.p;
    g.brow = b->brow.p;
    g.pblk = b->pblk.p;
    g.Ntot = N;
    g.m = m;
    g.P = P;
    g.nblk = b->nblk;
    return g;
}

// Every problem's GMRES in lockstep on concatenated leaf-order vectors: bl
// right-hand sides, xl initial guesses (updated; x0_zero: no initial product).
int gms_run(h2w_batch *b, const double *bl, double *xl, int max_iter, double tol, int prec, bool x0_zero, int *iters,
            double *resid) {
    if (max_iter < 1 || max_iter > 400) throw ApiError(H2W_ERR_ARG, "batch GMRES: max_iter must be in 1..400");
    const int P = (int)b->hs.size();
    GmresSeg g = gms_state(b, max_iter);
    cudaStream_t st = b->stream;
    CK(gms_norms(g, bl, g.normb, 1, st));
    if (x0_zero) {
        CK(gms_start(g, bl, nullptr, tol, st));
    } else {
        run_batch(b, prec, xl, b->r.p, true);
        CK(gms_start(g, bl, b->r.p, tol, st));
    }
    std::vector<int32_t> conv((size_t)P);
    auto read_conv = [&] {
        CK(cudaMemcpyAsync(conv.data(), g.conv, (size_t)P * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int p = 0; p < P; ++p)
            if (conv[(size_t)p] == -1) return false;
        return true;
    };
    bool done = read_conv();
    int last = -1;
    for (int i = 0; i < max_iter && !done; ++i) {
        run_batch(b, prec, g.vcur, g.w, true, g.conv);  // converged problems are skipped
        CK(gms_arnoldi(g, tol, st));
        last = i;
        done = read_conv();
    }
    int kmax = -1;
    for (int p = 0; p < P; ++p) {
        const int cv = conv[(size_t)p];
        kmax = std::max(kmax, cv >= 0 ? cv : (cv == -1 ? last : -1));
    }
    CK(gms_finish(g, xl, last, kmax, st));
    std::vector<double> rs((size_t)P);
    CK(cudaMemcpyAsync(rs.data(), g.resid, (size_t)P * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    batch_check_error(b);
    bool all = true;
    for (int p = 0; p < P; ++p) {
        const int cv = conv[(size_t)p];
        if (iters) iters[p] = cv >= 0 ? cv + 1 : (cv == -2 ? 0 : last + 1);
        if (resid) resid[p] = rs[(size_t)p];
        if (cv == -1) all = false;
    }
    return all ? H2W_OK : H2W_ERR_NOT_CONVERGED;
}

// Concatenated vectors in (stage from host) and out, gathered to leaf order
// for the solvers.
void batch_in(h2w_batch *b, const double *v, double *leaf, int where) {
    const double *src = v;
    if (where == H2W_HOST) {
        CK(cudaMemcpyAsync(b->sx.p, v, (size_t)b->Ntot * 8, cudaMemcpyHostToDevice, b->stream));
        src = b->sx.p;
    }
    CK(launch_gather64(src, leaf, b->perm_all.p, b->Ntot, b->stream));
}
void batch_out(h2w_batch *b, const double *leaf, double *v, int where) {
    double *dst = where == H2W_HOST ? b->sy.p : v;
    CK(launch_scatter64(leaf, dst, b->perm_all.p, b->Ntot, b->stream));
    if (where == H2W_HOST) CK(cudaMemcpyAsync(v, b->sy.p, (size_t)b->Ntot * 8, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
}

// Column blocks of up to 64 right-hand sides: stage (host) and pack into
// interleaved leaf order, run f on the block, unpack x back.
template <class F>
void for_rhs_blocks(h2w_handle *h, const double *b, double *x, int nrhs, int where, F &&f) {
    const int64_t N = h->tree.N;
    cudaStream_t st = h->stream;
    ensure_multi_vectors(h);
    if (h->m_bi.n < (size_t)N * MR_MAX) h->m_bi.alloc((size_t)N * MR_MAX);
    if (where == H2W_HOST) {
        if (h->m_stage_x.n < (size_t)N * MR_MAX) h->m_stage_x.alloc((size_t)N * MR_MAX);
        if (h->m_stage_y.n < (size_t)N * MR_MAX) h->m_stage_y.alloc((size_t)N * MR_MAX);
    }
    for (int c0 = 0; c0 < nrhs; c0 += MR_MAX) {
        const int nc = std::min(MR_MAX, nrhs - c0), rp = rp_for(nc);
        const double *bc = b + (size_t)c0 * N;
        double *xc = x + (size_t)c0 * N;
        const double *xsrc = xc;
        if (where == H2W_HOST) {
            CK(cudaMemcpyAsync(h->m_stage_x.p, bc, (size_t)N * nc * 8, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(h->m_stage_y.p, xc, (size_t)N * nc * 8, cudaMemcpyHostToDevice, st));
            bc = h->m_stage_x.p;
            xsrc = h->m_stage_y.p;
        }
        CK(launch_mr_pack(bc, N, h->m_bi.p, h->d_perm.p, N, nc, rp, st));
        CK(launch_mr_pack(xsrc, N, h->m_xi.p, h->d_perm.p, N, nc, rp, st));
        f(c0, nc, rp, h->m_bi.p, h->m_xi.p);
        CK(launch_mr_unpack(h->m_xi.p, where == H2W_HOST ? h->m_stage_y.p : xc, N, h->d_perm.p, N, nc, rp, st));
        if (where == H2W_HOST)
            CK(cudaMemcpyAsync(xc, h->m_stage_y.p, (size_t)N * nc * 8, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    check_device_error(h);
}

int fail(h2w_handle *h, int code, const std::string &m) {
    if (h) h->err = m;
    return code;
}

template <class F>
int guarded(h2w_handle *h, F &&f) {
    if (!h) return H2W_ERR_ARG;
    try {
        if (h->cfg.device >= 0 && cudaSetDevice(h->cfg.device) != cudaSuccess)
            return fail(h, H2W_ERR_CUDA, "cudaSetDevice failed");
        return f();
    } catch (const ApiError &e) {
        return fail(h, e.code, e.what());
    } catch (const CudaError &e) {
        return fail(h, H2W_ERR_CUDA, e.what());
    } catch (const std::bad_alloc &) {
        return fail(h, H2W_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(h, H2W_ERR_ARG, e.what());
    }
}

void require_points(h2w_handle *h) {
    if (h->pts.empty()) throw ApiError(H2W_ERR_STATE, "no points set");
}
void require_tree(h2w_handle *h) {
    if (!h->has_tree) throw ApiError(H2W_ERR_STATE, "tree not built (call h2w_build_tree)");
}
void require_op(h2w_handle *h) {
    if (!h->has_op) throw ApiError(H2W_ERR_STATE, "operator not assembled (call h2w_assemble)");
}
// Entry points of the real kernels only (mixed precision, batched, learned,
// far field on the fly, allocation-free product).
void require_real(const h2w_handle *h, const char *what) {
    if (h->cplx) throw ApiError(H2W_ERR_ARG, std::string(what) + " is not available for the complex kernels (Helmholtz, Hankel)");
}

// The reference GMRES (3D/codes/gmres.hpp:92-200, USE_Helm / USE_Hankel) on
// the complex operator: restart = max_iter, x0 from x, H(k,i) = w.dot(v_k)
// with Eigen's conjugate-first dot (sum conj(w) v_k), modified Gram-Schmidt
// in the reference's order, the reference's complex Givens formulas
// (GeneratePlaneRotation, gmres.hpp:52-68; ApplyPlaneRotation, :70-75) and
// back substitution on the host in std::complex arithmetic, stop when
// |s(i+1)| / ||b|| < tol. With H2W_OPT_COMPLEX_ARNOLDI the projections are
// Hermitian (sum conj(v_k) w) and the rotations unitary (dy' = -conj(sn) dx
// + cs dy). Krylov vectors, products and Gram-Schmidt on the GPU; the
// Hessenberg column comes to the host once per step. b, x: leaf order,
// interleaved (re, im), device.
int cgmres_run(h2w_handle *h, const double *db, double *dx, int max_iter, double tol, int *iters, double *resid) {
    typedef std::complex<double> cd;
    cudaStream_t st = h->stream;
    const int64_t n = h->tree.N;
    const int m = max_iter;
    if (h->c_V.n < (size_t)n * (size_t)(m + 1)) h->c_V.alloc((size_t)n * (size_t)(m + 1));
    if (h->c_w.n < (size_t)n) h->c_w.alloc((size_t)n);
    if (h->c_r.n < (size_t)n) h->c_r.alloc((size_t)n);
    if (h->c_ax.n < (size_t)n) h->c_ax.alloc((size_t)n);
    if (h->c_part.n < (size_t)cgm_blocks()) h->c_part.alloc((size_t)cgm_blocks());
    if (h->c_h.n < (size_t)(m + 2)) h->c_h.alloc((size_t)(m + 2));
    if (h->c_y.n < (size_t)(m + 1)) h->c_y.alloc((size_t)(m + 1));
    const double2 *b = reinterpret_cast<const double2 *>(db);
    double2 *x = reinterpret_cast<double2 *>(dx);
    auto A = [&](const double2 *in, double2 *out) {
        run_matvec_f64(h, reinterpret_cast<const double *>(in), reinterpret_cast<double *>(out), st, true);
    };
    auto dot = [&](const double2 *a, const double2 *bb, double2 *out) { CK(cgm_dot(a, bb, n, h->c_part.p, out, st)); };
    auto fetch = [&](const double2 *src, int cnt, std::vector<cd> &o) {
        std::vector<double2> t((size_t)cnt);
        CK(cudaMemcpyAsync(t.data(), src, (size_t)cnt * 16, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        o.resize((size_t)cnt);
        for (int i = 0; i < cnt; ++i) o[(size_t)i] = cd(t[(size_t)i].x, t[(size_t)i].y);
    };
    auto norm = [&](const double2 *a) {
        dot(a, a, h->c_h.p + m + 1);
        std::vector<cd> o;
        fetch(h->c_h.p + m + 1, 1, o);
        return std::sqrt(o[0].real());
    };
    auto gen_rot = [](cd &dxv, cd &dyv, cd &cs, cd &sn) {
        if (dxv == cd(0)) {
            cs = cd(0);
            sn = cd(1);
        } else {
            double scale = std::abs(dxv) + std::abs(dyv);
            double nrm = scale * std::sqrt(std::abs(dxv / scale) * std::abs(dxv / scale) +
                                           std::abs(dyv / scale) * std::abs(dyv / scale));
            cd alpha = dxv / std::abs(dxv);
            cs = std::abs(dxv) / nrm;
            sn = alpha * std::conj(dyv) / nrm;
        }
    };
    const bool herm = h->cgm_hermitian;
    auto app_rot = [herm](cd &dxv, cd &dyv, cd &cs, cd &sn) {
        cd temp = cs * dxv + sn * dyv;
        dyv = (herm ? -std::conj(sn) : -sn) * dxv + cs * dyv;
        dxv = temp;
    };
    std::vector<cd> H((size_t)(m + 1) * m, cd(0)), s((size_t)m + 1), cs((size_t)m + 1), sn((size_t)m + 1);
    auto Hc = [&](int r, int c) -> cd & { return H[(size_t)c * (m + 1) + r]; };
    auto update = [&](int k) {  // Update(x, k, H, s, v): back substitution, then x += sum_j v_j y_j
        std::vector<cd> y(s);
        for (int i = k; i >= 0; i--) {
            y[(size_t)i] /= Hc(i, i);
            for (int j = i - 1; j >= 0; j--) y[(size_t)j] -= Hc(j, i) * y[(size_t)i];
        }
        std::vector<double2> yd((size_t)k + 1);
        for (int j = 0; j <= k; ++j) yd[(size_t)j] = make_double2(y[(size_t)j].real(), y[(size_t)j].imag());
        CK(cudaMemcpyAsync(h->c_y.p, yd.data(), yd.size() * 16, cudaMemcpyHostToDevice, st));
        CK(cgm_update_launch(x, h->c_V.p, h->c_y.p, k + 1, n, st));
        CK(cudaStreamSynchronize(st));
    };
    double normb = norm(b);
    A(x, h->c_ax.p);
    CK(cgm_resid_launch(h->c_r.p, b, h->c_ax.p, n, st));
    double beta = norm(h->c_r.p);
    if (normb == 0.0) normb = 1;
    double res = beta / normb;
    *resid = res;
    *iters = 0;
    if (res <= tol) return H2W_OK;
    int j = 1;
    while (j <= max_iter) {
        CK(cgm_scale_launch(h->c_V.p, h->c_r.p, 1.0 / beta, n, st));
        std::fill(s.begin(), s.end(), cd(0));
        s[0] = beta;
        int i;
        for (i = 0; i < m && j <= max_iter; i++, j++) {
            double2 *vi = h->c_V.p + (size_t)i * n;
            A(vi, h->c_w.p);
            for (int k = 0; k <= i; k++) {
                double2 *hk = h->c_h.p + k;
                if (herm) dot(h->c_V.p + (size_t)k * n, h->c_w.p, hk);
                else dot(h->c_w.p, h->c_V.p + (size_t)k * n, hk);
                CK(cgm_axpy_launch(h->c_w.p, h->c_V.p + (size_t)k * n, hk, n, st));
            }
            const double hn = norm(h->c_w.p);
            std::vector<cd> col;
            fetch(h->c_h.p, i + 1, col);
            for (int k = 0; k <= i; ++k) Hc(k, i) = col[(size_t)k];
            Hc(i + 1, i) = hn;
            CK(cgm_scale_launch(h->c_V.p + (size_t)(i + 1) * n, h->c_w.p, 1.0 / hn, n, st));
            for (int k = 0; k < i; k++) app_rot(Hc(k, i), Hc(k + 1, i), cs[(size_t)k], sn[(size_t)k]);
            gen_rot(Hc(i, i), Hc(i + 1, i), cs[(size_t)i], sn[(size_t)i]);
            app_rot(Hc(i, i), Hc(i + 1, i), cs[(size_t)i], sn[(size_t)i]);
            app_rot(s[(size_t)i], s[(size_t)i + 1], cs[(size_t)i], sn[(size_t)i]);
            res = std::abs(s[(size_t)i + 1]) / normb;
            if (res < tol) {
                update(i);
                *resid = res;
                *iters = j;
                return H2W_OK;
            }
        }
        update(m - 1);
        A(x, h->c_ax.p);
        CK(cgm_resid_launch(h->c_r.p, b, h->c_ax.p, n, st));
        beta = norm(h->c_r.p);
        res = beta / normb;
        if (res < tol) {
            *resid = res;
            *iters = j;
            return H2W_OK;
        }
    }
    *resid = res;
    *iters = max_iter;
    return H2W_OK;
}

}  // namespace

// The product of h2w_matvec (x, y device pointers, original point order) with
// a caller-provided workspace, barrier state and error word instead of the
// handle's: used by the allocation-free entry point (noalloc.cu). Allocates
// nothing: the FP32 form needs the FP32 operator copy to exist already.
// x and y must be device (or managed) memory that this handle's device can
// address; cudaPointerGetAttributes checks that before any launch, so a host
// pointer is refused instead of faulting the kernel. The call waits for its
// launches and reads the error word back: a grid-barrier wait that ran out
// (the result is then wrong) returns H2W_ERR_CUDA on this call.
namespace {
void require_device_vector(const h2w_handle *h, const void *p, const char *name) {
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw ApiError(H2W_ERR_ARG, std::string(name) + ": not a CUDA pointer");
    }
    if (a.type == cudaMemoryTypeManaged) return;
    if (a.type != cudaMemoryTypeDevice)
        throw ApiError(H2W_ERR_ARG, std::string(name) + " is not device memory (host or unregistered pointer)");
    if (a.device != h->cfg.device)
        throw ApiError(H2W_ERR_ARG, std::string(name) + " lives on device " + std::to_string(a.device) +
                                        ", the operator on device " + std::to_string(h->cfg.device));
}
}  // namespace

namespace h2w {
int handle_device(const h2w_handle *h) { return h ? h->cfg.device : -1; }
int handle_fail(h2w_handle *h, int code, const char *msg) { return h ? fail(h, code, msg) : code; }
int matvec_external_ws(h2w_handle *h, const double *x, double *y, int precision, void *stream, double *ws,
                       int64_t ws_cap, unsigned *bar, int32_t *err) {
    return guarded(h, [&] {
        require_op(h);
        require_real(h, "the allocation-free product");
        if (!x || !y || !ws || !bar || !err || (precision != H2W_PREC_FP64 && precision != H2W_PREC_FP32))
            throw ApiError(H2W_ERR_ARG, "bad matvec arguments");
        const bool f32 = precision == H2W_PREC_FP32;
        if (f32 && !h->d_op32.p)
            throw ApiError(H2W_ERR_STATE,
                           "FP32 operator copy not materialised (one h2w_matvec call with H2W_PREC_FP32 creates it)");
        if (h->fly_active)
            throw ApiError(H2W_ERR_STATE, "the far field is evaluated on the fly (H2W_OPT_FAR_ON_THE_FLY): "
                                          "this entry point needs the stored operator");
        const int64_t need = f32 ? (h->ws_n + 1) / 2 : h->ws_n;  // in doubles
        if (need > ws_cap)
            throw ApiError(H2W_ERR_ARG, "matvec workspace of " + std::to_string(h->ws_n) + (f32 ? " floats" : " doubles") +
                                            " exceeds the static scratch maximum of " + std::to_string(ws_cap) +
                                            " doubles");
        require_device_vector(h, x, "x");
        require_device_vector(h, y, "y");
        cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
        CK(cudaMemsetAsync(ws, 0, (size_t)need * 8, st));
        CK(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
        CK(cudaMemsetAsync(err, 0, sizeof(int32_t), st));
        const int32_t *perm = h->d_perm.p;
        const int nph = (int)h->phases.size();
        if (h->coop) {
            if (f32)
                CK(launch_coop_f32(h->d_roff.p, h->d_blob.p, h->d_pstart.p, nph, h->d_op32.p, (float *)ws, x, y, perm,
                                   bar, err, st, h->spin_limit));
            else
                CK(launch_coop_f64(h->d_roff.p, h->d_blob.p, h->d_pstart.p, nph, h->d_op.p, ws, x, y, perm, bar, err,
                                   st, h->spin_limit));
        } else {
            for (const Phase &ph : h->phases) {
                if (f32)
                    CK(launch_brg_f32(h->d_roff.p, h->d_blob.p, ph.t0, ph.t1, h->d_op32.p, (float *)ws, x, y, perm, st));
                else
                    CK(launch_brg_f64(h->d_roff.p, h->d_blob.p, ph.t0, ph.t1, h->d_op.p, ws, x, y, perm, st));
            }
        }
        if (!h->fused_scatter) {
            if (f32) CK(launch_scatter_f32((float *)ws + h->yperm_off, y, perm, h->tree.N, st));
            else CK(launch_scatter_f64(ws + h->yperm_off, y, perm, h->tree.N, st));
        }
        int32_t flag = 0;
        CK(cudaMemcpyAsync(&flag, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (flag)
            throw ApiError(H2W_ERR_CUDA, "a grid-barrier wait of the product ran out (device error " +
                                             std::to_string(flag) + "); y is not valid");
        return H2W_OK;
    });
}
}  // namespace h2w

// ================================================================ C ABI ===
extern "C" {

int h2w_create(const h2w_config *cfg, h2w_handle **out) {
    if (!cfg || !out) return H2W_ERR_ARG;
    *out = nullptr;
    if (cfg->dim < 1 || cfg->dim > 3 || (cfg->form != 0 && cfg->form != 1 && cfg->form != 2) || (cfg->form == 2 && cfg->dim == 1) ||
        (cfg->choice != 0 && cfg->choice != 1 && cfg->choice != H2W_KERNEL_HELMHOLTZ && cfg->choice != H2W_KERNEL_HANKEL) ||
        (cfg->choice == H2W_KERNEL_HELMHOLTZ && (cfg->dim != 3 || cfg->form == 2)) ||
        (cfg->choice == H2W_KERNEL_HANKEL && (cfg->dim != 2 || cfg->form == 2)) || cfg->nlevels < 1 ||
        cfg->tol_pow < 0 || cfg->rank_cap < 0)
        return H2W_ERR_ARG;
    h2w_handle *h = nullptr;
    if (cfg->device >= 0) {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return H2W_ERR_CUDA;
        if (cfg->device >= ndev) return H2W_ERR_ARG;
        h = new h2w_handle;
        h->cfg = *cfg;
        h->cplx = cfg->choice == H2W_KERNEL_HELMHOLTZ || cfg->choice == H2W_KERNEL_HANKEL;
        if (cudaSetDevice(cfg->device) != cudaSuccess ||
            cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete h;
            return H2W_ERR_CUDA;
        }
    } else {
        // host-only handle: points, tree and lists, no device work
        h = new h2w_handle;
        h->cfg = *cfg;
        h->cplx = cfg->choice == H2W_KERNEL_HELMHOLTZ || cfg->choice == H2W_KERNEL_HANKEL;
    }
    *out = h;
    return H2W_OK;
}

int h2w_destroy(h2w_handle *h) {
    if (!h) return H2W_OK;
    if (h->cfg.device >= 0) cudaSetDevice(h->cfg.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto &r : h->prof_recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    for (auto &g : h->loops) {
        cudaGraphExecDestroy(g.exec);
        cudaGraphDestroy(g.graph);
    }
    cudaStream_t st = h->stream;
    delete h;
    if (st) cudaStreamDestroy(st);
    return H2W_OK;
}

const char *h2w_last_error(const h2w_handle *h) { return h ? h->err.c_str() : "null handle"; }

int h2w_set_points(h2w_handle *h, const double *pts, int64_t n) {
    return guarded(h, [&] {
        if (!pts || n < 1 || n > INT32_MAX - 1) throw ApiError(H2W_ERR_ARG, "bad point array");
        h->pts.assign(pts, pts + (size_t)n * h->cfg.dim);
        for (double v : h->pts)
            if (!std::isfinite(v)) throw ApiError(H2W_ERR_ARG, "non-finite point coordinate");
        h->has_tree = h->has_op = false;
        return H2W_OK;
    });
}

int h2w_gen_grid(h2w_handle *h, int64_t n) {
    return guarded(h, [&] {
        const int d = h->cfg.dim;
        if (n < 1) throw ApiError(H2W_ERR_ARG, "bad grid size");
        int64_t N = d == 1 ? n : (d == 2 ? n * n : n * n * n);
        if (N > INT32_MAX - 1) throw ApiError(H2W_ERR_ARG, "grid too large");
        std::vector<double> node((size_t)n);
        const double L = 1.0;
        for (int64_t k = 0; k < n; ++k) node[(size_t)k] = -L + 2.0 * L * (k + 1.0) / (n + 1.0);
        h->pts.resize((size_t)N * d);
        if (d == 1) {
            for (int64_t k = 0; k < n; ++k) h->pts[(size_t)k] = -1.0 + 2.0 * (k + 1.0) / (n + 1.0);
        } else if (d == 2) {
            for (int64_t j = 0; j < n; ++j)
                for (int64_t k = 0; k < n; ++k) {
                    size_t i = (size_t)(j * n + k);
                    h->pts[2 * i] = node[(size_t)k];
                    h->pts[2 * i + 1] = node[(size_t)j];
                }
        } else {
            for (int64_t j = 0; j < n; ++j)
                for (int64_t k = 0; k < n; ++k)
                    for (int64_t i = 0; i < n; ++i) {
                        size_t q = (size_t)((j * n + k) * n + i);
                        h->pts[3 * q] = node[(size_t)k];
                        h->pts[3 * q + 1] = node[(size_t)j];
                        h->pts[3 * q + 2] = node[(size_t)i];
                    }
        }
        h->has_tree = h->has_op = false;
        return H2W_OK;
    });
}

int h2w_gen_uniform(h2w_handle *h, uint64_t seed, int64_t n) {
    return guarded(h, [&] {
        const int d = h->cfg.dim;
        if (n < 1 || n > INT32_MAX - 1) throw ApiError(H2W_ERR_ARG, "bad point count");
        h->pts.resize((size_t)n * d);
        for (int64_t i = 0; i < n * d; ++i) {
            uint64_t z = seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z = z ^ (z >> 31);
            double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
            h->pts[(size_t)i] = 2.0 * u - 1.0;
        }
        h->has_tree = h->has_op = false;
        return H2W_OK;
    });
}

int h2w_get_points(h2w_handle *h, double *pts) {
    return guarded(h, [&] {
        require_points(h);
        if (!pts) throw ApiError(H2W_ERR_ARG, "null output");
        std::memcpy(pts, h->pts.data(), h->pts.size() * 8);
        return H2W_OK;
    });
}

int h2w_num_points(h2w_handle *h, int64_t *n) {
    return guarded(h, [&] {
        if (!n) throw ApiError(H2W_ERR_ARG, "null output");
        *n = (int64_t)(h->pts.size() / (size_t)h->cfg.dim);
        return H2W_OK;
    });
}

int h2w_build_tree(h2w_handle *h) {
    return guarded(h, [&] {
        require_points(h);
        h->tree = Tree{};
        h->tree.dim = h->cfg.dim;
        h->tree.nL = h->cfg.nlevels;
        h->tree.N = (int64_t)(h->pts.size() / (size_t)h->cfg.dim);
        h->tree.pts = h->pts;
        build_tree(h->tree);
        h->has_tree = true;
        h->has_op = false;
        if (h->cfg.device >= 0) {
            h->d_pts.upload(h->pts, h->stream);
            if (h->cplx) {  // realified permutation: (re, im) of leaf position p -> of point perm[p]
                std::vector<int32_t> p2((size_t)(2 * h->tree.N));
                for (int64_t i = 0; i < h->tree.N; ++i) {
                    p2[(size_t)(2 * i)] = 2 * h->tree.perm[(size_t)i];
                    p2[(size_t)(2 * i + 1)] = 2 * h->tree.perm[(size_t)i] + 1;
                }
                h->d_perm.upload(p2, h->stream);
            } else {
                h->d_perm.upload(h->tree.perm, h->stream);
            }
            CK(cudaStreamSynchronize(h->stream));
        }
        setup_kernel(h);
        for (int w = 0; w < 10; ++w) h->imp[w] = false;
        h->imp_ptr.assign(10, {});
        h->imp_val.assign(10, {});
        return H2W_OK;
    });
}

int h2w_get_list(h2w_handle *h, int which, int64_t *ptr, int32_t *val, int64_t *nptr, int64_t *nval) {
    return guarded(h, [&] {
        require_tree(h);
        const Tree &t = h->tree;
        std::vector<int64_t> P{0};
        std::vector<int32_t> V;
        auto add = [&](const int32_t *v, int64_t n) {
            V.insert(V.end(), v, v + n);
            P.push_back((int64_t)V.size());
        };
        const bool op = h->has_op;
        for (int j = 0; j <= t.nL; ++j)
            for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
                switch (which) {
                case H2W_LIST_CHARGE:
                    if (j == 0) {
                        std::vector<int32_t> a((size_t)t.N);
                        for (int64_t i = 0; i < t.N; ++i) a[(size_t)i] = (int32_t)i;
                        add(a.data(), t.N);
                    } else add(t.perm.data() + t.off[(size_t)j][(size_t)k], t.cnt(j, k));
                    break;
                case H2W_LIST_NBR: add(t.nb[(size_t)j].data() + k * t.nnb, t.nnb); break;
                case H2W_LIST_IL:
                case H2W_LIST_ISVERTEX: {
                    int64_t a = t.ilp[(size_t)j][(size_t)k], b = t.ilp[(size_t)j][(size_t)k + 1];
                    if (j == 0) { add(nullptr, 0); break; }
                    if (which == H2W_LIST_IL) add(t.il[(size_t)j].data() + a, b - a);
                    else {
                        std::vector<int32_t> f;
                        for (int64_t e = a; e < b; ++e) f.push_back(t.ilv[(size_t)j][(size_t)e]);
                        add(f.data(), (int64_t)f.size());
                    }
                    break;
                }
                case H2W_LIST_FAR_CHECK:
                case H2W_LIST_FAR_CHARGE:
                case H2W_LIST_VER_CHECK:
                case H2W_LIST_VER_CHARGE: {
                    const bool farl = which == H2W_LIST_FAR_CHECK || which == H2W_LIST_FAR_CHARGE;
                    const bool chk = which == H2W_LIST_FAR_CHECK || which == H2W_LIST_VER_CHECK;
                    const std::vector<Skel> *S = nullptr;
                    if (op) {
                        if (t.dim == 1) S = farl && h->cfg.form == 0 ? &h->ver : nullptr;
                        else if (h->cfg.form == H2W_FORM_NONNESTED) S = nullptr;
                        else S = farl ? &h->far : (h->cfg.form == 0 ? &h->ver : nullptr);
                    }
                    if (!S || S->empty() || (*S)[(size_t)j].ptr.empty()) { add(nullptr, 0); break; }
                    const Skel &s = (*S)[(size_t)j];
                    add((chk ? s.chk.data() : s.chg.data()) + s.ptr[(size_t)k], s.rank(k));
                    break;
                }
                case H2W_LIST_SN_ROW:
                case H2W_LIST_SN_COL: {
                    int nslot = t.dim == 1 ? (j >= 1 ? 2 : 0)
                                           : (int)(t.ilp[(size_t)j][(size_t)k + 1] - t.ilp[(size_t)j][(size_t)k]);
                    if (t.dim == 1 && j == 0) break;
                    for (int sl = 0; sl < nslot; ++sl) {
                        bool done = false;
                        if (op && h->cfg.form != H2W_FORM_NESTED && j >= 1) {
                            // the box's pairs are contiguous, in slot order
                            const Pairs &Pp = h->pairs[(size_t)j];
                            const size_t p0 = (size_t)(std::lower_bound(Pp.box.begin(), Pp.box.end(), (int32_t)k) -
                                                       Pp.box.begin());
                            for (size_t p = p0; p < Pp.box.size() && Pp.box[p] == k; ++p)
                                if (Pp.slot[p] == sl) {
                                    const auto &src = which == H2W_LIST_SN_ROW ? Pp.row : Pp.col;
                                    add(src.data() + Pp.ptr[p], Pp.ptr[p + 1] - Pp.ptr[p]);
                                    done = true;
                                    break;
                                }
                        }
                        if (!done) add(nullptr, 0);
                    }
                    break;
                }
                default: throw ApiError(H2W_ERR_ARG, "unknown list");
                }
            }
        if (nptr) *nptr = (int64_t)P.size();
        if (nval) *nval = (int64_t)V.size();
        if (ptr) std::memcpy(ptr, P.data(), P.size() * 8);
        if (val && !V.empty()) std::memcpy(val, V.data(), V.size() * 4);
        return H2W_OK;
    });
}

int h2w_import_list(h2w_handle *h, int which, const int64_t *ptr, const int32_t *val, int64_t nptr) {
    return guarded(h, [&] {
        require_tree(h);
        if (which < H2W_LIST_FAR_CHECK || which > H2W_LIST_SN_COL || !ptr || nptr < 1)
            throw ApiError(H2W_ERR_ARG, "bad import");
        h->imp_ptr[(size_t)which].assign(ptr, ptr + nptr);
        int64_t nv = ptr[nptr - 1];
        h->imp_val[(size_t)which].assign(val, val + nv);
        for (int32_t v : h->imp_val[(size_t)which])
            if (v < 0 || v >= h->tree.N) throw ApiError(H2W_ERR_ARG, "imported pivot out of range");
        h->imp[which] = true;
        return H2W_OK;
    });
}

int h2w_assemble(h2w_handle *h, int mode) {
    return guarded(h, [&] {
        require_tree(h);
        if (h->cfg.device < 0) throw ApiError(H2W_ERR_STATE, "host-only handle (device < 0) cannot assemble");
        const Tree &t = h->tree;
        // (H2+H)* and H* both keep per-pair factors; H* has no nested far field
        const bool sn = h->cfg.form != H2W_FORM_NESTED;
        const bool nn = h->cfg.form == H2W_FORM_NONNESTED;
        h->phases.clear();
        h->has_op = false;
        if (mode == H2W_ASSEMBLE_LEARNED) require_real(h, "learned assembly");
        if (mode == H2W_ASSEMBLE_LEARNED && !h->d_mlp.p)
            throw ApiError(H2W_ERR_STATE, "learned assembly needs a model (h2w_learn_set_model)");
        h->learned = mode == H2W_ASSEMBLE_LEARNED;
        static const bool timing = getenv("H2W_TIMING") && std::string(getenv("H2W_TIMING")) == "1";
        const auto ta = std::chrono::steady_clock::now();
        if (mode == H2W_ASSEMBLE_NCA || mode == H2W_ASSEMBLE_LEARNED) {
            if (t.dim > 1 && !nn) nca_far(h);
            if (!sn) nca_ver(h);
            if (sn) {
                pair_layout(h);
                nca_pairs(h);
            }
        } else if (mode == H2W_ASSEMBLE_IMPORT) {
            if (t.dim > 1 && !nn) {
                if (!h->imp[H2W_LIST_FAR_CHECK] || !h->imp[H2W_LIST_FAR_CHARGE])
                    throw ApiError(H2W_ERR_STATE, "far pivots not imported");
                import_skel(h, H2W_LIST_FAR_CHECK, H2W_LIST_FAR_CHARGE, h->far, 2);
                if (!sn) {
                    if (!h->imp[H2W_LIST_VER_CHECK] || !h->imp[H2W_LIST_VER_CHARGE])
                        throw ApiError(H2W_ERR_STATE, "vertex pivots not imported");
                    import_skel(h, H2W_LIST_VER_CHECK, H2W_LIST_VER_CHARGE, h->ver, 1);
                }
            } else if (!sn) {
                if (!h->imp[H2W_LIST_FAR_CHECK] || !h->imp[H2W_LIST_FAR_CHARGE])
                    throw ApiError(H2W_ERR_STATE, "nested-basis pivots not imported");
                import_skel(h, H2W_LIST_FAR_CHECK, H2W_LIST_FAR_CHARGE, h->ver, 1);
            }
            if (sn) {
                if (!h->imp[H2W_LIST_SN_ROW] || !h->imp[H2W_LIST_SN_COL])
                    throw ApiError(H2W_ERR_STATE, "pair pivots not imported");
                pair_layout(h);
                import_pairs(h);
            }
        } else {
            throw ApiError(H2W_ERR_ARG, "unknown assembly mode");
        }
        if (nn) h->far.clear();
        if (t.dim == 1 || sn) {
            if (h->far.empty()) {
                h->far.assign((size_t)t.nL + 1, Skel{});
                for (int j = 0; j <= t.nL; ++j) h->far[(size_t)j].ptr.assign((size_t)t.nbox[(size_t)j] + 1, 0);
            }
        }
        if (sn && h->ver.empty()) {
            h->ver.assign((size_t)t.nL + 1, Skel{});
            for (int j = 0; j <= t.nL; ++j) h->ver[(size_t)j].ptr.assign((size_t)t.nbox[(size_t)j] + 1, 0);
        }
        if (!sn && h->pairs.empty()) h->pairs.assign((size_t)t.nL + 1, Pairs{});
        const auto tb = std::chrono::steady_clock::now();
        build_plan(h);
        if (timing)
            fprintf(stderr, "h2w assembly: pivots %.3f s, operator formation %.3f s\n",
                    std::chrono::duration<double>(tb - ta).count(),
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - tb).count());
        h->storage = storage_entries(h);
        h->has_op = true;
        h->g_m = -1;
        h->gbd.m = -1;
        h->gbf.m = -1;
        h->m_wsd.reset();
        h->m_wsf.reset();
        return H2W_OK;
    });
}

int h2w_storage_entries(h2w_handle *h, double *e) {
    return guarded(h, [&] {
        require_op(h);
        if (!e) throw ApiError(H2W_ERR_ARG, "null output");
        *e = h->storage;
        return H2W_OK;
    });
}

int h2w_operator_bytes(h2w_handle *h, int precision, int64_t *bytes) {
    return guarded(h, [&] {
        require_op(h);
        if (!bytes) throw ApiError(H2W_ERR_ARG, "null output");
        *bytes = h->op_bytes_read * (precision == H2W_PREC_FP32 ? 4 : 8);
        return H2W_OK;
    });
}

int h2w_matvec(h2w_handle *h, const double *x, double *y, int nrhs, int precision, int where, void *stream) {
    return guarded(h, [&] {
        require_op(h);
        if (!x || !y || nrhs < 1 || (where != H2W_HOST && where != H2W_DEVICE)) throw ApiError(H2W_ERR_ARG, "bad matvec arguments");
        cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;
        const int64_t N = h->tree.N;
        if (precision != H2W_PREC_FP64 && precision != H2W_PREC_FP32 && precision != H2W_PREC_DF64)
            throw ApiError(H2W_ERR_ARG, "unknown precision");
        if (h->cplx) {  // complex operator: one FP64 product of interleaved (re, im) vectors
            if (precision != H2W_PREC_FP64 || nrhs != 1)
                throw ApiError(H2W_ERR_ARG, "the complex kernels (Helmholtz, Hankel) have the FP64 single-vector product only");
            const int64_t nv = h->nv();
            const double *dx = x;
            double *dy = y;
            if (where == H2W_HOST) {
                h->d_x.n < (size_t)nv ? h->d_x.alloc((size_t)nv) : (void)0;
                h->d_y.n < (size_t)nv ? h->d_y.alloc((size_t)nv) : (void)0;
                CK(cudaMemcpyAsync(h->d_x.p, x, (size_t)nv * 8, cudaMemcpyHostToDevice, st));
                dx = h->d_x.p;
                dy = h->d_y.p;
            }
            run_matvec_f64(h, dx, dy, st);
            if (where == H2W_HOST) {
                CK(cudaMemcpyAsync(y, h->d_y.p, (size_t)nv * 8, cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                check_device_error(h);
            }
            return H2W_OK;
        }
        const bool df_single = nrhs == 1 && precision == H2W_PREC_DF64 && h->fly_active;
        if (nrhs > 1 || (precision == H2W_PREC_DF64 && !df_single)) {
            // blocks of up to 64 columns through the multi-vector kernel
            ensure_multi_vectors(h);
            if (where == H2W_HOST) {
                if (h->m_stage_x.n < (size_t)N * MR_MAX) h->m_stage_x.alloc((size_t)N * MR_MAX);
                if (h->m_stage_y.n < (size_t)N * MR_MAX) h->m_stage_y.alloc((size_t)N * MR_MAX);
            }
            for (int c0 = 0; c0 < nrhs; c0 += MR_MAX) {
                const int nc = std::min(MR_MAX, nrhs - c0), rp = rp_for(nc);
                const double *xc = x + (size_t)c0 * N;
                double *yc = y + (size_t)c0 * N;
                if (where == H2W_HOST) {
                    CK(cudaMemcpyAsync(h->m_stage_x.p, xc, (size_t)N * nc * 8, cudaMemcpyHostToDevice, st));
                    xc = h->m_stage_x.p;
                }
                CK(launch_mr_pack(xc, N, h->m_xi.p, h->d_perm.p, N, nc, rp, st));
                run_matvec_multi(h, precision, rp, h->m_xi.p, h->m_yi.p, st);
                CK(launch_mr_unpack(h->m_yi.p, where == H2W_HOST ? h->m_stage_y.p : yc, N, h->d_perm.p, N, nc, rp,
                                    st));
                if (where == H2W_HOST)
                    CK(cudaMemcpyAsync(yc, h->m_stage_y.p, (size_t)N * nc * 8, cudaMemcpyDeviceToHost, st));
            }
            if (where == H2W_HOST) CK(cudaStreamSynchronize(st));
            check_device_error(h);
            return H2W_OK;
        }
        if (where == H2W_HOST) {
            h->d_x.n < (size_t)N ? h->d_x.alloc((size_t)N) : (void)0;
            h->d_y.n < (size_t)N ? h->d_y.alloc((size_t)N) : (void)0;
        }
        for (int c = 0; c < nrhs; ++c) {
            const double *xc = x + (size_t)c * N;
            double *yc = y + (size_t)c * N;
            const double *dx = xc;
            double *dy = yc;
            if (where == H2W_HOST) {
                CK(cudaMemcpyAsync(h->d_x.p, xc, (size_t)N * 8, cudaMemcpyHostToDevice, st));
                dx = h->d_x.p;
                dy = h->d_y.p;
            }
            if (precision == H2W_PREC_FP32) {
                run_matvec_f32(h, dx, dy, st);
            } else {
                run_matvec_f64(h, dx, dy, st, false, df_single);
            }
            if (where == H2W_HOST) CK(cudaMemcpyAsync(yc, h->d_y.p, (size_t)N * 8, cudaMemcpyDeviceToHost, st));
        }
        if (where == H2W_HOST) {
            CK(cudaStreamSynchronize(st));
            check_device_error(h);
        }
        return H2W_OK;
    });
}

int h2w_gmres(h2w_handle *h, const double *b, double *x, int max_iter, int tol_pow, int where, int *iters,
              double *resid) {
    return guarded(h, [&] {
        require_op(h);
        if (!b || !x || max_iter < 1 || !iters || !resid) throw ApiError(H2W_ERR_ARG, "bad gmres arguments");
        const int64_t N = h->nv();  // doubles per vector (interleaved (re, im) for the complex kernel)
        double tol = std::pow(10, -1.0 * tol_pow);
        const double *db = b;
        double *dx = x;
        if (where == H2W_HOST) {
            h->g_b.n < (size_t)N ? h->g_b.alloc((size_t)N) : (void)0;
            h->d_x.n < (size_t)N ? h->d_x.alloc((size_t)N) : (void)0;
            CK(cudaMemcpyAsync(h->g_b.p, b, (size_t)N * 8, cudaMemcpyHostToDevice, h->stream));
            CK(cudaMemcpyAsync(h->d_x.p, x, (size_t)N * 8, cudaMemcpyHostToDevice, h->stream));
            db = h->g_b.p;
            dx = h->d_x.p;
        }
        DBuf<double> &bp = h->s_b, &xp = h->s_x;
        if (bp.n < (size_t)N) bp.alloc((size_t)N);
        if (xp.n < (size_t)N) xp.alloc((size_t)N);
        CK(launch_gather_f64(db, bp.p, h->d_perm.p, N, h->stream));
        CK(launch_gather_f64(dx, xp.p, h->d_perm.p, N, h->stream));
        int rc = h->cplx ? cgmres_run(h, bp.p, xp.p, max_iter, tol, iters, resid)
                         : gmres_run(h, bp.p, xp.p, max_iter, tol, H2W_PREC_FP64, iters, resid);
        CK(launch_scatter_f64(xp.p, dx, h->d_perm.p, N, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        check_device_error(h);
        if (where == H2W_HOST) {
            CK(cudaMemcpyAsync(x, h->d_x.p, (size_t)N * 8, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        }
        return rc;
    });
}

int h2w_gmres_ir(h2w_handle *h, const double *b, double *x, int max_outer, int inner_iter, int tol_pow, int where,
                 int *outer_iters, int *inner_total, double *resid) {
    return guarded(h, [&] {
        require_op(h);
        require_real(h, "h2w_gmres_ir");
        if (!b || !x || max_outer < 1 || inner_iter < 1 || !outer_iters || !inner_total || !resid)
            throw ApiError(H2W_ERR_ARG, "bad gmres_ir arguments");
        const int64_t N = h->tree.N;
        cudaStream_t st = h->stream;
        double tol = std::pow(10, -1.0 * tol_pow);
        const double *db = b;
        double *dx = x;
        if (where == H2W_HOST) {
            h->g_b.n < (size_t)N ? h->g_b.alloc((size_t)N) : (void)0;
            h->d_x.n < (size_t)N ? h->d_x.alloc((size_t)N) : (void)0;
            CK(cudaMemcpyAsync(h->g_b.p, b, (size_t)N * 8, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(h->d_x.p, x, (size_t)N * 8, cudaMemcpyHostToDevice, st));
            db = h->g_b.p;
            dx = h->d_x.p;
        }
        GmresDev g = gmres_state(h, inner_iter);
        (void)g;
        DBuf<double> &r = h->s_r, &d = h->s_d, &bp = h->s_b, &xp = h->s_x;
        for (DBuf<double> *v : {&r, &d, &bp, &xp, &h->s_t})
            if (v->n < (size_t)N) v->alloc((size_t)N);
        CK(launch_gather_f64(db, bp.p, h->d_perm.p, N, st));
        CK(launch_gather_f64(dx, xp.p, h->d_perm.p, N, st));
        const double *db_user = db;
        double *dx_user = dx;
        db = bp.p;
        dx = xp.p;
        double normb = dnorm(h, db);
        if (normb == 0.0) normb = 1;
        const bool x0_zero = dnorm(h, dx) == 0.0;
        *inner_total = 0;
        *outer_iters = 0;
        int rc = H2W_ERR_NOT_CONVERGED;
        const double eta = h->ir_update ? fp32_error_single(h, st) : 0.0;
        double drift = HUGE_VAL;  // error bound of r since the last accurate residual
        bool above_floor = false;  // the accurate residual's own error is far below the tolerance
        for (int o = 0; o <= max_outer; ++o) {
            // residual: FP32 operator at x0 (a correction only), then FP64 (the
            // stopping test), or r -= A32 d while its error bound allows
            double add = HUGE_VAL;
            if (h->ir_update && o >= 2 && above_floor) add = IR_UPDATE_SAFETY * eta * dnorm(h, d.p);
            if (drift + add <= IR_UPDATE_SHARE * tol * normb) {
                run_matvec_f32(h, d.p, h->s_t.p, st, true);
                CK(vec_axpby(1.0, r.p, -1.0, h->s_t.p, r.p, N, st));
                drift += add;
            } else if (o == 0 && x0_zero) {  // r = b without a product
                CK(cudaMemcpyAsync(r.p, db, (size_t)N * 8, cudaMemcpyDeviceToDevice, st));
                drift = HUGE_VAL;
            } else {
                if (o == 0) run_matvec_f32(h, dx, r.p, st, true);
                else run_matvec_f64(h, dx, r.p, st, true, h->ir_resid_prec == H2W_PREC_DF64);
                CK(vec_axpby(1.0, db, -1.0, r.p, r.p, N, st));
                drift = o == 0 ? HUGE_VAL : 0.0;
                if (o == 1 && h->ir_update)
                    above_floor = IR_UPDATE_SAFETY * eta * IR_U64_OVER_U32 * dnorm(h, dx) <= IR_UPDATE_FLOOR * tol * normb;
            }
            if (o > 0) {
                *resid = (dnorm(h, r.p) + drift) / normb;
                if (*resid < tol) { rc = H2W_OK; break; }
                if (o == max_outer) break;
            }
            CK(cudaMemsetAsync(d.p, 0, (size_t)N * 8, st));
            int it = 0;
            double ires = 0;
            // inner: FP32 operator, relative reduction of the current residual to a
            // tenth of the target (1e-6 in the first step)
            gmres_run(h, r.p, d.p, inner_iter, o == 0 ? 1e-6 : inner_tol(tol, 1.0, *resid), H2W_PREC_FP32, &it, &ires,
                      true);
            *inner_total += it;
            CK(vec_axpby(1.0, dx, 1.0, d.p, dx, N, st));
            *outer_iters = o + 1;
        }
        (void)db_user;
        CK(launch_scatter_f64(xp.p, dx_user, h->d_perm.p, N, st));
        if (where == H2W_HOST) {
            CK(cudaMemcpyAsync(x, h->d_x.p, (size_t)N * 8, cudaMemcpyDeviceToHost, st));
        }
        CK(cudaStreamSynchronize(st));
        check_device_error(h);
        return rc;
    });
}

int h2w_gmres_batch(h2w_handle *h, const double *b, double *x, int nrhs, int max_iter, int tol_pow, int where,
                    int *iters, double *resid) {
    return guarded(h, [&] {
        require_op(h);
        require_real(h, "h2w_gmres_batch");
        if (!b || !x || nrhs < 1 || max_iter < 1 || max_iter > 400 || !iters || !resid ||
            (where != H2W_HOST && where != H2W_DEVICE))
            throw ApiError(H2W_ERR_ARG, "bad gmres_batch arguments");
        const double tol = std::pow(10, -1.0 * tol_pow);
        int rc = H2W_OK;
        for_rhs_blocks(h, b, x, nrhs, where, [&](int c0, int nc, int rp, double *bi, double *xi) {
            int r = gmres_batch_run(h, bi, xi, rp, nc, max_iter, tol, H2W_PREC_FP64, false, iters + c0, resid + c0);
            if (r != H2W_OK) rc = r;
        });
        return rc;
    });
}

int h2w_gmres_ir_batch(h2w_handle *h, const double *b, double *x, int nrhs, int max_outer, int inner_iter,
                       int tol_pow, int where, int *outer_iters, int *inner_total, double *resid) {
    return guarded(h, [&] {
        require_op(h);
        require_real(h, "h2w_gmres_ir_batch");
        if (!b || !x || nrhs < 1 || max_outer < 1 || inner_iter < 1 || inner_iter > 400 || !outer_iters ||
            !inner_total || !resid || (where != H2W_HOST && where != H2W_DEVICE))
            throw ApiError(H2W_ERR_ARG, "bad gmres_ir_batch arguments");
        const int64_t N = h->tree.N;
        cudaStream_t st = h->stream;
        const double tol = std::pow(10, -1.0 * tol_pow);
        *outer_iters = 0;
        *inner_total = 0;
        int rc = H2W_OK;
        if (h->m_ri.n < (size_t)N * MR_MAX) h->m_ri.alloc((size_t)N * MR_MAX);
        if (h->m_di.n < (size_t)N * MR_MAX) h->m_di.alloc((size_t)N * MR_MAX);
        if (!h->m_onorm.p) h->m_onorm.alloc(MR_MAX);
        if (!h->m_ores.p) h->m_ores.alloc(MR_MAX);
        if (h->m_ti.n < (size_t)N * MR_MAX) h->m_ti.alloc((size_t)N * MR_MAX);
        if (h->m_dn.n < (size_t)2 * MR_MAX) h->m_dn.alloc((size_t)2 * MR_MAX);
        // g: the inner solves' state (FP32 or FP64 basis), here for its reductions
        auto block = [&](auto g, int c0, int nc, int rp, double *bi, double *xi) {
            const size_t len = (size_t)N * rp;
            CK(gmb_norms(g, bi, h->m_onorm.p, 1, st));
            std::vector<double> nb((size_t)rp), nr((size_t)rp);
            CK(cudaMemcpyAsync(nb.data(), h->m_onorm.p, (size_t)rp * 8, cudaMemcpyDeviceToHost, st));
            std::vector<int> it((size_t)rp);
            std::vector<double> ir((size_t)rp), nd((size_t)rp);
            std::vector<double> drift((size_t)rp, HUGE_VAL);  // error bound of r since the last accurate residual
            bool above_floor = false;  // every column's accurate-residual error far below its tolerance
            // a zero start block (the usual x0) has r = b without a product
            CK(gmb_norms(g, xi, h->m_dn.p, 0, st));
            CK(cudaMemcpyAsync(nd.data(), h->m_dn.p, (size_t)rp * 8, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            bool x0_zero = true;
            for (int c = 0; c < rp; ++c)
                if (nd[(size_t)c] != 0.0) x0_zero = false;
            const double eta = h->ir_update ? fp32_error_multi(h, g, rp, st) : 0.0;
            bool ok = false;
            for (int o = 0; o <= max_outer; ++o) {
                // residual r = b - A x: FP32 operator at x0 (a correction only), then
                // FP64 (or double-FP32) products, which are the stopping test, or
                // r - A32 d while every column's error bound allows it: from the inner
                // solve's Arnoldi relation (no product) or from an FP32 product
                using BT = typename std::remove_pointer<decltype(g.V)>::type;
                const int jres = gmb_store(h, (BT *)nullptr).jres;  // the inner state is g's
                bool upd = h->ir_update && o >= 2 && above_floor, arn = upd && jres >= 0;
                if (upd) {
                    CK(gmb_norms(g, h->m_di.p, h->m_dn.p, 0, st));
                    CK(cudaMemcpyAsync(nd.data(), h->m_dn.p, (size_t)rp * 8, cudaMemcpyDeviceToHost, st));
                    CK(cudaStreamSynchronize(st));
                    for (int c = 0; c < nc; ++c) {
                        const double budget = IR_UPDATE_SHARE * tol * nb[(size_t)c];
                        if (!(drift[(size_t)c] + IR_UPDATE_SAFETY * IR_UPDATE_ARNOLDI * eta * nd[(size_t)c] <= budget))
                            arn = false;
                        if (!(drift[(size_t)c] + IR_UPDATE_SAFETY * eta * nd[(size_t)c] <= budget)) upd = false;
                    }
                    arn = arn && upd;
                }
                if (arn) {  // r - A32 d = (r - r_f) + V z of the last inner solve
                    CK(gmb_residual(g, h->m_ri.p, h->m_ti.p, jres, st));
                    std::swap(h->m_ri.p, h->m_ti.p);
                    std::swap(h->m_ri.n, h->m_ti.n);
                    for (int c = 0; c < nc; ++c)
                        drift[(size_t)c] += IR_UPDATE_SAFETY * IR_UPDATE_ARNOLDI * eta * nd[(size_t)c];
                } else if (upd) {
                    run_matvec_multi(h, H2W_PREC_FP32, rp, h->m_di.p, h->m_ti.p, st);
                    CK(vec_axpby(1.0, h->m_ri.p, -1.0, h->m_ti.p, h->m_ri.p, (int64_t)len, st));
                    for (int c = 0; c < nc; ++c) drift[(size_t)c] += IR_UPDATE_SAFETY * eta * nd[(size_t)c];
                } else if (o == 0 && x0_zero) {
                    CK(cudaMemcpyAsync(h->m_ri.p, bi, len * 8, cudaMemcpyDeviceToDevice, st));
                } else {
                    run_matvec_multi(h, o == 0 ? H2W_PREC_FP32 : h->ir_resid_prec, rp, xi, h->m_ri.p, st);
                    CK(vec_axpby(1.0, bi, -1.0, h->m_ri.p, h->m_ri.p, (int64_t)len, st));
                    std::fill(drift.begin(), drift.end(), o == 0 ? HUGE_VAL : 0.0);
                    if (o == 1 && h->ir_update) {
                        CK(gmb_norms(g, xi, h->m_dn.p, 0, st));
                        CK(cudaMemcpyAsync(nd.data(), h->m_dn.p, (size_t)rp * 8, cudaMemcpyDeviceToHost, st));
                        CK(cudaStreamSynchronize(st));
                        above_floor = true;
                        for (int c = 0; c < nc; ++c)
                            if (!(IR_UPDATE_SAFETY * eta * IR_U64_OVER_U32 * nd[(size_t)c] <=
                                  IR_UPDATE_FLOOR * tol * nb[(size_t)c]))
                                above_floor = false;
                    }
                }
                if (o > 0) {
                    CK(gmb_norms(g, h->m_ri.p, h->m_ores.p, 0, st));
                    CK(cudaMemcpyAsync(nr.data(), h->m_ores.p, (size_t)rp * 8, cudaMemcpyDeviceToHost, st));
                    CK(cudaStreamSynchronize(st));
                    ok = true;
                    for (int c = 0; c < nc; ++c) {
                        resid[c0 + c] = (nr[(size_t)c] + drift[(size_t)c]) / nb[(size_t)c];
                        if (!(resid[c0 + c] < tol)) ok = false;
                    }
                    if (ok || o == max_outer) break;
                }
                // FP32-operator inner GMRES on A d = r from d = 0; relative tolerance: the
                // strictest column's need (1e-6 in the first step)
                double tin = o == 0 ? 1e-6 : 0.1;
                if (o > 0)
                    for (int c = 0; c < nc; ++c)
                        tin = std::min(tin, inner_tol(tol, 1.0, resid[c0 + c]));
                CK(cudaMemsetAsync(h->m_di.p, 0, len * 8, st));
                gmres_batch_run(h, h->m_ri.p, h->m_di.p, rp, nc, inner_iter, tin, H2W_PREC_FP32, true, it.data(),
                                ir.data());
                int mx = 0;
                for (int c = 0; c < nc; ++c) mx = std::max(mx, it[(size_t)c]);
                *inner_total += mx;
                CK(vec_axpby(1.0, xi, 1.0, h->m_di.p, xi, (int64_t)len, st));
                *outer_iters = std::max(*outer_iters, o + 1);
            }
            if (!ok) rc = H2W_ERR_NOT_CONVERGED;
        };
        for_rhs_blocks(h, b, x, nrhs, where, [&](int c0, int nc, int rp, double *bi, double *xi) {
            if (h->f32_basis) block(gmb_state<float>(h, inner_iter, rp, nc), c0, nc, rp, bi, xi);
            else block(gmb_state<double>(h, inner_iter, rp, nc), c0, nc, rp, bi, xi);
        });
        return rc;
    });
}

int h2w_set_option(h2w_handle *h, int option, int64_t value) {
    return guarded(h, [&] {
        if (option == H2W_OPT_GRAPH) {
            h->use_graphs = value != 0;
            h->graph_failed = false;
        } else if (option == H2W_OPT_IR_RESIDUAL) {
            if (value != H2W_PREC_FP64 && value != H2W_PREC_DF64)
                throw ApiError(H2W_ERR_ARG, "IR residual precision must be FP64 or DF64");
            h->ir_resid_prec = (int)value;
        } else if (option == H2W_OPT_MULTI_XW) {
            if (h->has_op) realize_multi(h, value);
            else if (value < 32 || value > MR_XS_ELEMS || value % 4) throw ApiError(H2W_ERR_ARG, "column cap out of range");
            h->mr_xw = value;
        } else if (option == H2W_OPT_ROW_SPLIT) {
            if (h->has_op) realize_single(h, value);
            else if (value < 256 || value > (int64_t(1) << 24)) throw ApiError(H2W_ERR_ARG, "row split out of range");
            h->row_split = value;
        } else if (option == H2W_OPT_IR_UPDATE) {
            h->ir_update = value != 0;
        } else if (option == H2W_OPT_F32_BASIS) {
            h->f32_basis = value != 0;
        } else if (option == H2W_OPT_DATAFLOW) {
            h->dataflow = value != 0;
            h->eta_multi = -1.0;
            for (auto &g : h->loops) {  // captured steps hold the other launch form
                cudaGraphExecDestroy(g.exec);
                cudaGraphDestroy(g.graph);
            }
            h->loops.clear();
        } else if (option == H2W_OPT_PRODUCER_WARP) {
            h->producer_warp = value != 0;
            h->eta_multi = -1.0;
            for (auto &g : h->loops) {  // captured steps hold the other kernel
                cudaGraphExecDestroy(g.exec);
                cudaGraphDestroy(g.graph);
            }
            h->loops.clear();
        } else if (option == H2W_OPT_TENSOR) {
            h->tensor = value != 0;
            h->eta_multi = -1.0;
            for (auto &g : h->loops) {  // captured steps hold the other kernel
                cudaGraphExecDestroy(g.exec);
                cudaGraphDestroy(g.graph);
            }
            h->loops.clear();
        } else if (option == H2W_OPT_SPIN_LIMIT) {
            if (value < 0) throw ApiError(H2W_ERR_ARG, "spin limit must be >= 0");
            h->spin_limit = value;
        } else if (option == H2W_OPT_NCA_DF) {
            h->nca_df = value != 0;
        } else if (option == H2W_OPT_COMPLEX_ARNOLDI) {
            h->cgm_hermitian = value != 0;
        } else if (option == H2W_OPT_FAR_ON_THE_FLY) {
            if (value != 0) require_real(h, "the far field on the fly");
            h->far_fly = value != 0;  // takes effect at the next h2w_assemble
        } else if (option == H2W_OPT_COOP) {
            h->coop = value != 0;
            for (auto &g : h->loops) {  // captured steps hold the other launch form
                cudaGraphExecDestroy(g.exec);
                cudaGraphDestroy(g.graph);
            }
            h->loops.clear();
        } else {
            throw ApiError(H2W_ERR_ARG, "unknown option");
        }
        return H2W_OK;
    });
}

int h2w_get_option(h2w_handle *h, int option, int64_t *value) {
    return guarded(h, [&] {
        if (!value) throw ApiError(H2W_ERR_ARG, "null value");
        if (option == H2W_OPT_GRAPH) *value = (h->use_graphs && !h->graph_failed) ? 1 : 0;
        else if (option == H2W_OPT_COOP) *value = h->coop ? 1 : 0;
        else if (option == H2W_OPT_IR_RESIDUAL) *value = h->ir_resid_prec;
        else if (option == H2W_OPT_MULTI_XW) *value = h->mr_xw;
        else if (option == H2W_OPT_ROW_SPLIT) *value = h->row_split;
        else if (option == H2W_OPT_IR_UPDATE) *value = h->ir_update ? 1 : 0;
        else if (option == H2W_OPT_TENSOR) *value = h->tensor ? 1 : 0;
        else if (option == H2W_OPT_F32_BASIS) *value = h->f32_basis ? 1 : 0;
        else if (option == H2W_OPT_DATAFLOW) *value = h->dataflow ? 1 : 0;
        else if (option == H2W_OPT_PRODUCER_WARP) *value = h->producer_warp ? 1 : 0;
        else if (option == H2W_OPT_SPIN_LIMIT) *value = h->spin_limit;
        else if (option == H2W_OPT_FAR_ON_THE_FLY) *value = h->far_fly ? 1 : 0;
        else if (option == H2W_OPT_NCA_DF) *value = h->nca_df ? 1 : 0;
        else if (option == H2W_OPT_COMPLEX_ARNOLDI) *value = h->cgm_hermitian ? 1 : 0;
        else throw ApiError(H2W_ERR_ARG, "unknown option");
        return H2W_OK;
    });
}

int h2w_autotune(h2w_handle *h, int nrhs, int precision, int reps, int64_t *chosen, double *best_ms) {
    return guarded(h, [&] {
        require_op(h);
        require_real(h, "h2w_autotune");
        const bool mix = precision == H2W_TUNE_IR_MIX;
        if (nrhs < 1 || reps < 1 ||
            (precision != H2W_PREC_FP64 && precision != H2W_PREC_FP32 && precision != H2W_PREC_DF64 && !mix) ||
            (nrhs == 1 && (precision == H2W_PREC_DF64 || mix)))
            throw ApiError(H2W_ERR_ARG, "bad autotune arguments");
        cudaStream_t st = h->stream;
        const int64_t N = h->tree.N;
        const bool multi = nrhs > 1;
        const int rp = rp_for(std::min(nrhs, MR_MAX));
        // inputs: zeros (the products' cost does not depend on the values)
        if (multi) {
            ensure_multi_vectors(h);
            CK(cudaMemsetAsync(h->m_xi.p, 0, (size_t)N * rp * 8, st));
        } else {
            if (h->d_x.n < (size_t)N) h->d_x.alloc((size_t)N);
            if (h->d_y.n < (size_t)N) h->d_y.alloc((size_t)N);
            CK(cudaMemsetAsync(h->d_x.p, 0, (size_t)N * 8, st));
        }
        const std::vector<int64_t> cand = multi ? std::vector<int64_t>{256, 512, 1024, 2048}
                                                : std::vector<int64_t>{4096, 8192, 16384, 32768, 65536};
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        int64_t best = multi ? h->mr_xw : h->row_split;
        // the FP32 dataflow product's two forms (producer warp or not) are candidates too
        const bool forms = multi && (mix || precision == H2W_PREC_FP32) && h->dataflow && h->coop && !h->tensor;
        const bool pw0 = h->producer_warp;
        bool best_pw = pw0;
        double bms = 1e300;
        const bool prof = h->prof;
        h->prof = false;
        try {
            for (int f = 0; f < (forms ? 2 : 1); ++f)
            for (int64_t c : cand) {
                h->producer_warp = forms ? f == 0 : pw0;
                if (multi) realize_multi(h, c);
                else realize_single(h, c);
                auto once = [&] {
                    if (mix) {  // the batched refinement's mix: four FP32 products per DF64 residual
                        for (int q = 0; q < 4; ++q) run_matvec_multi(h, H2W_PREC_FP32, rp, h->m_xi.p, h->m_yi.p, st);
                        run_matvec_multi(h, H2W_PREC_DF64, rp, h->m_xi.p, h->m_yi.p, st);
                    } else if (multi) run_matvec_multi(h, precision, rp, h->m_xi.p, h->m_yi.p, st);
                    else if (precision == H2W_PREC_FP32) run_matvec_f32(h, h->d_x.p, h->d_y.p, st, true);
                    else run_matvec_f64(h, h->d_x.p, h->d_y.p, st, true);
                };
                once();  // first use (workspace, attributes) outside the timing
                CK(cudaEventRecord(e0, st));
                for (int r = 0; r < reps; ++r) once();
                CK(cudaEventRecord(e1, st));
                CK(cudaEventSynchronize(e1));
                float ms = 0.f;
                CK(cudaEventElapsedTime(&ms, e0, e1));
                check_device_error(h);
                if (ms / reps < bms) {
                    bms = ms / reps;
                    best = c;
                    best_pw = h->producer_warp;
                }
            }
        } catch (...) {
            h->producer_warp = pw0;
            h->prof = prof;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        h->prof = prof;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (h->producer_warp != best_pw || pw0 != best_pw) {
            h->producer_warp = best_pw;
            for (auto &g : h->loops) {  // captured steps hold the other kernel
                cudaGraphExecDestroy(g.exec);
                cudaGraphDestroy(g.graph);
            }
            h->loops.clear();
        }
        if (multi) realize_multi(h, best);
        else realize_single(h, best);
        if (chosen) *chosen = best;
        if (best_ms) *best_ms = bms;
        return H2W_OK;
    });
}

int h2w_batch_create(h2w_handle *const *handles, int n, h2w_batch **out) {
    if (!handles || n < 1 || !out) return H2W_ERR_ARG;
    *out = nullptr;
    if (n >= (1 << 22)) return H2W_ERR_ARG;
    auto *b = new h2w_batch();
    b->hs.assign(handles, handles + n);
    for (h2w_handle *h : b->hs)
        if (!h || !h->has_op || !h->plan || h->cfg.device != b->hs[0]->cfg.device || h->fly_active || h->cplx) {
            delete b;
            return H2W_ERR_STATE;
        }
    b->device = b->hs[0]->cfg.device;
    int rc = bguarded(b, [&] {
        CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        const int P = n;
        b->off.assign((size_t)P + 1, 0);
        b->wsoff.assign((size_t)P + 1, 0);
        for (int p = 0; p < P; ++p) {
            b->off[(size_t)p + 1] = b->off[(size_t)p] + b->hs[(size_t)p]->tree.N;
            b->wsoff[(size_t)p + 1] = b->wsoff[(size_t)p] + b->hs[(size_t)p]->ws_n;
        }
        b->Ntot = b->off[(size_t)P];
        // per problem: its single-vector stream with the problem index in the flags
        struct Rec { int slot; double size; std::vector<int64_t> words; };
        std::vector<std::vector<Rec>> per((size_t)P);
        size_t maxph = 0;
        std::vector<size_t> nph((size_t)P);
        for (int p = 0; p < P; ++p) {
            h2w_handle *h = b->hs[(size_t)p];
            PlanBuilder &pb = *h->plan;
            std::vector<Phase> ph;
            bool fused = true;
            pb.realize(h->row_split, 4, XW_CAP);
            assign_phases(h, pb, h->nph_total, ph, fused);
            validate_plan(pb, h, ph);
            if (!fused) b->unfused.push_back(p);
            for (Target &t : pb.T) t.flags |= (p << 8);
            std::vector<int64_t> ro, bl, ps;
            pack_records(pb, ph, ro, bl, ps);
            first_writers_overwrite(ro, bl, h->ws_n);
            nph[(size_t)p] = ph.size();
            maxph = std::max(maxph, ph.size());
            for (size_t j = 0; j < ph.size(); ++j)
                for (int64_t t = ph[j].t0; t < ph[j].t1; ++t) {
                    const Target &tg = pb.T[(size_t)t];
                    Rec r;
                    r.slot = (int)j;
                    r.size = (double)tg.nrows * (double)tg.xw;
                    r.words.assign(bl.begin() + ro[(size_t)t], bl.begin() + ro[(size_t)t + 1]);
                    per[(size_t)p].push_back(std::move(r));
                }
            pb.T = std::vector<Target>();
            pb.P = std::vector<Panel>();
            pb.S = std::vector<Seg>();
        }
        // merged phases, aligned at the leaf end; heaviest first within a phase
        std::vector<std::vector<std::pair<double, const Rec *>>> slots(maxph);
        for (int p = 0; p < P; ++p)
            for (const Rec &r : per[(size_t)p])
                slots[(size_t)r.slot + (maxph - nph[(size_t)p])].push_back({r.size, &r});
        std::vector<int64_t> roff{0}, blob, pstart;
        for (auto &sl : slots) {
            std::stable_sort(sl.begin(), sl.end(), [](const auto &a, const auto &c) { return a.first > c.first; });
            pstart.push_back((int64_t)roff.size() - 1);
            for (auto &e : sl) {
                blob.insert(blob.end(), e.second->words.begin(), e.second->words.end());
                roff.push_back((int64_t)blob.size());
            }
        }
        pstart.push_back((int64_t)roff.size() - 1);
        b->nphase = (int)maxph;
        cudaStream_t st = b->stream;
        b->roff.upload(roff, st);
        b->blob.upload(blob, st);
        b->pstart.upload(pstart, st);
        b->ws64.alloc((size_t)b->wsoff[(size_t)P]);
        std::vector<BatchProb> to((size_t)P), tl((size_t)P);
        for (int p = 0; p < P; ++p) {
            h2w_handle *h = b->hs[(size_t)p];
            to[(size_t)p] = {h->d_op.p, b->ws64.p + b->wsoff[(size_t)p], h->d_perm.p, b->off[(size_t)p]};
            tl[(size_t)p] = to[(size_t)p];
            tl[(size_t)p].perm = nullptr;
        }
        b->tab64_orig.upload(to, st);
        b->tab64_leaf.upload(tl, st);
        std::vector<int64_t> pa((size_t)b->Ntot);
        for (int p = 0; p < P; ++p) {
            const auto &pm = b->hs[(size_t)p]->tree.perm;
            for (size_t t = 0; t < pm.size(); ++t) pa[(size_t)b->off[(size_t)p] + t] = b->off[(size_t)p] + pm[t];
        }
        b->perm_all.upload(pa, st);
        b->bar.alloc(2);
        CK(cudaMemsetAsync(b->bar.p, 0, 8, st));
        b->errf.alloc(1);
        CK(cudaMemsetAsync(b->errf.p, 0, 4, st));
        for (DBuf<double> *v : {&b->sx, &b->sy, &b->bl, &b->xl, &b->r, &b->d}) v->alloc((size_t)b->Ntot);
        // segmented GMRES blocks: about 2048 rows each, never across problems
        std::vector<int32_t> bprob, pblk{0};
        std::vector<int64_t> brow{0};
        for (int p = 0; p < P; ++p) {
            const int64_t Np = b->hs[(size_t)p]->tree.N;
            const int64_t nb = std::max<int64_t>(1, (Np + 2047) / 2048);
            for (int64_t q = 0; q < nb; ++q) {
                bprob.push_back(p);
                brow.push_back(b->off[(size_t)p] + std::min(Np, (q + 1) * ((Np + nb - 1) / nb)));
            }
            pblk.push_back((int32_t)bprob.size());
        }
        b->nblk = (int)bprob.size();
        b->bprob.upload(bprob, st);
        b->brow.upload(brow, st);
        b->pblk.upload(pblk, st);
        for (DBuf<double> *v : {&b->normb, &b->resid, &b->onorm, &b->ores}) v->alloc((size_t)P);
        b->conv.alloc((size_t)P);
        b->iter.alloc(2);
        CK(cudaStreamSynchronize(st));
        return H2W_OK;
    });
    if (rc != H2W_OK) {
        if (b->stream) cudaStreamDestroy(b->stream);
        delete b;
        return rc;
    }
    *out = b;
    return H2W_OK;
}

int h2w_batch_destroy(h2w_batch *b) {
    if (!b) return H2W_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    cudaStream_t st = b->stream;
    delete b;
    if (st) cudaStreamDestroy(st);
    return H2W_OK;
}

const char *h2w_batch_last_error(const h2w_batch *b) { return b ? b->err.c_str() : "null batch"; }

int h2w_batch_offsets(h2w_batch *b, int64_t *offsets) {
    return bguarded(b, [&] {
        if (!offsets) throw ApiError(H2W_ERR_ARG, "null offsets");
        for (size_t p = 0; p < b->off.size(); ++p) offsets[p] = b->off[p];
        return H2W_OK;
    });
}

int h2w_batch_matvec(h2w_batch *b, const double *x, double *y, int precision, int where) {
    return bguarded(b, [&] {
        if (!x || !y || (precision != H2W_PREC_FP64 && precision != H2W_PREC_FP32) ||
            (where != H2W_HOST && where != H2W_DEVICE))
            throw ApiError(H2W_ERR_ARG, "bad batch matvec arguments");
        const double *dx = x;
        double *dy = y;
        if (where == H2W_HOST) {
            CK(cudaMemcpyAsync(b->sx.p, x, (size_t)b->Ntot * 8, cudaMemcpyHostToDevice, b->stream));
            dx = b->sx.p;
            dy = b->sy.p;
        }
        run_batch(b, precision, dx, dy, false);
        if (where == H2W_HOST) CK(cudaMemcpyAsync(y, b->sy.p, (size_t)b->Ntot * 8, cudaMemcpyDeviceToHost, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        batch_check_error(b);
        return H2W_OK;
    });
}

int h2w_batch_gmres(h2w_batch *b, const double *rhs, double *x, int max_iter, int tol_pow, int where, int *iters,
                    double *resid) {
    return bguarded(b, [&] {
        if (!rhs || !x || (where != H2W_HOST && where != H2W_DEVICE)) throw ApiError(H2W_ERR_ARG, "bad arguments");
        batch_in(b, rhs, b->bl.p, where);
        batch_in(b, x, b->xl.p, where);
        const int rc = gms_run(b, b->bl.p, b->xl.p, max_iter, std::pow(10, -1.0 * tol_pow), H2W_PREC_FP64, false,
                               iters, resid);
        batch_out(b, b->xl.p, x, where);
        return rc;
    });
}

int h2w_batch_gmres_ir(h2w_batch *b, const double *rhs, double *x, int max_outer, int inner_iter, int tol_pow,
                       int where, int *outer_iters, int *inner_total, double *resid) {
    return bguarded(b, [&] {
        if (!rhs || !x || max_outer < 1 || inner_iter < 1 || !outer_iters || !inner_total || !resid ||
            (where != H2W_HOST && where != H2W_DEVICE))
            throw ApiError(H2W_ERR_ARG, "bad arguments");
        const int P = (int)b->hs.size();
        const double tol = std::pow(10, -1.0 * tol_pow);
        cudaStream_t st = b->stream;
        batch_in(b, rhs, b->bl.p, where);
        batch_in(b, x, b->xl.p, where);
        GmresSeg g = gms_state(b, inner_iter);
        CK(gms_norms(g, b->bl.p, b->onorm.p, 1, st));
        std::vector<double> nb((size_t)P), nr((size_t)P);
        CK(cudaMemcpyAsync(nb.data(), b->onorm.p, (size_t)P * 8, cudaMemcpyDeviceToHost, st));
        *outer_iters = 0;
        *inner_total = 0;
        std::vector<int> it((size_t)P);
        bool ok = false;
        for (int o = 0; o <= max_outer; ++o) {
            // residual: FP32 operators at x0 (a correction only), then FP64 (the stopping test)
            run_batch(b, o == 0 ? H2W_PREC_FP32 : H2W_PREC_FP64, b->xl.p, b->r.p, true);
            CK(vec_axpby(1.0, b->bl.p, -1.0, b->r.p, b->r.p, b->Ntot, st));
            if (o > 0) {
                CK(gms_norms(g, b->r.p, b->ores.p, 0, st));
                CK(cudaMemcpyAsync(nr.data(), b->ores.p, (size_t)P * 8, cudaMemcpyDeviceToHost, st));
                CK(cudaStreamSynchronize(st));
                ok = true;
                for (int p = 0; p < P; ++p) {
                    resid[p] = nr[(size_t)p] / nb[(size_t)p];
                    if (!(resid[p] < tol)) ok = false;
                }
                if (ok || o == max_outer) break;
            }
            double tin = o == 0 ? 1e-6 : 0.1;  // the strictest problem's need (1e-6 in the first step)
            if (o > 0)
                for (int p = 0; p < P; ++p) tin = std::min(tin, inner_tol(tol, 1.0, resid[p]));
            CK(cudaMemsetAsync(b->d.p, 0, (size_t)b->Ntot * 8, st));
            gms_run(b, b->r.p, b->d.p, inner_iter, tin, H2W_PREC_FP32, true, it.data(), nullptr);
            int mx = 0;
            for (int p = 0; p < P; ++p) mx = std::max(mx, it[(size_t)p]);
            *inner_total += mx;
            CK(vec_axpby(1.0, b->xl.p, 1.0, b->d.p, b->xl.p, b->Ntot, st));
            *outer_iters = o + 1;
        }
        batch_out(b, b->xl.p, x, where);
        return ok ? H2W_OK : H2W_ERR_NOT_CONVERGED;
    });
}

int h2w_learn_record(h2w_handle *h, int enable) {
    return guarded(h, [&] {
        h->learn_rec = enable != 0;
        h->rec_X.clear();
        h->rec_y.clear();
        return H2W_OK;
    });
}

int h2w_learn_data(h2w_handle *h, float *X, uint8_t *y, int64_t *count) {
    return guarded(h, [&] {
        if (!count) throw ApiError(H2W_ERR_ARG, "null count");
        *count = (int64_t)h->rec_y.size();
        if (X) std::memcpy(X, h->rec_X.data(), h->rec_X.size() * 4);
        if (y) std::memcpy(y, h->rec_y.data(), h->rec_y.size());
        return H2W_OK;
    });
}

int h2w_learn_set_model(h2w_handle *h, const float *params, float calib, int margin) {
    return guarded(h, [&] {
        if (!params || !(calib > 0.f) || margin < 0) throw ApiError(H2W_ERR_ARG, "bad model arguments");
        if (h->cfg.device < 0) throw ApiError(H2W_ERR_STATE, "host-only handle");
        std::vector<float> v(params, params + LRN_NPARAM);
        h->d_mlp.upload(v, h->stream);
        CK(cudaStreamSynchronize(h->stream));
        h->mlp_calib = calib;
        h->mlp_margin = margin;
        return H2W_OK;
    });
}

int h2w_learn_stats(h2w_handle *h, int64_t *blocks, int64_t *accepted) {
    return guarded(h, [&] {
        if (blocks) *blocks = h->learn_blocks;
        if (accepted) *accepted = h->learn_accepted;
        h->learn_blocks = h->learn_accepted = 0;
        h->learn_reject[0] = h->learn_reject[1] = h->learn_reject[2] = 0;
        h->learn_rhat = h->learn_r1 = 0.0;
        return H2W_OK;
    });
}

int h2w_learn_detail(h2w_handle *h, int64_t *rejects, double *mean_rhat, double *mean_r1) {
    return guarded(h, [&] {
        const double nb = (double)std::max<int64_t>(h->learn_blocks, 1);
        if (rejects)
            for (int k = 0; k < 3; ++k) rejects[k] = h->learn_reject[k];
        if (mean_rhat) *mean_rhat = h->learn_rhat / nb;
        if (mean_r1) *mean_r1 = h->learn_r1 / nb;
        return H2W_OK;
    });
}

int h2w_mlp_nparam(void) { return LRN_NPARAM; }

int h2w_mlp_forward(const float *params, const float *X, int64_t n, float *logits, void *stream) {
    if (!params || !X || !logits || n < 0) return H2W_ERR_ARG;
    return launch_mlp_forward(params, X, n, logits, (cudaStream_t)stream) == cudaSuccess ? H2W_OK : H2W_ERR_CUDA;
}

int h2w_mlp_grad(const float *params, const float *X, const uint8_t *y, int64_t n, float pos_weight, float *grads,
                 float *loss, void *stream) {
    if (!params || !X || !y || !grads || !loss || n < 1 || !(pos_weight > 0.f)) return H2W_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(grads, 0, (size_t)LRN_NPARAM * 4, st) != cudaSuccess) return H2W_ERR_CUDA;
    if (cudaMemsetAsync(loss, 0, 4, st) != cudaSuccess) return H2W_ERR_CUDA;
    return launch_mlp_grad(params, X, y, n, pos_weight, grads, loss, st) == cudaSuccess ? H2W_OK : H2W_ERR_CUDA;
}

int h2w_mlp_adam(float *params, const float *grads, float *m, float *v, int step, float lr, void *stream) {
    if (!params || !grads || !m || !v || step < 1 || !(lr > 0.f)) return H2W_ERR_ARG;
    return launch_mlp_adam(params, grads, m, v, step, lr, (cudaStream_t)stream) == cudaSuccess ? H2W_OK
                                                                                                : H2W_ERR_CUDA;
}

int h2w_profile(h2w_handle *h, int enable) {
    return guarded(h, [&] {
        if (h->cfg.device < 0) throw ApiError(H2W_ERR_STATE, "host-only handle");
        CK(cudaStreamSynchronize(h->stream));
        for (auto &r : h->prof_recs) {
            h->ev_pool.push_back(r.a);
            h->ev_pool.push_back(r.b);
        }
        h->prof_recs.clear();
        h->prof = enable != 0;
        return H2W_OK;
    });
}

int h2w_profile_phases(h2w_handle *h, int precision, int max_phases, int64_t *launches, double *ms, double *bytes,
                       int *nphases) {
    return guarded(h, [&] {
        require_op(h);
        const int np = (int)h->phases.size() + 1;  // last entry: whole-matvec (cooperative) launches
        if (nphases) *nphases = np;
        if (!launches || !ms || !bytes) return H2W_OK;
        CK(cudaDeviceSynchronize());
        const double w = precision == H2W_PREC_FP32 ? 4.0 : 8.0;
        double tot = 0.0;
        for (int q = 0; q < std::min(np, max_phases); ++q) {
            launches[q] = 0;
            ms[q] = 0.0;
            if (q < np - 1) {
                bytes[q] = (double)(h->ph_op[(size_t)q] + h->ph_vec[(size_t)q]) * w;
                tot += bytes[q];
            }
        }
        if (np - 1 < max_phases) bytes[np - 1] = tot;
        for (auto &r : h->prof_recs) {
            if (r.prec != precision || r.phase >= max_phases) continue;
            float t = 0.f;
            CK(cudaEventElapsedTime(&t, r.a, r.b));
            launches[r.phase] += 1;
            ms[r.phase] += (double)t;
        }
        return H2W_OK;
    });
}

int h2w_profile_multi(h2w_handle *h, int precision, int64_t *launches, double *ms, double *bytes) {
    return guarded(h, [&] {
        require_op(h);
        if (!launches || !ms || !bytes) throw ApiError(H2W_ERR_ARG, "null output");
        CK(cudaDeviceSynchronize());
        const double w = precision == H2W_PREC_FP32 ? 4.0 : 8.0;
        *launches = 0;
        *ms = 0.0;
        double by = 0.0;
        for (auto &r : h->prof_recs) {
            if (r.prec != precision + 2 || r.phase == FLY_PHASE) continue;
            float t = 0.f;
            CK(cudaEventElapsedTime(&t, r.a, r.b));
            *launches += 1;
            *ms += (double)t;
            // operator once, the input block once (kernel precision), the FP64 result block once
            by += (double)h->op_bytes_read * w + (double)h->tree.N * r.rp * (w + 8.0);
        }
        *bytes = *launches ? by / (double)*launches : 0.0;
        return H2W_OK;
    });
}

int h2w_profile_fly(h2w_handle *h, int precision, int64_t *launches, double *ms, int64_t *entries) {
    return guarded(h, [&] {
        require_op(h);
        if (!launches || !ms || !entries) throw ApiError(H2W_ERR_ARG, "null output");
        CK(cudaDeviceSynchronize());
        *launches = 0;
        *ms = 0.0;
        *entries = h->fly_active ? h->fly_entries : 0;
        for (auto &r : h->prof_recs) {
            if (r.phase != FLY_PHASE || r.prec != precision) continue;
            float t = 0.f;
            CK(cudaEventElapsedTime(&t, r.a, r.b));
            *launches += 1;
            *ms += (double)t;
        }
        return H2W_OK;
    });
}

int h2w_plan_stats(h2w_handle *h, int64_t *stats, int n) {
    return guarded(h, [&] {
        require_op(h);
        if (!stats || n < 1 || n > 6) throw ApiError(H2W_ERR_ARG, "bad plan stats arguments");
        std::copy(h->mstats, h->mstats + n, stats);
        return H2W_OK;
    });
}

int64_t h2w_launch_count(void) { return launch_count(); }

int h2w_dense_matvec(h2w_handle *h, const double *x, double *y, int64_t row0, int64_t nrows, int where) {
    return guarded(h, [&] {
        require_tree(h);
        const int64_t N = h->tree.N;
        if (!x || !y || row0 < 0 || nrows < 0 || row0 + nrows > N) throw ApiError(H2W_ERR_ARG, "bad dense arguments");
        cudaStream_t st = h->stream;
        const int cw = h->cplx ? 2 : 1;  // doubles per entry
        const double *dx = x;
        double *dy = y;
        DBuf<double> bx, by;
        if (where == H2W_HOST) {
            bx.alloc((size_t)N * cw);
            by.alloc((size_t)std::max<int64_t>(nrows, 1) * cw);
            CK(cudaMemcpyAsync(bx.p, x, (size_t)N * 8 * cw, cudaMemcpyHostToDevice, st));
            dx = bx.p;
            dy = by.p;
        }
        if (h->cplx)
            CK(launch_dense_c(h->kparams(), N, reinterpret_cast<const double2 *>(dx), reinterpret_cast<double2 *>(dy),
                              row0, nrows, st));
        else
            CK(launch_dense_matvec(h->kparams(), N, dx, dy, row0, nrows, st));
        if (where == H2W_HOST) CK(cudaMemcpyAsync(y, by.p, (size_t)nrows * 8 * cw, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        return H2W_OK;
    });
}

// ------------------------------------------------------- operator files ---
// An operator file holds what determines the compressed operator: the
// configuration, the points, and every pivot list of the NCA (the skeletons
// of each level and the pair pivots), little-endian, closed by an FNV-1a
// checksum of everything before it. Opening rebuilds the tree from the
// points, imports the pivots and forms the operator from them on the GPU
// (H2W_ASSEMBLE_IMPORT): the pivot search, the costly part of assembly, is
// skipped, and the operator is bitwise the one that was saved.
}  // extern "C"

namespace {
constexpr char H2W_OPFILE_MAGIC[8] = {'H', '2', 'W', 'O', 'P', 'E', 'R', '1'};

struct OpWriter {
    std::vector<unsigned char> buf;
    template <class T> void put(const T &v) {
        const unsigned char *c = reinterpret_cast<const unsigned char *>(&v);
        buf.insert(buf.end(), c, c + sizeof(T));
    }
    template <class T> void put_n(const T *v, size_t n) {
        const unsigned char *c = reinterpret_cast<const unsigned char *>(v);
        buf.insert(buf.end(), c, c + n * sizeof(T));
    }
};
struct OpReader {
    const std::vector<unsigned char> &buf;
    size_t pos = 0, end;
    template <class T> T get() {
        if (pos + sizeof(T) > end) throw ApiError(H2W_ERR_ARG, "operator file is truncated");
        T v;
        std::memcpy(&v, buf.data() + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    template <class T> void get_n(T *v, size_t n) {
        if (n > (end - pos) / sizeof(T)) throw ApiError(H2W_ERR_ARG, "operator file is truncated");
        std::memcpy(v, buf.data() + pos, n * sizeof(T));
        pos += n * sizeof(T);
    }
};
uint64_t fnv1a(const unsigned char *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}
}  // namespace

extern "C" {

int h2w_get_config(h2w_handle *h, h2w_config *out) {
    return guarded(h, [&] {
        if (!out) throw ApiError(H2W_ERR_ARG, "null output");
        *out = h->cfg;
        return H2W_OK;
    });
}

int h2w_save_operator(h2w_handle *h, const char *path) {
    return guarded(h, [&] {
        require_op(h);
        if (!path) throw ApiError(H2W_ERR_ARG, "null path");
        OpWriter w;
        w.put_n(H2W_OPFILE_MAGIC, 8);
        const h2w_config &c = h->cfg;
        for (int32_t v : {c.dim, c.form, c.choice, c.tol_pow, c.nlevels, c.rank_cap}) w.put(v);
        w.put(c.kernel_n);
        w.put(c.diag_n);
        const int64_t N = h->tree.N;
        w.put(N);
        w.put_n(h->pts.data(), h->pts.size());
        std::vector<int32_t> lists;
        for (int which = H2W_LIST_FAR_CHECK; which <= H2W_LIST_SN_COL; ++which) lists.push_back(which);
        w.put((int32_t)lists.size());
        for (int which : lists) {
            int64_t np = 0, nv = 0;
            if (h2w_get_list(h, which, nullptr, nullptr, &np, &nv) != H2W_OK) throw ApiError(H2W_ERR_STATE, h->err);
            std::vector<int64_t> ptr((size_t)np);
            std::vector<int32_t> val((size_t)std::max<int64_t>(nv, 1));
            if (h2w_get_list(h, which, ptr.data(), val.data(), nullptr, nullptr) != H2W_OK)
                throw ApiError(H2W_ERR_STATE, h->err);
            w.put((int32_t)which);
            w.put(np);
            w.put_n(ptr.data(), ptr.size());
            w.put(nv);
            w.put_n(val.data(), (size_t)nv);
        }
        w.put(h->storage);
        w.put(fnv1a(w.buf.data(), w.buf.size()));
        FILE *f = std::fopen(path, "wb");
        if (!f) throw ApiError(H2W_ERR_ARG, std::string("cannot write ") + path);
        const size_t n = std::fwrite(w.buf.data(), 1, w.buf.size(), f);
        const bool ok = n == w.buf.size() && std::fclose(f) == 0;
        if (!ok) throw ApiError(H2W_ERR_ARG, std::string("write to ") + path + " failed");
        return H2W_OK;
    });
}

int h2w_open_operator(const char *path, int device, h2w_handle **out) {
    if (!path || !out) return H2W_ERR_ARG;
    *out = nullptr;
    std::vector<unsigned char> buf;
    {
        FILE *f = std::fopen(path, "rb");
        if (!f) return H2W_ERR_ARG;
        unsigned char tmp[1 << 16];
        size_t n;
        while ((n = std::fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + n);
        std::fclose(f);
    }
    if (buf.size() < 8 + 8 || std::memcmp(buf.data(), H2W_OPFILE_MAGIC, 8) != 0) return H2W_ERR_ARG;
    uint64_t sum;
    std::memcpy(&sum, buf.data() + buf.size() - 8, 8);
    if (fnv1a(buf.data(), buf.size() - 8) != sum) return H2W_ERR_ARG;
    OpReader r{buf, 8, buf.size() - 8};
    h2w_config c{};
    try {
        c.dim = r.get<int32_t>();
        c.form = r.get<int32_t>();
        c.choice = r.get<int32_t>();
        c.tol_pow = r.get<int32_t>();
        c.nlevels = r.get<int32_t>();
        c.rank_cap = r.get<int32_t>();
        c.kernel_n = r.get<int64_t>();
        c.diag_n = r.get<int64_t>();
    } catch (const ApiError &) {
        return H2W_ERR_ARG;
    }
    c.device = device;
    h2w_handle *h = nullptr;
    int rc = h2w_create(&c, &h);
    if (rc != H2W_OK) return rc;
    rc = guarded(h, [&] {
        const int64_t N = r.get<int64_t>();
        if (N < 1 || N > INT32_MAX - 1) throw ApiError(H2W_ERR_ARG, "operator file: bad point count");
        std::vector<double> pts((size_t)N * (size_t)c.dim);
        r.get_n(pts.data(), pts.size());
        if (h2w_set_points(h, pts.data(), N) != H2W_OK || h2w_build_tree(h) != H2W_OK) throw ApiError(H2W_ERR_ARG, h->err);
        const int32_t nl = r.get<int32_t>();
        for (int32_t q = 0; q < nl; ++q) {
            const int32_t which = r.get<int32_t>();
            const int64_t np = r.get<int64_t>();
            if (np < 1 || np > (int64_t)buf.size()) throw ApiError(H2W_ERR_ARG, "operator file: bad list");
            std::vector<int64_t> ptr((size_t)np);
            r.get_n(ptr.data(), ptr.size());
            const int64_t nv = r.get<int64_t>();
            if (nv < 0 || nv != ptr.back() || nv > (int64_t)buf.size()) throw ApiError(H2W_ERR_ARG, "operator file: bad list");
            std::vector<int32_t> val((size_t)std::max<int64_t>(nv, 1));
            r.get_n(val.data(), (size_t)nv);
            for (int64_t i = 1; i < np; ++i)
                if (ptr[(size_t)i] < ptr[(size_t)i - 1]) throw ApiError(H2W_ERR_ARG, "operator file: bad list");
            if (h2w_import_list(h, which, ptr.data(), val.data(), np) != H2W_OK) throw ApiError(H2W_ERR_ARG, h->err);
        }
        const double storage = r.get<double>();
        if (device >= 0) {
            if (h2w_assemble(h, H2W_ASSEMBLE_IMPORT) != H2W_OK) throw ApiError(H2W_ERR_ARG, h->err);
            if (h->storage != storage)
                throw ApiError(H2W_ERR_ARG, "operator file: the formed operator's storage differs from the saved one");
        }
        return H2W_OK;
    });
    if (rc != H2W_OK) {
        h2w_destroy(h);
        return rc;
    }
    *out = h;
    return H2W_OK;
}

int h2w_total_error(h2w_handle *h, const double *x, int64_t nrows, int where, double *err) {
    return guarded(h, [&] {
        require_op(h);
        require_real(h, "h2w_total_error");
        if (!x || !err || (where != H2W_HOST && where != H2W_DEVICE)) throw ApiError(H2W_ERR_ARG, "bad error arguments");
        const int64_t N = h->tree.N;
        cudaStream_t st = h->stream;
        DBuf<double> bx, byh, byd;
        DBuf<int64_t> brows;
        const double *dx = x;
        if (where == H2W_HOST) {
            bx.alloc((size_t)N);
            CK(cudaMemcpyAsync(bx.p, x, (size_t)N * 8, cudaMemcpyHostToDevice, st));
            dx = bx.p;
        }
        byh.alloc((size_t)N);
        run_matvec_f64(h, dx, byh.p, st);
        const bool all = nrows <= 0 || nrows >= N;
        const int64_t nr = all ? N : nrows;
        std::vector<int64_t> rows((size_t)nr);
        for (int64_t i = 0; i < nr; ++i) rows[(size_t)i] = all ? i : (int64_t)((__int128)i * N / nr);
        byd.alloc((size_t)nr);
        if (all) {
            CK(launch_dense_matvec(h->kparams(), N, dx, byd.p, 0, N, st));
        } else {
            brows.upload(rows, st);
            CK(launch_dense_rows(h->kparams(), N, dx, brows.p, nr, byd.p, st));
        }
        std::vector<double> yh((size_t)N), yd((size_t)nr);
        CK(cudaMemcpyAsync(yh.data(), byh.p, (size_t)N * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(yd.data(), byd.p, (size_t)nr * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        check_device_error(h);
        long double num = 0.0L, den = 0.0L;
        for (int64_t i = 0; i < nr; ++i) {
            const long double d = (long double)yd[(size_t)i] - (long double)yh[(size_t)rows[(size_t)i]];
            num += d * d;
            den += (long double)yd[(size_t)i] * (long double)yd[(size_t)i];
        }
        *err = den > 0.0L ? (double)std::sqrt(num / den) : 0.0;
        return H2W_OK;
    });
}

}  // extern "C"
