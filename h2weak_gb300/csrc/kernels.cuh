// Device-side entry points of the GB300 H2* / (H2+H)* library (sm_103a).
// Host code calls these launch wrappers; every pointer is a device pointer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "h2w_internal.h"

namespace h2w {

// Number of kernel launches issued by this library (all kernels).
int64_t launch_count();
void count_launch(int64_t n = 1);

// Kernel-matrix entry parameters (reference kernel.hpp getMatrixEntry).
struct KParams {
    const double *pts;   // N*dim, original order
    int dim, choice;
    double diag;         // value on the diagonal
    double c2d;          // 2D IE: (-1/(2 pi)) * 0.5
    double four_pi;      // 3D IE: 4 pi
    double loga;         // 3D RBF: log(a)
    double den_small;    // 3D RBF: a log(a) - 1
    double diag_im;      // complex kernels: imaginary part of the diagonal value
};

struct NcaProb {
    int64_t ri, ci;      // row / column index lists in the index buffer
    int64_t u, v;        // scratch offsets: U (n1 x rcap, column l at u + l*n1), V (rcap x n2)
    int64_t piv;         // output pivot offset (rcap entries)
    int32_t n1, n2, rcap, pad;
};

// Assembly
cudaError_t launch_nca(const NcaProb *probs, int nprob, const int32_t *idx, const KParams &kp, double tol,
                       double *scratch, int32_t *rank, int32_t *prow, int32_t *pcol, int32_t *status,
                       int max_n1, int max_n2, int max_rcap, cudaStream_t st);
// The NCA for large blocks: the CTAs of one cooperative launch in G groups,
// each group on one block at a time (same pivots as launch_nca). moff: per
// block, offset of its row+column pivot masks (uint32 words) in masks;
// partial buffers of nca_group_part_bytes() x grid each; dots: grid x 2*dcap
// (df: the scratch holds double-FP32 pairs and the residuals are formed in
// double-FP32 arithmetic, for kernels built on log, see ncabig.cu)
// + G x dcap doubles (dcap >= every block's rcap). A block whose rank reaches
// its rcap reports -rank in rank (launch_nca does the same).
int nca_group_grid(int dcap, bool df);
size_t nca_group_part_bytes();
cudaError_t launch_nca_group(const NcaProb *probs, const int64_t *moff, int nprob, int G, int grid,
                             const int32_t *idx, const KParams &kp, double tol, double *scr, uint32_t *masks,
                             int32_t *rank, int32_t *prow, int32_t *pcol, int32_t *status, unsigned *bars,
                             int32_t *err, void *prow_part, void *pcol_part, double *dots, int dcap, bool df,
                             const void *logtab, cudaStream_t st);
cudaError_t launch_factor(const FactorJob *jobs, int njobs, const int32_t *idx, const KParams &kp, double *F,
                          cudaStream_t st);
cudaError_t launch_xfer(const XferJob *jobs, int njobs, int max_n, const int32_t *idx, const KParams &kp,
                        const double *F, double *op, cudaStream_t st);
cudaError_t launch_fill(const FillJob *jobs, int njobs, const int32_t *idx, const KParams &kp, double *op,
                        cudaStream_t st);
cudaError_t launch_convert_f32(const double *src, float *dst, int64_t n, cudaStream_t st);

// Matvec: one block-row GEMV launch over targets [t0, t1) of the packed
// target records (roff: record offsets, blob: records). xin / yout are FP64
// in original point order when perm != NULL, in leaf order when perm == NULL.
cudaError_t launch_brg_f64(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t t1, const double *A,
                           double *ws, const double *xin, double *yout, const int32_t *perm, cudaStream_t st);
cudaError_t launch_brg_f32(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t t1, const float *A,
                           float *ws, const double *xin, double *yout, const int32_t *perm, cudaStream_t st);
// Dataflow form of the single-vector product (see launch_mr_f32_flow):
// targets [t0, nt) in stored order, ctr a zeroed claim counter, rem the producer
// counts (reset before every launch), consumers in cidx[coff[t] .. coff[t+1])
cudaError_t launch_brg_flow_f64(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t nt, int32_t *ctr, int32_t *rem,
                                const int64_t *coff, const int32_t *cidx, const double *A, double *ws,
                                const double *xin, double *yout, const int32_t *perm, int32_t *err, cudaStream_t st);
cudaError_t launch_brg_flow_f32(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t nt, int32_t *ctr, int32_t *rem,
                                const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const double *xin,
                                double *yout, const int32_t *perm, int32_t *err, cudaStream_t st);
// The whole matvec as one cooperative launch: phase p covers targets
// [pstart[p], pstart[p+1]); bar (2 unsigned, zero) is the grid barrier state;
// spin bounds each grid-barrier wait in polls (<= 0: the built-in limit).
cudaError_t launch_coop_f64(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const double *A, double *ws, const double *xin, double *yout, const int32_t *perm,
                            unsigned *bar, int32_t *err, cudaStream_t st, long long spin = 0);
cudaError_t launch_coop_f32(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const float *A, float *ws, const double *xin, double *yout, const int32_t *perm,
                            unsigned *bar, int32_t *err, cudaStream_t st, long long spin = 0);
cudaError_t launch_scatter_f64(const double *yp, double *y, const int32_t *perm, int64_t n, cudaStream_t st);
cudaError_t launch_gather_f64(const double *x, double *xp, const int32_t *perm, int64_t n, cudaStream_t st);
cudaError_t launch_scatter_f32(const float *yp, double *y, const int32_t *perm, int64_t n, cudaStream_t st);
constexpr int BRG_XS_ELEMS = 4096;    // gathered source width per target (elements)
constexpr int BRG_MAX_PANELS = 32;    // panels per target
constexpr int BRG_REC_WORDS = 1024;   // packed record of one target (int64 words)
constexpr int MR_XS_ELEMS = 2048;     // gathered source width per multi-vector target (elements)

// Far-field M2L evaluated during the product (m2lfly.cu). One work item: a
// block of <= FLY_ROWS rows of one target box: rows[i] (point ids at rowpid[rows
// + i]) get ws[dst + i] = sum_c K(row point, cpid[cbeg + c]) ws[cws[cbeg + c]].
constexpr int FLY_ROWS = 32;  // rows per work item
struct FlyItem {
    int64_t dst, rows, cbeg;
    int32_t nrows, ncols;
};
// FP32 constants of the kernel functions (3D/2D, choice 0/1)
struct FlyK32 {
    float c2d, inv4pi, inv_loga, inv_den, a, a2, inv_a;
    int32_t sep;  // every far pair is farther apart than a (deepest box wider than a)
};
cudaError_t launch_fly_f64(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                           const int32_t *cpid, const int32_t *cws, double *ws, const KParams &kp, cudaStream_t st);
cudaError_t launch_fly_f32(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                           const int32_t *cpid, const int32_t *cws, const float *pts4, float *ws, const KParams &kp,
                           const FlyK32 &k32, cudaStream_t st);
// (x, y, z, 0) FP32 coordinates of the FP64 points (N x dim) for the FP32 form.
cudaError_t launch_pts4(const double *pts, int dim, int64_t n, float *out, cudaStream_t st);
// The FP64-accurate form on the FP32 pipes (double-FP32 arithmetic) for the
// kernels built on log(R^2) when every far pair is farther apart than a (else
// the FP64 form): ptsdf = (hi, lo) FP32 quadruples of the points
// (launch_ptsdf, 8 floats per point), logtab = fly_df_logtab's 128 x 8 floats.
bool fly_df_supported(const KParams &kp, const FlyK32 &k32);
cudaError_t launch_fly_df64(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                            const int32_t *cpid, const int32_t *cws, const float *ptsdf, const void *logtab,
                            double *ws, const KParams &kp, const FlyK32 &k32, cudaStream_t st);
void fly_df_logtab(float *out);
cudaError_t launch_ptsdf(const double *pts, int dim, int64_t n, float *out, cudaStream_t st);

// Complex Helmholtz kernels (helm.cu). Positions of the assembly jobs are in
// complex units of a complex operator image opc; launch_realify expands each
// complex block (a, lda, cols triples in blk, complex units) into the real
// block [[Re, -Im], [Im, Re]] with interleaved rows and columns at 4a,
// leading dimension 2 lda, of the real operator.
size_t nca_c_smem(int max_n1, int max_n2, int max_rcap);
cudaError_t launch_nca_c(const NcaProb *probs, int nprob, const int32_t *idx, const KParams &kp, double tol,
                         double2 *scratch, int32_t *rank, int32_t *prow, int32_t *pcol, int32_t *status, int max_n1,
                         int max_n2, int max_rcap, cudaStream_t st);
cudaError_t launch_assemble_c(const FactorJob *fac, int nfac, const XferJob *xf, int nxf, int max_n,
                              const FillJob *fill, int nfill, const int32_t *idx, const KParams &kp, double2 *F,
                              double2 *opc, cudaStream_t st);
cudaError_t launch_realify(const int64_t *blk, int64_t nblk, const double2 *opc, double *op, cudaStream_t st);
cudaError_t launch_dense_c(const KParams &kp, int64_t N, const double2 *x, double2 *y, int64_t row0, int64_t nrows,
                           cudaStream_t st);
// The reference GMRES's complex vector operations (n complex entries):
// out = sum conj(a_i) b_i (part: cgm_blocks() scratch entries), w -= (*h) v,
// dst = s src (s real), x += sum_j V[:, j] y_j, r = b - ax.
int cgm_blocks();
cudaError_t cgm_dot(const double2 *a, const double2 *b, int64_t n, double2 *part, double2 *out, cudaStream_t st);
cudaError_t cgm_axpy_launch(double2 *w, const double2 *v, const double2 *h, int64_t n, cudaStream_t st);
cudaError_t cgm_scale_launch(double2 *dst, const double2 *src, double s, int64_t n, cudaStream_t st);
cudaError_t cgm_update_launch(double2 *x, const double2 *V, const double2 *y, int k, int64_t n, cudaStream_t st);
cudaError_t cgm_resid_launch(double2 *r, const double2 *b, const double2 *ax, int64_t n, cudaStream_t st);

// Dense FP64 oracle rows y[r] = sum_j K(r, j) x[j], r in [row0, row0+nrows).
cudaError_t launch_dense_matvec(const KParams &kp, int64_t N, const double *x, double *y, int64_t row0,
                                int64_t nrows, cudaStream_t st);
// The same for a list of rows (each in [0, N)): y[i] = sum_j K(rows[i], j) x[j].
cudaError_t launch_dense_rows(const KParams &kp, int64_t N, const double *x, const int64_t *rows, int64_t nrows,
                              double *y, cudaStream_t st);

// GMRES building blocks (FP64). V is column-major N x (m+1).
struct GmresDev {
    double *V, *w, *vcur, *H, *cs, *sn, *s;  // V: N x (m+1); H: (m+1) x m column-major
    double *part;                             // 3 * nblk * (m+1) partial sums
    double *scal;                             // [0] ||b||, [1] resid, [2] converged flag, [3] beta,
                                              // [6] stopping tolerance (read by the Givens step)
    int32_t *iter;                            // [0] current Arnoldi column i, [1] steps taken
    int64_t N;
    int m, nblk;
};
void gmres_prepare();                                             // one-time kernel attributes
cudaError_t gmres_cgs2(const GmresDev &g, cudaStream_t st);      // orthogonalise w against V[:, 0..i], H column
cudaError_t gmres_finish_iter(const GmresDev &g, cudaStream_t st);  // normalise, Givens, residual (tol: scal[6])
cudaError_t gmres_start(const GmresDev &g, const double *b, const double *Ax, double normb, cudaStream_t st);
cudaError_t gmres_update(const GmresDev &g, double *x, const double *y, int k, cudaStream_t st);
// last node of a graph-captured Arnoldi step: sets the while-loop condition
cudaError_t gmres_loop_cond(const GmresDev &g, cudaGraphConditionalHandle hnd, cudaStream_t st);
cudaError_t vec_norm(const double *x, int64_t n, double *part, int nblk, double *out, cudaStream_t st);
cudaError_t vec_axpby(double a, const double *x, double b, const double *y, double *z, int64_t n, cudaStream_t st);
cudaError_t vec_f64_to_f32(const double *x, float *y, int64_t n, cudaStream_t st);
cudaError_t vec_f32_to_f64(const float *x, double *y, int64_t n, cudaStream_t st);

// ------------------------------------------------------- learned NCA
// A per-point MLP (features -> 128 -> 128 -> logit, BF16 weights, FP32
// accumulation) scores the candidate row and column points of NCA blocks;
// the top-scored points form a cross-approximation proposal that the NCA's
// own stopping test accepts or rejects.
constexpr int LRN_F = 16, LRN_H = 128;
constexpr int LRN_W1 = 0, LRN_B1 = LRN_F * LRN_H, LRN_W2 = LRN_B1 + LRN_H, LRN_B2 = LRN_W2 + LRN_H * LRN_H,
              LRN_W3 = LRN_B2 + LRN_H, LRN_B3 = LRN_W3 + LRN_H, LRN_NPARAM = LRN_B3 + 1;
constexpr int LRN_CAP = 128;  // most pivots a proposal holds

struct LearnProb {
    int64_t ri, ci;        // row / column point lists in the index buffer
    int64_t xo;            // feature / logit offset: n1 rows then n2 columns
    int64_t ac, ar;        // K(R, J): n1 x cap, column l at ac + l*n1; K(I, C): cap x n2, row l at ar + l*n2
    int64_t uu, vv;        // U (n1 x cap), V (cap x n2), same layouts
    int64_t ff, gu, gv;    // LU of K(I', J') and the Gram matrices U^T U, V V^T (cap x cap, row-major)
    int64_t piv;           // proposal / pivot lists (cap + 1 entries)
    int32_t n1, n2, cap, pad;
};
struct LearnState {
    int32_t rhat, r1, accept, rank;  // proposal size, pivots kept, accepted, final rank
};
struct LearnTile {
    int32_t b, kind, start, count;  // kind 0: K(R,J') entries, 1: K(I,C) entries, 2: U rows, 3: V columns
};
// rows_only: features of the rows alone (inference scores rows only)
cudaError_t launch_learn_features(const LearnProb *probs, int nprob, const int32_t *idx, const KParams &kp,
                                  int tol_pow, float *X, int rows_only, cudaStream_t st);
cudaError_t launch_mlp_forward(const float *params, const float *X, int64_t n, float *logits, cudaStream_t st);
cudaError_t launch_mlp_grad(const float *params, const float *X, const uint8_t *y, int64_t n, float pos_weight,
                            float *grads, float *loss, cudaStream_t st);
cudaError_t launch_mlp_adam(float *params, const float *grads, float *m, float *v, int step, float lr,
                            cudaStream_t st);
cudaError_t launch_learn_propose(const LearnProb *probs, int nprob, const float *logits, float calib, int margin,
                                 int32_t *prop_r, int32_t *prop_c, LearnState *lst, int mask_words, cudaStream_t st);
cudaError_t launch_learn_fill(const LearnTile *tiles, int ntiles, const LearnProb *probs, const int32_t *idx,
                              const KParams &kp, const int32_t *prop_r, const int32_t *ordJ, const LearnState *lst,
                              double *scr, int only, cudaStream_t st);
cudaError_t launch_learn_aca(const LearnProb *probs, int nprob, double tol, double *scr, int32_t *ordI,
                             int32_t *ordJ, LearnState *lst, int mask_words, cudaStream_t st);
cudaError_t launch_learn_solve(const LearnTile *tiles, int ntiles, const LearnProb *probs, const int32_t *ordI,
                               const int32_t *ordJ, const LearnState *lst, double *scr, cudaStream_t st);
cudaError_t launch_learn_gram(const LearnTile *tiles, int ntiles, const LearnProb *probs, const LearnState *lst,
                              double *scr, cudaStream_t st);
cudaError_t launch_learn_test(const LearnProb *probs, int nprob, const int32_t *idx, const KParams &kp, double tol,
                              const int32_t *prop_r, const int32_t *prop_c, const int32_t *ordI, const int32_t *ordJ,
                              LearnState *lst, double *scr, int32_t *prow, int32_t *pcol, int mask_words,
                              cudaStream_t st);

// ------------------------------------------------ many independent problems
// One problem of a batch: its packed operator (FP64 or FP32 copy), its
// workspace, its leaf permutation (NULL: vectors in leaf order) and the
// offset of its segment in the concatenated input / output vectors.
struct BatchProb {
    const void *A;
    void *ws;
    const int32_t *perm;
    int64_t xoff;
};
// The single-vector matvec of every problem of a batch in one cooperative
// launch; records carry the problem index in bits 8.. of their flag word.
// active (may be NULL): problems whose entry is not -1 are skipped.
cudaError_t launch_brgb_f64(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const BatchProb *probs, const int32_t *active, const double *xin, double *yout,
                            unsigned *bar, int32_t *err, cudaStream_t st);
cudaError_t launch_brgb_f32(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const BatchProb *probs, const int32_t *active, const double *xin, double *yout,
                            unsigned *bar, int32_t *err, cudaStream_t st);

// Segmented GMRES: P independent systems in lockstep over one concatenated
// vector (problem p owns a contiguous row range); block b works on rows
// [brow[b], brow[b+1]) of problem bprob[b], problem p owns blocks
// [pblk[p], pblk[p+1]).
struct GmresSeg {
    double *V;               // (m+1) blocks of Ntot
    double *w, *vcur;        // Ntot
    double *H;               // per problem p: (m+1) x m column-major at p*m*(m+1)
    double *cs, *sn, *s;     // per problem: m+1 at p*(m+1)
    double *part;            // nblk x (m+1) block partial sums
    double *hsum;            // P x (m+1) per-problem sums
    double *normb, *resid;   // P
    double *y;               // P x (m+1) back-substituted coefficients
    int32_t *conv;           // P: -1 running, k >= 0 converged at column k, -2 at the start
    int32_t *iter;           // [0] current Arnoldi column, [1] steps taken
    const int32_t *bprob;    // nblk
    const int64_t *brow;     // nblk + 1
    const int32_t *pblk;     // P + 1
    int64_t Ntot;
    int m, P, nblk;
};
bool gms_attr(const GmresSeg &g);
cudaError_t gms_norms(const GmresSeg &g, const double *v, double *out, int zero_to_one, cudaStream_t st);
cudaError_t gms_start(const GmresSeg &g, const double *b, const double *Ax, double tol, cudaStream_t st);
cudaError_t gms_arnoldi(const GmresSeg &g, double tol, cudaStream_t st);
cudaError_t gms_loop(const GmresSeg &g, cudaGraphConditionalHandle hnd, cudaStream_t st);
cudaError_t gms_finish(const GmresSeg &g, double *x, int last, int kmax, cudaStream_t st);
// y[idx[t]] = x[t] (scatter) / y[t] = x[idx[t]] (gather) over n elements with
// 64-bit indices (concatenated permutations of a batch)
cudaError_t launch_gather64(const double *x, double *y, const int64_t *idx, int64_t n, cudaStream_t st);
cudaError_t launch_scatter64(const double *x, double *y, const int64_t *idx, int64_t n, cudaStream_t st);

// ------------------------------------------------ multiple right-hand sides
// Blocks of rp vectors are interleaved: element (t, c) at t*rp + c
// (rp = 16, 32 or 64). The workspace holds ws_n rows of rp values.
// ctr: one int per phase, zero at launch (the phase's target counter).
struct MrPhases {          // per-phase launches instead of one cooperative launch
    const int64_t *t0, *t1;
    int n;
};
cudaError_t launch_mr_f64(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                          const MrPhases *phased, int32_t *ctr, const double *A, double *ws, const double *xin, double *yout,
                          unsigned *bar, int32_t *err, cudaStream_t st);
cudaError_t launch_mr_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                          const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin, double *yout,
                          unsigned *bar, int32_t *err, cudaStream_t st);
// the same with a float result (interleaved FP32 blocks)
cudaError_t launch_mr_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                          const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin, float *yout,
                          unsigned *bar, int32_t *err, cudaStream_t st);
// Dataflow launch of the FP32 multi-vector stream (no grid barriers): nt
// targets in stored order, ctr a zeroed claim counter, rem the targets'
// producer counts (reset before every launch), consumers of target t in
// cidx[coff[t] .. coff[t+1]); err = 3 if a wait timed out
cudaError_t launch_mr_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr, int32_t *rem,
                               const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const float *xin,
                               double *yout, int32_t *err, cudaStream_t st);
cudaError_t launch_mr_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr, int32_t *rem,
                               const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const float *xin,
                               float *yout, int32_t *err, cudaStream_t st);
// the slices of an FP32 operator, 6 words each (source offset, leading
// dimension, rows, columns, destination offset, destination leading
// dimension), copied to dst with zeros in the destination's padding rows
cudaError_t launch_slice_copy_f32(const float *src, const int64_t *slices, int64_t n, float *dst, cudaStream_t st);
// warp-specialised form of launch_mr_f32_flow (a producer warp streams each
// CTA's chunks by bulk asynchronous copies; mrws.cu); A and blob: the
// slice-contiguous operator copy and its records
cudaError_t launch_mw_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr,
                               int32_t *rem, const int64_t *coff, const int32_t *cidx, const float *A, float *ws,
                               const float *xin, double *yout, int32_t *err, cudaStream_t st);
cudaError_t launch_mw_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr,
                               int32_t *rem, const int64_t *coff, const int32_t *cidx, const float *A, float *ws,
                               const float *xin, float *yout, int32_t *err, cudaStream_t st);
// the same for the FP64 (df = false) and double-FP32 (df = true, A and xin
// pre-split pairs as for launch_mr_df64) products
cudaError_t launch_mr_f64_flow(int rp, bool df, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr,
                               int32_t *rem, const int64_t *coff, const int32_t *cidx, const double *A, double *ws,
                               const double *xin, double *yout, int32_t *err, cudaStream_t st);
// Double-FP32 arithmetic on the FP32 pipes (each product and sum carried as
// an FP32 pair; about 2^-44 relative per term instead of FP64's 2^-53): A and
// xin are (hi, lo) pairs (launch_mr_split of the FP64 operator and input),
// the workspace and the result FP64.
// FP32 multi-vector product on the tensor cores (tcgen05 kind::tf32 with
// hi/lo operand splitting), same records and arguments as launch_mr_f32
cudaError_t launch_mrt_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                           const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin,
                           double *yout, unsigned *bar, int32_t *err, cudaStream_t st);
cudaError_t launch_mrt_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                           const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin,
                           float *yout, unsigned *bar, int32_t *err, cudaStream_t st);
cudaError_t launch_mr_df64(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                           const MrPhases *phased, int32_t *ctr, const double *A, double *ws, const double *xin, double *yout,
                           unsigned *bar, int32_t *err, cudaStream_t st);
// (hi, lo) FP32 pairs of n doubles (8 bytes each, the double-FP32 product's
// operator and input formats)
cudaError_t launch_mr_split(const double *a, void *b, int64_t n, cudaStream_t st);
// calibration vectors (even columns pseudo-random, odd columns smooth), n x rp interleaved
cudaError_t launch_calib_fill(double *z, int64_t n, int rp, int c0, cudaStream_t st);
cudaError_t launch_mr_pack(const double *x, int64_t ldx, double *xi, const int32_t *perm, int64_t n, int nrhs,
                           int rp, cudaStream_t st);
cudaError_t launch_mr_unpack(const double *yi, double *y, int64_t ldy, const int32_t *perm, int64_t n, int nrhs,
                             int rp, cudaStream_t st);
cudaError_t launch_mr_widen_f64(const double *a, double *b, int64_t n, cudaStream_t st);
cudaError_t launch_mr_widen_f32(const float *a, double *b, int64_t n, cudaStream_t st);

// Batched GMRES state (rp interleaved systems, Krylov dimension m).
// Lockstep GMRES state for RP systems (gmbatch.cu). T: type of the Krylov
// vectors (double for FP64 solves, float for FP32-operator inner solves);
// Hessenberg, rotations and reductions are double.
template <class T>
struct GmbT {
    T *V;                    // (m+1) blocks of N*rp
    T *w, *vcur;             // N*rp
    double *H;               // per column c: (m+1) x m column-major at c*m*(m+1)
    double *cs, *sn, *s;     // per column c: m+1 at c*(m+1)
    double *part;            // nblk x (m+1) x rp block partial sums
    double *hsum;            // (m+1) x rp reduced sums
    double *normb, *resid;   // rp
    double *y;               // (m+1) x rp back-substituted coefficients
    double *z;               // (m+2) x rp: beta e1 - Hbar y of each column (its residual in the basis)
    int32_t *conv;           // rp: -1 running, k >= 0 converged at Arnoldi column k, -2 at the start, -3 padding
    int32_t *iter;           // [0] current Arnoldi column, [1] steps taken
    double *tolp;            // stopping tolerance (device, so that captured steps do not hold it)
    int64_t N;
    int m, rp, nrhs, nblk;
};
using GmresBatch = GmbT<double>;
template <class T>
cudaError_t gmb_norms(const GmbT<T> &g, const double *v, double *out, int zero_to_one, cudaStream_t st);
// w = b - Ax (Ax NULL: w = b, and normb = ||b|| is set here), V[:, 0], rotations, state
template <class T>
cudaError_t gmb_start(const GmbT<T> &g, const double *b, const double *Ax, double tol, cudaStream_t st);
template <class T>
cudaError_t gmb_arnoldi(const GmbT<T> &g, cudaStream_t st);
template <class T>
cudaError_t gmb_loop(const GmbT<T> &g, cudaGraphConditionalHandle hnd, cudaStream_t st);
// x += V y (and z = beta e1 - Hbar y per column)
template <class T>
cudaError_t gmb_finish(const GmbT<T> &g, double *x, int last, int kmax, cudaStream_t st);
// after gmb_finish: rout = (rin - T(rin)) + sum_{j <= jmax} V_j z_j, the solved system's
// residual rin - A d from the Arnoldi relation (rin: the right-hand side the solve started
// from at x0 = 0; jmax: the largest Arnoldi index + 1 over the columns)
template <class T>
cudaError_t gmb_residual(const GmbT<T> &g, const double *rin, double *rout, int jmax, cudaStream_t st);

}  // namespace h2w
