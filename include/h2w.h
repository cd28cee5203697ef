/* h2w.h — C ABI of the GB300-native H2* / (H2+H)* HODLRdD operator and solver.
 *
 * Drop-in boundary for the hot path of H2weak: the operator object that the
 * reference's GMRES drives (class initialisation, {1D,2D,3D}/codes/matvec.hpp) and the
 * GMRES itself (class iterative_solver, {1D,2D,3D}/codes/gmres.hpp). Plain pointers and
 * sizes only; no C++ or torch types cross this boundary. Every function
 * returns H2W_OK (0) or a negative status; h2w_last_error() gives the text.
 *
 * Ownership and threading: the handle owns all device memory (tree tables,
 * packed operator, work vectors, CUDA graphs). Callers own x, y, b. One handle
 * is used by one host thread at a time; distinct handles are independent and
 * may share a device.
 */
#ifndef H2W_H
#define H2W_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct h2w_handle h2w_handle;

enum {
    H2W_OK = 0,
    H2W_ERR_ARG = -1,        /* bad argument or call order */
    H2W_ERR_CUDA = -2,       /* CUDA runtime error (message has the call) */
    H2W_ERR_NOMEM = -3,      /* device allocation failed */
    H2W_ERR_RANK = -4,       /* an NCA rank exceeded the configured cap */
    H2W_ERR_NOT_CONVERGED = -5,
    H2W_ERR_STATE = -6       /* call needs an earlier step (tree, assembly) */
};

/* -DUSE_nHODLRdD (H2*), -DUSE_snHODLRdD ((H2+H)*), -DUSE_HODLRdD (H*, non-nested:
 * every interaction-list pair compressed on its own, 2D and 3D only,
 * 2D/codes/matvec.hpp:136-172, 3D/codes/matvec.hpp:138-180) */
enum { H2W_FORM_NESTED = 0, H2W_FORM_SEMINESTED = 1, H2W_FORM_NONNESTED = 2 };
/* reference "choice". The complex kernels (nested or semi-nested forms):
 *  H2W_KERNEL_HELMHOLTZ (3D): the reference's USE_Helm build, exp(iR)/(4 pi)
 *    off the diagonal and 500 sqrt(N) on it (3D/codes/kernel.hpp:132-144,195-208);
 *  H2W_KERNEL_HANKEL (2D): the reference's USE_Hankel build, i H0^(1)(R) / 4
 *    = (-Y0(R) + i J0(R)) / 4 off the diagonal and (1 + 15 ln N + Kii) / h^2 on
 *    it (2D/codes/kernel.hpp:126-144,321-333, 2D/codes/integral2d.hpp:16-90),
 *    with the library's own J0 and Y0 where the reference calls Boost;
 * complex scalars throughout (3D/codes/headers.hpp:35-40, 2D/codes/headers.hpp:34-40),
 * in the nested and semi-nested forms (H2W_FORM_NONNESTED with a complex kernel is
 * refused at h2w_create with H2W_ERR_ARG). A handle with a complex kernel takes and returns complex vectors as N
 * interleaved (re, im) pairs of doubles (the layout of std::complex<double>)
 * in h2w_matvec (FP64, one right-hand side), h2w_gmres and h2w_dense_matvec;
 * the mixed-precision, many-right-hand-side, learned, far-field-on-the-fly
 * and allocation-free entry points refuse it with H2W_ERR_ARG, and
 * h2w_batch_create with H2W_ERR_STATE. */
enum { H2W_KERNEL_IE = 0, H2W_KERNEL_RBF = 1, H2W_KERNEL_HELMHOLTZ = 2, H2W_KERNEL_HANKEL = 10 };
enum { H2W_ASSEMBLE_NCA = 0, H2W_ASSEMBLE_IMPORT = 1, H2W_ASSEMBLE_LEARNED = 2 };
/* FP64: FP64 operator and arithmetic. FP32: FP32 operator copy and arithmetic.
 * DF64 (multi-vector products only: h2w_matvec with nrhs > 1 and the batched
 * solvers): the FP64 operator with double-FP32 arithmetic (each operand split
 * into an FP32 pair, products and sums carried as FP32 pairs), about 2^-44
 * relative per term, on the FP32 pipes. */
enum { H2W_PREC_FP64 = 0, H2W_PREC_FP32 = 1, H2W_PREC_DF64 = 2 };
/* pointer-location flags for vectors */
enum { H2W_HOST = 0, H2W_DEVICE = 1 };

/* Lists exported by h2w_get_list / accepted by h2w_import_list: CSR over
 * (level 0..L, box in numbering order); per (level, box, interaction-list
 * slot) for SN_ROW/SN_COL in 2D/3D and per (level >= 1, box, sibling slot)
 * in 1D. Values are original point indices except NBR/IL (box numbers) and
 * ISVERTEX (0/1). */
enum {
    H2W_LIST_CHARGE = 0, H2W_LIST_NBR = 1, H2W_LIST_IL = 2, H2W_LIST_ISVERTEX = 3,
    H2W_LIST_FAR_CHECK = 4, H2W_LIST_FAR_CHARGE = 5, H2W_LIST_VER_CHECK = 6, H2W_LIST_VER_CHARGE = 7,
    H2W_LIST_SN_ROW = 8, H2W_LIST_SN_COL = 9
};

typedef struct h2w_config {
    int dim;          /* 1, 2 or 3 */
    int form;         /* H2W_FORM_* */
    int choice;       /* H2W_KERNEL_*: kernel.hpp getMatrixEntry choice 0 / 1 / 2 / 10 */
    int tol_pow;      /* NCA/ACA tolerance 10^-tol_pow (aca.hpp LowRank) */
    int nlevels;      /* tree depth (main.cpp computes it from N and nmax) */
    int rank_cap;     /* max NCA rank per block; 0 = min(rows, cols) */
    int64_t kernel_n; /* particles.size() when the kernel object is built (0 = N) */
    int64_t diag_n;   /* particles.size() when entries are evaluated (0 = N; 1D drivers: 2N) */
    int device;       /* CUDA device ordinal; -1 = host-only handle (points, tree, lists) */
} h2w_config;

/* Replaces: new initialisation(N|sqrtN|cbrtN, nLevels, nParticlesInLeaf, L, TOL_POW, choice)
 * (1D/codes/matvec.hpp:85-93, 2D/codes/matvec.hpp:120-129, 3D/codes/matvec.hpp:19-29). */
int h2w_create(const h2w_config *cfg, h2w_handle **out);
/* Replaces the destructor (the reference leaks; this frees everything). */
int h2w_destroy(h2w_handle *h);
const char *h2w_last_error(const h2w_handle *h);

/* Points, row-major n x dim, host memory. Replaces the point generation of
 * set_Uniform_Nodes (1D/codes/HODLR1Dtree.hpp:59-66, 2D :75-91, 3D :82-102). */
int h2w_set_points(h2w_handle *h, const double *pts, int64_t n);
/* The reference's uniform grid: n_per_axis^dim interior points of [-1,1]^dim,
 * -1 + 2(k+1)/(n+1), with the reference's point numbering. */
int h2w_gen_grid(h2w_handle *h, int64_t n_per_axis);
/* n points uniform in [-1,1)^dim from the counter-based splitmix64 stream `seed`. */
int h2w_gen_uniform(h2w_handle *h, uint64_t seed, int64_t n);
/* Copy the current points out (row-major n x dim). */
int h2w_get_points(h2w_handle *h, double *pts);
int h2w_num_points(h2w_handle *h, int64_t *n);

/* Tree, neighbour slots, ordered interaction lists, vertex flags and charge
 * locations. Replaces createTree + assign_*Interaction* + assign_center_location
 * + separate_vertex_interaction + assignChargeLocations + assignNonLeafChargeLocations
 * (1D/codes/HODLR1Dtree.hpp:79-212, 2D/codes/HODLR2Dtree.hpp:104-534, 3D/codes/HODLR3Dtree.hpp:116-1852). */
int h2w_build_tree(h2w_handle *h);
/* CSR export of a list; call with NULL arrays to get the sizes. */
int h2w_get_list(h2w_handle *h, int which, int64_t *ptr, int32_t *val, int64_t *nptr, int64_t *nval);

/* Skeleton import (pivots of another NCA run, e.g. the oracle's), same CSR
 * layout as h2w_get_list; used by H2W_ASSEMBLE_IMPORT. */
int h2w_import_list(h2w_handle *h, int which, const int64_t *ptr, const int32_t *val, int64_t nptr);

/* Compress the operator on the GPU. Replaces tree_initialisation's assembly
 * calls: getNodes / getNodes_ver / assemble_M2L_* / assemble_M2M_ver /
 * assemble_NearField / getUVtTree_sn / assembleAcAr_sn (and the 1D forms). */
int h2w_assemble(h2w_handle *h, int mode);
/* Stored-entry count, exactly findMemory_n / findMemory_sn
 * (1D/codes/HODLR1Dtree.hpp:535-588, 2D :1207-1305, 3D :2505-2628). */
int h2w_storage_entries(h2w_handle *h, double *entries);
/* Bytes of packed operator data one FP64 / FP32 matvec reads. */
int h2w_operator_bytes(h2w_handle *h, int precision, int64_t *bytes);

/* y = A x for nrhs right-hand sides (column-major N x nrhs, leading dim N),
 * x and y in original point order. Replaces initialisation::mat_vec_prod
 * (1D/codes/matvec.hpp:121-138,163-178; 2D :163-182,212-233; 3D :63-83,115-136).
 * where = H2W_HOST or H2W_DEVICE; stream = cudaStream_t or NULL (default).
 * Complex kernels (H2W_KERNEL_HELMHOLTZ / _HANKEL): nrhs = 1, H2W_PREC_FP64,
 * x and y N interleaved (re, im) pairs. */
int h2w_matvec(h2w_handle *h, const double *x, double *y, int nrhs, int precision, int where, void *stream);

/* y = A x like h2w_matvec (one right-hand side, x and y DEVICE pointers in
 * original point order), but allocating nothing on any call: the workspace
 * is a fixed device array of 2^21 doubles (16 MiB) inside the library, not
 * handle memory. No counterpart in the reference (its mat_vec_prod keeps its
 * work vectors in the tree nodes). Limits and rules:
 *  - an operator whose workspace exceeds the array (more than 2^21 doubles
 *    FP64, 2^22 floats FP32) is rejected with H2W_ERR_ARG;
 *  - H2W_PREC_FP32 needs the FP32 operator copy, which this call does not
 *    create: one h2w_matvec FP32 call creates it, otherwise H2W_ERR_STATE;
 *  - the first call on a device looks up the array's device address (set-up,
 *    once per device); make that first call before any stream capture;
 *  - every call and every handle on a device shares the array, which keeps
 *    the last call's contents (each call clears what must start at zero):
 *    calls that overlap on the GPU race on it;
 *  - x and y must be device (or managed) memory of the handle's device;
 *    anything else (a host pointer) is refused with H2W_ERR_ARG before any
 *    launch;
 *  - the product is enqueued on `stream` (NULL: the handle's stream) and the
 *    call returns once it has finished: it reads the product's device error
 *    word back, so a grid-barrier wait that ran out (y then invalid) returns
 *    H2W_ERR_CUDA from this call rather than H2W_OK;
 *  - the array's cached device address does not survive cudaDeviceReset
 *    (or a new primary context) on that device: do not call it after one. */
int h2w_matvec_static(h2w_handle *h, const double *x, double *y, int precision, void *stream);

/* GMRES, unrestarted, FP64, device-resident. Replaces iterative_solver::GMRES
 * ({1D,2D,3D}/codes/gmres.hpp:92-200): x0 = x on entry, stops when |s(i+1)|/||b|| < 10^-tol_pow.
 * Complex kernels: b and x N interleaved (re, im) pairs; the reference's
 * complex GMRES (H2W_OPT_COMPLEX_ARNOLDI selects GMRES proper). */
int h2w_gmres(h2w_handle *h, const double *b, double *x, int max_iter, int tol_pow, int where, int *iters,
              double *resid);
/* Mixed precision: FP32 inner GMRES (FP32 operator, from d = 0; relative
 * tolerance 1e-6 in the first step, later a tenth of tol * ||b|| / ||r||,
 * within [1e-6, 0.1]) wrapped in FP64 iterative refinement; the first
 * residual (at the caller's x0) is formed with the FP32 operator and only
 * corrects, later residuals use the FP64 operator (or an update under
 * H2W_OPT_IR_UPDATE) and are the stopping test: FP64 relative residual
 * ||b - A x|| / ||b|| < 10^-tol_pow. */
int h2w_gmres_ir(h2w_handle *h, const double *b, double *x, int max_outer, int inner_iter, int tol_pow, int where,
                 int *outer_iters, int *inner_total, double *resid);

/* Many right-hand sides at once. b and x are column-major N x nrhs (leading
 * dimension N, original point order); x holds the initial guesses on entry.
 * Columns go through the solver in blocks of up to 64 that share every
 * operator read (one multi-vector matvec per Arnoldi step); each column runs
 * its own GMRES (the reference's iterative_solver::GMRES,
 * {1D,2D,3D}/codes/gmres.hpp:92-200, applied per column: own Krylov basis,
 * Givens rotations and stopping test) and stops updating when it converges.
 * iters / resid: nrhs entries. max_iter <= 400. The reference solves one
 * right-hand side per call; this replaces a loop of such calls. */
int h2w_gmres_batch(h2w_handle *h, const double *b, double *x, int nrhs, int max_iter, int tol_pow, int where,
                    int *iters, double *resid);
/* Mixed precision for many right-hand sides: per block of up to 64 columns,
 * refinement residuals from one multi-vector matvec per outer step (the first
 * with the FP32 operator, the later ones FP64, or DF64 by H2W_OPT_IR_RESIDUAL,
 * and only those tested against the tolerance) and a batched
 * FP32-operator inner GMRES (x0 = 0; relative tolerance 1e-6 in the first
 * step, later the strictest column's need: a tenth of tol * ||b|| / ||r||,
 * within [1e-6, 0.1]). resid: final
 * FP64 relative residual per column (nrhs entries); outer_iters: largest
 * outer count over the blocks; inner_total: inner Arnoldi steps summed over
 * outer steps and blocks (lockstep steps, not per column). */
int h2w_gmres_ir_batch(h2w_handle *h, const double *b, double *x, int nrhs, int max_outer, int inner_iter,
                       int tol_pow, int where, int *outer_iters, int *inner_total, double *resid);

/* Execution options of a handle (no counterpart in the reference, whose
 * only switches are compile-time macros):
 *  H2W_OPT_GRAPH  1 (default): GMRES runs its Arnoldi steps as one CUDA graph
 *                 launch (a conditional while node whose body is one step:
 *                 matvec + orthogonalisation + rotations + loop test), so
 *                 the host does not wait on each step; 0: host-driven loop.
 *                 Both run the same kernels in the same order.
 *  H2W_OPT_COOP   1 (default): a matvec is one cooperative launch with grid
 *                 barriers between its phases; 0: one launch per phase.
 *  H2W_OPT_MULTI_XW  gathered columns per target of the multi-vector
 *                 stream before a target is split into atomically
 *                 accumulated column chunks (multiple of 4, 32..2048;
 *                 default 1024). Setting it after assembly re-cuts the
 *                 stream (host work and small uploads; the operator is kept).
 *  H2W_OPT_ROW_SPLIT  rows x width per target of the single-vector stream
 *                 before it is cut into row chunks (default 16384); also
 *                 re-cuts after assembly.
 *  H2W_OPT_IR_RESIDUAL  precision of the refinement residuals after the
 *                 first in h2w_gmres_ir_batch (and in h2w_gmres_ir with the
 *                 far field on the fly): H2W_PREC_FP64 (default) or
 *                 H2W_PREC_DF64. (The first residual, at the caller's x0, is
 *                 formed with the FP32 operator and is not tested for
 *                 convergence; the inner solve only needs it to the inner
 *                 tolerance.)
 *  H2W_OPT_IR_UPDATE  1 (default): in the refinement solvers, after an
 *                 accurate residual r = b - A x, later residuals may be
 *                 updated as r - A32 d (d the last correction, A32 the FP32
 *                 operator) while the error bound of those updates,
 *                 10 * eta * ||d|| summed, stays below 25 % of
 *                 tol * ||b|| per column; eta = ||A32 z - A z|| / ||z||,
 *                 measured once per operator on pseudo-random and smooth z.
 *                 The stopping test and the reported residual add that
 *                 bound to ||r||. Not used near the FP64 floor (where
 *                 10 * eta * 2^-29 * ||x|| exceeds 1 % of tol * ||b||).
 *                 0: every residual after the first is formed from x.
 *  H2W_OPT_TENSOR  1: FP32 multi-vector products (nrhs > 1) run on the tensor
 *                 cores: tcgen05 TF32 MMAs on hi/lo-split operands
 *                 (a = tf32(a) + rest; all four partial products), FP32
 *                 accuracy; 0 (default): the FP32 FMA kernel, which is
 *                 faster on the operators measured (one tensor-memory CTA
 *                 per SM; targets of 20-64 rows fill half of an M = 128
 *                 MMA at best).
 *  H2W_OPT_F32_BASIS  1 (default): the inner solves of h2w_gmres_ir_batch
 *                 (FP32 operator, x0 = 0) keep their Krylov vectors and do
 *                 their orthogonalisation in FP32 (Hessenberg, rotations and
 *                 block sums in FP64); 0: FP64 Krylov vectors.
 *  H2W_OPT_DATAFLOW  1 (default): the products (single-vector FP64 / FP32,
 *                 multi-vector FP32 / FP64 / double-FP32) run as one
 *                 cooperative launch without grid barriers: each target waits
 *                 for the targets that produce the workspace rows it uses
 *                 (dependencies derived on the host from the rows each target
 *                 reads and writes) and releases its consumers; 0: phases
 *                 separated by grid barriers.
 *  H2W_OPT_PRODUCER_WARP  1 (default): the dataflow form of the FP32
 *                 multi-vector product splits each CTA into a producer warp
 *                 (claims targets, waits for their producers, streams their
 *                 chunks into a ring of shared-memory stages by bulk
 *                 asynchronous copies) and multiplying warps; 0: every warp
 *                 stages and multiplies its CTA's current target.
 *  H2W_OPT_SPIN_LIMIT  polls allowed per grid-barrier wait of the
 *                 single-vector product's cooperative launch with grid
 *                 barriers (H2W_OPT_DATAFLOW 0, and h2w_matvec_static);
 *                 0 (default): the built-in limit (2^26 polls, seconds). A
 *                 wait that runs out lets the kernel finish with an invalid
 *                 result and makes the call fail with H2W_ERR_CUDA; a tiny
 *                 limit is how that error path is exercised.
 *  H2W_OPT_FAR_ON_THE_FLY  1: the far-field M2L blocks (kernel entries between
 *                 the check points of interacting boxes, assemble_M2L_far,
 *                 3D/codes/HODLR3Dtree.hpp:1978-1998) are not stored; every
 *                 single-vector product evaluates them from the point
 *                 coordinates (FP64: the stored entries bitwise; FP32: FP32
 *                 entries from FP32 coordinates) between its upward and
 *                 downward passes. For operators whose stored form exceeds
 *                 device memory (3D, tight tolerances: the far M2L blocks
 *                 are most of the entries). Takes effect at the next
 *                 h2w_assemble; multi-vector products and many-problem
 *                 batches need the stored form (H2W_ERR_STATE). 0 (default):
 *                 stored. The storage count stays the reference's. In this
 *                 mode one-column products also take H2W_PREC_DF64 (the far
 *                 M2L in double-FP32 arithmetic on the FP32 pipes, FP64
 *                 accuracy, for the kernels built on log(R^2); the stored
 *                 passes in FP64), and h2w_gmres_ir forms its accurate
 *                 residuals that way when H2W_OPT_IR_RESIDUAL is DF64.
 *  H2W_OPT_NCA_DF  1 (default): the pivot search on groups of CTAs for the
 *                 kernels built on log (1D and 2D integral equation, 3D
 *                 RBF), whose entries already differ from the reference's
 *                 in the last bit, runs in double-FP32 arithmetic (about
 *                 2^-48 relative) on the FP32 pipes instead of FP64: the
 *                 residuals, the entries (FP64 coordinate differences, then
 *                 R^2 and the logarithm as pairs), and the stopping test's
 *                 dots, which are summed inside the next pivot's residual
 *                 passes; every block of 2048 or more rows + columns is
 *                 searched on groups then. 0: FP64. The other kernels always
 *                 search in FP64 (their pivots are bitwise the reference's).
 *  H2W_OPT_COMPLEX_ARNOLDI  complex kernels only. 0 (default): h2w_gmres is
 *                 the reference's GMRES as written (3D/codes/gmres.hpp:52-68,
 *                 :92-200): its Gram-Schmidt coefficients are Eigen's
 *                 w.dot(v_k) = sum conj(w) v_k, the conjugates of the
 *                 projections, and its rotations apply -sn dx where a unitary
 *                 rotation has -conj(sn) dx, so for complex operators the
 *                 Krylov vectors are not orthogonal and |s(i+1)| / ||b|| is
 *                 not the true residual (iteration counts and results match
 *                 the reference's). 1: Hermitian projections sum conj(v_k) w
 *                 and unitary rotations: GMRES proper, whose stopping test
 *                 bounds the true residual. */
enum { H2W_OPT_GRAPH = 0, H2W_OPT_COOP = 1, H2W_OPT_IR_RESIDUAL = 2, H2W_OPT_MULTI_XW = 3, H2W_OPT_ROW_SPLIT = 4,
       H2W_OPT_IR_UPDATE = 5, H2W_OPT_TENSOR = 6, H2W_OPT_F32_BASIS = 7, H2W_OPT_DATAFLOW = 8,
       H2W_OPT_PRODUCER_WARP = 9, H2W_OPT_SPIN_LIMIT = 10, H2W_OPT_FAR_ON_THE_FLY = 11, H2W_OPT_NCA_DF = 12,
       H2W_OPT_COMPLEX_ARNOLDI = 13 };
int h2w_set_option(h2w_handle *h, int option, int64_t value);
int h2w_get_option(h2w_handle *h, int option, int64_t *value);

/* Many independent problems at once (no counterpart in the reference, which
 * runs one problem per process): a batch groups assembled handles of one
 * device; their single-vector products run as ONE cooperative launch over a
 * merged target stream (every problem's levels, aligned at the leaf end), and
 * the solvers run every problem's GMRES in lockstep over concatenated vectors
 * (each problem with its own Krylov basis, rotations and stopping test).
 * Vectors are the problems' vectors concatenated in handle order, each in its
 * own original point order; h2w_batch_offsets gives the n+1 offsets. The
 * handles must outlive the batch and must not be re-assembled meanwhile. */
typedef struct h2w_batch h2w_batch;
int h2w_batch_create(h2w_handle *const *handles, int n, h2w_batch **out);
int h2w_batch_destroy(h2w_batch *b);
const char *h2w_batch_last_error(const h2w_batch *b);
int h2w_batch_offsets(h2w_batch *b, int64_t *offsets);
/* y = A_p x for every problem p (mat_vec_prod of each), FP64 or FP32. */
int h2w_batch_matvec(h2w_batch *b, const double *x, double *y, int precision, int where);
/* FP64 GMRES of every problem (iterative_solver::GMRES of each), x0 = x on
 * entry; iters / resid: n entries. max_iter <= 400. */
int h2w_batch_gmres(h2w_batch *b, const double *rhs, double *x, int max_iter, int tol_pow, int where, int *iters,
                    double *resid);
/* Mixed precision for every problem: batched FP32-operator inner GMRES (x0 =
 * 0; relative tolerance 1e-6 in the first step, later the strictest
 * problem's need, as in h2w_gmres_ir_batch) and FP64 refinement (first residual with the
 * FP32 operators, the later ones FP64 and tested); resid: n final FP64
 * relative residuals. */
int h2w_batch_gmres_ir(h2w_batch *b, const double *rhs, double *x, int max_outer, int inner_iter, int tol_pow,
                       int where, int *outer_iters, int *inner_total, double *resid);

/* Learned NCA proposals (no counterpart in the reference). A small network
 * (per candidate point: 16 geometric features -> 128 -> 128 -> 1, ReLU, BF16
 * weights, FP32 accumulation) scores the row and column points of every NCA
 * block; with H2W_ASSEMBLE_LEARNED the top-scored points form a cross
 * approximation that the NCA's own stopping test (1D/codes/aca.hpp:363,
 * 404-409) checks on the full block with one further ACA step; blocks that
 * fail it get the plain pivot search, so every block meets the NCA tolerance.
 * Parameters: h2w_mlp_nparam() floats, W1 (16 x 128, row-major), b1 (128),
 * W2 (128 x 128), b2 (128), w3 (128), b3 (1).
 *  h2w_learn_record     while enabled, plain NCA assembly records training
 *                       data: features of every candidate point (16 floats)
 *                       and a label (1 = chosen as a pivot); enabling clears it
 *  h2w_learn_data       copies it out (NULL arrays: count only)
 *  h2w_learn_set_model  installs a trained model; rank estimate per block =
 *                       ceil(calib * sum of the rows' probabilities) + margin
 *  h2w_learn_stats      blocks proposed / accepted since the last call
 *  h2w_mlp_forward / h2w_mlp_grad / h2w_mlp_adam   the network's training
 *                       kernels on device pointers: logits; the gradient of
 *                       the mean weighted binary cross-entropy (positives
 *                       weighted by pos_weight) into grads, and the loss; an
 *                       Adam step (beta 0.9 / 0.999, eps 1e-8) */
int h2w_learn_record(h2w_handle *h, int enable);
int h2w_learn_data(h2w_handle *h, float *X, uint8_t *y, int64_t *count);
int h2w_learn_set_model(h2w_handle *h, const float *params, float calib, int margin);
int h2w_learn_stats(h2w_handle *h, int64_t *blocks, int64_t *accepted);
/* Since the last h2w_learn_stats: rejections by cause (rejects[0] no usable
 * pivots in the proposal, [1] non-finite factors, [2] the stopping test
 * failed) and the mean proposal size and pivots kept per block. */
int h2w_learn_detail(h2w_handle *h, int64_t *rejects, double *mean_rhat, double *mean_r1);
int h2w_mlp_nparam(void);
int h2w_mlp_forward(const float *params, const float *X, int64_t n, float *logits, void *stream);
int h2w_mlp_grad(const float *params, const float *X, const uint8_t *y, int64_t n, float pos_weight, float *grads,
                 float *loss, void *stream);
int h2w_mlp_adam(float *params, const float *grads, float *m, float *v, int step, float lr, void *stream);

/* Autotuner (no counterpart in the reference): times `reps` products per
 * candidate target granularity on this operator and this GPU and keeps the
 * fastest. nrhs > 1: the multi-vector stream's column cap (256, 512, 1024,
 * 2048) at `precision` (FP32, FP64 or DF64) for blocks of nrhs columns;
 * nrhs == 1: the single-vector stream's row split (4096 ... 65536) at FP32 or
 * FP64. precision H2W_TUNE_IR_MIX (nrhs > 1): the batched refinement's mix,
 * four FP32 products and one DF64 product per timed repetition. With FP32
 * or the mix on the dataflow launch, both forms of the FP32 product
 * (H2W_OPT_PRODUCER_WARP on and off) are candidates as well, and the faster
 * one stays set. chosen / best_ms (may be NULL): the kept column cap or row
 * split and its ms per repetition. */
enum { H2W_TUNE_IR_MIX = 16 };
int h2w_autotune(h2w_handle *h, int nrhs, int precision, int reps, int64_t *chosen, double *best_ms);

/* Launch statistics of the block-row GEMV kernel that performs every matvec
 * pass. While enabled, each phase launch is bracketed by CUDA events on its
 * own stream; enabling (or disabling) resets the record. (No counterpart in
 * the reference, whose only instrumentation is clock() accumulators.) */
int h2w_profile(h2w_handle *h, int enable);
/* Per phase of one matvec: launches recorded, total device ms, and the
 * algorithmic bytes one launch moves (operator panels + gathered sources +
 * destination rows) at the given precision. nphases receives the count. */
int h2w_profile_phases(h2w_handle *h, int precision, int max_phases, int64_t *launches, double *ms, double *bytes,
                       int *nphases);
/* Launch statistics of the multi-vector matvec kernel (h2w_matvec with
 * nrhs > 1, batched solvers) at one precision while profiling is enabled:
 * launches, total device ms and the algorithmic bytes of one launch (packed
 * operator once, the input block in the kernel's precision, the FP64 result
 * block). */
int h2w_profile_multi(h2w_handle *h, int precision, int64_t *launches, double *ms, double *bytes);
/* Launch statistics of the far-field M2L kernel of single-vector products
 * with H2W_OPT_FAR_ON_THE_FLY (precision H2W_PREC_FP32, H2W_PREC_FP64 or
 * H2W_PREC_DF64) while profiling is enabled: launches, total device ms, and
 * the kernel entries one launch evaluates (the far M2L blocks the reference
 * stores, evaluateFarField / assemble_M2L_far in 3D/codes/HODLR3Dtree.hpp,
 * formed from the points instead of read). entries is 0 when the operator
 * stores its far field. (No counterpart in the reference.) */
int h2w_profile_fly(h2w_handle *h, int precision, int64_t *launches, double *ms, int64_t *entries);
/* Shape of the multi-vector product's plan (host-side figures, no device
 * work): stats[0] targets, [1] operator panels, [2] operator entries read per
 * column, [3] entries the kernel multiplies per column (rows rounded to the
 * 8 rows of a warp, each panel's columns to 32-column chunks), [4] targets
 * accumulated atomically (column-split block rows), [5] entries spanned by
 * the kernel's 64-row tiles (the share of [3] in [5] is the share of busy
 * warps). n (1..6) entries are written. */
int h2w_plan_stats(h2w_handle *h, int64_t *stats, int n);
/* Kernel launches issued by this library since it was loaded. */
int64_t h2w_launch_count(void);

/* Dense FP64 product with the exact kernel matrix (getTruePoten,
 * 1D/codes/HODLR1Dtree.hpp:590-604), on the GPU, rows [row0, row0 + nrows).
 * Complex kernels: x (N) and y (nrows) interleaved (re, im) pairs. */
int h2w_dense_matvec(h2w_handle *h, const double *x, double *y, int64_t row0, int64_t nrows, int where);
/* Operator files (no counterpart in the reference, which re-assembles on
 * every run, 3D/codes/main.cpp:21-25). h2w_save_operator writes the
 * configuration, the points and every NCA pivot list of an assembled handle,
 * closed by a checksum. h2w_open_operator creates a handle on `device` from
 * such a file, rebuilds the tree and forms the operator from the saved pivots
 * (H2W_ASSEMBLE_IMPORT: the pivot search is skipped; the operator is bitwise
 * the saved one, its storage count checked); device = -1 gives a host-only
 * handle with the points, tree and imported lists. A missing, truncated or
 * corrupted file is refused with H2W_ERR_ARG. */
int h2w_save_operator(h2w_handle *h, const char *path);
/* The configuration a handle was created with (e.g. one opened from a file). */
int h2w_get_config(h2w_handle *h, h2w_config *out);
int h2w_open_operator(const char *path, int device, h2w_handle **out);

/* Relative error of the compressed FP64 product against the exact dense
 * product on the same vector, ||y_dense - A x|| / ||y_dense||: the reference's
 * compute_total_error (3D/codes/HODLR3Dtree.hpp:2645-2662, 2D/codes/HODLR2Dtree.hpp:1347,
 * on the charge of the last mat_vec_prod), on the GPU.
 * nrows <= 0 or >= N: every row (O(N^2) kernel entries, as the reference);
 * otherwise nrows rows evenly spaced in original point order
 * (row i * N / nrows), the sampled form for large N. x host or device (where). */
int h2w_total_error(h2w_handle *h, const double *x, int64_t nrows, int where, double *err);

#ifdef __cplusplus
}
#endif
#endif
