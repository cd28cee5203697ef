/* CPU oracle for the H2* / (H2+H)* HODLRdD matvec and GMRES of H2weak.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py, always as the checker or
 * the timed CPU baseline, never by the GPU library.
 *
 * Parity pinning: this restatement is checked against (a) the reference's
 * own headers compiled against an Eigen-subset shim (oracle/_ref, golden
 * dumps under tests/golden/) and (b) the storage known-answer values the
 * reference publishes in {1D,2D,3D}/results/*.txt.
 */
#ifndef H2W_ORACLE_H
#define H2W_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct h2wo h2wo;

/* dim 1..3; form 0 = nested H2*, 1 = semi-nested (H2+H)*, 2 = H*;
 * choice 0 / 1 (real kernels), 2 (the complex Helmholtz kernel of the
 * reference's USE_Helm build, 3D) or 10 (the complex Hankel kernel of its
 * USE_Hankel build, 2D), in every form, whose vectors (x, y, b in
 * matvec, dense_matvec, gmres; out in entries) are interleaved (re, im)
 * doubles; pts n*dim
 * row-major; kernel_n = particles.size() when the reference kernel object
 * is built (sets h), diag_n = particles.size() when entries are evaluated
 * (1D drivers push the grid twice, so diag_n = 2N there). */
h2wo *h2wo_create(int dim, int form, int64_t n, const double *pts, int nlevels, int tol_pow, int choice,
                  int64_t kernel_n, int64_t diag_n);
void h2wo_destroy(h2wo *o);
int h2wo_assemble(h2wo *o);
int h2wo_matvec(h2wo *o, const double *x, double *y);
int h2wo_dense_matvec(h2wo *o, const double *x, double *y);
int h2wo_gmres(h2wo *o, const double *b, double *x, int max_iter, int tol_pow, int *iters, double *resid);
double h2wo_memory(h2wo *o);
double h2wo_kii(h2wo *o);
int h2wo_entries(h2wo *o, const int32_t *rows, int64_t nr, const int32_t *cols, int64_t nc, double *out);
/* CSR export of per-(level, box) lists, levels 0..L, boxes in numbering
 * order (per (level, box, interaction-list slot) for sn_row / sn_col).
 * which: 0 charge, 1 nbr, 2 il, 3 isvertex, 4 far_check, 5 far_charge,
 * 6 ver_check, 7 ver_charge, 8 sn_row, 9 sn_col, 10 uv_rank.
 * Returns the number of values; ptr/val may be NULL to query sizes
 * (h2wo_list_nptr gives the ptr length). */
int64_t h2wo_list(h2wo *o, int which, int64_t *ptr, int32_t *val);
/* 1 for the complex kernel */
int h2wo_is_complex(h2wo *o);
/* Summation order of every block product (process-wide): 0 = ascending, the
 * reference build's order (the default); 1 = descending, for tests of how much
 * a product depends on its summation order. */
void h2wo_set_sum_order(int reverse);
int64_t h2wo_list_nptr(h2wo *o, int which);

#ifdef __cplusplus
}
#endif
#endif
