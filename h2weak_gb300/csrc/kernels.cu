// sm_103a kernels of the GB300 H2* / (H2+H)* library.
//
//  * kentry            kernel-matrix entries, operation order and rounding of
//                      the reference's getMatrixEntry (no FMA contraction)
//  * nca_kernel        batched NCA/ACA pivot search, one CTA per block
//                      (1D/codes/aca.hpp:296-446 pivoting and stopping rule)
//  * factor_kernel     LU of K(I,J) in pivot order = the ACA's L and R
//  * xfer_kernel       rows K(p,J) R^-1 L^-1 (transfer matrices), columns
//                      R^-1 L^-1 K(I,p), and the 1D U / V^T factors
//  * fill_kernel       dense blocks K(I,J) straight into the packed operator
//  * brg_kernel        the matvec: block-row GEMV over a work list of targets,
//                      each the sum of row-major panels times gathered sources
//  * GMRES kernels     CGS2 Arnoldi step, normalisation, Givens rotations
#include <atomic>
#include <cfloat>
#include <climits>

#include "kernels.cuh"
#include "sync.cuh"
#include "entry.cuh"

namespace h2w {

static std::atomic<int64_t> g_launches{0};
int64_t launch_count() { return g_launches.load(); }
void count_launch(int64_t n) { g_launches.fetch_add(n); }

// ---------------------------------------------------------- reductions ---
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ bool amax_better(double va, int ia, double vb, int ib) {
    return va > vb || (va == vb && ia < ib);
}
__device__ __forceinline__ void warp_amax(double &v, int &i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, v, o);
        int oi = __shfl_xor_sync(0xffffffffu, i, o);
        if (amax_better(ov, oi, v, i)) { v = ov; i = oi; }
    }
}
// Block-wide sum; every thread gets the total. sh: >= 32 doubles.
__device__ double block_sum(double v, double *sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t += sh[q];
    return t;
}
// Block-wide argmax of (value, lowest index); every thread gets the result.
__device__ void block_amax(double &v, int &i, double *shv, int *shi) {
    warp_amax(v, i);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) { shv[w] = v; shi[w] = i; }
    __syncthreads();
    v = shv[0];
    i = shi[0];
    for (int q = 1; q < nw; ++q)
        if (amax_better(shv[q], shi[q], v, i)) { v = shv[q]; i = shi[q]; }
}

__device__ __forceinline__ bool bit_get(const uint32_t *m, int i) { return (m[i >> 5] >> (i & 31)) & 1u; }

// ----------------------------------------------------------------- NCA ---
// One CTA per block (I, J). Pivoting and stopping follow ACA_only_nodes:
// first row with a non-negligible entry, column pivot = first largest |.|
// among unused columns of the residual row, row pivot = first largest |.|
// among unused rows of the residual column, stop when ||u|| ||v|| <= tol
// normS or the rank reaches min(n1, n2) (a block whose rank reaches its
// scratch capacity rcap first reports -rcap). Residual rows and columns are
// formed entry by entry in pivot order with separate multiply and subtract,
// so for identical entries they are bitwise those of the reference; norms
// and dot products are tree reductions (they only enter the stopping test).
constexpr int NCA_THREADS = 256;
constexpr int GM_THREADS = 256;

__global__ void __launch_bounds__(NCA_THREADS) nca_kernel(const NcaProb *__restrict__ probs,
                                                          const int32_t *__restrict__ idx, KParams kp, double tol,
                                                          double *__restrict__ scr, int32_t *__restrict__ rank_out,
                                                          int32_t *__restrict__ prow, int32_t *__restrict__ pcol,
                                                          int32_t *status, int mask1_words, int mask2_words,
                                                          int coef_len) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *rmask = reinterpret_cast<uint32_t *>(smem);
    uint32_t *cmask = rmask + mask1_words;
    double *coef = reinterpret_cast<double *>(cmask + mask2_words + ((mask1_words + mask2_words) & 1));
    double *red = coef + coef_len;                       // coef_len * 8 (per-warp partial dots)
    __shared__ double shv[32];
    __shared__ int shi[32];
    __shared__ double shs[32];

    const NcaProb pb = probs[blockIdx.x];
    const int n1 = pb.n1, n2 = pb.n2, rcap = pb.rcap;
    const int32_t *I = idx + pb.ri;
    const int32_t *J = idx + pb.ci;
    double *U = scr + pb.u;
    double *V = scr + pb.v;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;

    for (int q = tid; q < mask1_words; q += nt) rmask[q] = 0u;
    for (int q = tid; q < mask2_words; q += nt) cmask[q] = 0u;
    __syncthreads();
    if (tid == 0) rank_out[blockIdx.x] = 0;
    const int mn = n1 < n2 ? n1 : n2;
    if (mn == 0 || rcap == 0) return;

    // first pivot row: first row whose largest |entry| exceeds 1e-36
    const double tiny = 1e-36;
    int ri = -1, ci = -1;
    for (int l = 0; l < n1; ++l) {
        double bv = -1.0;
        int bi = INT_MAX;
        const int gi = I[l];
        for (int s = tid; s < n2; s += nt) {
            double v = kentry(kp, gi, J[s]);
            V[s] = v;
            double a = fabs(v);
            if (amax_better(a, s, bv, bi)) { bv = a; bi = s; }
        }
        block_amax(bv, bi, shv, shi);
        if (bv > tiny) { ri = l; ci = bi; break; }
    }
    if (ri < 0) return;
    __syncthreads();
    double piv = V[ci];
    double usq = 0.0, vsq = 0.0;
    int nri = INT_MAX;
    {
        double bv = -1.0;
        int bi = INT_MAX;
        const int gj = J[ci];
        for (int t = tid; t < n1; t += nt) {
            double c = kentry(kp, I[t], gj);
            double u = __ddiv_rn(c, piv);
            U[t] = u;
            usq += u * u;
            if (t != ri) {
                double a = fabs(c);
                if (amax_better(a, t, bv, bi)) { bv = a; bi = t; }
            }
        }
        for (int s = tid; s < n2; s += nt) vsq += V[s] * V[s];
        block_amax(bv, bi, shv, shi);
        nri = bi;
    }
    double nu = sqrt(block_sum(usq, shs));
    double nv = sqrt(block_sum(vsq, shs));
    if (tid == 0) {
        prow[pb.piv] = ri;
        pcol[pb.piv] = ci;
        rmask[ri >> 5] |= 1u << (ri & 31);
        cmask[ci >> 5] |= 1u << (ci & 31);
    }
    int rank = 1;
    double normS = 0.0;
    ri = nri;
    __syncthreads();

    bool over = false;  // the block needs more pivots than its scratch holds
    while (nu * nv > tol * normS && rank < mn) {
        if (rank >= rcap) {
            over = true;
            break;
        }
        if (ri < 0 || ri >= n1) {  // no finite candidate row
            if (tid == 0) atomicOr(status, 2);
            break;
        }
        // residual row ri
        for (int l = tid; l < rank; l += nt) coef[l] = U[(size_t)l * n1 + ri];
        __syncthreads();
        double *Vr = V + (size_t)rank * n2;
        double bv = -1.0;
        int bi = INT_MAX;
        vsq = 0.0;
        {
            const int gi = I[ri];
            for (int s = tid; s < n2; s += nt) {
                double v = kentry(kp, gi, J[s]);
                for (int l = 0; l < rank; ++l) v = __dsub_rn(v, __dmul_rn(coef[l], V[(size_t)l * n2 + s]));
                Vr[s] = v;
                vsq += v * v;
                if (!bit_get(cmask, s)) {
                    double a = fabs(v);
                    if (amax_better(a, s, bv, bi)) { bv = a; bi = s; }
                }
            }
        }
        block_amax(bv, bi, shv, shi);
        if (bi < 0 || bi >= n2) {  // no finite candidate column (non-finite entries)
            if (tid == 0) atomicOr(status, 2);
            break;
        }
        ci = bi;
        nv = sqrt(block_sum(vsq, shs));
        // residual column ci
        piv = Vr[ci];
        for (int l = tid; l < rank; l += nt) coef[l] = V[(size_t)l * n2 + ci];
        __syncthreads();
        double *Ur = U + (size_t)rank * n1;
        usq = 0.0;
        bv = -1.0;
        bi = INT_MAX;
        {
            const int gj = J[ci];
            for (int t = tid; t < n1; t += nt) {
                double c = kentry(kp, I[t], gj);
                for (int l = 0; l < rank; ++l) c = __dsub_rn(c, __dmul_rn(coef[l], U[(size_t)l * n1 + t]));
                double u = __ddiv_rn(c, piv);
                Ur[t] = u;
                usq += u * u;
                if (t != ri && !bit_get(rmask, t)) {
                    double a = fabs(c);
                    if (amax_better(a, t, bv, bi)) { bv = a; bi = t; }
                }
            }
        }
        block_amax(bv, bi, shv, shi);
        nri = bi;
        nu = sqrt(block_sum(usq, shs));
        if (nu < 1e-36 || nv < 1e-36) break;
        if (tid == 0) {
            prow[pb.piv + rank] = ri;
            pcol[pb.piv + rank] = ci;
            rmask[ri >> 5] |= 1u << (ri & 31);
            cmask[ci >> 5] |= 1u << (ci & 31);
        }
        ++rank;
        // normS update: dots of every stored u and v with the new ones
        for (int l = 0; l < rank; ++l) {
            const double *Ul = U + (size_t)l * n1, *Vl = V + (size_t)l * n2;
            double du = 0.0, dv = 0.0;
            for (int t = tid; t < n1; t += nt) du += Ul[t] * Ur[t];
            for (int s = tid; s < n2; s += nt) dv += Vl[s] * Vr[s];
            du = warp_sum(du);
            dv = warp_sum(dv);
            if (lane == 0) {
                red[(size_t)(2 * l) * nw + warp] = du;
                red[(size_t)(2 * l + 1) * nw + warp] = dv;
            }
        }
        __syncthreads();
        for (int l = tid; l < rank; l += nt) {
            double du = 0.0, dv = 0.0;
            for (int q = 0; q < nw; ++q) {
                du += red[(size_t)(2 * l) * nw + q];
                dv += red[(size_t)(2 * l + 1) * nw + q];
            }
            coef[l] = 2.0 * fabs(du * dv);
        }
        __syncthreads();
        if (tid == 0) {
            double uv = nu * nv;
            double ns = normS * normS + uv * uv;
            for (int l = 0; l < rank; ++l) ns += coef[l];
            shs[0] = sqrt(ns);
        }
        __syncthreads();
        normS = shs[0];
        ri = nri;
        __syncthreads();
    }
    // an overflowing block reports -rank: the host runs it again with more scratch
    if (tid == 0) rank_out[blockIdx.x] = over ? -rank : rank;
}

cudaError_t launch_nca(const NcaProb *probs, int nprob, const int32_t *idx, const KParams &kp, double tol,
                       double *scratch, int32_t *rank, int32_t *prow, int32_t *pcol, int32_t *status, int max_n1,
                       int max_n2, int max_rcap, cudaStream_t st) {
    if (nprob == 0) return cudaSuccess;
    int m1 = (max_n1 + 31) / 32, m2 = (max_n2 + 31) / 32;
    int coef_len = max_rcap + 1;
    size_t smem = (size_t)(m1 + m2 + 1) * 4 + (size_t)coef_len * 8 + (size_t)coef_len * 2 * (NCA_THREADS / 32) * 8;
    cudaError_t e = cudaFuncSetAttribute(nca_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    nca_kernel<<<nprob, NCA_THREADS, smem, st>>>(probs, idx, kp, tol, scratch, rank, prow, pcol, status, m1, m2,
                                                 coef_len);
    count_launch(); return cudaGetLastError();
}

// ------------------------------------------------------------- factors ---
// F (r x r, row-major) <- K(I,J) factorised in pivot order: R on and above
// the diagonal, unit-lower L below it, with the ACA's operation order
// (R(l,j) = A(l,j) - sum_m L(l,m) R(m,j); L(t,l) = (A(t,l) - sum_m R(m,l) L(t,m)) / R(l,l)).
__global__ void factor_kernel(const FactorJob *__restrict__ jobs, const int32_t *__restrict__ idx, KParams kp,
                              double *__restrict__ F) {
    const FactorJob jb = jobs[blockIdx.x];
    const int r = jb.r;
    double *A = F + jb.f;
    const int32_t *I = idx + jb.ii, *J = idx + jb.jj;
    for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
        int i = e / r, j = e % r;
        A[e] = kentry(kp, I[i], J[j]);
    }
    __syncthreads();
    for (int l = 0; l < r; ++l) {
        for (int j = l + threadIdx.x; j < r; j += blockDim.x) {
            double v = A[l * r + j];
            for (int m = 0; m < l; ++m) v = __dsub_rn(v, __dmul_rn(A[l * r + m], A[m * r + j]));
            A[l * r + j] = v;
        }
        __syncthreads();
        const double piv = A[l * r + l];
        for (int t = l + 1 + threadIdx.x; t < r; t += blockDim.x) {
            double v = A[t * r + l];
            for (int m = 0; m < l; ++m) v = __dsub_rn(v, __dmul_rn(A[m * r + l], A[t * r + m]));
            A[t * r + l] = __ddiv_rn(v, piv);
        }
        __syncthreads();
    }
}

cudaError_t launch_factor(const FactorJob *jobs, int njobs, const int32_t *idx, const KParams &kp, double *F,
                          cudaStream_t st) {
    if (njobs == 0) return cudaSuccess;
    factor_kernel<<<njobs, 128, 0, st>>>(jobs, idx, kp, F);
    count_launch(); return cudaGetLastError();
}

// ----------------------------------------------------------- transfers ---
// One thread per point p of a job.
//  X_ROW_RL: y = K(p,J) R^-1 L^-1  (far L2P rows; vertex / 1D M2M^T rows)
//  X_ROW_R : y = K(p,J) R^-1       (1D U rows)
//  X_COL_LR: y = R^-1 L^-1 K(I,p)  (semi-nested R^-1 L^-1 Ar columns)
//  X_COL_L : y = L^-1 K(I,p)       (1D V^T columns)
// The substitutions follow Eigen's triangularView::solve order as restated
// in the oracle, so transfer rows are bitwise the reference's for equal entries.
__global__ void xfer_kernel(const XferJob *__restrict__ jobs, const int32_t *__restrict__ idx, KParams kp,
                            const double *__restrict__ F, double *__restrict__ op) {
    const XferJob jb = jobs[blockIdx.y];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= jb.n) return;
    const int r = jb.r;
    const double *A = F + jb.f;  // row-major r x r: R upper, L strictly lower
    const int32_t *J = idx + jb.jj;
    const int gp = idx[jb.pi + p];
    const bool row = jb.mode == X_ROW_RL || jb.mode == X_ROW_R;
    // Column-major outputs. ROW modes: element (p, j) of the n x r result at
    // a1 + j*ld1 + p; COL modes: element (i, p) of the r x n result at
    // a1 + p*ld1 + i. The output location is the working vector.
    double *y = row ? op + jb.a1 + p : op + jb.a1 + (int64_t)p * jb.ld1;
    const int64_t ys = row ? jb.ld1 : 1;
    for (int j = 0; j < r; ++j) y[j * ys] = kentry(kp, gp, J[j]);  // K(p,J) == K(J,p) bitwise
    if (row) {
        // z R = b (forward), then y L = z (backward, unit diagonal)
        for (int j = 0; j < r; ++j) {
            double s = y[j * ys];
            for (int q = 0; q < j; ++q) s = __dsub_rn(s, __dmul_rn(y[q * ys], A[q * r + j]));
            y[j * ys] = __ddiv_rn(s, A[j * r + j]);
        }
        if (jb.mode == X_ROW_RL)
            for (int j = r - 1; j >= 0; --j) {
                double s = y[j * ys];
                for (int q = j + 1; q < r; ++q) s = __dsub_rn(s, __dmul_rn(y[q * ys], A[q * r + j]));
                y[j * ys] = s;
            }
        // transposed copy: element (j, p) of the r x n result at a2 + p*ld2 + j
        if (jb.a2 >= 0)
            for (int j = 0; j < r; ++j) op[jb.a2 + (int64_t)p * jb.ld2 + j] = y[j * ys];
    } else {
        // L x = b (forward, unit diagonal), then R x = x (backward)
        for (int i = 0; i < r; ++i) {
            double s = y[i];
            for (int q = 0; q < i; ++q) s = __dsub_rn(s, __dmul_rn(A[i * r + q], y[q]));
            y[i] = s;
        }
        if (jb.mode == X_COL_LR)
            for (int i = r - 1; i >= 0; --i) {
                double s = y[i];
                for (int q = i + 1; q < r; ++q) s = __dsub_rn(s, __dmul_rn(A[i * r + q], y[q]));
                y[i] = __ddiv_rn(s, A[i * r + i]);
            }
    }
}

cudaError_t launch_xfer(const XferJob *jobs, int njobs, int max_n, const int32_t *idx, const KParams &kp,
                        const double *F, double *op, cudaStream_t st) {
    if (njobs == 0 || max_n == 0) return cudaSuccess;
    const int bs = 64;
    for (int j0 = 0; j0 < njobs; j0 += 65535) {
        int nj = njobs - j0 < 65535 ? njobs - j0 : 65535;
        dim3 grid((unsigned)((max_n + bs - 1) / bs), (unsigned)nj);
        xfer_kernel<<<grid, bs, 0, st>>>(jobs + j0, idx, kp, F, op);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// --------------------------------------------------------------- fills ---
__global__ void fill_kernel(const FillJob *__restrict__ jobs, const int32_t *__restrict__ idx, KParams kp,
                            double *__restrict__ op) {
    const FillJob jb = jobs[blockIdx.y];
    const int64_t total = (int64_t)jb.nr * jb.nc;
    const int32_t *R = idx + jb.ri, *C = idx + jb.ci;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int c = (int)(e / jb.nr), i = (int)(e % jb.nr);
        op[jb.a + (int64_t)c * jb.lda + i] = kentry(kp, R[i], C[c]);
    }
}

cudaError_t launch_fill(const FillJob *jobs, int njobs, const int32_t *idx, const KParams &kp, double *op,
                        cudaStream_t st) {
    if (njobs == 0) return cudaSuccess;
    for (int j0 = 0; j0 < njobs; j0 += 65535) {
        int nj = njobs - j0 < 65535 ? njobs - j0 : 65535;
        dim3 grid(8, (unsigned)nj);
        fill_kernel<<<grid, 256, 0, st>>>(jobs + j0, idx, kp, op);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

__global__ void convert_f32_kernel(const double *__restrict__ s, float *__restrict__ d, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}
cudaError_t launch_convert_f32(const double *src, float *dst, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    convert_f32_kernel<<<1216, 256, 0, st>>>(src, dst, n);
    count_launch(); return cudaGetLastError();
}

// ------------------------------------------------------- block-row GEMV ---
// Persistent block-row GEMV over column-major panels. A CTA takes targets
// t0 + blockIdx.x, + gridDim.x, ... (heaviest first, the host sorts them),
// copies the target's packed record into shared memory, gathers its sources
// (x through perm, or the workspace) into shared memory, then lets
// lane l of a warp own row l of a 32-row group while the warps of the CTA
// split the columns: every load is a coalesced 32-row column segment and
// each lane keeps several independent loads in flight. Partial sums of the
// column slices meet in shared memory.
constexpr int BRG_THREADS = 256;
constexpr int BRG_WARPS = BRG_THREADS / 32;

// Target record (int64 words), built by the host plan:
//   [0] dst   [1] nrows | flags << 32   [2] np | ns << 32
//   np panels x 3 words: a, lda | w << 32, xoff
//   ns segments x 2 words: src, len | (xoff << 1 | gather) << 32  (xoff: offset in the target's gathered x)
template <class T> struct Vec16;
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
__device__ __forceinline__ void vfma(double *acc, const double2 v, const double x) {
    acc[0] += v.x * x;
    acc[1] += v.y * x;
}
__device__ __forceinline__ void vfma(float *acc, const float4 v, const float x) {
    acc[0] += v.x * x;
    acc[1] += v.y * x;
    acc[2] += v.z * x;
    acc[3] += v.w * x;
}

template <class T> struct BrgShared {
    T xs[BRG_XS_ELEMS];
    T red[BRG_WARPS * 32 * Vec16<T>::n];
    int64_t rec[BRG_REC_WORDS];
};

// One target: rows [dst, dst+nrows) from its packed record (see above).
template <class T>
__device__ __forceinline__ void brg_target(BrgShared<T> &sh, int64_t t, const int64_t *__restrict__ roff,
                                           const int64_t *__restrict__ blob, const T *__restrict__ A, T *ws,
                                           const double *__restrict__ xin, double *yout,
                                           const int32_t *__restrict__ perm) {
    T *xs = sh.xs;
    T *red = sh.red;
    int64_t *rec = sh.rec;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t o = roff[t];
    const int nw = (int)(roff[t + 1] - o);
    for (int q = tid; q < nw; q += BRG_THREADS) rec[q] = blob[o + q];
    __syncthreads();
    const int64_t dst = rec[0];
    const int nrows = (int)(rec[1] & 0xffffffff), flags = (int)(rec[1] >> 32);
    const int np = (int)(rec[2] & 0xffffffff), ns = (int)(rec[2] >> 32);
    const int64_t *pan = rec + 3;
    const int64_t *seg = pan + 3 * np;
    // gather: every thread walks the segments for its elements
    {
        int sidx = 0;
        int64_t s_src = 0;
        int s_lo = 0, s_hi = -1, s_g = 0;
        auto seek = [&](int e) {
            while (e >= s_hi && sidx < ns) {
                const int64_t w1 = seg[2 * sidx + 1];
                s_src = seg[2 * sidx];
                const int len = (int)(w1 & 0xffffffff);
                const int code = (int)(w1 >> 32);
                s_lo = code >> 1;
                s_hi = s_lo + len;
                s_g = code & 1;
                ++sidx;
            }
        };
        // elements of the concatenated sources, in segment order
        int total = 0;
        if (ns > 0) {
            const int64_t wl = seg[2 * (ns - 1) + 1];
            total = (int)(wl >> 33) + (int)(wl & 0xffffffff);
        }
        for (int e0 = tid; e0 < total; e0 += 4 * BRG_THREADS) {
            int64_t idx4[4];
            int xo4[4], g4[4];
            int cnt = 0;
            for (int u = 0; u < 4; ++u) {
                const int e = e0 + u * BRG_THREADS;
                if (e >= total) break;
                seek(e);
                if (e < s_lo) {  // padding gap between panels
                    idx4[u] = -1;
                } else {
                    idx4[u] = s_src + (e - s_lo);
                }
                xo4[u] = e;
                g4[u] = s_g;
                ++cnt;
            }
            T v4[4];
            for (int u = 0; u < cnt; ++u) {
                const int64_t ix = idx4[u];
                if (ix < 0) v4[u] = T(0);
                else if (g4[u]) v4[u] = (T)xin[perm ? (int64_t)perm[ix] : ix];
                else v4[u] = ws[ix];
            }
            for (int u = 0; u < cnt; ++u) xs[xo4[u]] = v4[u];
        }
    }
    __syncthreads();
    // Rows in blocks of RB = 32*VN. Within a block, a warp's lane l owns the
    // VN-row slice rq = l % RQ (16-byte vector loads down a column) and
    // column phase cs = l / RQ, so one load instruction covers 32/RQ columns.
    // The warps of the CTA split the columns of each block.
    using V16 = typename Vec16<T>::type;
    constexpr int VN = Vec16<T>::n;
    constexpr int RB = 32 * VN;
    const int nblk = (nrows + RB - 1) / RB;
    for (int bb = 0; bb < nblk; bb += BRG_WARPS) {
        const int nb_here = nblk - bb < BRG_WARPS ? nblk - bb : BRG_WARPS;
        const int S = BRG_WARPS / nb_here;        // warps (column slices) per row block
        const int myb = warp % nb_here, sl = warp / nb_here;
        const int rb = (bb + myb) * RB;
        const int rows = nrows - rb < RB ? nrows - rb : RB;
        int RQ = 1;
        while (RQ * VN < rows) RQ <<= 1;          // row slices of this block (power of two <= 32)
        const int CS = 32 / RQ;                   // column phases per load
        const int rq = lane % RQ, cs = lane / RQ;
        const int r_lo = rb + rq * VN;            // first row of the lane's slice
        T acc[VN];
#pragma unroll
        for (int v = 0; v < VN; ++v) acc[v] = T(0);
        if (sl < S && r_lo < nrows) {
            for (int q = 0; q < np; ++q) {
                const int64_t pa = pan[3 * q];
                const int lda = (int)(pan[3 * q + 1] & 0xffffffff), w = (int)(pan[3 * q + 1] >> 32);
                const int xoff = (int)pan[3 * q + 2];
                const int c0 = (int)(((int64_t)w * sl) / S), c1 = (int)(((int64_t)w * (sl + 1)) / S);
                const T *xp = xs + xoff;
                const int64_t ld = lda;
                const T *base = A + pa + r_lo;
                if (((pa & 3) == 0) && ((lda & 3) == 0)) {
                    int c = c0 + cs;
                    for (; c + 3 * CS < c1; c += 4 * CS) {
                        const V16 v0 = *reinterpret_cast<const V16 *>(base + (int64_t)c * ld);
                        const V16 v1 = *reinterpret_cast<const V16 *>(base + (int64_t)(c + CS) * ld);
                        const V16 v2 = *reinterpret_cast<const V16 *>(base + (int64_t)(c + 2 * CS) * ld);
                        const V16 v3 = *reinterpret_cast<const V16 *>(base + (int64_t)(c + 3 * CS) * ld);
                        const T x0 = xp[c], x1 = xp[c + CS], x2 = xp[c + 2 * CS], x3 = xp[c + 3 * CS];
                        vfma(acc, v0, x0);
                        vfma(acc, v1, x1);
                        vfma(acc, v2, x2);
                        vfma(acc, v3, x3);
                    }
                    for (; c < c1; c += CS) vfma(acc, *reinterpret_cast<const V16 *>(base + (int64_t)c * ld), xp[c]);
                } else {
                    const int nv = nrows - r_lo < VN ? nrows - r_lo : VN;
                    for (int c = c0 + cs; c < c1; c += CS) {
                        const T xc = xp[c];
                        const T *col = base + (int64_t)c * ld;
#pragma unroll
                        for (int v = 0; v < VN; ++v)
                            if (v < nv) acc[v] += col[v] * xc;
                    }
                }
            }
        }
        // reduce over the column phases of the warp
#pragma unroll
        for (int v = 0; v < VN; ++v)
            for (int o = RQ; o < 32; o <<= 1) acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], o);
        if (cs == 0 && sl < S)
#pragma unroll
            for (int v = 0; v < VN; ++v) red[warp * RB + rq * VN + v] = acc[v];
        __syncthreads();
        // combine the column slices of each block and write
        for (int e = tid; e < nb_here * RB; e += BRG_THREADS) {
            const int mb = e / RB, r = e % RB;
            const int i = (bb + mb) * RB + r;
            if (i >= nrows) continue;
            T v = T(0);
            for (int q = 0; q < S; ++q) v += red[(mb + q * nb_here) * RB + r];
            const int64_t d = dst + i;
            if (flags & T_SCATTER) {
                const T ov = (flags & T_ACCUM) ? ws[d] + v : v;
                yout[perm ? (int64_t)perm[d] : d] = (double)ov;
            } else if (flags & T_ATOMIC) {
                atomicAdd(ws + d, v);
            } else if (flags & T_ACCUM) {
                ws[d] += v;
            } else {
                ws[d] = v;
            }
        }
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(BRG_THREADS, 4)
    brg_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob, int64_t t0, int64_t t1,
               const T *__restrict__ A, T *ws, const double *__restrict__ xin, double *yout,
               const int32_t *__restrict__ perm) {
    __shared__ BrgShared<T> sh;
    for (int64_t t = t0 + blockIdx.x; t < t1; t += gridDim.x) brg_target<T>(sh, t, roff, blob, A, ws, xin, yout, perm);
}

// The whole matvec in one cooperative launch: phases separated by grid
// barriers; targets of a phase striped over the CTAs.
template <class T>
__global__ void __launch_bounds__(BRG_THREADS, 4)
    brg_coop_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob,
                    const int64_t *__restrict__ pstart, int nphase, const T *__restrict__ A, T *ws,
                    const double *__restrict__ xin, double *yout, const int32_t *__restrict__ perm, unsigned *bar,
                    int32_t *err, long long spin) {
    __shared__ BrgShared<T> sh;
    for (int p = 0; p < nphase; ++p) {
        const int64_t t1 = pstart[p + 1];
        for (int64_t t = pstart[p] + blockIdx.x; t < t1; t += gridDim.x)
            brg_target<T>(sh, t, roff, blob, A, ws, xin, yout, perm);
        if (p + 1 < nphase) grid_barrier(bar, gridDim.x, err, spin);
    }
}

// Dataflow form of brg_coop_kernel (no grid barriers): targets claimed in
// stored (topological) order from a global counter; each waits until its
// producer count rem[t] is zero (bounded spin: on timeout *err = 3 and the
// CTA proceeds), runs, fences its writes and decrements the counts of its
// consumers cidx[coff[t] .. coff[t+1]). Cooperative launch: every CTA is
// resident, so the producers of a waiting target are all claimed and running.
template <class T>
__global__ void __launch_bounds__(BRG_THREADS, 4)
    brg_flow_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob, int64_t t0, int64_t nt,
                    int32_t *ctr, int32_t *rem, const int64_t *__restrict__ coff, const int32_t *__restrict__ cidx,
                    const T *__restrict__ A, T *ws, const double *__restrict__ xin, double *yout,
                    const int32_t *__restrict__ perm, int32_t *err) {
    __shared__ BrgShared<T> sh;
    __shared__ int64_t s_next;
    int64_t t = t0 + blockIdx.x;
    while (t < nt) {
        if (threadIdx.x == 0) {
            long long it = 0;
            while (*((volatile int32_t *)(rem + t)) > 0) {
                if (++it > (1LL << 20)) {  // about 0.1 s
                    atomicExch(err, 3);
                    break;
                }
                __nanosleep(32);
            }
            __threadfence();
        }
        __syncthreads();
        brg_target<T>(sh, t, roff, blob, A, ws, xin, yout, perm);
        __syncthreads();
        if (threadIdx.x < 32) {
            __threadfence();  // this CTA's results are visible before its consumers are released
            for (int64_t e = coff[t] + threadIdx.x; e < coff[t + 1]; e += 32) atomicSub(rem + cidx[e], 1);
            if (threadIdx.x == 0) s_next = t0 + gridDim.x + atomicAdd(ctr, 1);
        }
        __syncthreads();
        t = s_next;
    }
}

// Many independent problems in one cooperative launch: the problem index of
// a target sits in bits 8.. of its record's flag word, and the target runs
// on that problem's operator, workspace, point permutation and vector
// segment (xoff into the concatenated input and output vectors). active
// (may be NULL): a problem whose entry is not -1 (a converged system of the
// lockstep solver) is skipped.
template <class T>
__global__ void __launch_bounds__(BRG_THREADS, 4)
    brgb_coop_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob,
                     const int64_t *__restrict__ pstart, int nphase, const BatchProb *__restrict__ probs,
                     const int32_t *__restrict__ active, const double *__restrict__ xin, double *yout,
                     unsigned *bar, int32_t *err) {
    __shared__ BrgShared<T> sh;
    for (int p = 0; p < nphase; ++p) {
        const int64_t t1 = pstart[p + 1];
        for (int64_t t = pstart[p] + blockIdx.x; t < t1; t += gridDim.x) {
            const int pid = (int)(blob[roff[t] + 1] >> 40);
            if (active && active[pid] != -1) continue;
            const BatchProb pr = probs[pid];
            brg_target<T>(sh, t, roff, blob, reinterpret_cast<const T *>(pr.A), reinterpret_cast<T *>(pr.ws),
                          xin + pr.xoff, yout + pr.xoff, pr.perm);
        }
        if (p + 1 < nphase) grid_barrier(bar, gridDim.x, err);
    }
}

static int g_num_sms = 0;

template <class T>
static cudaError_t launch_brg_t(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t t1, const T *A, T *ws,
                                const double *xin, double *yout, const int32_t *perm, cudaStream_t st) {
    if (t1 <= t0) return cudaSuccess;
    static int per_sm = 0;
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, brg_kernel<T>, BRG_THREADS, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    const int64_t nt = t1 - t0;
    const int64_t cap = (int64_t)g_num_sms * per_sm;
    const int grid = (int)(nt < cap ? nt : cap);
    brg_kernel<T><<<grid, BRG_THREADS, 0, st>>>(roff, blob, t0, t1, A, ws, xin, yout, perm);
    count_launch();
    return cudaGetLastError();
}

template <class T>
static cudaError_t launch_coop_t(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                                 const T *A, T *ws, const double *xin, double *yout, const int32_t *perm,
                                 unsigned *bar, int32_t *err, long long spin, cudaStream_t st) {
    if (nphase <= 0) return cudaSuccess;
    if (spin <= 0) spin = GRID_SPIN_LIMIT;
    static int per_sm = 0;
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, brg_coop_kernel<T>, BRG_THREADS, 0);
        if (per_sm <= 0) return cudaErrorCooperativeLaunchTooLarge;
    }
    const int grid = g_num_sms * per_sm;
    void *args[] = {(void *)&roff, (void *)&blob, (void *)&pstart, (void *)&nphase, (void *)&A, (void *)&ws,
                    (void *)&xin, (void *)&yout, (void *)&perm, (void *)&bar, (void *)&err, (void *)&spin};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)brg_coop_kernel<T>, dim3(grid), dim3(BRG_THREADS), args,
                                                0, st);
    count_launch();
    return e;
}

template <class T>
static cudaError_t launch_brg_flow_t(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t nt, int32_t *ctr,
                                     int32_t *rem,
                                     const int64_t *coff, const int32_t *cidx, const T *A, T *ws, const double *xin,
                                     double *yout, const int32_t *perm, int32_t *err, cudaStream_t st) {
    if (nt <= t0) return cudaSuccess;
    static int per_sm = 0;
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, brg_flow_kernel<T>, BRG_THREADS, 0);
        if (per_sm <= 0) return cudaErrorCooperativeLaunchTooLarge;
    }
    const int grid = g_num_sms * per_sm;
    void *args[] = {(void *)&roff, (void *)&blob, (void *)&t0, (void *)&nt,   (void *)&ctr,  (void *)&rem,
                    (void *)&coff, (void *)&cidx, (void *)&A,    (void *)&ws,   (void *)&xin,
                    (void *)&yout, (void *)&perm, (void *)&err};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)brg_flow_kernel<T>, dim3(grid), dim3(BRG_THREADS), args,
                                                0, st);
    count_launch();
    return e;
}
cudaError_t launch_brg_flow_f64(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t nt, int32_t *ctr, int32_t *rem,
                                const int64_t *coff, const int32_t *cidx, const double *A, double *ws,
                                const double *xin, double *yout, const int32_t *perm, int32_t *err, cudaStream_t st) {
    return launch_brg_flow_t<double>(roff, blob, t0, nt, ctr, rem, coff, cidx, A, ws, xin, yout, perm, err, st);
}
cudaError_t launch_brg_flow_f32(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t nt, int32_t *ctr, int32_t *rem,
                                const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const double *xin,
                                double *yout, const int32_t *perm, int32_t *err, cudaStream_t st) {
    return launch_brg_flow_t<float>(roff, blob, t0, nt, ctr, rem, coff, cidx, A, ws, xin, yout, perm, err, st);
}

cudaError_t launch_coop_f64(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const double *A, double *ws, const double *xin, double *yout, const int32_t *perm,
                            unsigned *bar, int32_t *err, cudaStream_t st, long long spin) {
    return launch_coop_t<double>(roff, blob, pstart, nphase, A, ws, xin, yout, perm, bar, err, spin, st);
}
cudaError_t launch_coop_f32(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const float *A, float *ws, const double *xin, double *yout, const int32_t *perm,
                            unsigned *bar, int32_t *err, cudaStream_t st, long long spin) {
    return launch_coop_t<float>(roff, blob, pstart, nphase, A, ws, xin, yout, perm, bar, err, spin, st);
}

template <class T>
static cudaError_t launch_brgb_t(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                                 const BatchProb *probs, const int32_t *active, const double *xin, double *yout,
                                 unsigned *bar, int32_t *err, cudaStream_t st) {
    if (nphase <= 0) return cudaSuccess;
    static int per_sm = 0;
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, brgb_coop_kernel<T>, BRG_THREADS, 0);
        if (per_sm <= 0) return cudaErrorCooperativeLaunchTooLarge;
    }
    const int grid = g_num_sms * per_sm;
    void *args[] = {(void *)&roff, (void *)&blob, (void *)&pstart, (void *)&nphase, (void *)&probs,
                    (void *)&active, (void *)&xin, (void *)&yout,  (void *)&bar,    (void *)&err};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)brgb_coop_kernel<T>, dim3(grid), dim3(BRG_THREADS), args,
                                                0, st);
    count_launch();
    return e;
}
cudaError_t launch_brgb_f64(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const BatchProb *probs, const int32_t *active, const double *xin, double *yout,
                            unsigned *bar, int32_t *err, cudaStream_t st) {
    return launch_brgb_t<double>(roff, blob, pstart, nphase, probs, active, xin, yout, bar, err, st);
}
cudaError_t launch_brgb_f32(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                            const BatchProb *probs, const int32_t *active, const double *xin, double *yout,
                            unsigned *bar, int32_t *err, cudaStream_t st) {
    return launch_brgb_t<float>(roff, blob, pstart, nphase, probs, active, xin, yout, bar, err, st);
}

cudaError_t launch_brg_f64(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t t1, const double *A,
                           double *ws, const double *xin, double *yout, const int32_t *perm, cudaStream_t st) {
    return launch_brg_t<double>(roff, blob, t0, t1, A, ws, xin, yout, perm, st);
}
cudaError_t launch_brg_f32(const int64_t *roff, const int64_t *blob, int64_t t0, int64_t t1, const float *A,
                           float *ws, const double *xin, double *yout, const int32_t *perm, cudaStream_t st) {
    return launch_brg_t<float>(roff, blob, t0, t1, A, ws, xin, yout, perm, st);
}

template <class T>
__global__ void scatter_kernel2(const T *__restrict__ yp, double *__restrict__ y, const int32_t *__restrict__ perm,
                                int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[perm[i]] = (double)yp[i];
}
cudaError_t launch_scatter_f64(const double *yp, double *y, const int32_t *perm, int64_t n, cudaStream_t st) {
    scatter_kernel2<double><<<608, 256, 0, st>>>(yp, y, perm, n);
    count_launch(); return cudaGetLastError();
}
__global__ void gather_kernel(const double *__restrict__ x, double *__restrict__ xp, const int32_t *__restrict__ perm,
                              int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        xp[i] = x[perm[i]];
}
cudaError_t launch_gather_f64(const double *x, double *xp, const int32_t *perm, int64_t n, cudaStream_t st) {
    gather_kernel<<<608, 256, 0, st>>>(x, xp, perm, n);
    count_launch(); return cudaGetLastError();
}
cudaError_t launch_scatter_f32(const float *yp, double *y, const int32_t *perm, int64_t n, cudaStream_t st) {
    scatter_kernel2<float><<<608, 256, 0, st>>>(yp, y, perm, n);
    count_launch(); return cudaGetLastError();
}

// -------------------------------------------------------- dense oracle ---
__global__ void dense_kernel(KParams kp, int64_t N, const double *__restrict__ x, double *__restrict__ y,
                             int64_t row0) {
    __shared__ double sh[32];
    const int64_t r = row0 + blockIdx.x;
    double acc = 0.0;
    for (int64_t j = threadIdx.x; j < N; j += blockDim.x) acc += kentry(kp, (int)r, (int)j) * x[j];
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) y[blockIdx.x] = acc;
}
// Dense FP64 rows y[i] = sum_j K(rows[i], j) x[j] for a list of rows.
__global__ void dense_rows_kernel(KParams kp, int64_t N, const double *__restrict__ x,
                                  const int64_t *__restrict__ rows, double *__restrict__ y) {
    __shared__ double sh[32];
    const int64_t r = rows[blockIdx.x];
    double acc = 0.0;
    for (int64_t j = threadIdx.x; j < N; j += blockDim.x) acc += kentry(kp, (int)r, (int)j) * x[j];
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) y[blockIdx.x] = acc;
}
cudaError_t launch_dense_rows(const KParams &kp, int64_t N, const double *x, const int64_t *rows, int64_t nrows,
                              double *y, cudaStream_t st) {
    for (int64_t b = 0; b < nrows; b += 2147483647LL) {
        int64_t nb = nrows - b < 2147483647LL ? nrows - b : 2147483647LL;
        dense_rows_kernel<<<(unsigned)nb, 256, 0, st>>>(kp, N, x, rows + b, y + b);
        count_launch();
    }
    return cudaGetLastError();
}
cudaError_t launch_dense_matvec(const KParams &kp, int64_t N, const double *x, double *y, int64_t row0, int64_t nrows,
                                cudaStream_t st) {
    for (int64_t b = 0; b < nrows; b += 2147483647LL) {
        int64_t nb = nrows - b < 2147483647LL ? nrows - b : 2147483647LL;
        dense_kernel<<<(unsigned)nb, 256, 0, st>>>(kp, N, x, y + b, row0 + b);
        count_launch();
    }
    return cudaGetLastError();
}

// --------------------------------------------------------------- GMRES ---
// Classical Gram-Schmidt with one reorthogonalisation (CGS2), FP64, on a
// device-resident Krylov basis. Block b owns rows [b*chunk, (b+1)*chunk);
// per-block partial sums go through three buffers so that no block
// overwrites a partial another block still reads.
__device__ __forceinline__ void gm_rows(int64_t N, int nblk, int64_t &r0, int64_t &r1) {
    int64_t chunk = (N + nblk - 1) / nblk;
    r0 = (int64_t)blockIdx.x * chunk;
    r1 = r0 + chunk < N ? r0 + chunk : N;
}

// out[b*(m+1)+k] = sum_{t in block b} V[t,k] w[t], k <= i
__device__ void gm_block_dots(const GmresDev &g, int i, int64_t r0, int64_t r1, double *red, double *out) {
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = 0; k <= i; ++k) {
        const double *Vk = g.V + (size_t)k * g.N;
        double acc = 0.0;
        for (int64_t t = r0 + threadIdx.x; t < r1; t += blockDim.x) acc += Vk[t] * g.w[t];
        acc = warp_sum(acc);
        if (lane == 0) red[k * nw + warp] = acc;
    }
    __syncthreads();
    for (int k = threadIdx.x; k <= i; k += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < nw; ++q) s += red[k * nw + q];
        out[(size_t)blockIdx.x * (g.m + 1) + k] = s;
    }
}

__global__ void gm_dots(GmresDev g) {
    extern __shared__ double red[];
    const int i = *g.iter;
    int64_t r0, r1;
    gm_rows(g.N, g.nblk, r0, r1);
    gm_block_dots(g, i, r0, r1, red, g.part);
}

// h = sum_b in; w -= V h; H(:,i) (=|+=) h; out <- new dots (pass 0) or ||w||^2 partials (pass 1)
__global__ void gm_update(GmresDev g, int pass) {
    extern __shared__ double shm[];
    double *h = shm;
    double *red = shm + (g.m + 1);
    const double *in = g.part + (size_t)pass * g.nblk * (g.m + 1);
    double *out = g.part + (size_t)(pass + 1) * g.nblk * (g.m + 1);
    const int i = *g.iter;
    for (int k = threadIdx.x; k <= i; k += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < g.nblk; ++b) s += in[(size_t)b * (g.m + 1) + k];
        h[k] = s;
    }
    __syncthreads();
    if (blockIdx.x == 0)
        for (int k = threadIdx.x; k <= i; k += blockDim.x) {
            double *Hk = g.H + (size_t)i * (g.m + 1) + k;
            *Hk = pass == 0 ? h[k] : *Hk + h[k];
        }
    int64_t r0, r1;
    gm_rows(g.N, g.nblk, r0, r1);
    for (int64_t t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
        double v = g.w[t];
        for (int k = 0; k <= i; ++k) v -= g.V[(size_t)k * g.N + t] * h[k];
        g.w[t] = v;
    }
    __syncthreads();
    if (pass == 0) {
        gm_block_dots(g, i, r0, r1, red, out);
    } else {
        const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        double acc = 0.0;
        for (int64_t t = r0 + threadIdx.x; t < r1; t += blockDim.x) acc += g.w[t] * g.w[t];
        acc = warp_sum(acc);
        if (lane == 0) red[warp] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int q = 0; q < nw; ++q) s += red[q];
            out[(size_t)blockIdx.x * (g.m + 1)] = s;
        }
    }
}

// H(i+1,i) = ||w||; V[:,i+1] = vcur = (1/H(i+1,i)) w
__global__ void gm_normalise(GmresDev g) {
    __shared__ double hn;
    const double *in = g.part + (size_t)2 * g.nblk * (g.m + 1);
    const int i = *g.iter;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < g.nblk; ++b) s += in[(size_t)b * (g.m + 1)];
        hn = sqrt(s);
        if (blockIdx.x == 0) g.H[(size_t)i * (g.m + 1) + i + 1] = hn;
    }
    __syncthreads();
    const double ih = 1.0 / hn;
    int64_t r0, r1;
    gm_rows(g.N, g.nblk, r0, r1);
    double *Vn = g.V + (size_t)(i + 1) * g.N;
    for (int64_t t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
        double v = ih * g.w[t];
        Vn[t] = v;
        g.vcur[t] = v;
    }
}

__device__ void gm_apply(double &dx, double &dy, double cs, double sn) {
    double temp = __dadd_rn(__dmul_rn(cs, dx), __dmul_rn(sn, dy));
    dy = __dadd_rn(__dmul_rn(-sn, dx), __dmul_rn(cs, dy));
    dx = temp;
}

// Givens rotations on column i (*/codes/gmres.hpp:30-75,156-162); resid = |s(i+1)| / ||b||.
__global__ void gm_givens(GmresDev g) {
    const int i = *g.iter;
    const double tol = g.scal[6];
    double *Hc = g.H + (size_t)i * (g.m + 1);
    if (g.scal[2] != 0.0) return;  // already converged: leave state untouched
    for (int k = 0; k < i; ++k) gm_apply(Hc[k], Hc[k + 1], g.cs[k], g.sn[k]);
    double dx = Hc[i], dy = Hc[i + 1], cs, sn;
    if (dy == 0.0) { cs = 1.0; sn = 0.0; }
    else if (fabs(dy) > fabs(dx)) {
        double temp = dx / dy;
        sn = 1.0 / sqrt(1.0 + temp * temp);
        cs = temp * sn;
    } else {
        double temp = dy / dx;
        cs = 1.0 / sqrt(1.0 + temp * temp);
        sn = temp * cs;
    }
    g.cs[i] = cs;
    g.sn[i] = sn;
    gm_apply(Hc[i], Hc[i + 1], cs, sn);
    gm_apply(g.s[i], g.s[i + 1], cs, sn);
    double resid = fabs(g.s[i + 1]) / g.scal[0];
    g.scal[1] = resid;
    if (resid < tol) g.scal[2] = 1.0;
    else if (i + 1 < g.m) *g.iter = i + 1;
}

// One-time function attributes of the Arnoldi kernels (done before any
// stream capture of an Arnoldi step).
void gmres_prepare() {
    static bool cfg = false;
    if (!cfg) {
        cudaFuncSetAttribute(gm_dots, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(gm_update, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cfg = true;
    }
}

cudaError_t gmres_cgs2(const GmresDev &g, cudaStream_t st) {
    const int nw = GM_THREADS / 32;
    size_t sm_dots = (size_t)(g.m + 1) * nw * sizeof(double);
    size_t sm_upd = (size_t)(g.m + 1) * (nw + 1) * sizeof(double);
    gmres_prepare();
    gm_dots<<<g.nblk, GM_THREADS, sm_dots, st>>>(g);
    gm_update<<<g.nblk, GM_THREADS, sm_upd, st>>>(g, 0);
    gm_update<<<g.nblk, GM_THREADS, sm_upd, st>>>(g, 1);
    count_launch(3); return cudaGetLastError();
}

cudaError_t gmres_finish_iter(const GmresDev &g, cudaStream_t st) {
    gm_normalise<<<g.nblk, GM_THREADS, 0, st>>>(g);
    gm_givens<<<1, 1, 0, st>>>(g);
    count_launch(2); return cudaGetLastError();
}

// r = b - Ax (Ax NULL: r = b); beta = ||r||; V[:,0] = vcur = r / beta; s = beta e1; iter = 0
__global__ void gm_resid_part(GmresDev g, const double *__restrict__ b, const double *__restrict__ Ax) {
    __shared__ double sh[32];
    int64_t r0, r1;
    gm_rows(g.N, g.nblk, r0, r1);
    double acc = 0.0;
    for (int64_t t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
        double r = Ax ? b[t] - Ax[t] : b[t];  // Ax == NULL: x0 = 0
        g.w[t] = r;
        acc += r * r;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) g.part[blockIdx.x] = acc;
}
__global__ void gm_start_fin(GmresDev g, double normb) {
    __shared__ double beta;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < g.nblk; ++b) s += g.part[b];
        beta = sqrt(s);
        if (blockIdx.x == 0) {
            for (int k = 0; k <= g.m; ++k) { g.s[k] = 0.0; g.cs[k] = 0.0; g.sn[k] = 0.0; }
            g.s[0] = beta;
            g.scal[0] = normb;
            g.scal[1] = beta / normb;
            g.scal[2] = 0.0;
            g.scal[3] = beta;
            g.iter[0] = 0;
            g.iter[1] = 0;  // Arnoldi steps taken (graph loop counter)
        }
    }
    __syncthreads();
    const double ib = 1.0 / beta;
    int64_t r0, r1;
    gm_rows(g.N, g.nblk, r0, r1);
    for (int64_t t = r0 + threadIdx.x; t < r1; t += blockDim.x) {
        double v = g.w[t] * ib;
        g.V[t] = v;
        g.vcur[t] = v;
    }
}
// Loop condition of the graph-captured Arnoldi step: run another step while
// not converged and fewer than m steps were taken.
__global__ void gm_loop_cond(GmresDev g, cudaGraphConditionalHandle hnd) {
    const int c = ++g.iter[1];
    cudaGraphSetConditional(hnd, (g.scal[2] == 0.0 && c < g.m) ? 1u : 0u);
}
cudaError_t gmres_loop_cond(const GmresDev &g, cudaGraphConditionalHandle hnd, cudaStream_t st) {
    gm_loop_cond<<<1, 1, 0, st>>>(g, hnd);
    count_launch();
    return cudaGetLastError();
}

cudaError_t gmres_start(const GmresDev &g, const double *b, const double *Ax, double normb, cudaStream_t st) {
    gm_resid_part<<<g.nblk, GM_THREADS, 0, st>>>(g, b, Ax);
    gm_start_fin<<<g.nblk, GM_THREADS, 0, st>>>(g, normb);
    count_launch(2); return cudaGetLastError();
}

// x += sum_{j<=k} V[:,j] y[j]  (y precomputed by the back-substitution, in g.s)
__global__ void gm_xupdate(GmresDev g, double *__restrict__ x, const double *__restrict__ y, int k) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < g.N; t += (int64_t)gridDim.x * blockDim.x) {
        double v = x[t];
        for (int j = 0; j <= k; ++j) v += g.V[(size_t)j * g.N + t] * y[j];
        x[t] = v;
    }
}
cudaError_t gmres_update(const GmresDev &g, double *x, const double *y, int k, cudaStream_t st) {
    gm_xupdate<<<g.nblk, GM_THREADS, 0, st>>>(g, x, y, k);
    count_launch(); return cudaGetLastError();
}

__global__ void norm_part(const double *__restrict__ x, int64_t n, double *part) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        acc += x[t] * x[t];
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}
__global__ void norm_fin(const double *part, int nblk, double *out) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += part[b];
    *out = sqrt(s);
}
cudaError_t vec_norm(const double *x, int64_t n, double *part, int nblk, double *out, cudaStream_t st) {
    norm_part<<<nblk, GM_THREADS, 0, st>>>(x, n, part);
    norm_fin<<<1, 1, 0, st>>>(part, nblk, out);
    count_launch(2); return cudaGetLastError();
}

__global__ void axpby_kernel(double a, const double *x, double b, const double *y, double *z, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        z[t] = a * x[t] + b * y[t];
}
cudaError_t vec_axpby(double a, const double *x, double b, const double *y, double *z, int64_t n, cudaStream_t st) {
    axpby_kernel<<<608, 256, 0, st>>>(a, x, b, y, z, n);
    count_launch(); return cudaGetLastError();
}
__global__ void d2f_kernel(const double *x, float *y, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        y[t] = (float)x[t];
}
__global__ void f2d_kernel(const float *x, double *y, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        y[t] = (double)x[t];
}
cudaError_t vec_f64_to_f32(const double *x, float *y, int64_t n, cudaStream_t st) {
    d2f_kernel<<<608, 256, 0, st>>>(x, y, n);
    count_launch(); return cudaGetLastError();
}
cudaError_t vec_f32_to_f64(const float *x, double *y, int64_t n, cudaStream_t st) {
    f2d_kernel<<<608, 256, 0, st>>>(x, y, n);
    count_launch(); return cudaGetLastError();
}

}  // namespace h2w
