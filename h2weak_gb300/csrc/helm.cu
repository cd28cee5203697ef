// Complex Helmholtz kernels of the GB300 H2* library (sm_103a): the
// reference's USE_Helm build in 3D (3D/codes/kernel.hpp:132-144,195-208) and
// USE_Hankel build in 2D (2D/codes/kernel.hpp:126-144,321-333,
// 2D/codes/integral2d.hpp:16-57), complex scalars throughout
// (3D/codes/headers.hpp:35-40, 2D/codes/headers.hpp:34-40).
//
//  * kentry_c          3D: exp(iR)/(4 pi) off the diagonal, 500 sqrt(N) on it;
//                      2D: i H0^(1)(R) / 4 with J0, Y0 of bessel.cuh
//  * nca_c_kernel      the NCA/ACA pivot search in complex arithmetic, one CTA
//                      per block (3D/codes/aca.hpp:180-275)
//  * factor_c / xfer_c / fill_c   operator formation into a complex image
//  * realify_kernel    each complex block C (m x n) into the real block
//                      [[Re C, -Im C], [Im C, Re C]] with rows and columns
//                      interleaved (2i, 2i+1), so that the real FP64 product
//                      kernels apply the complex operator to interleaved
//                      (re, im) vectors unchanged
//  * dense_c_kernel    dense complex rows (getTruePoten)
//  * cgm_*             the reference GMRES's complex vector operations
//
// Complex arithmetic follows the C++ runtime the reference is built with:
// products (ac - bd, ad + bc) with every multiply and add rounded
// separately, quotients by Smith's algorithm (R. L. Smith, "Algorithm 116:
// Complex division", CACM 5(8), 1962), magnitudes by hypot; Eigen's complex
// dot product is conjugate-linear in its first argument.
#include <cfloat>
#include <climits>

#include "bessel.cuh"
#include "kernels.cuh"

namespace h2w {

// ------------------------------------------------------------ arithmetic ---
__device__ __forceinline__ double2 c_mul(double2 a, double2 b) {
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 c_sub(double2 a, double2 b) {
    return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y));
}
__device__ __forceinline__ double2 c_add(double2 a, double2 b) {
    return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}
// n / d by Smith's algorithm
__device__ __forceinline__ double2 c_div(double2 n, double2 d) {
    const double a = n.x, b = n.y, c = d.x, e = d.y;
    if (fabs(c) < fabs(e)) {
        const double r = __ddiv_rn(c, e);
        const double den = __dadd_rn(__dmul_rn(c, r), e);
        return make_double2(__ddiv_rn(__dadd_rn(__dmul_rn(a, r), b), den),
                            __ddiv_rn(__dsub_rn(__dmul_rn(b, r), a), den));
    }
    const double r = __ddiv_rn(e, c);
    const double den = __dadd_rn(__dmul_rn(e, r), c);
    return make_double2(__ddiv_rn(__dadd_rn(__dmul_rn(b, r), a), den), __ddiv_rn(__dsub_rn(b, __dmul_rn(a, r)), den));
}
__device__ __forceinline__ double c_abs(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double c_abs2(double2 a) { return __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)); }
// conj(a) * b
__device__ __forceinline__ double2 c_cmul(double2 a, double2 b) {
    return make_double2(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

// --------------------------------------------------------------- entries ---
// Helmholtz3D (3D/codes/kernel.hpp:133-144): R2 = (dx^2 + dy^2) + dz^2,
// exp(i R) = (cos R, sin R), each part divided by 4 pi; diagonal 500 sqrt(N).
// Helmholtz2D (2D/codes/kernel.hpp:126-144): R2 = dx^2 + dy^2,
// i (J0(R) + i Y0(R)) / 4 = (-Y0(R) / 4, J0(R) / 4); diagonal
// (1 + 15 ln N + Kii) / h^2 with the complex self term Kii.
__device__ __forceinline__ double2 kentry_c(const KParams &k, int i, int j) {
    if (i == j) return make_double2(k.diag, k.diag_im);
    if (k.dim == 2) {
        const double *a = k.pts + (size_t)i * 2, *b = k.pts + (size_t)j * 2;
        const double dx = __dsub_rn(a[0], b[0]), dy = __dsub_rn(a[1], b[1]);
        const double R = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
        double j0, y0;
        bessel::j0y0(R, j0, y0);
        return make_double2(__ddiv_rn(-y0, 4.0), __ddiv_rn(j0, 4.0));
    }
    const double *a = k.pts + (size_t)i * 3, *b = k.pts + (size_t)j * 3;
    const double dx = __dsub_rn(a[0], b[0]), dy = __dsub_rn(a[1], b[1]), dz = __dsub_rn(a[2], b[2]);
    const double R2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const double R = __dsqrt_rn(R2);
    double s, c;
    sincos(R, &s, &c);
    return make_double2(__ddiv_rn(c, k.four_pi), __ddiv_rn(s, k.four_pi));
}

// ------------------------------------------------------------ reductions ---
__device__ __forceinline__ double c_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ bool c_amax_better(double va, int ia, double vb, int ib) {
    return va > vb || (va == vb && ia < ib);
}
// Block-wide sum; every thread gets the total. sh: >= 32 doubles.
__device__ double c_block_sum(double v, double *sh) {
    v = c_warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t += sh[q];
    return t;
}
// Block-wide argmax of (value, lowest index); every thread gets the result.
__device__ void c_block_amax(double &v, int &i, double *shv, int *shi) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, v, o);
        int oi = __shfl_xor_sync(0xffffffffu, i, o);
        if (c_amax_better(ov, oi, v, i)) { v = ov; i = oi; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) { shv[w] = v; shi[w] = i; }
    __syncthreads();
    v = shv[0];
    i = shi[0];
    for (int q = 1; q < nw; ++q)
        if (c_amax_better(shv[q], shi[q], v, i)) { v = shv[q]; i = shi[q]; }
}
__device__ __forceinline__ bool c_bit_get(const uint32_t *m, int i) { return (m[i >> 5] >> (i & 31)) & 1u; }

// ------------------------------------------------------------------- NCA ---
// One CTA per block (I, J), the pivoting and stopping rule of the real
// nca_kernel with complex residuals: first row whose largest |entry|
// exceeds 1e-36, column pivot = first largest |.| among unused columns of the
// residual row, row pivot = first largest |.| among unused rows of the
// residual column (before the division by the pivot), residual entries
// formed in pivot order (r - U_l(i) V_l(s), separately rounded), u = col /
// pivot, stop when ||u|| ||v|| <= tol normS or the rank reaches min(n1, n2);
// normS^2 = normS^2 + (||u|| ||v||)^2 + sum_l 2 |(U_l . u)(V_l . v)| with
// conjugate-first dots. U and V: complex scratch at pb.u / pb.v (complex units).
constexpr int NCAC_THREADS = 256;

__global__ void __launch_bounds__(NCAC_THREADS) nca_c_kernel(const NcaProb *__restrict__ probs,
                                                             const int32_t *__restrict__ idx, KParams kp, double tol,
                                                             double2 *__restrict__ scr, int32_t *__restrict__ rank_out,
                                                             int32_t *__restrict__ prow, int32_t *__restrict__ pcol,
                                                             int32_t *status, int mask1_words, int mask2_words,
                                                             int coef_len) {
    extern __shared__ __align__(16) unsigned char smem[];
    double2 *coef = reinterpret_cast<double2 *>(smem);                 // coef_len
    double2 *red = coef + coef_len;                                     // 2 * coef_len * nw
    uint32_t *rmask = reinterpret_cast<uint32_t *>(red + (size_t)2 * coef_len * (NCAC_THREADS / 32));
    uint32_t *cmask = rmask + mask1_words;
    __shared__ double shv[32];
    __shared__ int shi[32];
    __shared__ double shs[32];

    const NcaProb pb = probs[blockIdx.x];
    const int n1 = pb.n1, n2 = pb.n2, rcap = pb.rcap;
    const int32_t *I = idx + pb.ri;
    const int32_t *J = idx + pb.ci;
    double2 *U = scr + pb.u;
    double2 *V = scr + pb.v;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;

    for (int q = tid; q < mask1_words; q += nt) rmask[q] = 0u;
    for (int q = tid; q < mask2_words; q += nt) cmask[q] = 0u;
    __syncthreads();
    if (tid == 0) rank_out[blockIdx.x] = 0;
    const int mn = n1 < n2 ? n1 : n2;
    if (mn == 0 || rcap == 0) return;

    const double tiny = 1e-36;
    int ri = -1, ci = -1;
    for (int l = 0; l < n1; ++l) {
        double bv = -1.0;
        int bi = INT_MAX;
        const int gi = I[l];
        for (int s = tid; s < n2; s += nt) {
            double2 v = kentry_c(kp, gi, J[s]);
            V[s] = v;
            double a = c_abs(v);
            if (c_amax_better(a, s, bv, bi)) { bv = a; bi = s; }
        }
        c_block_amax(bv, bi, shv, shi);
        if (bv > tiny) { ri = l; ci = bi; break; }
    }
    if (ri < 0) return;
    __syncthreads();
    double2 piv = V[ci];
    double usq = 0.0, vsq = 0.0;
    int nri = INT_MAX;
    {
        double bv = -1.0;
        int bi = INT_MAX;
        const int gj = J[ci];
        for (int t = tid; t < n1; t += nt) {
            double2 c = kentry_c(kp, I[t], gj);
            double2 u = c_div(c, piv);
            U[t] = u;
            usq += c_abs2(u);
            if (t != ri) {
                double a = c_abs(c);
                if (c_amax_better(a, t, bv, bi)) { bv = a; bi = t; }
            }
        }
        for (int s = tid; s < n2; s += nt) vsq += c_abs2(V[s]);
        c_block_amax(bv, bi, shv, shi);
        nri = bi;
    }
    double nu = sqrt(c_block_sum(usq, shs));
    double nv = sqrt(c_block_sum(vsq, shs));
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

    bool over = false;
    while (nu * nv > tol * normS && rank < mn) {
        if (rank >= rcap) {
            over = true;
            break;
        }
        if (ri < 0 || ri >= n1) {
            if (tid == 0) atomicOr(status, 2);
            break;
        }
        for (int l = tid; l < rank; l += nt) coef[l] = U[(size_t)l * n1 + ri];
        __syncthreads();
        double2 *Vr = V + (size_t)rank * n2;
        double bv = -1.0;
        int bi = INT_MAX;
        vsq = 0.0;
        {
            const int gi = I[ri];
            for (int s = tid; s < n2; s += nt) {
                double2 v = kentry_c(kp, gi, J[s]);
                for (int l = 0; l < rank; ++l) v = c_sub(v, c_mul(coef[l], V[(size_t)l * n2 + s]));
                Vr[s] = v;
                vsq += c_abs2(v);
                if (!c_bit_get(cmask, s)) {
                    double a = c_abs(v);
                    if (c_amax_better(a, s, bv, bi)) { bv = a; bi = s; }
                }
            }
        }
        c_block_amax(bv, bi, shv, shi);
        if (bi < 0 || bi >= n2) {
            if (tid == 0) atomicOr(status, 2);
            break;
        }
        ci = bi;
        nv = sqrt(c_block_sum(vsq, shs));
        piv = Vr[ci];
        for (int l = tid; l < rank; l += nt) coef[l] = V[(size_t)l * n2 + ci];
        __syncthreads();
        double2 *Ur = U + (size_t)rank * n1;
        usq = 0.0;
        bv = -1.0;
        bi = INT_MAX;
        {
            const int gj = J[ci];
            for (int t = tid; t < n1; t += nt) {
                double2 c = kentry_c(kp, I[t], gj);
                for (int l = 0; l < rank; ++l) c = c_sub(c, c_mul(coef[l], U[(size_t)l * n1 + t]));
                double2 u = c_div(c, piv);
                Ur[t] = u;
                usq += c_abs2(u);
                if (t != ri && !c_bit_get(rmask, t)) {
                    double a = c_abs(c);
                    if (c_amax_better(a, t, bv, bi)) { bv = a; bi = t; }
                }
            }
        }
        c_block_amax(bv, bi, shv, shi);
        nri = bi;
        nu = sqrt(c_block_sum(usq, shs));
        if (nu < 1e-36 || nv < 1e-36) break;
        if (tid == 0) {
            prow[pb.piv + rank] = ri;
            pcol[pb.piv + rank] = ci;
            rmask[ri >> 5] |= 1u << (ri & 31);
            cmask[ci >> 5] |= 1u << (ci & 31);
        }
        ++rank;
        // conjugate-first dots of every stored u and v with the new ones
        for (int l = 0; l < rank; ++l) {
            const double2 *Ul = U + (size_t)l * n1, *Vl = V + (size_t)l * n2;
            double2 du = make_double2(0.0, 0.0), dv = make_double2(0.0, 0.0);
            for (int t = tid; t < n1; t += nt) {
                double2 p = c_cmul(Ul[t], Ur[t]);
                du.x += p.x;
                du.y += p.y;
            }
            for (int s = tid; s < n2; s += nt) {
                double2 p = c_cmul(Vl[s], Vr[s]);
                dv.x += p.x;
                dv.y += p.y;
            }
            du.x = c_warp_sum(du.x);
            du.y = c_warp_sum(du.y);
            dv.x = c_warp_sum(dv.x);
            dv.y = c_warp_sum(dv.y);
            if (lane == 0) {
                red[(size_t)(2 * l) * nw + warp] = du;
                red[(size_t)(2 * l + 1) * nw + warp] = dv;
            }
        }
        __syncthreads();
        for (int l = tid; l < rank; l += nt) {
            double2 du = make_double2(0.0, 0.0), dv = make_double2(0.0, 0.0);
            for (int q = 0; q < nw; ++q) {
                double2 a = red[(size_t)(2 * l) * nw + q], b = red[(size_t)(2 * l + 1) * nw + q];
                du.x += a.x;
                du.y += a.y;
                dv.x += b.x;
                dv.y += b.y;
            }
            coef[l] = make_double2(2.0 * c_abs(c_mul(du, dv)), 0.0);
        }
        __syncthreads();
        if (tid == 0) {
            double uv = nu * nv;
            double ns = normS * normS + uv * uv;
            for (int l = 0; l < rank; ++l) ns += coef[l].x;
            shs[0] = sqrt(ns);
        }
        __syncthreads();
        normS = shs[0];
        ri = nri;
        __syncthreads();
    }
    if (tid == 0) rank_out[blockIdx.x] = over ? -rank : rank;
}

size_t nca_c_smem(int max_n1, int max_n2, int max_rcap) {
    const int m1 = (max_n1 + 31) / 32, m2 = (max_n2 + 31) / 32;
    const size_t coef_len = (size_t)max_rcap + 1;
    return coef_len * 16 + coef_len * 2 * (NCAC_THREADS / 32) * 16 + (size_t)(m1 + m2) * 4;
}

cudaError_t launch_nca_c(const NcaProb *probs, int nprob, const int32_t *idx, const KParams &kp, double tol,
                         double2 *scratch, int32_t *rank, int32_t *prow, int32_t *pcol, int32_t *status, int max_n1,
                         int max_n2, int max_rcap, cudaStream_t st) {
    if (nprob == 0) return cudaSuccess;
    const int m1 = (max_n1 + 31) / 32, m2 = (max_n2 + 31) / 32;
    const size_t smem = nca_c_smem(max_n1, max_n2, max_rcap);
    cudaError_t e = cudaFuncSetAttribute(nca_c_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    nca_c_kernel<<<nprob, NCAC_THREADS, smem, st>>>(probs, idx, kp, tol, scratch, rank, prow, pcol, status, m1, m2,
                                                    max_rcap + 1);
    count_launch();
    return cudaGetLastError();
}

// -------------------------------------------------------- factors, etc. ---
// The complex forms of factor_kernel, xfer_kernel and fill_kernel: the same
// job descriptors, positions in complex units of the complex operator image.
__global__ void factor_c_kernel(const FactorJob *__restrict__ jobs, const int32_t *__restrict__ idx, KParams kp,
                                double2 *__restrict__ F) {
    const FactorJob jb = jobs[blockIdx.x];
    const int r = jb.r;
    double2 *A = F + jb.f;
    const int32_t *I = idx + jb.ii, *J = idx + jb.jj;
    for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
        int i = e / r, j = e % r;
        A[e] = kentry_c(kp, I[i], J[j]);
    }
    __syncthreads();
    for (int l = 0; l < r; ++l) {
        for (int j = l + threadIdx.x; j < r; j += blockDim.x) {
            double2 v = A[l * r + j];
            for (int m = 0; m < l; ++m) v = c_sub(v, c_mul(A[l * r + m], A[m * r + j]));
            A[l * r + j] = v;
        }
        __syncthreads();
        const double2 piv = A[l * r + l];
        for (int t = l + 1 + threadIdx.x; t < r; t += blockDim.x) {
            double2 v = A[t * r + l];
            for (int m = 0; m < l; ++m) v = c_sub(v, c_mul(A[m * r + l], A[t * r + m]));
            A[t * r + l] = c_div(v, piv);
        }
        __syncthreads();
    }
}

__global__ void xfer_c_kernel(const XferJob *__restrict__ jobs, const int32_t *__restrict__ idx, KParams kp,
                              const double2 *__restrict__ F, double2 *__restrict__ op) {
    const XferJob jb = jobs[blockIdx.y];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= jb.n) return;
    const int r = jb.r;
    const double2 *A = F + jb.f;
    const int32_t *J = idx + jb.jj;
    const int gp = idx[jb.pi + p];
    const bool row = jb.mode == X_ROW_RL || jb.mode == X_ROW_R;
    double2 *y = row ? op + jb.a1 + p : op + jb.a1 + (int64_t)p * jb.ld1;
    const int64_t ys = row ? jb.ld1 : 1;
    for (int j = 0; j < r; ++j) y[j * ys] = kentry_c(kp, gp, J[j]);  // K(p,J) == K(J,p): the kernel is symmetric
    if (row) {
        for (int j = 0; j < r; ++j) {
            double2 s = y[j * ys];
            for (int q = 0; q < j; ++q) s = c_sub(s, c_mul(y[q * ys], A[q * r + j]));
            y[j * ys] = c_div(s, A[j * r + j]);
        }
        if (jb.mode == X_ROW_RL)
            for (int j = r - 1; j >= 0; --j) {
                double2 s = y[j * ys];
                for (int q = j + 1; q < r; ++q) s = c_sub(s, c_mul(y[q * ys], A[q * r + j]));
                y[j * ys] = s;
            }
        if (jb.a2 >= 0)
            for (int j = 0; j < r; ++j) op[jb.a2 + (int64_t)p * jb.ld2 + j] = y[j * ys];
    } else {
        for (int i = 0; i < r; ++i) {
            double2 s = y[i];
            for (int q = 0; q < i; ++q) s = c_sub(s, c_mul(A[i * r + q], y[q]));
            y[i] = s;
        }
        if (jb.mode == X_COL_LR)
            for (int i = r - 1; i >= 0; --i) {
                double2 s = y[i];
                for (int q = i + 1; q < r; ++q) s = c_sub(s, c_mul(A[i * r + q], y[q]));
                y[i] = c_div(s, A[i * r + i]);
            }
    }
}

__global__ void fill_c_kernel(const FillJob *__restrict__ jobs, const int32_t *__restrict__ idx, KParams kp,
                              double2 *__restrict__ op) {
    const FillJob jb = jobs[blockIdx.y];
    const int64_t total = (int64_t)jb.nr * jb.nc;
    const int32_t *R = idx + jb.ri, *C = idx + jb.ci;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int c = (int)(e / jb.nr), i = (int)(e % jb.nr);
        op[jb.a + (int64_t)c * jb.lda + i] = kentry_c(kp, R[i], C[c]);
    }
}

cudaError_t launch_assemble_c(const FactorJob *fac, int nfac, const XferJob *xf, int nxf, int max_n,
                              const FillJob *fill, int nfill, const int32_t *idx, const KParams &kp, double2 *F,
                              double2 *opc, cudaStream_t st) {
    if (nfac > 0) {
        factor_c_kernel<<<nfac, 128, 0, st>>>(fac, idx, kp, F);
        count_launch();
    }
    if (nxf > 0 && max_n > 0) {
        const int bs = 64;
        for (int j0 = 0; j0 < nxf; j0 += 65535) {
            int nj = nxf - j0 < 65535 ? nxf - j0 : 65535;
            dim3 grid((unsigned)((max_n + bs - 1) / bs), (unsigned)nj);
            xfer_c_kernel<<<grid, bs, 0, st>>>(xf + j0, idx, kp, F, opc);
            count_launch();
        }
    }
    for (int j0 = 0; j0 < nfill; j0 += 65535) {
        int nj = nfill - j0 < 65535 ? nfill - j0 : 65535;
        dim3 grid(8, (unsigned)nj);
        fill_c_kernel<<<grid, 256, 0, st>>>(fill + j0, idx, kp, opc);
        count_launch();
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------- realified ---
// Block q: complex column-major (element (i, c) at a + c*lda + i, lda rows,
// cols columns) -> real block at 4a, leading dimension 2*lda: (2i, 2c) = re,
// (2i+1, 2c) = im, (2i, 2c+1) = -im, (2i+1, 2c+1) = re.
__global__ void realify_kernel(const int64_t *__restrict__ blk, int64_t nblk, const double2 *__restrict__ opc,
                               double *__restrict__ op) {
    for (int64_t q = blockIdx.x; q < nblk; q += gridDim.x) {
        const int64_t a = blk[3 * q], lda = blk[3 * q + 1], cols = blk[3 * q + 2];
        const int64_t n = lda * cols;
        double *o = op + 4 * a;
        for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
            const int64_t c = e / lda, i = e - c * lda;
            const double2 z = opc[a + e];
            double *c0 = o + (2 * c) * (2 * lda) + 2 * i;
            double *c1 = c0 + 2 * lda;
            c0[0] = z.x;
            c0[1] = z.y;
            c1[0] = -z.y;
            c1[1] = z.x;
        }
    }
}
cudaError_t launch_realify(const int64_t *blk, int64_t nblk, const double2 *opc, double *op, cudaStream_t st) {
    if (nblk <= 0) return cudaSuccess;
    const int64_t grid = nblk < 4096 ? nblk : 4096;
    realify_kernel<<<(unsigned)grid, 256, 0, st>>>(blk, nblk, opc, op);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ dense rows ---
// y[r] = sum_j K(r, j) x[j] (complex, original order), r in [row0, row0+nrows):
// getTruePoten (3D/codes/HODLR3Dtree.hpp:2630-2643).
__global__ void dense_c_kernel(KParams kp, int64_t N, const double2 *__restrict__ x, double2 *__restrict__ y,
                               int64_t row0) {
    __shared__ double sh[32];
    const int64_t r = row0 + blockIdx.x;
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t j = threadIdx.x; j < N; j += blockDim.x) {
        double2 p = c_mul(kentry_c(kp, (int)r, (int)j), x[j]);
        acc.x += p.x;
        acc.y += p.y;
    }
    acc.x = c_block_sum(acc.x, sh);
    acc.y = c_block_sum(acc.y, sh);
    if (threadIdx.x == 0) y[blockIdx.x] = acc;
}
cudaError_t launch_dense_c(const KParams &kp, int64_t N, const double2 *x, double2 *y, int64_t row0, int64_t nrows,
                           cudaStream_t st) {
    for (int64_t b = 0; b < nrows; b += 2147483647LL) {
        int64_t nb = nrows - b < 2147483647LL ? nrows - b : 2147483647LL;
        dense_c_kernel<<<(unsigned)nb, 256, 0, st>>>(kp, N, x, y + b, row0 + b);
        count_launch();
    }
    return cudaGetLastError();
}

// ----------------------------------------------------------------- GMRES ---
// Vector operations of the reference GMRES (3D/codes/gmres.hpp:92-200) on
// complex vectors of n entries. Reductions: per-block partials, then one
// block sums them in order.
constexpr int CGM_THREADS = 256;
constexpr int CGM_BLOCKS = 304;

// part[b] = sum over the block's entries of conj(a_i) b_i  (Eigen's a.dot(b))
__global__ void cgm_dot_part(const double2 *__restrict__ a, const double2 *__restrict__ b, int64_t n,
                             double2 *__restrict__ part) {
    __shared__ double sh[32];
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 p = c_cmul(a[i], b[i]);
        acc.x += p.x;
        acc.y += p.y;
    }
    acc.x = c_block_sum(acc.x, sh);
    acc.y = c_block_sum(acc.y, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}
// out = sum of part[0..nb)
__global__ void cgm_dot_fin(const double2 *__restrict__ part, int nb, double2 *__restrict__ out) {
    __shared__ double sh[32];
    double2 acc = make_double2(0.0, 0.0);
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        acc.x += part[i].x;
        acc.y += part[i].y;
    }
    acc.x = c_block_sum(acc.x, sh);
    acc.y = c_block_sum(acc.y, sh);
    if (threadIdx.x == 0) *out = acc;
}
// w -= (*h) v
__global__ void cgm_axpy(double2 *__restrict__ w, const double2 *__restrict__ v, const double2 *__restrict__ h,
                         int64_t n) {
    const double2 c = *h;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = c_sub(w[i], c_mul(c, v[i]));
}
// dst = src * s (s real)
__global__ void cgm_scale(double2 *__restrict__ dst, const double2 *__restrict__ src, double s, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = make_double2(__dmul_rn(src[i].x, s), __dmul_rn(src[i].y, s));
}
// x += sum_j v_j y_j (y: k complex coefficients, v: column-major n x k)
__global__ void cgm_update(double2 *__restrict__ x, const double2 *__restrict__ V, const double2 *__restrict__ y,
                           int k, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 a = x[i];
        for (int j = 0; j < k; ++j) a = c_add(a, c_mul(V[(size_t)j * n + i], y[j]));
        x[i] = a;
    }
}
// r = b - Ax
__global__ void cgm_resid(double2 *__restrict__ r, const double2 *__restrict__ b, const double2 *__restrict__ ax,
                          int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = c_sub(b[i], ax[i]);
}

cudaError_t cgm_dot(const double2 *a, const double2 *b, int64_t n, double2 *part, double2 *out, cudaStream_t st) {
    cgm_dot_part<<<CGM_BLOCKS, CGM_THREADS, 0, st>>>(a, b, n, part);
    cgm_dot_fin<<<1, CGM_THREADS, 0, st>>>(part, CGM_BLOCKS, out);
    count_launch(2);
    return cudaGetLastError();
}
cudaError_t cgm_axpy_launch(double2 *w, const double2 *v, const double2 *h, int64_t n, cudaStream_t st) {
    cgm_axpy<<<CGM_BLOCKS, CGM_THREADS, 0, st>>>(w, v, h, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t cgm_scale_launch(double2 *dst, const double2 *src, double s, int64_t n, cudaStream_t st) {
    cgm_scale<<<CGM_BLOCKS, CGM_THREADS, 0, st>>>(dst, src, s, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t cgm_update_launch(double2 *x, const double2 *V, const double2 *y, int k, int64_t n, cudaStream_t st) {
    if (k <= 0) return cudaSuccess;
    cgm_update<<<CGM_BLOCKS, CGM_THREADS, 0, st>>>(x, V, y, k, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t cgm_resid_launch(double2 *r, const double2 *b, const double2 *ax, int64_t n, cudaStream_t st) {
    cgm_resid<<<CGM_BLOCKS, CGM_THREADS, 0, st>>>(r, b, ax, n);
    count_launch();
    return cudaGetLastError();
}
int cgm_blocks() { return CGM_BLOCKS; }

}  // namespace h2w
