// Segmented GMRES for many independent problems (sm_103a).
//
// P systems of different sizes run the reference's unrestarted GMRES
// (*/codes/gmres.hpp:92-200) in lockstep over one concatenated vector:
// problem p owns a contiguous row range, every CTA works on rows of one
// problem only, so a CTA's partial sums belong to one problem and a
// per-problem reduction over that problem's CTAs gives its dot products.
// CGS2 orthogonalisation, Givens rotations, stopping test and back
// substitution are per problem; one problem's numbers never mix with
// another's. A converged problem keeps its state.
#include "kernels.cuh"

namespace h2w {

constexpr int GMS_THREADS = 256;
constexpr int GMS_WARPS = GMS_THREADS / 32;

__device__ __forceinline__ double gms_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ size_t gms_h(const GmresSeg &g, int p, int row, int col) {
    return ((size_t)p * g.m + col) * (g.m + 1) + row;
}

// out[blk*(m+1) + k] = sum over the block's rows of a_k[t] * b[t], k < kn,
// a_k = a + k*Ntot; four a_k per sweep. red: 4 * GMS_WARPS doubles.
__device__ void gms_block_dots(const GmresSeg &g, const double *a, const double *b, int kn, double *red,
                               double *out) {
    const int64_t r0 = g.brow[blockIdx.x], r1 = g.brow[blockIdx.x + 1];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k0 = 0; k0 < kn; k0 += 4) {
        const int kc = kn - k0 < 4 ? kn - k0 : 4;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 2
        for (int64_t t = r0 + threadIdx.x; t < r1; t += GMS_THREADS) {
            const double bv = b[t];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j < kc) acc[j] += a[(size_t)(k0 + j) * g.Ntot + t] * bv;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double v = gms_warp_sum(acc[j]);
            if (lane == 0) red[j * GMS_WARPS + warp] = v;
        }
        __syncthreads();
        if (threadIdx.x < kc) {
            double s = 0.0;
            for (int q = 0; q < GMS_WARPS; ++q) s += red[threadIdx.x * GMS_WARPS + q];
            out[(size_t)blockIdx.x * (g.m + 1) + k0 + threadIdx.x] = s;
        }
        __syncthreads();
    }
}

// Blocks of problems that are no longer running (converged) skip the
// Arnoldi step's vector work: their state is frozen.
__global__ void gms_dots(GmresSeg g) {
    __shared__ double red[4 * GMS_WARPS];
    if (g.conv[g.bprob[blockIdx.x]] != -1) return;
    gms_block_dots(g, g.V, g.w, *g.iter + 1, red, g.part);
}

// hsum[p*(m+1) + k] = sum over problem p's blocks of part[b*(m+1) + k], k <= i
// (all = 1) or k = 0 (all = 0); block p
__global__ void gms_reduce(GmresSeg g, int all) {
    const int p = blockIdx.x;
    const int kn = all ? *g.iter + 1 : 1;
    const int b0 = g.pblk[p], b1 = g.pblk[p + 1];
    for (int k = threadIdx.x; k < kn; k += blockDim.x) {
        double s = 0.0;
        for (int b = b0; b < b1; ++b) s += g.part[(size_t)b * (g.m + 1) + k];
        g.hsum[(size_t)p * (g.m + 1) + k] = s;
    }
}

// h = hsum of the block's problem; H(:, i) (=|+=) h (the problem's first
// block); w -= V h; then new dots (pass 0) or ||w||^2 partials (pass 1)
__global__ void gms_update(GmresSeg g, int pass) {
    extern __shared__ double gms_sm[];
    double *h = gms_sm;
    double *red = gms_sm + (g.m + 1);
    const int i = *g.iter, p = g.bprob[blockIdx.x];
    if (g.conv[p] != -1) return;
    for (int k = threadIdx.x; k <= i; k += blockDim.x) h[k] = g.hsum[(size_t)p * (g.m + 1) + k];
    __syncthreads();
    if (blockIdx.x == g.pblk[p])
        for (int k = threadIdx.x; k <= i; k += blockDim.x) {
            double *Hk = g.H + gms_h(g, p, k, i);
            *Hk = pass == 0 ? h[k] : *Hk + h[k];
        }
    const int64_t r0 = g.brow[blockIdx.x], r1 = g.brow[blockIdx.x + 1];
    for (int64_t t = r0 + threadIdx.x; t < r1; t += GMS_THREADS) {
        double v = g.w[t];
        for (int k = 0; k <= i; ++k) v -= g.V[(size_t)k * g.Ntot + t] * h[k];
        g.w[t] = v;
    }
    __syncthreads();
    if (pass == 0) gms_block_dots(g, g.V, g.w, i + 1, red, g.part);
    else gms_block_dots(g, g.w, g.w, 1, red, g.part);
}

// H(i+1, i) = ||w||; V[:, i+1] = vcur = w / ||w|| (a zero segment stays zero)
__global__ void gms_normalise(GmresSeg g) {
    const int i = *g.iter, p = g.bprob[blockIdx.x];
    if (g.conv[p] != -1) return;
    const double hn = sqrt(g.hsum[(size_t)p * (g.m + 1)]);
    if (blockIdx.x == g.pblk[p] && threadIdx.x == 0) g.H[gms_h(g, p, i + 1, i)] = hn;
    const double ih = hn > 0.0 ? 1.0 / hn : 0.0;
    double *Vn = g.V + (size_t)(i + 1) * g.Ntot;
    const int64_t r0 = g.brow[blockIdx.x], r1 = g.brow[blockIdx.x + 1];
    for (int64_t t = r0 + threadIdx.x; t < r1; t += GMS_THREADS) {
        const double v = ih * g.w[t];
        Vn[t] = v;
        g.vcur[t] = v;
    }
}

__device__ __forceinline__ void gms_apply(double &dx, double &dy, double cs, double sn) {
    const double temp = __dadd_rn(__dmul_rn(cs, dx), __dmul_rn(sn, dy));
    dy = __dadd_rn(__dmul_rn(-sn, dx), __dmul_rn(cs, dy));
    dx = temp;
}

// Givens rotations of column i for every running problem
// (*/codes/gmres.hpp:30-75,156-162); one CTA, problems strided over threads.
__global__ void gms_givens(GmresSeg g, double tol) {
    const int i = *g.iter;
    for (int p = threadIdx.x; p < g.P; p += blockDim.x) {
        if (g.conv[p] != -1) continue;
        double *cs = g.cs + (size_t)p * (g.m + 1), *sn = g.sn + (size_t)p * (g.m + 1), *s = g.s + (size_t)p * (g.m + 1);
        double *Hc = g.H + gms_h(g, p, 0, i);
        for (int k = 0; k < i; ++k) gms_apply(Hc[k], Hc[k + 1], cs[k], sn[k]);
        double dx = Hc[i], dy = Hc[i + 1], c_, s_;
        if (dy == 0.0) { c_ = 1.0; s_ = 0.0; }
        else if (fabs(dy) > fabs(dx)) {
            const double temp = dx / dy;
            s_ = 1.0 / sqrt(1.0 + temp * temp);
            c_ = temp * s_;
        } else {
            const double temp = dy / dx;
            c_ = 1.0 / sqrt(1.0 + temp * temp);
            s_ = temp * c_;
        }
        cs[i] = c_;
        sn[i] = s_;
        gms_apply(Hc[i], Hc[i + 1], c_, s_);
        gms_apply(s[i], s[i + 1], c_, s_);
        const double resid = fabs(s[i + 1]) / g.normb[p];
        g.resid[p] = resid;
        if (resid < tol) g.conv[p] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0 && i + 1 < g.m) *g.iter = i + 1;
}

// w = b - Ax (Ax == NULL: w = b) and per-block partials of ||w||^2
__global__ void gms_resid(GmresSeg g, const double *__restrict__ b, const double *__restrict__ Ax) {
    __shared__ double red[4 * GMS_WARPS];
    const int64_t r0 = g.brow[blockIdx.x], r1 = g.brow[blockIdx.x + 1];
    for (int64_t t = r0 + threadIdx.x; t < r1; t += GMS_THREADS) g.w[t] = Ax ? b[t] - Ax[t] : b[t];
    __syncthreads();
    gms_block_dots(g, g.w, g.w, 1, red, g.part);
}
__global__ void gms_colnorm_part(GmresSeg g, const double *__restrict__ v) {
    __shared__ double red[4 * GMS_WARPS];
    gms_block_dots(g, v, v, 1, red, g.part);
}
// out[p] = sqrt(sum of problem p's partials); zero_to_one: a zero norm becomes 1
__global__ void gms_colnorm_fin(GmresSeg g, double *out, int zero_to_one) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < g.P; p += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = g.pblk[p]; b < g.pblk[p + 1]; ++b) s += g.part[(size_t)b * (g.m + 1)];
        s = sqrt(s);
        out[p] = (zero_to_one && s == 0.0) ? 1.0 : s;
    }
}
// beta = ||w|| (hsum); V[:, 0] = vcur = w / beta; s = beta e1; per-problem state
__global__ void gms_start_fin(GmresSeg g, double tol) {
    const int p = g.bprob[blockIdx.x];
    const double beta = sqrt(g.hsum[(size_t)p * (g.m + 1)]);
    if (blockIdx.x == g.pblk[p] && threadIdx.x == 0) {
        double *cs = g.cs + (size_t)p * (g.m + 1), *sn = g.sn + (size_t)p * (g.m + 1), *s = g.s + (size_t)p * (g.m + 1);
        for (int k = 0; k <= g.m; ++k) { s[k] = 0.0; cs[k] = 0.0; sn[k] = 0.0; }
        s[0] = beta;
        const double r = beta / g.normb[p];
        g.resid[p] = r;
        g.conv[p] = r <= tol ? -2 : -1;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        g.iter[0] = 0;
        g.iter[1] = 0;
    }
    const double ib = beta > 0.0 ? 1.0 / beta : 0.0;
    const int64_t r0 = g.brow[blockIdx.x], r1 = g.brow[blockIdx.x + 1];
    for (int64_t t = r0 + threadIdx.x; t < r1; t += GMS_THREADS) {
        const double v = g.w[t] * ib;
        g.V[t] = v;
        g.vcur[t] = v;
    }
}
// y_p = H_p(0:k, 0:k) \ s_p(0:k), k = the problem's last Arnoldi column
// (converged: conv; running: last; converged at the start: none), in the
// reference's back-substitution order (*/codes/gmres.hpp:77-90)
__global__ void gms_backsolve(GmresSeg g, int last) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < g.P; p += gridDim.x * blockDim.x) {
        const int cv = g.conv[p];
        const int k = cv >= 0 ? cv : (cv == -1 ? last : -1);
        const double *s = g.s + (size_t)p * (g.m + 1);
        double *y = g.y + (size_t)p * (g.m + 1);
        for (int j = 0; j <= g.m; ++j) y[j] = j <= k ? s[j] : 0.0;
        for (int i = k; i >= 0; --i) {
            const double yi = y[i] / g.H[gms_h(g, p, i, i)];
            y[i] = yi;
            for (int j = i - 1; j >= 0; --j) y[j] -= g.H[gms_h(g, p, j, i)] * yi;
        }
    }
}
// x += V y over the Arnoldi columns of each row's problem (0..k_p: its
// converged column, `last` while running, none when converged at the start;
// later columns of a converged problem are never written and never read)
__global__ void gms_xupdate(GmresSeg g, double *__restrict__ x, int last) {
    const int p = g.bprob[blockIdx.x];
    const int cv = g.conv[p];
    const int kp = cv >= 0 ? cv : (cv == -1 ? last : -1);
    const double *y = g.y + (size_t)p * (g.m + 1);
    const int64_t r0 = g.brow[blockIdx.x], r1 = g.brow[blockIdx.x + 1];
    for (int64_t t = r0 + threadIdx.x; t < r1; t += GMS_THREADS) {
        double v = x[t];
        for (int j = 0; j <= kp; ++j) v += g.V[(size_t)j * g.Ntot + t] * y[j];
        x[t] = v;
    }
}
// Loop condition of the graph-captured segmented Arnoldi step.
__global__ void gms_loop_cond(GmresSeg g, cudaGraphConditionalHandle hnd) {
    const int c = ++g.iter[1];
    int running = 0;
    for (int p = 0; p < g.P; ++p) running |= g.conv[p] == -1;
    cudaGraphSetConditional(hnd, (running && c < g.m) ? 1u : 0u);
}

__global__ void gather64_kernel(const double *__restrict__ x, double *__restrict__ y, const int64_t *__restrict__ idx,
                                int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        y[t] = x[idx[t]];
}
__global__ void scatter64_kernel(const double *__restrict__ x, double *__restrict__ y, const int64_t *__restrict__ idx,
                                 int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        y[idx[t]] = x[t];
}
cudaError_t launch_gather64(const double *x, double *y, const int64_t *idx, int64_t n, cudaStream_t st) {
    gather64_kernel<<<1216, 256, 0, st>>>(x, y, idx, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_scatter64(const double *x, double *y, const int64_t *idx, int64_t n, cudaStream_t st) {
    scatter64_kernel<<<1216, 256, 0, st>>>(x, y, idx, n);
    count_launch();
    return cudaGetLastError();
}

bool gms_attr(const GmresSeg &g) { return ((size_t)(g.m + 1) + 4 * GMS_WARPS) * 8 <= 48 * 1024; }

static unsigned gms_pgrid(const GmresSeg &g) { return (unsigned)((g.P + GMS_THREADS - 1) / GMS_THREADS); }

cudaError_t gms_norms(const GmresSeg &g, const double *v, double *out, int zero_to_one, cudaStream_t st) {
    gms_colnorm_part<<<g.nblk, GMS_THREADS, 0, st>>>(g, v);
    gms_colnorm_fin<<<gms_pgrid(g), GMS_THREADS, 0, st>>>(g, out, zero_to_one);
    count_launch(2);
    return cudaGetLastError();
}
cudaError_t gms_start(const GmresSeg &g, const double *b, const double *Ax, double tol, cudaStream_t st) {
    gms_resid<<<g.nblk, GMS_THREADS, 0, st>>>(g, b, Ax);
    gms_reduce<<<g.P, 32, 0, st>>>(g, 0);
    gms_start_fin<<<g.nblk, GMS_THREADS, 0, st>>>(g, tol);
    count_launch(3);
    return cudaGetLastError();
}
cudaError_t gms_arnoldi(const GmresSeg &g, double tol, cudaStream_t st) {
    const size_t smu = ((size_t)(g.m + 1) + 4 * GMS_WARPS) * 8;
    gms_dots<<<g.nblk, GMS_THREADS, 0, st>>>(g);
    gms_reduce<<<g.P, 128, 0, st>>>(g, 1);
    gms_update<<<g.nblk, GMS_THREADS, smu, st>>>(g, 0);
    gms_reduce<<<g.P, 128, 0, st>>>(g, 1);
    gms_update<<<g.nblk, GMS_THREADS, smu, st>>>(g, 1);
    gms_reduce<<<g.P, 32, 0, st>>>(g, 0);
    gms_normalise<<<g.nblk, GMS_THREADS, 0, st>>>(g);
    gms_givens<<<1, 1024, 0, st>>>(g, tol);
    count_launch(8);
    return cudaGetLastError();
}
cudaError_t gms_loop(const GmresSeg &g, cudaGraphConditionalHandle hnd, cudaStream_t st) {
    gms_loop_cond<<<1, 1, 0, st>>>(g, hnd);
    count_launch();
    return cudaGetLastError();
}
cudaError_t gms_finish(const GmresSeg &g, double *x, int last, int kmax, cudaStream_t st) {
    gms_backsolve<<<gms_pgrid(g), GMS_THREADS, 0, st>>>(g, last);
    count_launch();
    if (kmax >= 0) {
        gms_xupdate<<<g.nblk, GMS_THREADS, 0, st>>>(g, x, last);
        count_launch();
    }
    return cudaGetLastError();
}

}  // namespace h2w
