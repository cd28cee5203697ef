// Lockstep GMRES over RP systems (the reference's unrestarted GMRES,
// */codes/gmres.hpp:92-200, per column): CGS2 Arnoldi, Givens rotations,
// per-column convergence; one column's numbers never mix with another's.
//
// The Krylov vectors are interleaved blocks (element (t, c) at t*RP + c) of
// type T: double for FP64 solves, float for the inner solves of the
// mixed-precision refinement, whose operator is FP32 anyway. GB300 runs FP64
// arithmetic at 1/64 of the FP32 rate, so double sweeps that multiply every
// element are bounded by the FP64 pipe, not by HBM; the float basis halves
// the bytes and moves the arithmetic to the FP32 pipes. Dots and norms are
// summed per thread in T (double when either operand is double), per block in
// double, and over blocks in a fixed order (deterministic). The number of
// basis vectors a sweep handles (1-4) is a template parameter, so no
// multiply-add is issued for an empty slot.
#include <algorithm>
#include <type_traits>

#include "kernels.cuh"

namespace h2w {

constexpr int GMB_THREADS = 256;
constexpr int GMB_RED = 1024;

template <class TA, class TB> struct GmbAcc { using type = double; };
template <> struct GmbAcc<float, float> { using type = float; };

template <class T>
__device__ __forceinline__ void gmb_rows(const GmbT<T> &g, int64_t &r0, int64_t &r1) {
    const int64_t chunk = (g.N + g.nblk - 1) / g.nblk;
    r0 = (int64_t)blockIdx.x * chunk;
    r1 = r0 + chunk < g.N ? r0 + chunk : g.N;
}
template <class T>
__device__ __forceinline__ size_t gmb_h(const GmbT<T> &g, int c, int row, int col) {
    return ((size_t)c * g.m + col) * (g.m + 1) + row;
}

// out[(blk*(m+1) + j)*rp + c] = this block's sum of acc[j] over its threads, j < nout
template <class T, class Acc>
__device__ __forceinline__ void gmb_block_sum(const GmbT<T> &g, const Acc (&acc)[4], int nout, double *red,
                                              double *out) {
    const int rp = g.rp, c = threadIdx.x % rp, rl = threadIdx.x / rp, RL = GMB_THREADS / rp;
#pragma unroll
    for (int j = 0; j < 4; ++j) red[(j * RL + rl) * rp + c] = (double)acc[j];
    __syncthreads();
    if (rl == 0)
        for (int j = 0; j < nout; ++j) {
            double s2 = 0.0;
            for (int q = 0; q < RL; ++q) s2 += red[(j * RL + q) * rp + c];
            out[((size_t)blockIdx.x * (g.m + 1) + j) * rp + c] = s2;
        }
    __syncthreads();
}

// acc[j] += sum over this thread's rows of a_j[t, c] * b[t, c], j < KC
// (a_j = a + j*stride); four rows per iteration
template <int KC, class TA, class TB, class Acc>
__device__ __forceinline__ void gmb_dots_sweep(const TA *__restrict__ a, size_t stride, const TB *__restrict__ b,
                                               int64_t r0, int64_t r1, int rp, Acc (&acc)[4]) {
    const int c = threadIdx.x % rp, rl = threadIdx.x / rp, RL = GMB_THREADS / rp;
    const int64_t step = (int64_t)RL * rp;
    int64_t t = r0 + rl;
    for (; t + 3 * RL < r1; t += 4 * RL) {
        const int64_t o = t * rp + c;
        Acc bv[4], av[4][KC];
#pragma unroll
        for (int u = 0; u < 4; ++u) bv[u] = (Acc)b[o + u * step];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < KC; ++j) av[u][j] = (Acc)a[j * stride + o + u * step];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < KC; ++j) acc[j] += av[u][j] * bv[u];
    }
    for (; t < r1; t += RL) {
        const Acc bv = (Acc)b[t * rp + c];
#pragma unroll
        for (int j = 0; j < KC; ++j) acc[j] += (Acc)a[j * stride + t * rp + c] * bv;
    }
}

// block partials of a_k . b, k = 0..kn-1 (a_k = a + k*N*rp), four a_k per
// sweep over the rows (b read once per four); red: 4*GMB_THREADS
template <class T, class TA, class TB>
__device__ void gmb_block_dots(const GmbT<T> &g, const TA *a, const TB *b, int kn, int64_t r0, int64_t r1,
                               double *red, double *out) {
    using Acc = typename GmbAcc<TA, TB>::type;
    const size_t stride = (size_t)g.N * g.rp;
    for (int k0 = 0; k0 < kn; k0 += 4) {
        const int kc = kn - k0 < 4 ? kn - k0 : 4;
        const TA *ak = a + (size_t)k0 * stride;
        Acc acc[4] = {Acc(0), Acc(0), Acc(0), Acc(0)};
        switch (kc) {
        case 1: gmb_dots_sweep<1>(ak, stride, b, r0, r1, g.rp, acc); break;
        case 2: gmb_dots_sweep<2>(ak, stride, b, r0, r1, g.rp, acc); break;
        case 3: gmb_dots_sweep<3>(ak, stride, b, r0, r1, g.rp, acc); break;
        default: gmb_dots_sweep<4>(ak, stride, b, r0, r1, g.rp, acc); break;
        }
        gmb_block_sum(g, acc, kc, red, out + (size_t)k0 * g.rp);
    }
}

template <class T>
__global__ void __launch_bounds__(GMB_THREADS, 3) gmb_dots(GmbT<T> g) {
    __shared__ double red[4 * GMB_THREADS];
    int64_t r0, r1;
    gmb_rows(g, r0, r1);
    gmb_block_dots(g, (const T *)g.V, (const T *)g.w, *g.iter + 1, r0, r1, red, g.part);
}

// sum over blocks of part[(b*(m+1) + k)*rp + c], in a fixed order: 1024 / rp
// lanes per column split the blocks (four loads in flight each), then meet in
// shared memory; valid in the threads with threadIdx.x < rp
template <class T>
__device__ __forceinline__ double gmb_sum_parts(const GmbT<T> &g, int k, double *red) {
    const int rp = g.rp, c = threadIdx.x % rp, bl = threadIdx.x / rp, BL = GMB_RED / rp;
    const size_t st = (size_t)(g.m + 1) * rp;
    const double *p = g.part + (size_t)k * rp + c;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int b = bl;
    for (; b + 3 * BL < g.nblk; b += 4 * BL) {
        s0 += p[(size_t)b * st];
        s1 += p[(size_t)(b + BL) * st];
        s2 += p[(size_t)(b + 2 * BL) * st];
        s3 += p[(size_t)(b + 3 * BL) * st];
    }
    for (; b < g.nblk; b += BL) s0 += p[(size_t)b * st];
    red[threadIdx.x] = (s0 + s1) + (s2 + s3);
    __syncthreads();
    double s = 0.0;
    if (bl == 0)
        for (int q = 0; q < BL; ++q) s += red[q * rp + c];
    return s;
}
// hsum[k*rp + c] for k <= i (all = 1) or k = 0 (all = 0); block k
template <class T>
__global__ void gmb_reduce(GmbT<T> g, int all) {
    __shared__ double red[GMB_RED];
    const int kn = all ? *g.iter + 1 : 1;
    const int k = blockIdx.x;
    if (k >= kn) return;
    const double s = gmb_sum_parts(g, k, red);
    if (threadIdx.x < g.rp) g.hsum[(size_t)k * g.rp + threadIdx.x] = s;
}

// w -= sum_j V_j h_j (j < KC) over this thread's rows; FUSE 1: acc[j] += V_j . w
// (the new w), FUSE 2: acc[0] += w . w, from the values already in registers
template <int KC, int FUSE, class T>
__device__ __forceinline__ void gmb_update_sweep(T *__restrict__ w, const T *__restrict__ Vk, size_t stride,
                                                 const T (&hk)[4], int64_t r0, int64_t r1, int rp, T (&acc)[4]) {
    const int c = threadIdx.x % rp, rl = threadIdx.x / rp, RL = GMB_THREADS / rp;
    const int64_t step = (int64_t)RL * rp;
    int64_t t = r0 + rl;
    for (; t + 3 * RL < r1; t += 4 * RL) {
        const int64_t o = t * rp + c;
        T wv[4], vk[4][KC];
#pragma unroll
        for (int u = 0; u < 4; ++u) wv[u] = w[o + u * step];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < KC; ++j) vk[u][j] = Vk[j * stride + o + u * step];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            T v = wv[u];
#pragma unroll
            for (int j = 0; j < KC; ++j) v -= vk[u][j] * hk[j];
            w[o + u * step] = v;
            if (FUSE == 1) {
#pragma unroll
                for (int j = 0; j < KC; ++j) acc[j] += vk[u][j] * v;
            } else if (FUSE == 2) {
                acc[0] += v * v;
            }
        }
    }
    for (; t < r1; t += RL) {
        const int64_t o = t * rp + c;
        T vk[KC];
#pragma unroll
        for (int j = 0; j < KC; ++j) vk[j] = Vk[j * stride + o];
        T v = w[o];
#pragma unroll
        for (int j = 0; j < KC; ++j) v -= vk[j] * hk[j];
        w[o] = v;
        if (FUSE == 1) {
#pragma unroll
            for (int j = 0; j < KC; ++j) acc[j] += vk[j] * v;
        } else if (FUSE == 2) {
            acc[0] += v * v;
        }
    }
}

// h = hsum; H(:, i) (=|+=) h; w -= V h; then new dots (pass 0) or ||w||^2 partials (pass 1).
// With at most four basis vectors the dots are formed in the same sweep from
// the basis values already in registers (the basis is read once); with more,
// w is updated four basis vectors at a time and a second sweep forms the dots.
template <class T>
__global__ void __launch_bounds__(GMB_THREADS, 3) gmb_update(GmbT<T> g, int pass) {
    __shared__ double red[4 * GMB_THREADS];
    const int i = *g.iter, rp = g.rp, kn = i + 1;
    if (blockIdx.x == 0)
        for (int e = threadIdx.x; e < kn * rp; e += blockDim.x) {
            const int k = e / rp, c = e % rp;
            double *Hk = g.H + gmb_h(g, c, k, i);
            *Hk = pass == 0 ? g.hsum[e] : *Hk + g.hsum[e];
        }
    int64_t r0, r1;
    gmb_rows(g, r0, r1);
    const int c = threadIdx.x % rp;
    const size_t stride = (size_t)g.N * rp;
    for (int k0 = 0; k0 < kn; k0 += 4) {
        const int kc = kn - k0 < 4 ? kn - k0 : 4;
        const T *Vk = g.V + (size_t)k0 * stride;
        T hk[4], acc[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int j = 0; j < 4; ++j) hk[j] = j < kc ? (T)g.hsum[(size_t)(k0 + j) * rp + c] : T(0);
        if (kn <= 4) {  // one sweep with the dots (pass 0) or the norm (pass 1) fused
            if (pass == 0) {
                switch (kc) {
                case 1: gmb_update_sweep<1, 1>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                case 2: gmb_update_sweep<2, 1>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                case 3: gmb_update_sweep<3, 1>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                default: gmb_update_sweep<4, 1>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                }
            } else {
                switch (kc) {
                case 1: gmb_update_sweep<1, 2>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                case 2: gmb_update_sweep<2, 2>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                case 3: gmb_update_sweep<3, 2>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                default: gmb_update_sweep<4, 2>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
                }
            }
            gmb_block_sum(g, acc, pass == 0 ? kn : 1, red, g.part);
            return;
        }
        switch (kc) {
        case 1: gmb_update_sweep<1, 0>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
        case 2: gmb_update_sweep<2, 0>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
        case 3: gmb_update_sweep<3, 0>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
        default: gmb_update_sweep<4, 0>(g.w, Vk, stride, hk, r0, r1, rp, acc); break;
        }
    }
    __syncthreads();
    if (pass == 0) gmb_block_dots(g, (const T *)g.V, (const T *)g.w, kn, r0, r1, red, g.part);
    else gmb_block_dots(g, (const T *)g.w, (const T *)g.w, 1, r0, r1, red, g.part);
}

// H(i+1, i) = ||w||; V[:, i+1] = vcur = w / ||w|| (a zero column stays zero)
template <class T>
__global__ void __launch_bounds__(GMB_THREADS, 3) gmb_normalise(GmbT<T> g) {
    const int i = *g.iter, rp = g.rp;
    const int c = threadIdx.x % rp, rl = threadIdx.x / rp, RL = GMB_THREADS / rp;
    const double hn = sqrt(g.hsum[c]);
    if (blockIdx.x == 0 && rl == 0) g.H[gmb_h(g, c, i + 1, i)] = hn;
    const T ih = hn > 0.0 ? (T)(1.0 / hn) : T(0);
    int64_t r0, r1;
    gmb_rows(g, r0, r1);
    T *__restrict__ Vn = g.V + (size_t)(i + 1) * g.N * rp;
    T *__restrict__ vc = g.vcur;
    const T *__restrict__ wr = g.w;
    const int64_t step = (int64_t)RL * rp;
    int64_t t = r0 + rl;
    for (; t + 3 * RL < r1; t += 4 * RL) {
        const int64_t o = t * rp + c;
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = ih * wr[o + u * step];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            Vn[o + u * step] = v[u];
            vc[o + u * step] = v[u];
        }
    }
    for (; t < r1; t += RL) {
        const T v = ih * wr[t * rp + c];
        Vn[t * rp + c] = v;
        vc[t * rp + c] = v;
    }
}

__device__ __forceinline__ void gmb_apply(double &dx, double &dy, double cs, double sn) {
    const double temp = __dadd_rn(__dmul_rn(cs, dx), __dmul_rn(sn, dy));
    dy = __dadd_rn(__dmul_rn(-sn, dx), __dmul_rn(cs, dy));
    dx = temp;
}

// Givens rotations of column i for every running system
// (*/codes/gmres.hpp:30-75,156-162); one thread per column.
template <class T>
__global__ void gmb_givens(GmbT<T> g) {
    const int i = *g.iter, c = threadIdx.x;
    const double tol = *g.tolp;
    if (c < g.rp && g.conv[c] == -1) {
        double *cs = g.cs + (size_t)c * (g.m + 1), *sn = g.sn + (size_t)c * (g.m + 1), *s = g.s + (size_t)c * (g.m + 1);
        double *Hc = g.H + gmb_h(g, c, 0, i);
        for (int k = 0; k < i; ++k) gmb_apply(Hc[k], Hc[k + 1], cs[k], sn[k]);
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
        gmb_apply(Hc[i], Hc[i + 1], c_, s_);
        gmb_apply(s[i], s[i + 1], c_, s_);
        const double resid = fabs(s[i + 1]) / g.normb[c];
        g.resid[c] = resid;
        if (resid < tol) g.conv[c] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0 && i + 1 < g.m) *g.iter = i + 1;
}

// w = b - Ax (Ax == NULL: w = b), stored as T, and block partials of ||w||^2
template <class T>
__global__ void __launch_bounds__(GMB_THREADS, 3)
    gmb_resid(GmbT<T> g, const double *__restrict__ b, const double *__restrict__ Ax) {
    __shared__ double red[4 * GMB_THREADS];
    int64_t r0, r1;
    gmb_rows(g, r0, r1);
    const int rp = g.rp, c = threadIdx.x % rp, rl = threadIdx.x / rp, RL = GMB_THREADS / rp;
    T acc[4] = {T(0), T(0), T(0), T(0)};
    const int64_t step = (int64_t)RL * rp;
    int64_t t = r0 + rl;
    for (; t + 3 * RL < r1; t += 4 * RL) {  // four rows per iteration: the loads of all four in flight
        const int64_t o = t * rp + c;
        double bv[4], av[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            bv[u] = b[o + u * step];
            av[u] = Ax ? Ax[o + u * step] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const T v = (T)(Ax ? bv[u] - av[u] : bv[u]);
            g.w[o + u * step] = v;
            acc[0] += v * v;
        }
    }
    for (; t < r1; t += RL) {
        const T v = (T)(Ax ? b[t * rp + c] - Ax[t * rp + c] : b[t * rp + c]);
        g.w[t * rp + c] = v;
        acc[0] += v * v;
    }
    gmb_block_sum(g, acc, 1, red, g.part);
}
// block partials of ||v[:, c]||^2 (v double)
template <class T>
__global__ void __launch_bounds__(GMB_THREADS, 3) gmb_colnorm_part(GmbT<T> g, const double *__restrict__ v) {
    __shared__ double red[4 * GMB_THREADS];
    int64_t r0, r1;
    gmb_rows(g, r0, r1);
    gmb_block_dots(g, v, v, 1, r0, r1, red, g.part);
}
// out[c] = sqrt(sum of the partials); zero_to_one: a zero norm becomes 1
template <class T>
__global__ void gmb_colnorm_fin(GmbT<T> g, double *out, int zero_to_one) {
    __shared__ double red[GMB_RED];
    const double s = sqrt(gmb_sum_parts(g, 0, red));
    if (threadIdx.x < g.rp) out[threadIdx.x] = (zero_to_one && s == 0.0) ? 1.0 : s;
}
// beta = ||w|| (hsum); V[:, 0] = vcur = w / beta; s = beta e1; per-column state.
// set_normb (x0 = 0, where w = b): ||b|| = beta (a zero norm becomes 1)
template <class T>
__global__ void __launch_bounds__(GMB_THREADS, 3) gmb_start_fin(GmbT<T> g, double tol, int set_normb) {
    const int rp = g.rp, c = threadIdx.x % rp, rl = threadIdx.x / rp, RL = GMB_THREADS / rp;
    const double beta = sqrt(g.hsum[c]);
    if (blockIdx.x == 0 && rl == 0) {
        if (set_normb) g.normb[c] = beta == 0.0 ? 1.0 : beta;
        double *cs = g.cs + (size_t)c * (g.m + 1), *sn = g.sn + (size_t)c * (g.m + 1), *s = g.s + (size_t)c * (g.m + 1);
        for (int k = 0; k <= g.m; ++k) { s[k] = 0.0; cs[k] = 0.0; sn[k] = 0.0; }
        s[0] = beta;
        const double r = beta / g.normb[c];
        g.resid[c] = r;
        g.conv[c] = c >= g.nrhs ? -3 : (r <= tol ? -2 : -1);
        if (c == 0) {
            g.iter[0] = 0;
            g.iter[1] = 0;  // Arnoldi steps taken (graph loop counter)
        }
    }
    const T ib = beta > 0.0 ? (T)(1.0 / beta) : T(0);
    int64_t r0, r1;
    gmb_rows(g, r0, r1);
    const int64_t step = (int64_t)RL * rp;
    int64_t t = r0 + rl;
    for (; t + 3 * RL < r1; t += 4 * RL) {
        const int64_t o = t * rp + c;
        T v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = g.w[o + u * step] * ib;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            g.V[o + u * step] = v[u];
            g.vcur[o + u * step] = v[u];
        }
    }
    for (; t < r1; t += RL) {
        const T v = g.w[t * rp + c] * ib;
        g.V[t * rp + c] = v;
        g.vcur[t * rp + c] = v;
    }
}
// y_c = H_c(0:k, 0:k) \ s_c(0:k), k = the column's last Arnoldi index
// (converged: conv; still running: last; converged at the start / padding: none),
// in the reference's back-substitution order (*/codes/gmres.hpp:77-90). Also
// z_c = beta e1 - Hbar y = Q^T (s_{k+1} e_{k+1}): the rotations undone on the
// last rotated residual entry (padding: z = 0).
template <class T>
__global__ void gmb_backsolve(GmbT<T> g, int last) {
    const int c = threadIdx.x;
    if (c >= g.rp) return;
    const int cv = g.conv[c];
    const int k = cv >= 0 ? cv : (cv == -1 ? last : -1);
    const double *s = g.s + (size_t)c * (g.m + 1);
    for (int j = 0; j <= g.m; ++j) g.y[(size_t)j * g.rp + c] = j <= k ? s[j] : 0.0;
    for (int i = k; i >= 0; --i) {
        double *y = g.y;
        const double yi = y[(size_t)i * g.rp + c] / g.H[gmb_h(g, c, i, i)];
        y[(size_t)i * g.rp + c] = yi;
        for (int j = i - 1; j >= 0; --j) y[(size_t)j * g.rp + c] -= g.H[gmb_h(g, c, j, i)] * yi;
    }
    double *z = g.z;
    const double *cs = g.cs + (size_t)c * (g.m + 1), *sn = g.sn + (size_t)c * (g.m + 1);
    for (int j = 0; j <= g.m + 1; ++j) z[(size_t)j * g.rp + c] = 0.0;
    if (cv == -3 || k + 1 > g.m) return;
    z[(size_t)(k + 1) * g.rp + c] = s[k + 1];
    for (int i = k; i >= 0; --i) {  // (z_i, z_{i+1}) <- G_i^T (z_i, z_{i+1})
        const double a = z[(size_t)i * g.rp + c], b = z[(size_t)(i + 1) * g.rp + c];
        z[(size_t)i * g.rp + c] = cs[i] * a - sn[i] * b;
        z[(size_t)(i + 1) * g.rp + c] = sn[i] * a + cs[i] * b;
    }
}
// x += V y over Arnoldi columns 0..kmax (x double; with a float basis the
// combination V y is formed in float and added in double); launched with
// about one element per thread (GMB_XU_BLOCKS)
template <class T>
__global__ void __launch_bounds__(GMB_THREADS) gmb_xupdate(GmbT<T> g, double *__restrict__ x, int kmax) {
    const int rp = g.rp;
    const size_t stride = (size_t)g.N * rp;
    const int64_t tot = g.N * rp;
    const T *__restrict__ V = g.V;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % rp);
        if constexpr (std::is_same<T, float>::value) {
            float v = 0.f;
            for (int j = 0; j <= kmax; ++j) v += V[j * stride + e] * (float)g.y[(size_t)j * rp + c];
            x[e] += (double)v;
        } else {
            double v = x[e];
            for (int j = 0; j <= kmax; ++j) v += V[j * stride + e] * g.y[(size_t)j * rp + c];
            x[e] = v;
        }
    }
}

// rout = (rin - T(rin)) + sum_{j <= jmax} V_j z_j: the residual of the solved
// system rin - A d (the right-hand side was rin rounded to T), one element per thread
template <class T>
__global__ void __launch_bounds__(GMB_THREADS)
    gmb_resvec(GmbT<T> g, const double *__restrict__ rin, double *__restrict__ rout, int jmax) {
    const int rp = g.rp;
    const size_t stride = (size_t)g.N * rp;
    const int64_t tot = g.N * rp;
    const T *__restrict__ V = g.V;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % rp);
        T v = T(0);
        for (int j = 0; j <= jmax; ++j) v += V[j * stride + e] * (T)g.z[(size_t)j * rp + c];
        const double r = rin[e];
        rout[e] = (r - (double)(T)r) + (double)v;
    }
}

// Loop condition of the graph-captured batched Arnoldi step: run another
// step while a column is still running and fewer than m steps were taken.
template <class T>
__global__ void gmb_loop_cond(GmbT<T> g, cudaGraphConditionalHandle hnd) {
    const int c = ++g.iter[1];
    int running = 0;
    for (int q = 0; q < g.nrhs; ++q) running |= g.conv[q] == -1;
    cudaGraphSetConditional(hnd, (running && c < g.m) ? 1u : 0u);
}

template <class T>
cudaError_t gmb_norms(const GmbT<T> &g, const double *v, double *out, int zero_to_one, cudaStream_t st) {
    gmb_colnorm_part<T><<<g.nblk, GMB_THREADS, 0, st>>>(g, v);
    gmb_colnorm_fin<T><<<1, GMB_RED, 0, st>>>(g, out, zero_to_one);
    count_launch(2);
    return cudaGetLastError();
}
template <class T>
cudaError_t gmb_start(const GmbT<T> &g, const double *b, const double *Ax, double tol, cudaStream_t st) {
    gmb_resid<T><<<g.nblk, GMB_THREADS, 0, st>>>(g, b, Ax);
    gmb_reduce<T><<<1, GMB_RED, 0, st>>>(g, 0);
    gmb_start_fin<T><<<g.nblk, GMB_THREADS, 0, st>>>(g, tol, Ax == nullptr ? 1 : 0);
    count_launch(3);
    return cudaGetLastError();
}
template <class T>
cudaError_t gmb_arnoldi(const GmbT<T> &g, cudaStream_t st) {
    gmb_dots<T><<<g.nblk, GMB_THREADS, 0, st>>>(g);
    gmb_reduce<T><<<g.m + 1, GMB_RED, 0, st>>>(g, 1);
    gmb_update<T><<<g.nblk, GMB_THREADS, 0, st>>>(g, 0);
    gmb_reduce<T><<<g.m + 1, GMB_RED, 0, st>>>(g, 1);
    gmb_update<T><<<g.nblk, GMB_THREADS, 0, st>>>(g, 1);
    gmb_reduce<T><<<1, GMB_RED, 0, st>>>(g, 0);
    gmb_normalise<T><<<g.nblk, GMB_THREADS, 0, st>>>(g);
    gmb_givens<T><<<1, 64, 0, st>>>(g);
    count_launch(8);
    return cudaGetLastError();
}
template <class T>
cudaError_t gmb_loop(const GmbT<T> &g, cudaGraphConditionalHandle hnd, cudaStream_t st) {
    gmb_loop_cond<T><<<1, 1, 0, st>>>(g, hnd);
    count_launch();
    return cudaGetLastError();
}
template <class T>
cudaError_t gmb_finish(const GmbT<T> &g, double *x, int last, int kmax, cudaStream_t st) {
    gmb_backsolve<T><<<1, 64, 0, st>>>(g, last);
    count_launch();
    if (kmax >= 0) {
        const int64_t tot = g.N * g.rp;
        const int nb = (int)std::min<int64_t>((tot + GMB_THREADS - 1) / GMB_THREADS, 152 * 64);
        gmb_xupdate<T><<<nb, GMB_THREADS, 0, st>>>(g, x, kmax);
        count_launch();
    }
    return cudaGetLastError();
}
template <class T>
cudaError_t gmb_residual(const GmbT<T> &g, const double *rin, double *rout, int jmax, cudaStream_t st) {
    if (jmax < 0 || jmax > g.m) return cudaErrorInvalidValue;
    const int64_t tot = g.N * g.rp;
    const int nb = (int)std::min<int64_t>((tot + GMB_THREADS - 1) / GMB_THREADS, 152 * 64);
    gmb_resvec<T><<<nb, GMB_THREADS, 0, st>>>(g, rin, rout, jmax);
    count_launch();
    return cudaGetLastError();
}

#define GMB_INSTANTIATE(T)                                                                                         \
    template cudaError_t gmb_norms<T>(const GmbT<T> &, const double *, double *, int, cudaStream_t);              \
    template cudaError_t gmb_start<T>(const GmbT<T> &, const double *, const double *, double, cudaStream_t);     \
    template cudaError_t gmb_arnoldi<T>(const GmbT<T> &, cudaStream_t);                                           \
    template cudaError_t gmb_loop<T>(const GmbT<T> &, cudaGraphConditionalHandle, cudaStream_t);                  \
    template cudaError_t gmb_finish<T>(const GmbT<T> &, double *, int, int, cudaStream_t);                       \
    template cudaError_t gmb_residual<T>(const GmbT<T> &, const double *, double *, int, cudaStream_t);
GMB_INSTANTIATE(double)
GMB_INSTANTIATE(float)
#undef GMB_INSTANTIATE

}  // namespace h2w
