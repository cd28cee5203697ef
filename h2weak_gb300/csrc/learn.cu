// Learned NCA proposals (sm_103a).
//
//  * learn_features   16 geometric features per candidate point of an NCA
//                     block (position in its own set's bounding box, relation
//                     to the other set, set sizes, dimension, kernel, tolerance)
//  * mlp_forward / mlp_grad / mlp_adam   the scoring network 16 -> 128 -> 128
//                     -> 1 (ReLU) with BF16-rounded weights and FP32
//                     accumulation: inference, the gradient of the weighted
//                     binary cross-entropy (forward recomputed per 64-point
//                     tile in shared memory), and the Adam update
//  * learn_propose    per block: rank estimate from the row scores, the
//                     top-scored rows (oversampled)
//  * learn_fill / learn_aca / learn_solve / learn_gram   the cross
//                     approximation: K(I, C) of the proposed rows over all SMs,
//                     the reference's ACA restricted to those rows on it
//                     (column pivots over every column, no new entries), K(R, J')
//                     for the chosen columns over all SMs, the LU of K(I', J'),
//                     U = K(R, J') R^-1 and V = L^-1 K(I', C), Gram matrices
//  * learn_test       the NCA's stopping test on the full block: one further
//                     ACA step (row pivot = argmax of the last residual column,
//                     column pivot = argmax of that residual row) and
//                     ||u|| ||v|| <= tol * normS (1D/codes/aca.hpp:363,404-409);
//                     an accepted block keeps that step's pivot, as the ACA
//                     would, a rejected one goes to the plain pivot search
#include <climits>
#include <cmath>

#include <cuda_bf16.h>

#include "entry.cuh"

namespace h2w {

constexpr int LT = 256;  // threads of the learned-NCA kernels

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ------------------------------------------------------------ features ---
__global__ void __launch_bounds__(LT)
    learn_features_kernel(const LearnProb *__restrict__ probs, const int32_t *__restrict__ idx, KParams kp,
                          int tol_pow, float *__restrict__ X, int rows_only) {
    __shared__ double part[LT][12];
    __shared__ double st[12];  // row: min[3] max[3]; col: min[3] max[3]
    __shared__ double cen[6];  // row centroid, col centroid
    const LearnProb pb = probs[blockIdx.x];
    const int d = kp.dim, tid = threadIdx.x;
    const int32_t *R = idx + pb.ri, *C = idx + pb.ci;
    for (int set = 0; set < 2; ++set) {
        const int32_t *P = set == 0 ? R : C;
        const int n = set == 0 ? pb.n1 : pb.n2;
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300}, sm[3] = {0.0, 0.0, 0.0};
        for (int t = tid; t < n; t += LT) {
            const double *q = kp.pts + (size_t)P[t] * d;
            for (int k = 0; k < d; ++k) {
                mn[k] = fmin(mn[k], q[k]);
                mx[k] = fmax(mx[k], q[k]);
                sm[k] += q[k];
            }
        }
        for (int k = 0; k < 3; ++k) {
            part[tid][k] = mn[k];
            part[tid][3 + k] = mx[k];
            part[tid][6 + k] = sm[k];
        }
        __syncthreads();
        if (tid < 9) {
            double v = tid < 3 ? 1e300 : (tid < 6 ? -1e300 : 0.0);
            for (int q = 0; q < LT; ++q) {
                const double w = part[q][tid];
                v = tid < 3 ? fmin(v, w) : (tid < 6 ? fmax(v, w) : v + w);
            }
            if (tid < 6) st[6 * set + tid] = v;
            else cen[3 * set + tid - 6] = n > 0 ? v / n : 0.0;
        }
        __syncthreads();
    }
    const float lg1 = log2f((float)pb.n1 + 1.f) / 16.f, lg2 = log2f((float)pb.n2 + 1.f) / 16.f;
    for (int e = tid; e < pb.n1 + (rows_only ? 0 : pb.n2); e += LT) {
        const bool row = e < pb.n1;
        const int set = row ? 0 : 1;
        const int gp = row ? R[e] : C[e - pb.n1];
        const double *q = kp.pts + (size_t)gp * d;
        double hw = 0.0, ctr[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < d; ++k) {
            ctr[k] = 0.5 * (st[6 * set + k] + st[6 * set + 3 + k]);
            hw = fmax(hw, 0.5 * (st[6 * set + 3 + k] - st[6 * set + k]));
        }
        hw = fmax(hw, 1e-12);
        double rel[3] = {0.0, 0.0, 0.0}, o[3] = {0.0, 0.0, 0.0};
        double rinf = 0.0, r2 = 0.0, o2 = 0.0, ro = 0.0;
        for (int k = 0; k < d; ++k) {
            rel[k] = (q[k] - ctr[k]) / hw;
            o[k] = (cen[3 * (1 - set) + k] - ctr[k]) / hw;
            rinf = fmax(rinf, fabs(rel[k]));
            r2 += rel[k] * rel[k];
            o2 += o[k] * o[k];
            ro += rel[k] * o[k];
        }
        const double on = sqrt(o2), rn = sqrt(r2);
        float *x = X + (size_t)(pb.xo + e) * LRN_F;
        x[0] = (float)rel[0];
        x[1] = (float)rel[1];
        x[2] = (float)rel[2];
        x[3] = (float)rinf;
        x[4] = (float)(rn / sqrt((double)d));
        x[5] = (float)(ro / (rn * on + 1e-30));
        x[6] = (float)log1p(on);
        x[7] = row ? 1.f : 0.f;
        x[8] = lg1;
        x[9] = lg2;
        x[10] = (float)d / 3.f;
        x[11] = (float)kp.choice;
        x[12] = (float)tol_pow / 16.f;
        x[13] = (float)(ro / (on + 1e-30));
        x[14] = row ? lg1 : lg2;
        x[15] = 1.f;
    }
}

cudaError_t launch_learn_features(const LearnProb *probs, int nprob, const int32_t *idx, const KParams &kp,
                                  int tol_pow, float *X, int rows_only, cudaStream_t st) {
    for (int b0 = 0; b0 < nprob; b0 += 65535) {
        const int nb = nprob - b0 < 65535 ? nprob - b0 : 65535;
        learn_features_kernel<<<nb, LT, 0, st>>>(probs + b0, idx, kp, tol_pow, X, rows_only);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// ----------------------------------------------------------------- MLP ---
constexpr int MT_P = 64;  // points per tile

struct MlpSmem {
    __nv_bfloat16 w1[LRN_F * LRN_H];
    __nv_bfloat16 w2[LRN_H * LRN_H];
    float w3[LRN_H], b1[LRN_H], b2[LRN_H];
    float x[MT_P * LRN_F];
    float h1[MT_P * LRN_H];
};

__device__ void mlp_load(MlpSmem &sm, const float *params) {
    for (int e = threadIdx.x; e < LRN_F * LRN_H; e += blockDim.x) sm.w1[e] = __float2bfloat16_rn(params[LRN_W1 + e]);
    for (int e = threadIdx.x; e < LRN_H * LRN_H; e += blockDim.x) sm.w2[e] = __float2bfloat16_rn(params[LRN_W2 + e]);
    for (int e = threadIdx.x; e < LRN_H; e += blockDim.x) {
        sm.w3[e] = bf16r(params[LRN_W3 + e]);
        sm.b1[e] = params[LRN_B1 + e];
        sm.b2[e] = params[LRN_B2 + e];
    }
}

// logits of points [p0, p0 + np): thread (u = tid & 127, pp = tid >> 7)
__global__ void __launch_bounds__(LT) mlp_forward_kernel(const float *__restrict__ params, const float *__restrict__ X,
                                                         int64_t n, float *__restrict__ out) {
    extern __shared__ __align__(16) unsigned char mlp_raw[];
    MlpSmem &sm = *reinterpret_cast<MlpSmem *>(mlp_raw);
    __shared__ float red[MT_P][4];
    mlp_load(sm, params);
    const float b3 = params[LRN_B3];
    const int tid = threadIdx.x, u = tid & (LRN_H - 1), pp = tid >> 7, w = (tid >> 5) & 3;
    for (int64_t p0 = (int64_t)blockIdx.x * MT_P; p0 < n; p0 += (int64_t)gridDim.x * MT_P) {
        const int np = n - p0 < MT_P ? (int)(n - p0) : MT_P;
        __syncthreads();
        for (int e = tid; e < MT_P * LRN_F; e += LT) sm.x[e] = e < np * LRN_F ? X[p0 * LRN_F + e] : 0.f;
        __syncthreads();
        for (int p = pp; p < MT_P; p += 2) {
            float a = sm.b1[u];
            for (int f = 0; f < LRN_F; ++f) a += sm.x[p * LRN_F + f] * __bfloat162float(sm.w1[f * LRN_H + u]);
            sm.h1[p * LRN_H + u] = fmaxf(a, 0.f);
        }
        __syncthreads();
        for (int p = pp; p < MT_P; p += 2) {
            float a = sm.b2[u];
            for (int j = 0; j < LRN_H; ++j) a += sm.h1[p * LRN_H + j] * __bfloat162float(sm.w2[j * LRN_H + u]);
            float c = fmaxf(a, 0.f) * sm.w3[u];
            for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
            if ((tid & 31) == 0) red[p][w] = c;
        }
        __syncthreads();
        if (tid < np) out[p0 + tid] = b3 + red[tid][0] + red[tid][1] + red[tid][2] + red[tid][3];
    }
}

cudaError_t launch_mlp_forward(const float *params, const float *X, int64_t n, float *logits, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(MlpSmem));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int64_t tiles = (n + MT_P - 1) / MT_P;
    const int grid = (int)(tiles < 4 * 152 ? tiles : 4 * 152);
    mlp_forward_kernel<<<grid, LT, sizeof(MlpSmem), st>>>(params, X, n, logits);
    count_launch();
    return cudaGetLastError();
}

// Gradient of mean_p w_p (softplus(z_p) - y_p z_p), w_p = pos_weight for
// y_p = 1, with respect to the parameters (the weights' BF16 values), summed
// into grads; loss accumulates the same mean.
struct MlpGradSmem {
    MlpSmem f;
    float h2[MT_P * LRN_H];   // ReLU outputs, then dL/dh2 (pre-activation)
    float dh1[MT_P * LRN_H];  // dL/dh1 (pre-activation)
    float dz[MT_P];
};

__global__ void __launch_bounds__(LT) mlp_grad_kernel(const float *__restrict__ params, const float *__restrict__ X,
                                                      const uint8_t *__restrict__ y, int64_t n, float pos_weight,
                                                      float *__restrict__ grads, float *__restrict__ loss) {
    extern __shared__ __align__(16) unsigned char mlp_raw[];
    MlpGradSmem &sm = *reinterpret_cast<MlpGradSmem *>(mlp_raw);
    __shared__ float red[MT_P][4];
    mlp_load(sm.f, params);
    const float b3 = params[LRN_B3];
    const int tid = threadIdx.x, u = tid & (LRN_H - 1), pp = tid >> 7, w = (tid >> 5) & 3;
    const float inv_n = 1.f / (float)n;
    for (int64_t p0 = (int64_t)blockIdx.x * MT_P; p0 < n; p0 += (int64_t)gridDim.x * MT_P) {
        const int np = n - p0 < MT_P ? (int)(n - p0) : MT_P;
        __syncthreads();
        for (int e = tid; e < MT_P * LRN_F; e += LT) sm.f.x[e] = e < np * LRN_F ? X[p0 * LRN_F + e] : 0.f;
        __syncthreads();
        for (int p = pp; p < MT_P; p += 2) {
            float a = sm.f.b1[u];
            for (int f = 0; f < LRN_F; ++f) a += sm.f.x[p * LRN_F + f] * __bfloat162float(sm.f.w1[f * LRN_H + u]);
            sm.f.h1[p * LRN_H + u] = fmaxf(a, 0.f);
        }
        __syncthreads();
        for (int p = pp; p < MT_P; p += 2) {
            float a = sm.f.b2[u];
            for (int j = 0; j < LRN_H; ++j) a += sm.f.h1[p * LRN_H + j] * __bfloat162float(sm.f.w2[j * LRN_H + u]);
            const float h = fmaxf(a, 0.f);
            sm.h2[p * LRN_H + u] = h;
            float c = h * sm.f.w3[u];
            for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
            if ((tid & 31) == 0) red[p][w] = c;
        }
        __syncthreads();
        if (tid < MT_P) {
            float dz = 0.f;
            if (tid < np) {
                const float z = b3 + red[tid][0] + red[tid][1] + red[tid][2] + red[tid][3];
                const float yy = y[p0 + tid] ? 1.f : 0.f;
                const float wt = yy > 0.f ? pos_weight : 1.f;
                const float sp = z > 0.f ? z + log1pf(expf(-z)) : log1pf(expf(z));
                atomicAdd(loss, wt * (sp - yy * z) * inv_n);
                const float sg = 1.f / (1.f + expf(-z));
                dz = wt * (sg - yy) * inv_n;
            }
            sm.dz[tid] = dz;
        }
        __syncthreads();
        // W3, b3
        {
            float g = 0.f;
            for (int p = pp; p < MT_P; p += 2) g += sm.dz[p] * sm.h2[p * LRN_H + u];
            atomicAdd(grads + LRN_W3 + u, g);
            if (tid == 0) {
                float gb = 0.f;
                for (int p = 0; p < MT_P; ++p) gb += sm.dz[p];
                atomicAdd(grads + LRN_B3, gb);
            }
        }
        __syncthreads();
        // dL/d(pre-activation of h2), in place
        for (int p = pp; p < MT_P; p += 2) {
            const float h = sm.h2[p * LRN_H + u];
            sm.h2[p * LRN_H + u] = h > 0.f ? sm.dz[p] * sm.f.w3[u] : 0.f;
        }
        __syncthreads();
        // W2 (j, u2) pairs strided over threads, b2
        for (int e = tid; e < LRN_H * LRN_H; e += LT) {
            const int j = e / LRN_H, u2 = e % LRN_H;
            float g = 0.f;
            for (int p = 0; p < MT_P; ++p) g += sm.f.h1[p * LRN_H + j] * sm.h2[p * LRN_H + u2];
            atomicAdd(grads + LRN_W2 + e, g);
        }
        if (tid < LRN_H) {
            float g = 0.f;
            for (int p = 0; p < MT_P; ++p) g += sm.h2[p * LRN_H + tid];
            atomicAdd(grads + LRN_B2 + tid, g);
        }
        // dL/d(pre-activation of h1)
        for (int p = pp; p < MT_P; p += 2) {
            float a = 0.f;
            for (int u2 = 0; u2 < LRN_H; ++u2) a += sm.h2[p * LRN_H + u2] * __bfloat162float(sm.f.w2[u * LRN_H + u2]);
            sm.dh1[p * LRN_H + u] = sm.f.h1[p * LRN_H + u] > 0.f ? a : 0.f;
        }
        __syncthreads();
        for (int e = tid; e < LRN_F * LRN_H; e += LT) {
            const int f = e / LRN_H, j = e % LRN_H;
            float g = 0.f;
            for (int p = 0; p < MT_P; ++p) g += sm.f.x[p * LRN_F + f] * sm.dh1[p * LRN_H + j];
            atomicAdd(grads + LRN_W1 + e, g);
        }
        if (tid < LRN_H) {
            float g = 0.f;
            for (int p = 0; p < MT_P; ++p) g += sm.dh1[p * LRN_H + tid];
            atomicAdd(grads + LRN_B1 + tid, g);
        }
    }
}

cudaError_t launch_mlp_grad(const float *params, const float *X, const uint8_t *y, int64_t n, float pos_weight,
                            float *grads, float *loss, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(MlpGradSmem));
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int64_t tiles = (n + MT_P - 1) / MT_P;
    const int grid = (int)(tiles < 2 * 152 ? tiles : 2 * 152);
    mlp_grad_kernel<<<grid, LT, sizeof(MlpGradSmem), st>>>(params, X, y, n, pos_weight, grads, loss);
    count_launch();
    return cudaGetLastError();
}

__global__ void mlp_adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                                float *__restrict__ v, int step, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < LRN_NPARAM; e += gridDim.x * blockDim.x) {
        const float ge = g[e];
        const float me = b1 * m[e] + (1.f - b1) * ge, ve = b2 * v[e] + (1.f - b2) * ge * ge;
        m[e] = me;
        v[e] = ve;
        p[e] -= lr * (me / c1) / (sqrtf(ve / c2) + eps);
    }
}
cudaError_t launch_mlp_adam(float *params, const float *grads, float *m, float *v, int step, float lr,
                            cudaStream_t st) {
    mlp_adam_kernel<<<(LRN_NPARAM + 255) / 256, 256, 0, st>>>(params, grads, m, v, step, lr);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ proposal ---
__device__ __forceinline__ void lblock_argmax(float &v, int &i, float *shv, int *shi) {
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, i, o);
        if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { shv[w] = v; shi[w] = i; }
    __syncthreads();
    v = shv[0];
    i = shi[0];
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        if (shv[q] > v || (shv[q] == v && shi[q] < i)) { v = shv[q]; i = shi[q]; }
}
__device__ __forceinline__ bool lbit(const uint32_t *m, int i) { return (m[i >> 5] >> (i & 31)) & 1u; }

// rank estimate r = clamp(ceil(calib * sum_rows sigmoid) + margin, 2, cap),
// top-r rows and columns by score (ties: lower index), in score order
__global__ void __launch_bounds__(LT)
    learn_propose_kernel(const LearnProb *__restrict__ probs, const float *__restrict__ logits, float calib, int margin,
                         int32_t *__restrict__ prop_r, int32_t *__restrict__ prop_c, LearnState *lst) {
    extern __shared__ uint32_t lmask[];
    __shared__ float shv[32];
    __shared__ int shi[32];
    __shared__ float ssum[32];
    const LearnProb pb = probs[blockIdx.x];
    const float *zr = logits + pb.xo, *zc = logits + pb.xo + pb.n1;
    float s = 0.f;
    for (int t = threadIdx.x; t < pb.n1; t += LT) s += 1.f / (1.f + expf(-zr[t]));
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ssum[threadIdx.x >> 5] = s;
    __syncthreads();
    float tot = 0.f;
    for (int q = 0; q < LT / 32; ++q) tot += ssum[q];
    int r = (int)ceilf(calib * tot) + margin;
    r = r < 2 ? 2 : r;
    r = r > pb.cap ? pb.cap : r;
    r = r < 1 ? 1 : r;
    for (int set = 0; set < 1; ++set) {  // rows; the columns are chosen by the restricted ACA
        const int n = set == 0 ? pb.n1 : pb.n2;
        const float *z = set == 0 ? zr : zc;
        int32_t *out = (set == 0 ? prop_r : prop_c) + pb.piv;
        const int words = (n + 31) >> 5;
        for (int q = threadIdx.x; q < words; q += LT) lmask[q] = 0u;
        __syncthreads();
        for (int k = 0; k < r; ++k) {
            float bv = -INFINITY;
            int bi = INT_MAX;
            for (int t = threadIdx.x; t < n; t += LT) {
                const float zt = z[t] == z[t] ? z[t] : -INFINITY;  // a NaN score ranks last
                if (!lbit(lmask, t) && (zt > bv || (zt == bv && t < bi))) { bv = zt; bi = t; }
            }
            lblock_argmax(bv, bi, shv, shi);
            if (bi < 0 || bi >= n) bi = 0;  // unreachable while r <= n; keeps every index in range
            if (threadIdx.x == 0) {
                out[k] = bi;
                lmask[bi >> 5] |= 1u << (bi & 31);
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) lst[blockIdx.x] = {r, 0, 0, 0};
}

cudaError_t launch_learn_propose(const LearnProb *probs, int nprob, const float *logits, float calib, int margin,
                                 int32_t *prop_r, int32_t *prop_c, LearnState *lst, int mask_words, cudaStream_t st) {
    const size_t sm = (size_t)mask_words * 4;
    static size_t set = 0;
    if (sm > 48 * 1024 && sm > set) {
        cudaError_t e = cudaFuncSetAttribute(learn_propose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        set = sm;
    }
    for (int b0 = 0; b0 < nprob; b0 += 65535) {
        const int nb = nprob - b0 < 65535 ? nprob - b0 : 65535;
        learn_propose_kernel<<<nb, LT, sm, st>>>(probs + b0, logits, calib, margin, prop_r, prop_c, lst + b0);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Tiles over all SMs: kind 1, K(I, C) for the proposed rows (rhat of them);
// kind 0, K(R, J') for the ACA's pivot columns (r1 of them, column k = k-th
// pivot). only: the kind this launch fills.
__global__ void learn_fill_kernel(const LearnTile *__restrict__ tiles, const LearnProb *__restrict__ probs,
                                  const int32_t *__restrict__ idx, KParams kp, const int32_t *__restrict__ prop_r,
                                  const int32_t *__restrict__ ordJ, const LearnState *__restrict__ lst,
                                  double *__restrict__ scr, int only) {
    const LearnTile tl = tiles[blockIdx.x];
    if (tl.kind != only) return;
    const LearnProb pb = probs[tl.b];
    const int32_t *R = idx + pb.ri, *C = idx + pb.ci;
    if (tl.kind == 0) {
        const int r1 = lst[tl.b].r1;
        for (int e = tl.start + threadIdx.x; e < tl.start + tl.count; e += blockDim.x) {
            const int c = e / pb.n1, i = e % pb.n1;
            if (c < r1) scr[pb.ac + (int64_t)c * pb.n1 + i] = kentry(kp, R[i], C[ordJ[pb.piv + c]]);
        }
    } else {
        const int rh = lst[tl.b].rhat;
        for (int e = tl.start + threadIdx.x; e < tl.start + tl.count; e += blockDim.x) {
            const int l = e / pb.n2, s = e % pb.n2;
            if (l < rh) scr[pb.ar + (int64_t)l * pb.n2 + s] = kentry(kp, R[prop_r[pb.piv + l]], C[s]);
        }
    }
}
cudaError_t launch_learn_fill(const LearnTile *tiles, int ntiles, const LearnProb *probs, const int32_t *idx,
                              const KParams &kp, const int32_t *prop_r, const int32_t *ordJ, const LearnState *lst,
                              double *scr, int only, cudaStream_t st) {
    for (int t0 = 0; t0 < ntiles; t0 += 65535) {
        const int nt = ntiles - t0 < 65535 ? ntiles - t0 : 65535;
        learn_fill_kernel<<<nt, LT, 0, st>>>(tiles + t0, probs, idx, kp, prop_r, ordJ, lst, scr, only);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The reference's ACA (1D/codes/aca.hpp:296-446) restricted to the proposal's
// rows, on the precomputed K(I, C) (rhat x n2, row l at ar + l*n2): column
// pivots by argmax of the residual row over every column, row pivots by argmax
// of the residual column over the proposed rows, the stopping test with
// normS over these vectors; at most cap - 1 pivots (one column is kept for the
// full-block test; normS here only trims, without the cross terms). ordI:
// pivot rows as proposal indices, ordJ: pivot columns
// as local column indices, both in pivot order; then the LU (no pivoting) of
// K(I', J') in that order at ff (L unit lower / R upper, row-major cap x cap).
// Scratch: the residual rows at vv, the restricted residual columns at gu
// (zeroed again for the Gram matrices).
__global__ void __launch_bounds__(LT)
    learn_aca_kernel(const LearnProb *__restrict__ probs, double tol, double *__restrict__ scr,
                     int32_t *__restrict__ ordI, int32_t *__restrict__ ordJ, LearnState *lst) {
    extern __shared__ uint32_t acm[];  // column mask, n2 bits
    __shared__ double coef[LRN_CAP], shv[32], shd[2 * LT / 32];
    __shared__ int shi[32], crow[LRN_CAP];
    __shared__ double s_norm;
    const LearnProb pb = probs[blockIdx.x];
    const int rh = lst[blockIdx.x].rhat, cap = pb.cap, n2 = pb.n2, tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5, nw = LT / 32;
    const double *M = scr + pb.ar;
    double *Vr = scr + pb.vv;  // residual rows, row l at l*n2
    double *Ur = scr + pb.gu;  // restricted residual columns, column l at l*cap
    const double tiny = 1e-36;
    for (int q = tid; q < (n2 + 31) / 32; q += LT) acm[q] = 0u;
    for (int k = tid; k < LRN_CAP; k += LT) crow[k] = 0;
    if (tid == 0) s_norm = 0.0;
    __syncthreads();
    auto dmax = [&](double &v, int &i) {  // block argmax, lowest index on ties
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, v, o);
            const int oi = __shfl_xor_sync(0xffffffffu, i, o);
            if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
        }
        __syncthreads();
        if (lane == 0) { shv[warp] = v; shi[warp] = i; }
        __syncthreads();
        v = shv[0];
        i = shi[0];
        for (int q = 1; q < nw; ++q)
            if (shv[q] > v || (shv[q] == v && shi[q] < i)) { v = shv[q]; i = shi[q]; }
        __syncthreads();
    };
    auto dsum = [&](double v) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        __syncthreads();
        if (lane == 0) shv[warp] = v;
        __syncthreads();
        double t = 0.0;
        for (int q = 0; q < nw; ++q) t += shv[q];
        __syncthreads();
        return t;
    };
    // first row (score order) with a non-negligible entry
    int row = -1;
    for (int k = 0; k < rh && row < 0; ++k) {
        double bv = -1.0;
        int bi = INT_MAX;
        for (int s2 = tid; s2 < n2; s2 += LT) {
            const double a = fabs(M[(int64_t)k * n2 + s2]);
            if (a > bv || (a == bv && s2 < bi)) { bv = a; bi = s2; }
        }
        dmax(bv, bi);
        if (bv > tiny) row = k;
    }
    int r1 = 0;
    double normS = 0.0;
    const int rmax = rh < cap - 1 ? rh : cap - 1;
    while (row >= 0 && row < rh && r1 < rmax) {
        // residual row of `row` over every column; column pivot
        for (int l = tid; l < r1; l += LT) coef[l] = Ur[(int64_t)l * cap + row];
        __syncthreads();
        double *v = Vr + (int64_t)r1 * n2;
        double vsq = 0.0, bv = -1.0;
        int bi = INT_MAX;
        for (int s2 = tid; s2 < n2; s2 += LT) {
            double x = M[(int64_t)row * n2 + s2];
            for (int l = 0; l < r1; ++l) x -= coef[l] * Vr[(int64_t)l * n2 + s2];
            v[s2] = x;
            vsq += x * x;
            if (!lbit(acm, s2)) {
                const double a = fabs(x);
                if (a > bv || (a == bv && s2 < bi)) { bv = a; bi = s2; }
            }
        }
        dmax(bv, bi);
        const double nv = sqrt(dsum(vsq));
        if (bi < 0 || bi >= n2 || !(nv == nv)) break;
        const int cj = bi;
        const double piv = v[cj];
        if (fabs(piv) <= tiny) break;
        // residual column at cj over the proposed rows; next row pivot
        for (int l = tid; l < r1; l += LT) coef[l] = Vr[(int64_t)l * n2 + cj];
        __syncthreads();
        double *u = Ur + (int64_t)r1 * cap;
        double usq = 0.0;
        bv = -1.0;
        bi = INT_MAX;
        for (int m = tid; m < rh; m += LT) {
            double c = M[(int64_t)m * n2 + cj];
            for (int l = 0; l < r1; ++l) c -= coef[l] * Ur[(int64_t)l * cap + m];
            const double uu = c / piv;
            u[m] = uu;
            usq += uu * uu;
            if (m != row && !crow[m]) {
                const double a = fabs(c);
                if (a > bv || (a == bv && m < bi)) { bv = a; bi = m; }
            }
        }
        dmax(bv, bi);
        const double nu = sqrt(dsum(usq));
        if (nu < tiny || nv < tiny) break;
        if (tid == 0) {
            ordI[pb.piv + r1] = row;
            ordJ[pb.piv + r1] = cj;
            crow[row] = 1;
            acm[cj >> 5] |= 1u << (cj & 31);
        }
        // normS for trimming the proposal (the full-block test recomputes it
        // exactly from the Gram matrices)
        const double cross = 0.0;
        ++r1;
        const double uv = nu * nv;
        normS = sqrt(normS * normS + uv * uv + cross);
        __syncthreads();
        if (uv <= tol * normS) break;
        row = bi;
    }
    // LU of K(I', J') in pivot order
    double *F = scr + pb.ff;
    for (int e = tid; e < r1 * r1; e += LT) {
        const int k = e / r1, l = e % r1;
        F[(size_t)k * cap + l] = M[(int64_t)ordI[pb.piv + k] * n2 + ordJ[pb.piv + l]];
    }
    __syncthreads();
    for (int k = 0; k < r1; ++k) {
        const double d = F[(size_t)k * cap + k];
        for (int i = k + 1 + tid; i < r1; i += LT) F[(size_t)i * cap + k] /= d;
        __syncthreads();
        for (int e = tid; e < (r1 - k - 1) * (r1 - k - 1); e += LT) {
            const int i = k + 1 + e / (r1 - k - 1), j = k + 1 + e % (r1 - k - 1);
            F[(size_t)i * cap + j] -= F[(size_t)i * cap + k] * F[(size_t)k * cap + j];
        }
        __syncthreads();
    }
    for (int e = tid; e < cap * cap; e += LT) Ur[e] = 0.0;  // the Gram buffers start at zero
    if (tid == 0) lst[blockIdx.x].r1 = r1;
}
cudaError_t launch_learn_aca(const LearnProb *probs, int nprob, double tol, double *scr, int32_t *ordI,
                             int32_t *ordJ, LearnState *lst, int mask_words, cudaStream_t st) {
    const size_t sm = (size_t)mask_words * 4;
    static size_t set = 0;
    if (sm > 48 * 1024 && sm > set) {
        cudaError_t e = cudaFuncSetAttribute(learn_aca_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        set = sm;
    }
    for (int b0 = 0; b0 < nprob; b0 += 65535) {
        const int nb = nprob - b0 < 65535 ? nprob - b0 : 65535;
        learn_aca_kernel<<<nb, LT, sm, st>>>(probs + b0, tol, scr, ordI, ordJ, lst + b0);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// U rows: u R = K(R_i, J') (forward over the pivot columns); V columns:
// L v = K(I', C_s) (forward over the pivot rows)
__global__ void learn_solve_kernel(const LearnTile *__restrict__ tiles, const LearnProb *__restrict__ probs,
                                   const int32_t *__restrict__ ordI, const int32_t *__restrict__ ordJ,
                                   const LearnState *__restrict__ lst, double *__restrict__ scr) {
    const LearnTile tl = tiles[blockIdx.x];
    if (tl.kind < 2) return;
    const LearnProb pb = probs[tl.b];
    const int r1 = lst[tl.b].r1, cap = pb.cap;
    const double *F = scr + pb.ff;
    for (int e = tl.start + threadIdx.x; e < tl.start + tl.count; e += blockDim.x) {
        if (tl.kind == 2) {
            const int i = e;
            for (int k = 0; k < r1; ++k) {
                double a = scr[pb.ac + (int64_t)k * pb.n1 + i];
                for (int l = 0; l < k; ++l) a -= scr[pb.uu + (int64_t)l * pb.n1 + i] * F[(size_t)l * cap + k];
                scr[pb.uu + (int64_t)k * pb.n1 + i] = a / F[(size_t)k * cap + k];
            }
        } else {
            const int s = e;
            for (int k = 0; k < r1; ++k) {
                double a = scr[pb.ar + (int64_t)ordI[pb.piv + k] * pb.n2 + s];
                for (int l = 0; l < k; ++l) a -= F[(size_t)k * cap + l] * scr[pb.vv + (int64_t)l * pb.n2 + s];
                scr[pb.vv + (int64_t)k * pb.n2 + s] = a;
            }
        }
    }
}
cudaError_t launch_learn_solve(const LearnTile *tiles, int ntiles, const LearnProb *probs, const int32_t *ordI,
                               const int32_t *ordJ, const LearnState *lst, double *scr, cudaStream_t st) {
    for (int t0 = 0; t0 < ntiles; t0 += 65535) {
        const int nt = ntiles - t0 < 65535 ? ntiles - t0 : 65535;
        learn_solve_kernel<<<nt, 64, 0, st>>>(tiles + t0, probs, ordI, ordJ, lst, scr);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Gram matrices U^T U and V V^T (r1 x r1), partial sums of a tile's rows or
// columns added into the block's buffers (zero beforehand)
__global__ void learn_gram_kernel(const LearnTile *__restrict__ tiles, const LearnProb *__restrict__ probs,
                                  const LearnState *__restrict__ lst, double *__restrict__ scr) {
    const LearnTile tl = tiles[blockIdx.x];
    if (tl.kind < 2) return;
    const LearnProb pb = probs[tl.b];
    const int r1 = lst[tl.b].r1, cap = pb.cap;
    const bool rows = tl.kind == 2;
    const int64_t base = rows ? pb.uu : pb.vv;
    const int64_t ld = rows ? pb.n1 : pb.n2;
    double *G = scr + (rows ? pb.gu : pb.gv);
    for (int e = threadIdx.x; e < r1 * r1; e += blockDim.x) {
        const int k = e / r1, l = e % r1;
        if (l < k) continue;
        double a = 0.0;
        for (int t = tl.start; t < tl.start + tl.count; ++t) a += scr[base + k * ld + t] * scr[base + l * ld + t];
        atomicAdd(G + (size_t)k * cap + l, a);
        if (l != k) atomicAdd(G + (size_t)l * cap + k, a);
    }
}
cudaError_t launch_learn_gram(const LearnTile *tiles, int ntiles, const LearnProb *probs, const LearnState *lst,
                              double *scr, cudaStream_t st) {
    for (int t0 = 0; t0 < ntiles; t0 += 65535) {
        const int nt = ntiles - t0 < 65535 ? ntiles - t0 : 65535;
        learn_gram_kernel<<<nt, 256, 0, st>>>(tiles + t0, probs, lst, scr);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The NCA stopping test on the full block after the proposal's r1 pivots.
__global__ void __launch_bounds__(LT)
    learn_test_kernel(const LearnProb *__restrict__ probs, const int32_t *__restrict__ idx, KParams kp, double tol,
                      const int32_t *__restrict__ prop_r, const int32_t *__restrict__ prop_c,
                      const int32_t *__restrict__ ordI, const int32_t *__restrict__ ordJ, LearnState *lst,
                      double *__restrict__ scr, int32_t *__restrict__ prow, int32_t *__restrict__ pcol) {
    extern __shared__ uint32_t tmask[];  // rows (n1 bits) then columns (n2 bits)
    __shared__ double shv[32], shd[2 * LRN_CAP], shc[LRN_CAP];
    __shared__ int shi[32];
    const LearnProb pb = probs[blockIdx.x];
    const int r1 = lst[blockIdx.x].r1, cap = pb.cap, tid = threadIdx.x;
    const int w1 = (pb.n1 + 31) >> 5, w2 = (pb.n2 + 31) >> 5;
    uint32_t *rm = tmask, *cm = tmask + w1;
    const int32_t *R = idx + pb.ri, *C = idx + pb.ci;
    if (r1 < 1 || r1 >= cap) {  // nothing usable, or no room for the test step: plain search
        if (tid == 0) {
            lst[blockIdx.x].accept = 0;
            lst[blockIdx.x].rank = -1;
        }
        return;
    }
    for (int q = tid; q < w1 + w2; q += LT) tmask[q] = 0u;
    __syncthreads();
    if (tid == 0)
        for (int k = 0; k < r1; ++k) {
            const int i = prop_r[pb.piv + ordI[pb.piv + k]], j = ordJ[pb.piv + k];
            rm[i >> 5] |= 1u << (i & 31);
            cm[j >> 5] |= 1u << (j & 31);
        }
    __syncthreads();
    // normS^2 = ||U V||_F^2 = sum_kl Gu(k,l) Gv(k,l)
    double ns = 0.0;
    for (int e = tid; e < r1 * r1; e += LT) {
        const int k = e / r1, l = e % r1;
        ns += scr[pb.gu + (size_t)k * cap + l] * scr[pb.gv + (size_t)k * cap + l];
    }
    for (int o = 16; o > 0; o >>= 1) ns += __shfl_xor_sync(0xffffffffu, ns, o);
    if ((tid & 31) == 0) shv[tid >> 5] = ns;
    __syncthreads();
    double normS2 = 0.0;
    for (int q = 0; q < LT / 32; ++q) normS2 += shv[q];
    __syncthreads();
    // next row pivot: argmax |last residual column| over rows not chosen
    const double *Ulast = scr + pb.uu + (int64_t)(r1 - 1) * pb.n1;
    double bv = -1.0;
    int bi = INT_MAX;
    for (int t = tid; t < pb.n1; t += LT)
        if (!lbit(rm, t)) {
            const double a = fabs(Ulast[t]);
            if (a > bv || (a == bv && t < bi)) { bv = a; bi = t; }
        }
    // block argmax (doubles)
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    if ((tid & 31) == 0) { shv[tid >> 5] = bv; shi[tid >> 5] = bi; }
    __syncthreads();
    bv = shv[0];
    bi = shi[0];
    for (int q = 1; q < LT / 32; ++q)
        if (shv[q] > bv || (shv[q] == bv && shi[q] < bi)) { bv = shv[q]; bi = shi[q]; }
    __syncthreads();
    const int is = bi;
    int accept = 0, rank = r1;
    int js = -1;
    if (!isfinite(normS2)) {
        accept = 0;  // a non-finite factorisation: plain search
    } else if (is < 0 || is >= pb.n1) {
        accept = r1 >= pb.n1 ? 1 : 0;  // every row a pivot already, else non-finite residuals
    } else {
        // coefficients U(is, k)
        for (int k = tid; k < r1; k += LT) shc[k] = scr[pb.uu + (int64_t)k * pb.n1 + is];
        __syncthreads();
        // residual row at is -> V row r1; column pivot
        double *Vn = scr + pb.vv + (int64_t)r1 * pb.n2;
        double vsq = 0.0, cv = -1.0;
        int cj = INT_MAX;
        for (int s = tid; s < pb.n2; s += LT) {
            double v = kentry(kp, R[is], C[s]);
            for (int k = 0; k < r1; ++k) v -= shc[k] * scr[pb.vv + (int64_t)k * pb.n2 + s];
            Vn[s] = v;
            vsq += v * v;
            if (!lbit(cm, s)) {
                const double a = fabs(v);
                if (a > cv || (a == cv && s < cj)) { cv = a; cj = s; }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            vsq += __shfl_xor_sync(0xffffffffu, vsq, o);
            const double ov = __shfl_xor_sync(0xffffffffu, cv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, cj, o);
            if (ov > cv || (ov == cv && oi < cj)) { cv = ov; cj = oi; }
        }
        __syncthreads();
        if ((tid & 31) == 0) { shv[tid >> 5] = vsq; shd[tid >> 5] = cv; shi[tid >> 5] = cj; }
        __syncthreads();
        vsq = 0.0;
        cv = shd[0];
        cj = shi[0];
        for (int q = 0; q < LT / 32; ++q) {
            vsq += shv[q];
            if (q && (shd[q] > cv || (shd[q] == cv && shi[q] < cj))) { cv = shd[q]; cj = shi[q]; }
        }
        __syncthreads();
        const double nv = sqrt(vsq);
        if (!isfinite(nv)) {
            accept = 0;
        } else if (nv < 1e-36) {
            accept = 1;  // the ACA stops here without another term
        } else if (cj < 0 || cj >= pb.n2) {
            accept = r1 >= pb.n2 ? 1 : 0;
        } else {
            js = cj;
            const double piv = Vn[js];
            for (int k = tid; k < r1; k += LT) shc[k] = scr[pb.vv + (int64_t)k * pb.n2 + js];
            __syncthreads();
            double *Un = scr + pb.uu + (int64_t)r1 * pb.n1;
            double usq = 0.0;
            for (int t = tid; t < pb.n1; t += LT) {
                double c = kentry(kp, R[t], C[js]);
                for (int k = 0; k < r1; ++k) c -= shc[k] * scr[pb.uu + (int64_t)k * pb.n1 + t];
                const double uu = c / piv;
                Un[t] = uu;
                usq += uu * uu;
            }
            for (int o = 16; o > 0; o >>= 1) usq += __shfl_xor_sync(0xffffffffu, usq, o);
            __syncthreads();
            if ((tid & 31) == 0) shv[tid >> 5] = usq;
            __syncthreads();
            usq = 0.0;
            for (int q = 0; q < LT / 32; ++q) usq += shv[q];
            __syncthreads();
            const double nu = sqrt(usq);
            if (!isfinite(nu)) {
                accept = 0;
            } else if (nu < 1e-36) {
                accept = 1;
            } else {
                // cross terms 2 sum_k |<U_k, u><V_k, v>| (the reference's normS update)
                for (int k = 0; k < r1; ++k) {
                    double du = 0.0, dv = 0.0;
                    for (int t = tid; t < pb.n1; t += LT) du += scr[pb.uu + (int64_t)k * pb.n1 + t] * Un[t];
                    for (int s = tid; s < pb.n2; s += LT) dv += scr[pb.vv + (int64_t)k * pb.n2 + s] * Vn[s];
                    for (int o = 16; o > 0; o >>= 1) {
                        du += __shfl_xor_sync(0xffffffffu, du, o);
                        dv += __shfl_xor_sync(0xffffffffu, dv, o);
                    }
                    if ((tid & 31) == 0) { shd[2 * (tid >> 5)] = du; shd[2 * (tid >> 5) + 1] = dv; }
                    __syncthreads();
                    if (tid == 0) {
                        double a = 0.0, b = 0.0;
                        for (int q = 0; q < LT / 32; ++q) { a += shd[2 * q]; b += shd[2 * q + 1]; }
                        shc[k] = 2.0 * fabs(a * b);
                    }
                    __syncthreads();
                }
                double ns2 = normS2 + (nu * nv) * (nu * nv);
                for (int k = 0; k < r1; ++k) ns2 += shc[k];
                accept = (isfinite(ns2) && nu * nv <= tol * sqrt(ns2)) ? 1 : 0;
                rank = r1 + 1;
            }
        }
    }
    if (tid == 0) {
        LearnState &s = lst[blockIdx.x];
        s.accept = accept;
        s.rank = accept ? rank : (isfinite(normS2) ? -3 : -2);  // rejected: -3 test failed, -2 non-finite
        if (accept) {
            for (int k = 0; k < r1; ++k) {
                prow[pb.piv + k] = prop_r[pb.piv + ordI[pb.piv + k]];
                pcol[pb.piv + k] = ordJ[pb.piv + k];
            }
            if (rank > r1) {
                prow[pb.piv + r1] = is;
                pcol[pb.piv + r1] = js;
            }
        }
    }
}
cudaError_t launch_learn_test(const LearnProb *probs, int nprob, const int32_t *idx, const KParams &kp, double tol,
                              const int32_t *prop_r, const int32_t *prop_c, const int32_t *ordI, const int32_t *ordJ,
                              LearnState *lst, double *scr, int32_t *prow, int32_t *pcol, int mask_words,
                              cudaStream_t st) {
    const size_t sm = (size_t)mask_words * 4;
    static size_t set = 0;
    if (sm > 48 * 1024 && sm > set) {
        cudaError_t e = cudaFuncSetAttribute(learn_test_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        set = sm;
    }
    for (int b0 = 0; b0 < nprob; b0 += 65535) {
        const int nb = nprob - b0 < 65535 ? nprob - b0 : 65535;
        learn_test_kernel<<<nb, LT, sm, st>>>(probs + b0, idx, kp, tol, prop_r, prop_c, ordI, ordJ, lst + b0, scr,
                                              prow, pcol);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace h2w
