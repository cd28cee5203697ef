// Far-field M2L evaluated during the product (sm_103a).
//
// The far M2L blocks of the nested form are plain kernel entries between
// skeleton points: M2L[k][q] = K(check_k, check_q) (assemble_M2L_far,
// 2D/codes/HODLR2Dtree.hpp:655-675, 3D/codes/HODLR3Dtree.hpp:1978-1998), and
// they are most of the stored entries of a 3D operator (about 80 % for
// uniform random points at tol 1e-10). When the stored operator would not fit
// in device memory, the handle keeps the far check points instead and this
// kernel forms in_k = sum_q K(check_k, check_q) out_q (evaluate_M2L_far,
// 2D :678-699, 3D :2000-2021) from the point coordinates on every product.
//
// Work items are blocks of <= 32 rows of one target box (enough items to
// fill every SM); a persistent grid claims them largest first from a
// counter. A CTA stages the item's source columns 256 at a time in shared
// memory (coordinates and the workspace value out_q); four threads share a
// row, each over every fourth column with two independent accumulation
// chains, their partial sums met by shuffles, and the row is written once:
// the target's rows are written by no other item, and this kernel is the
// first writer of them in the product. The FP64 form evaluates the entries
// with a few ulps of the stored ones (fly_entry64); the FP32 form evaluates
// them in FP32 from FP32 coordinates.
#include <cmath>

#include "dfmath.cuh"
#include "entry.cuh"

namespace h2w {

constexpr int FLY_THREADS = 128;
constexpr int FLY_TILE = 256;
constexpr int FLY_TPR = 4;  // threads per row; FLY_ROWS = FLY_THREADS / FLY_TPR rows per work item
static_assert(FLY_ROWS * FLY_TPR == FLY_THREADS, "work item shape");

template <int DIM, int CH>
__device__ __forceinline__ float fly_entry32(const FlyK32 &k, float dx, float dy, float dz) {
    const float R2 = DIM == 3 ? fmaf(dz, dz, fmaf(dy, dy, dx * dx)) : fmaf(dy, dy, dx * dx);
    if (DIM == 2) {
        if (CH == 0) return k.c2d * __logf(R2);
        return R2 < k.a2 ? sqrtf(R2) * k.inv_a : k.a * rsqrtf(R2);
    }
    if (CH == 0) return k.inv4pi * rsqrtf(R2);
    if (R2 < k.a2) {
        const float R = sqrtf(R2);
        return (R * __logf(R) - 1.f) * k.inv_den;
    }
    return (0.5f * __logf(R2)) * k.inv_loga;
}

// one staged source column: coordinates and the workspace value out_q
template <class T> struct FlyCol { T x, y, z, v; };

// FP64 entries for the far field: the same functions with fewer FP64
// operations than the exact getMatrixEntry order (log R = log(R^2) / 2, a
// product by 1/log a, an rsqrt instead of a division by a square root);
// they differ from the stored entries by a few ulps. Far pairs never meet
// the R < a branch of the RBF kernels (boxes are separated by a box), which
// keeps the exact form.
template <int DIM, int CH>
__device__ __forceinline__ double fly_entry64(const KParams &k, const double *a, const double *b) {
    const double dx = a[0] - b[0], dy = a[1] - b[1];
    const double R2 = DIM == 3 ? fma(a[2] - b[2], a[2] - b[2], fma(dy, dy, dx * dx)) : fma(dy, dy, dx * dx);
    const double aa = 0.0001;
    if (DIM == 2) {
        if (CH == 0) return k.c2d * log(R2);
        if (R2 < aa * aa) return kentry_ab(k, a, b);
        return aa * rsqrt(R2);
    }
    if (CH == 0) return rsqrt(R2) / k.four_pi;
    if (R2 < aa * aa) return kentry_ab(k, a, b);
    return log(R2) * (0.5 / k.loga);
}

template <class T, int DIM, int CH>
__global__ void __launch_bounds__(FLY_THREADS)
    m2l_fly_kernel(const FlyItem *__restrict__ items, int64_t nitems, unsigned long long *ctr,
                   const int32_t *__restrict__ rowpid, const int32_t *__restrict__ cpid,
                   const int32_t *__restrict__ cws, const T *__restrict__ pts, T *ws, KParams kp, FlyK32 k32) {
    __shared__ __align__(16) FlyCol<T> sc[FLY_TILE];
    __shared__ long long s_it;
    // coordinates: FP32 as (x, y, z, 0) quadruples, FP64 as the points array (N x DIM)
    constexpr int PS = sizeof(T) == 4 ? 4 : DIM;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_it = (long long)atomicAdd(ctr, 1ull);
        __syncthreads();
        const long long it = s_it;
        if (it >= nitems) return;
        const FlyItem m = items[it];
        // FLY_ROWS rows per item, FLY_TPR threads per row over interleaved columns
        const int tpr = FLY_TPR;
        const int row = threadIdx.x / tpr, sub = threadIdx.x - row * tpr;
        const bool has = row < m.nrows;
        T a[3] = {T(0), T(0), T(0)};
        if (has) {
            const int64_t p = rowpid[m.rows + row];
#pragma unroll
            for (int d = 0; d < DIM; ++d) a[d] = pts[p * PS + d];
        }
        (void)PS;
        T acc = T(0), acc2 = T(0);  // two chains: the multiply-adds of neighbouring columns overlap
        for (int c0 = 0; c0 < m.ncols; c0 += FLY_TILE) {
            const int nc = m.ncols - c0 < FLY_TILE ? m.ncols - c0 : FLY_TILE;
            __syncthreads();
            for (int c = threadIdx.x; c < nc; c += FLY_THREADS) {
                const int64_t e = m.cbeg + c0 + c;
                const int64_t p = cpid[e];
                FlyCol<T> q;
                if constexpr (sizeof(T) == 4) {
                    const float4 f = reinterpret_cast<const float4 *>(pts)[p];
                    q.x = f.x;
                    q.y = f.y;
                    q.z = f.z;
                } else {
                    q.x = pts[p * PS];
                    q.y = pts[p * PS + 1];
                    q.z = DIM == 3 ? pts[p * PS + 2] : T(0);
                }
                q.v = ws[cws[e]];
                sc[c] = q;
            }
            __syncthreads();
            if (has) {
                if constexpr (sizeof(T) == 4) {
                    int c = sub;
                    for (; c + tpr < nc; c += 2 * tpr) {
                        const float4 q = reinterpret_cast<const float4 *>(sc)[c];
                        const float4 r = reinterpret_cast<const float4 *>(sc)[c + tpr];
                        acc = fmaf(fly_entry32<DIM, CH>(k32, a[0] - q.x, a[1] - q.y, DIM == 3 ? a[2] - q.z : 0.f), q.w,
                                   acc);
                        acc2 = fmaf(fly_entry32<DIM, CH>(k32, a[0] - r.x, a[1] - r.y, DIM == 3 ? a[2] - r.z : 0.f),
                                    r.w, acc2);
                    }
                    if (c < nc) {
                        const float4 q = reinterpret_cast<const float4 *>(sc)[c];
                        acc = fmaf(fly_entry32<DIM, CH>(k32, a[0] - q.x, a[1] - q.y, DIM == 3 ? a[2] - q.z : 0.f), q.w,
                                   acc);
                    }
                } else {
                    const double aa[3] = {(double)a[0], (double)a[1], (double)a[2]};
                    int c = sub;
                    for (; c + tpr < nc; c += 2 * tpr) {
                        const FlyCol<T> q = sc[c], r = sc[c + tpr];
                        const double b[3] = {(double)q.x, (double)q.y, (double)q.z};
                        const double e[3] = {(double)r.x, (double)r.y, (double)r.z};
                        acc = fma(fly_entry64<DIM, CH>(kp, aa, b), (double)q.v, (double)acc);
                        acc2 = fma(fly_entry64<DIM, CH>(kp, aa, e), (double)r.v, (double)acc2);
                    }
                    if (c < nc) {
                        const FlyCol<T> q = sc[c];
                        const double b[3] = {(double)q.x, (double)q.y, (double)q.z};
                        acc = fma(fly_entry64<DIM, CH>(kp, aa, b), (double)q.v, (double)acc);
                    }
                }
            }
        }
        // partial sums of a row's threads (adjacent lanes)
        acc += acc2;
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        if (has && sub == 0) ws[m.dst + row] = acc;
    }
}

// FP32 form for far pairs separated by more than the RBF kernels' radius a
// (every far pair of a tree whose deepest boxes are wider than a: a far pair's
// boxes are not adjacent, so its points are at least a box width apart). The
// entry is then one function of R^2 times a constant: log2(R^2) (3D RBF,
// 2D IE) or 1/sqrt(R^2) (3D IE, 2D RBF); the constant multiplies the row's
// sum once. Sixteen threads share four rows of the item (rows g, g + 8,
// g + 16, g + 24), each over every sixteenth staged column: one shared-memory
// load feeds four entries, whose sums are independent chains, and the
// function is one MUFU instruction without the subnormal fix-up (R^2 of a
// far pair is never subnormal). Measured on the 2^17-point 3D RBF operator:
// 1.57 -> 1.20 ms per launch against two rows per thread with the library
// log2 (profiles/m2l_fly32_sep_3d_rbf_131072.md). (Paired FP32 instructions,
// __ffma2_rn and kin, on the two rows of a thread measured 3.46 ms: issue
// fell to 28 %.)
template <int DIM, int CH>
__device__ __forceinline__ float fly_g32(float R2) {
    float y;
    if ((DIM == 3 && CH == 1) || (DIM == 2 && CH == 0)) asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(R2));
    else asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(R2));
    return y;
}

template <int DIM, int CH>
__global__ void __launch_bounds__(FLY_THREADS)
    m2l_fly32_sep_kernel(const FlyItem *__restrict__ items, int64_t nitems, unsigned long long *ctr,
                         const int32_t *__restrict__ rowpid, const int32_t *__restrict__ cpid,
                         const int32_t *__restrict__ cws, const float *__restrict__ pts4, float *ws, float scale) {
    constexpr int RPT = 4, TPR = 16, GROUPS = FLY_ROWS / RPT;  // rows per thread, threads per row group
    static_assert(GROUPS * TPR == FLY_THREADS, "four rows per thread");
    __shared__ __align__(16) float4 sc[FLY_TILE];
    __shared__ long long s_it;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_it = (long long)atomicAdd(ctr, 1ull);
        __syncthreads();
        const long long it = s_it;
        if (it >= nitems) return;
        const FlyItem m = items[it];
        const int grp = threadIdx.x / TPR, sub = threadIdx.x - grp * TPR;
        const bool any = grp < m.nrows;
        float ax[RPT], ay[RPT], az[RPT], acc[RPT];
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const int r = grp + k * GROUPS;
            // rows past the item's last repeat its first row's point: their sums are dropped
            const int rr = r < m.nrows ? r : grp;
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
            if (any) a = reinterpret_cast<const float4 *>(pts4)[rowpid[m.rows + rr]];
            ax[k] = a.x;
            ay[k] = a.y;
            az[k] = a.z;
            acc[k] = 0.f;
        }
        for (int c0 = 0; c0 < m.ncols; c0 += FLY_TILE) {
            const int nc = m.ncols - c0 < FLY_TILE ? m.ncols - c0 : FLY_TILE;
            __syncthreads();
            for (int c = threadIdx.x; c < nc; c += FLY_THREADS) {
                const int64_t e = m.cbeg + c0 + c;
                float4 q = reinterpret_cast<const float4 *>(pts4)[cpid[e]];
                q.w = ws[cws[e]];
                sc[c] = q;
            }
            __syncthreads();
            if (any) {
#pragma unroll 2
                for (int c = sub; c < nc; c += TPR) {
                    const float4 q = sc[c];
#pragma unroll
                    for (int k = 0; k < RPT; ++k) {
                        const float dx = ax[k] - q.x, dy = ay[k] - q.y;
                        float r2 = fmaf(dy, dy, dx * dx);
                        if (DIM == 3) {
                            const float dz = az[k] - q.z;
                            r2 = fmaf(dz, dz, r2);
                        }
                        acc[k] = fmaf(fly_g32<DIM, CH>(r2), q.w, acc[k]);
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < RPT; ++k)
#pragma unroll
            for (int o = 1; o < TPR; o <<= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
        if (sub == 0) {
#pragma unroll
            for (int k = 0; k < RPT; ++k)
                if (grp + k * GROUPS < m.nrows) ws[m.dst + grp + k * GROUPS] = acc[k] * scale;
        }
    }
}

// ---- double-FP32 form (FP64-accurate far M2L on the FP32 pipes) ---------
//
// GB300 runs FP64 at 1/64 of its FP32 rate, and the FP64 entries spend it on
// the logarithm. Here every value is an unevaluated pair of floats and every
// operation an error-free transformation (dfmath.cuh); the points are split
// once into (hi, lo) pairs, R^2 is formed from pair differences and log(R^2)
// by the table-driven pair logarithm. Each row's sum is a pair; the kernel's
// constant multiplies it once. For the kernels built on log(R^2) (3D RBF, 2D
// integral equation) with every far pair farther apart than a; the others
// keep the FP64 form.

// the FP64-accurate far M2L: rows' sums as pairs times `scale`, into an FP64 workspace
template <int DIM>
__global__ void __launch_bounds__(FLY_THREADS)
    m2l_flydf_kernel(const FlyItem *__restrict__ items, int64_t nitems, unsigned long long *ctr,
                     const int32_t *__restrict__ rowpid, const int32_t *__restrict__ cpid,
                     const int32_t *__restrict__ cws, const float *__restrict__ ptsdf, double *ws,
                     const DfLogTab *__restrict__ gtab, double scale) {
    __shared__ __align__(16) float sc[FLY_TILE][8];  // x, y, z hi; x, y, z lo; value hi, lo
    __shared__ __align__(16) DfLogTab tab[128];
    __shared__ long long s_it;
    for (int i = threadIdx.x; i < 128; i += FLY_THREADS) tab[i] = gtab[i];
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_it = (long long)atomicAdd(ctr, 1ull);
        __syncthreads();
        const long long it = s_it;
        if (it >= nitems) return;
        const FlyItem m = items[it];
        const int row = threadIdx.x / FLY_TPR, sub = threadIdx.x - row * FLY_TPR;
        const bool has = row < m.nrows;
        float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (has) {
            const float4 *q = reinterpret_cast<const float4 *>(ptsdf) + 2 * (int64_t)rowpid[m.rows + row];
            const float4 hi = q[0], lo = q[1];
            a[0] = hi.x; a[1] = hi.y; a[2] = hi.z; a[4] = lo.x; a[5] = lo.y; a[6] = lo.z;
        }
        Df acc{0.f, 0.f};
        for (int c0 = 0; c0 < m.ncols; c0 += FLY_TILE) {
            const int nc = m.ncols - c0 < FLY_TILE ? m.ncols - c0 : FLY_TILE;
            __syncthreads();
            for (int c = threadIdx.x; c < nc; c += FLY_THREADS) {
                const int64_t e = m.cbeg + c0 + c;
                const float4 *q = reinterpret_cast<const float4 *>(ptsdf) + 2 * (int64_t)cpid[e];
                const float4 hi = q[0], lo = q[1];
                const double v = ws[cws[e]];
                const float vh = (float)v;
                const float vl = (float)(v - (double)vh);
                reinterpret_cast<float4 *>(sc[c])[0] = make_float4(hi.x, hi.y, hi.z, lo.x);
                reinterpret_cast<float4 *>(sc[c])[1] = make_float4(lo.y, lo.z, vh, vl);
            }
            __syncthreads();
            if (has) {
                for (int c = sub; c < nc; c += FLY_TPR) {
                    const float4 p0 = reinterpret_cast<const float4 *>(sc[c])[0];
                    const float4 p1 = reinterpret_cast<const float4 *>(sc[c])[1];
                    const Df dx = df_sub(Df{a[0], a[4]}, Df{p0.x, p0.w});
                    const Df dy = df_sub(Df{a[1], a[5]}, Df{p0.y, p1.x});
                    const Df sx = df_sqr(dx), sy = df_sqr(dy);
                    Df r2 = df_add(sx, sy);
                    if (DIM == 3) r2 = df_add(r2, df_sqr(df_sub(Df{a[2], a[6]}, Df{p0.z, p1.y})));
                    const Df lg = df_log(r2, tab);
                    // acc += lg * v
                    const float ph = __fmul_rn(lg.h, p1.z);
                    float pe = __fmaf_rn(lg.h, p1.z, -ph);
                    pe = __fmaf_rn(lg.h, p1.w, pe);
                    pe = __fmaf_rn(lg.l, p1.z, pe);
                    const Df s2 = df_two_sum(acc.h, ph);
                    acc = df_fast(s2.h, __fadd_rn(s2.l, __fadd_rn(acc.l, pe)));
                }
            }
        }
        // partial sums of a row's four threads (pairs)
#pragma unroll
        for (int o = 1; o < FLY_TPR; o <<= 1) {
            const Df b{__shfl_xor_sync(0xffffffffu, acc.h, o), __shfl_xor_sync(0xffffffffu, acc.l, o)};
            acc = df_add(acc, b);
        }
        if (has && sub == 0) ws[m.dst + row] = ((double)acc.h + (double)acc.l) * scale;
    }
}

static int fly_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <class T, int DIM, int CH>
static cudaError_t fly_launch_t(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                                const int32_t *cpid, const int32_t *cws, const T *pts, T *ws, const KParams &kp,
                                const FlyK32 &k32, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, m2l_fly_kernel<T, DIM, CH>, FLY_THREADS, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    const int64_t cap = (int64_t)fly_sms() * per_sm;
    const int grid = (int)(nitems < cap ? nitems : cap);
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    m2l_fly_kernel<T, DIM, CH><<<grid, FLY_THREADS, 0, st>>>(items, nitems, ctr, rowpid, cpid, cws, pts, ws, kp, k32);
    count_launch();
    return cudaGetLastError();
}

template <class T>
static cudaError_t fly_dispatch(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                                const int32_t *cpid, const int32_t *cws, const T *pts, T *ws, const KParams &kp,
                                const FlyK32 &k32, cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    if (kp.dim == 2)
        return kp.choice == 0 ? fly_launch_t<T, 2, 0>(items, nitems, ctr, rowpid, cpid, cws, pts, ws, kp, k32, st)
                              : fly_launch_t<T, 2, 1>(items, nitems, ctr, rowpid, cpid, cws, pts, ws, kp, k32, st);
    if (kp.dim == 3)
        return kp.choice == 0 ? fly_launch_t<T, 3, 0>(items, nitems, ctr, rowpid, cpid, cws, pts, ws, kp, k32, st)
                              : fly_launch_t<T, 3, 1>(items, nitems, ctr, rowpid, cpid, cws, pts, ws, kp, k32, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_fly_f64(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                           const int32_t *cpid, const int32_t *cws, double *ws, const KParams &kp, cudaStream_t st) {
    return fly_dispatch<double>(items, nitems, ctr, rowpid, cpid, cws, kp.pts, ws, kp, FlyK32{}, st);
}

template <int DIM, int CH>
static cudaError_t fly32_sep_launch(const FlyItem *items, int64_t nitems, unsigned long long *ctr,
                                    const int32_t *rowpid, const int32_t *cpid, const int32_t *cws, const float *pts4,
                                    float *ws, float scale, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, m2l_fly32_sep_kernel<DIM, CH>, FLY_THREADS, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    const int64_t cap = (int64_t)fly_sms() * per_sm;
    const int grid = (int)(nitems < cap ? nitems : cap);
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    m2l_fly32_sep_kernel<DIM, CH><<<grid, FLY_THREADS, 0, st>>>(items, nitems, ctr, rowpid, cpid, cws, pts4, ws, scale);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_fly_f32(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                           const int32_t *cpid, const int32_t *cws, const float *pts4, float *ws, const KParams &kp,
                           const FlyK32 &k32, cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    if (k32.sep) {  // every far pair farther apart than a: one function of R^2 times a constant
        const double ln2 = 0.69314718055994530942;
        if (kp.dim == 3 && kp.choice == 1)
            return fly32_sep_launch<3, 1>(items, nitems, ctr, rowpid, cpid, cws, pts4, ws,
                                          (float)(0.5 * ln2 / kp.loga), st);
        if (kp.dim == 3 && kp.choice == 0)
            return fly32_sep_launch<3, 0>(items, nitems, ctr, rowpid, cpid, cws, pts4, ws, (float)(1.0 / kp.four_pi),
                                          st);
        if (kp.dim == 2 && kp.choice == 0)
            return fly32_sep_launch<2, 0>(items, nitems, ctr, rowpid, cpid, cws, pts4, ws, (float)(kp.c2d * ln2), st);
        if (kp.dim == 2 && kp.choice == 1)
            return fly32_sep_launch<2, 1>(items, nitems, ctr, rowpid, cpid, cws, pts4, ws, k32.a, st);
    }
    return fly_dispatch<float>(items, nitems, ctr, rowpid, cpid, cws, pts4, ws, kp, k32, st);
}

template <int DIM>
static cudaError_t flydf_launch(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                                const int32_t *cpid, const int32_t *cws, const float *ptsdf, double *ws,
                                const DfLogTab *tab, double scale, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, m2l_flydf_kernel<DIM>, FLY_THREADS, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    const int64_t cap = (int64_t)fly_sms() * per_sm;
    const int grid = (int)(nitems < cap ? nitems : cap);
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    m2l_flydf_kernel<DIM><<<grid, FLY_THREADS, 0, st>>>(items, nitems, ctr, rowpid, cpid, cws, ptsdf, ws, tab, scale);
    count_launch();
    return cudaGetLastError();
}

bool fly_df_supported(const KParams &kp, const FlyK32 &k32) {
    return k32.sep && ((kp.dim == 3 && kp.choice == 1) || (kp.dim == 2 && kp.choice == 0));
}

cudaError_t launch_fly_df64(const FlyItem *items, int64_t nitems, unsigned long long *ctr, const int32_t *rowpid,
                            const int32_t *cpid, const int32_t *cws, const float *ptsdf, const void *logtab,
                            double *ws, const KParams &kp, const FlyK32 &k32, cudaStream_t st) {
    if (nitems <= 0) return cudaSuccess;
    if (!fly_df_supported(kp, k32))
        return fly_dispatch<double>(items, nitems, ctr, rowpid, cpid, cws, kp.pts, ws, kp, FlyK32{}, st);
    const DfLogTab *tab = reinterpret_cast<const DfLogTab *>(logtab);
    if (kp.dim == 3) return flydf_launch<3>(items, nitems, ctr, rowpid, cpid, cws, ptsdf, ws, tab, 0.5 / kp.loga, st);
    return flydf_launch<2>(items, nitems, ctr, rowpid, cpid, cws, ptsdf, ws, tab, kp.c2d, st);
}

// The log table of the double-FP32 form: 128 bins of [1, 2), centre
// c_k = 1 + (2k + 1) / 256 (exact in FP32), log c_k and 1 / c_k as (hi, lo)
// pairs of their FP64 values. 8 floats per entry.
void fly_df_logtab(float *out) {
    for (int k = 0; k < 128; ++k) {
        const double c = 1.0 + (2.0 * k + 1.0) / 256.0, l = std::log(c), i = 1.0 / c;
        const float lh = (float)l, ih = (float)i;
        float *t = out + 8 * k;
        t[0] = (float)c;
        t[1] = lh;
        t[2] = (float)(l - (double)lh);
        t[3] = ih;
        t[4] = (float)(i - (double)ih);
        t[5] = t[6] = t[7] = 0.f;
    }
}

// (x, y, z, 0) hi and lo FP32 quadruples of the FP64 points (N x dim): x = hi + lo to 2^-48.
__global__ void ptsdf_kernel(const double *__restrict__ pts, int dim, int64_t n, float *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float h[4] = {0.f, 0.f, 0.f, 0.f}, l[4] = {0.f, 0.f, 0.f, 0.f};
        for (int d = 0; d < dim; ++d) {
            const double v = pts[i * dim + d];
            h[d] = (float)v;
            l[d] = (float)(v - (double)h[d]);
        }
        reinterpret_cast<float4 *>(out)[2 * i] = make_float4(h[0], h[1], h[2], h[3]);
        reinterpret_cast<float4 *>(out)[2 * i + 1] = make_float4(l[0], l[1], l[2], l[3]);
    }
}

cudaError_t launch_ptsdf(const double *pts, int dim, int64_t n, float *out, cudaStream_t st) {
    ptsdf_kernel<<<fly_sms() * 4, 256, 0, st>>>(pts, dim, n, out);
    count_launch();
    return cudaGetLastError();
}

// (x, y, z, 0) FP32 quadruples of the FP64 points (N x dim).
__global__ void pts4_kernel(const double *__restrict__ pts, int dim, int64_t n, float *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float q[4] = {0.f, 0.f, 0.f, 0.f};
        for (int d = 0; d < dim; ++d) q[d] = (float)pts[i * dim + d];
        reinterpret_cast<float4 *>(out)[i] = make_float4(q[0], q[1], q[2], q[3]);
    }
}

cudaError_t launch_pts4(const double *pts, int dim, int64_t n, float *out, cudaStream_t st) {
    pts4_kernel<<<fly_sms() * 4, 256, 0, st>>>(pts, dim, n, out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace h2w
