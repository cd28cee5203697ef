// Multi-right-hand-side matvec and batched GMRES (sm_103a).
//
//  * mr_kernel / mr_coop_kernel  Y = A X for RP right-hand sides at once, over
//      the same packed target records as the single-vector GEMV: a target is
//      a small GEMM (rows x RP) = sum_p A_p (rows x w_p) X_p (w_p x RP). The
//      operator panels and the gathered sources are staged through shared
//      memory in 32-column chunks (the next chunk is loaded into registers
//      while the current one is multiplied) and every thread keeps a 4-row x
//      4-column block of the result, so each operator element read from HBM
//      feeds RP fused multiply-adds. The input block is read in the
//      kernel's precision (FP32 kernel: an FP32 copy). Vectors are interleaved: element (t, c)
//      of a block of RP vectors sits at t*RP + c, so one source row is RP
//      contiguous values.
//  * mr_pack / mr_unpack  column-major vectors in the caller's point order
//      <-> interleaved leaf-order blocks.
//  (The lockstep GMRES over these blocks is in gmbatch.cu.)
#include <cfloat>
#include <type_traits>

#include "dfmath.cuh"
#include "kernels.cuh"
#include "sync.cuh"

namespace h2w {

constexpr int MR_MT = 64;  // result rows per tile
constexpr int MR_KC = 32;  // operator columns per staged chunk
constexpr int MR_NSA = 3;  // staging buffers of the FP32 kernel (two chunks in flight)

// 16-byte asynchronous global -> shared copy; bytes < 16 zero-fills the rest
// (bytes = 0: no global read, src may be any valid address)
__device__ __forceinline__ void mr_cp16(void *dst, const void *src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mr_cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void mr_cp_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <class T> struct MrVec;
template <> struct MrVec<double> { using type = double2; static constexpr int n = 2; };
template <> struct MrVec<float> { using type = float4; static constexpr int n = 4; };

template <class T, int RP> struct MrLayout {
    static constexpr int NT = 4 * RP;                  // 16 row quads x RP/4 column quads
    static constexpr int VN = MrVec<T>::n;             // elements per 16-byte vector
    static constexpr int NA = MR_KC * MR_MT / VN / NT; // A vectors per thread per chunk
    static constexpr int NX = MR_KC * RP / VN / NT;    // X vectors per thread per chunk
    static constexpr size_t rec_bytes = (size_t)BRG_REC_WORDS * 8;
    static constexpr size_t as_bytes = sizeof(T) * MR_KC * MR_MT;
    static constexpr size_t xs_bytes = sizeof(T) * MR_KC * RP;
    static constexpr size_t map_bytes = (size_t)4 * MR_XS_ELEMS;
    static constexpr size_t smem = rec_bytes + 2 * (as_bytes + xs_bytes) + map_bytes;  // two staging buffers
    // FP32 kernel: MR_NSA staging buffers filled by asynchronous copies
    static constexpr size_t smem_async = rec_bytes + MR_NSA * (as_bytes + xs_bytes) + map_bytes;
    static_assert(NA >= 1 && NA * VN * NT == MR_KC * MR_MT, "A chunk split");
    static_assert(NX >= 1 && NX * VN * NT == MR_KC * RP, "X chunk split");
};

__device__ __forceinline__ void mr_zero(double2 &v) { v = make_double2(0.0, 0.0); }
__device__ __forceinline__ void mr_zero(float4 &v) { v = make_float4(0.f, 0.f, 0.f, 0.f); }
__device__ __forceinline__ void mr_scalar(double2 &v, const double *p, int nv) {
    v.x = nv > 0 ? p[0] : 0.0;
    v.y = nv > 1 ? p[1] : 0.0;
}
__device__ __forceinline__ void mr_scalar(float4 &v, const float *p, int nv) {
    v.x = nv > 0 ? p[0] : 0.f;
    v.y = nv > 1 ? p[1] : 0.f;
    v.z = nv > 2 ? p[2] : 0.f;
    v.w = nv > 3 ? p[3] : 0.f;
}
__device__ __forceinline__ void mr_get4(double *o, const double *p) {
    const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
__device__ __forceinline__ void mr_get4(float *o, const float *p) {
    const float4 a = *reinterpret_cast<const float4 *>(p);
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
}

// Double-FP32 ("df64") arithmetic for an FP64-accurate product on the FP32
// pipes: a double a is carried as hi = fl32(a), lo = fl32(a - hi) (2^-48
// relative), a product a*x as p = hi_a*hi_x plus its exact FMA error and the
// two cross terms, and a sum as an unevaluated pair (sh, sl) advanced by
// Knuth's TwoSum, so every rounding of the FP32 sum is kept in sl. All
// operations are explicitly rounded (no contraction may merge them).
__device__ __forceinline__ void df_fma(float &sh, float &sl, const float2 a, const float2 x) {
    const float p = __fmul_rn(a.x, x.x);
    float e = __fmaf_rn(a.x, x.x, -p);
    e = __fmaf_rn(a.x, x.y, e);
    e = __fmaf_rn(a.y, x.x, e);
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(t, e));
}
// k-parts of a row tile: a tile of at most 32 (16) rows leaves half (three
// quarters) of the 16 row groups without rows, so the row groups split each
// chunk's columns into 2 (4) parts instead, summed through shared memory
// after the last chunk
__device__ __forceinline__ int mr_kparts(int rows) { return rows > 32 ? 1 : (rows > 16 ? 2 : 4); }
__device__ __forceinline__ void df_get4(float2 *o, const float2 *p) {
    const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
    o[0] = make_float2(a.x, a.y); o[1] = make_float2(a.z, a.w);
    o[2] = make_float2(b.x, b.y); o[3] = make_float2(b.z, b.w);
}

// One target of the packed record stream (record layout as the
// single-vector GEMV: header, panels, segments). DF (with T = double): A and
// xin hold (hi, lo) FP32 pairs in place of doubles (split once, mr_split),
// workspace values are split when staged, and the tiles are multiplied with
// double-FP32 arithmetic.
template <class T, int RP, bool DF = false, class YT = double>
__device__ __forceinline__ void mr_target(char *smem, int64_t t, const int64_t *__restrict__ roff,
                                          const int64_t *__restrict__ blob, const T *__restrict__ A, T *ws,
                                          const T *__restrict__ xin, YT *yout) {
    using Lay = MrLayout<T, RP>;
    using V = typename MrVec<T>::type;
    constexpr int NT = Lay::NT, VN = Lay::VN, NA = Lay::NA, NX = Lay::NX;
    int64_t *rec = reinterpret_cast<int64_t *>(smem);
    // staging buffer s: As + s * MR_KC * MR_MT, Xs + s * MR_KC * RP
    T *As = reinterpret_cast<T *>(smem + Lay::rec_bytes);
    T *Xs = reinterpret_cast<T *>(smem + Lay::rec_bytes + 2 * Lay::as_bytes);
    int32_t *map = reinterpret_cast<int32_t *>(smem + Lay::rec_bytes + 2 * (Lay::as_bytes + Lay::xs_bytes));
    const int tid = threadIdx.x;
    const int ty = tid / (RP / 4), tx = tid % (RP / 4);

    const int64_t o = roff[t];
    const int nw = (int)(roff[t + 1] - o);
    for (int q = tid; q < nw; q += NT) rec[q] = blob[o + q];
    __syncthreads();
    const int64_t dst = rec[0];
    const int nrows = (int)(rec[1] & 0xffffffff), flags = (int)(rec[1] >> 32);
    const int np = (int)(rec[2] & 0xffffffff), ns = (int)(rec[2] >> 32);
    const int64_t *pan = rec + 3;
    const int64_t *seg = pan + 3 * np;
    // source map: gathered row e -> workspace row (>= 0), input row (-2 - pos) or none (-1)
    int xend = 0;
    for (int q = 0; q < np; ++q) {
        const int e = (int)pan[3 * q + 2] + (int)(pan[3 * q + 1] >> 32);
        xend = e > xend ? e : xend;
    }
    for (int e = tid; e < xend; e += NT) map[e] = -1;
    __syncthreads();
    for (int s = 0; s < ns; ++s) {
        const int64_t src = seg[2 * s], w1 = seg[2 * s + 1];
        const int len = (int)(w1 & 0xffffffff), code = (int)(w1 >> 32);
        const int xo = code >> 1;
        const bool g = code & 1;
        for (int i = tid; i < len; i += NT) map[xo + i] = g ? -(2 + (int)(src + i)) : (int)(src + i);
    }
    __syncthreads();

    V ra[NA], rx[NX];
    bool xws[NX];  // DF: the source row came from the FP64 workspace (split on staging)
    // load chunk (panel q, columns c0 .. c0+KC) of row tile rt0 into registers
    auto load = [&](int q, int c0, int rt0) {
        const int64_t pa = pan[3 * q];
        const int lda = (int)(pan[3 * q + 1] & 0xffffffff), w = (int)(pan[3 * q + 1] >> 32);
        const int xoff = (int)pan[3 * q + 2];
        const bool vec = ((pa & 3) == 0) && ((lda & 3) == 0);  // the plan's 16-byte-row rule (4 elements)
#pragma unroll
        for (int u = 0; u < NA; ++u) {
            const int v = tid + NT * u;
            const int col = v / (MR_MT / VN), r = rt0 + (v % (MR_MT / VN)) * VN;
            const int c = c0 + col;
            if (c < w && r < nrows) {
                const T *p = A + pa + (int64_t)c * lda + r;
                if (vec) ra[u] = *reinterpret_cast<const V *>(p);
                else mr_scalar(ra[u], p, nrows - r);
            } else {
                mr_zero(ra[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < NX; ++u) {
            const int v = tid + NT * u;
            const int row = v / (RP / VN), cv = (v % (RP / VN)) * VN;
            mr_zero(rx[u]);
            xws[u] = false;
            if (c0 + row < w) {
                const int m = map[xoff + c0 + row];
                xws[u] = m >= 0;
                if (m >= 0) rx[u] = *reinterpret_cast<const V *>(ws + (int64_t)m * RP + cv);
                else if (m <= -2) rx[u] = *reinterpret_cast<const V *>(xin + (int64_t)(-2 - m) * RP + cv);
            }
        }
    };
    auto store = [&](int sb) {
#pragma unroll
        for (int u = 0; u < NA; ++u) {
            const int v = tid + NT * u;
            T *d = As + sb * (MR_KC * MR_MT) + (v / (MR_MT / VN)) * MR_MT + (v % (MR_MT / VN)) * VN;
            // DF: the operator is stored pre-split (hi, lo FP32 pairs): the bits go as they are
            *reinterpret_cast<V *>(d) = ra[u];
        }
#pragma unroll
        for (int u = 0; u < NX; ++u) {
            const int v = tid + NT * u;
            T *d = Xs + sb * (MR_KC * RP) + (v / (RP / VN)) * RP + (v % (RP / VN)) * VN;
            if constexpr (DF) {
                if (xws[u]) {  // FP64 workspace values: split here
                    const float2 h0 = df_split_fast(rx[u].x), h1 = df_split_fast(rx[u].y);
                    *reinterpret_cast<float4 *>(d) = make_float4(h0.x, h0.y, h1.x, h1.y);
                } else {  // the input block is pre-split
                    *reinterpret_cast<V *>(d) = rx[u];
                }
            } else {
                *reinterpret_cast<V *>(d) = rx[u];
            }
        }
    };

    for (int rt0 = 0; rt0 < nrows; rt0 += MR_MT) {
        T acc[4][4];
        float ah[4][4], al[4][4];  // DF: (hi, lo) pairs
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                acc[i][j] = T(0);
                ah[i][j] = 0.f;
                al[i][j] = 0.f;
            }
        // Two staging buffers: chunk i is multiplied from buffer i&1 while the
        // registers already hold chunk i+1, which then goes to the other buffer;
        // one barrier per chunk. Warps whose rows are all past the target's
        // last row skip the multiply (the SM's other CTA keeps the pipes busy:
        // this kernel is issue-bound, and splitting a short tile's chunks over
        // the idle warps, as the FP32 kernel does, measured no faster).
        int q = 0, c0 = 0, sb = 0;
        if (np > 0) {
            load(0, 0, rt0);
            store(0);
        }
        __syncthreads();
        const bool active = rt0 + ty * 4 < nrows;
        while (q < np) {
            int nq = q, nc0 = c0 + MR_KC;
            if (nc0 >= (int)(pan[3 * q + 1] >> 32)) { nq = q + 1; nc0 = 0; }
            const bool more = nq < np;
            if (more) load(nq, nc0, rt0);
            const T *Ab = As + sb * (MR_KC * MR_MT);
            const T *Xb = Xs + sb * (MR_KC * RP);
            if (!active) {
            } else if constexpr (DF) {
                // columns past the panel's width are zero: the 12-operation terms stop at the width
                const int kw = min(MR_KC, (int)(pan[3 * q + 1] >> 32) - c0);
#pragma unroll 4
                for (int k = 0; k < kw; ++k) {
                    float2 a4[4], x4[4];
                    df_get4(a4, reinterpret_cast<const float2 *>(Ab) + k * MR_MT + ty * 4);
                    df_get4(x4, reinterpret_cast<const float2 *>(Xb) + k * RP + tx * 4);
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) df_fma(ah[i][j], al[i][j], a4[i], x4[j]);
                }
            } else {
                const int kw = min(MR_KC, (int)(pan[3 * q + 1] >> 32) - c0);
#pragma unroll 8
                for (int k = 0; k < kw; ++k) {
                    T a4[4], x4[4];
                    mr_get4(a4, Ab + k * MR_MT + ty * 4);
                    mr_get4(x4, Xb + k * RP + tx * 4);
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] += a4[i] * x4[j];
                }
            }
            if (more) store(sb ^ 1);
            __syncthreads();
            q = nq;
            c0 = nc0;
            sb ^= 1;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = rt0 + ty * 4 + i;
            if (r >= nrows) continue;
            const int64_t d = (dst + r) * RP + tx * 4;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                T v;
                if constexpr (DF) v = (T)((double)ah[i][j] + (double)al[i][j]);
                else v = acc[i][j];
                if (flags & T_SCATTER) yout[d + j] = (YT)((flags & T_ACCUM) ? ws[d + j] + v : v);
                else if (flags & T_ATOMIC) atomicAdd(ws + d + j, v);
                else if (flags & T_ACCUM) ws[d + j] += v;
                else ws[d + j] = v;
            }
        }
    }
    __syncthreads();
}

// FP32 form of mr_target with the chunks staged by asynchronous copies
// (cp.async, zero-filled past a target's rows or a panel's columns) into
// MR_NSA buffers: the copies of chunks i+1 and i+2 are in flight while chunk
// i is multiplied, with no staging registers; one barrier per chunk.
template <int RP, class YT>
__device__ __forceinline__ void mr_target_async(char *smem, int64_t t, const int64_t *__restrict__ roff,
                                                const int64_t *__restrict__ blob, const float *__restrict__ A,
                                                float *ws, const float *__restrict__ xin, YT *yout) {
    using Lay = MrLayout<float, RP>;
    constexpr int NT = Lay::NT, NA = Lay::NA, NX = Lay::NX;
    int64_t *rec = reinterpret_cast<int64_t *>(smem);
    float *As = reinterpret_cast<float *>(smem + Lay::rec_bytes);
    float *Xs = reinterpret_cast<float *>(smem + Lay::rec_bytes + MR_NSA * Lay::as_bytes);
    int32_t *map = reinterpret_cast<int32_t *>(smem + Lay::rec_bytes + MR_NSA * (Lay::as_bytes + Lay::xs_bytes));
    const int tid = threadIdx.x;
    const int ty = tid / (RP / 4), tx = tid % (RP / 4);

    const int64_t o = roff[t];
    const int nw = (int)(roff[t + 1] - o);
    for (int q = tid; q < nw; q += NT) rec[q] = blob[o + q];
    __syncthreads();
    const int64_t dst = rec[0];
    const int nrows = (int)(rec[1] & 0xffffffff), flags = (int)(rec[1] >> 32);
    const int np = (int)(rec[2] & 0xffffffff), ns = (int)(rec[2] >> 32);
    const int64_t *pan = rec + 3;
    const int64_t *seg = pan + 3 * np;
    int xend = 0;
    for (int q = 0; q < np; ++q) {
        const int e = (int)pan[3 * q + 2] + (int)(pan[3 * q + 1] >> 32);
        xend = e > xend ? e : xend;
    }
    for (int e = tid; e < xend; e += NT) map[e] = -1;
    __syncthreads();
    for (int s = 0; s < ns; ++s) {
        const int64_t src = seg[2 * s], w1 = seg[2 * s + 1];
        const int len = (int)(w1 & 0xffffffff), code = (int)(w1 >> 32);
        const int xo = code >> 1;
        const bool g = code & 1;
        for (int i = tid; i < len; i += NT) map[xo + i] = g ? -(2 + (int)(src + i)) : (int)(src + i);
    }
    __syncthreads();

    auto advance = [&](int &q, int &c0) {
        if (q >= np) return;
        c0 += MR_KC;
        if (c0 >= (int)(pan[3 * q + 1] >> 32)) {
            ++q;
            c0 = 0;
        }
    };
    // copies of chunk (panel q, columns c0 .. c0+KC) of rows rt0 .. into buffer sb
    // (q >= np: none), committed as one group
    auto issue = [&](int q, int c0, int rt0, int sb) {
        if (q < np) {
            const int64_t pa = pan[3 * q];
            const int lda = (int)(pan[3 * q + 1] & 0xffffffff), w = (int)(pan[3 * q + 1] >> 32);
            const int xoff = (int)pan[3 * q + 2];
            const bool vec = ((pa & 3) == 0) && ((lda & 3) == 0);  // the plan's 16-byte-row rule (4 elements)
#pragma unroll
            for (int u = 0; u < NA; ++u) {
                const int v = tid + NT * u;
                const int col = v / (MR_MT / 4), r = rt0 + (v % (MR_MT / 4)) * 4;
                const int c = c0 + col;
                float *d = As + sb * (MR_KC * MR_MT) + col * MR_MT + (v % (MR_MT / 4)) * 4;
                if (c < w && r < nrows) {
                    const float *p = A + pa + (int64_t)c * lda + r;
                    const int nv = nrows - r < 4 ? nrows - r : 4;
                    if (vec) {
                        mr_cp16(d, p, 4 * nv);
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; ++j) d[j] = j < nv ? p[j] : 0.f;
                    }
                } else {
                    mr_cp16(d, A, 0);
                }
            }
#pragma unroll
            for (int u = 0; u < NX; ++u) {
                const int v = tid + NT * u;
                const int row = v / (RP / 4), cv = (v % (RP / 4)) * 4;
                const float *src = xin;
                int bytes = 0;
                if (c0 + row < w) {
                    const int m = map[xoff + c0 + row];
                    if (m >= 0) {
                        src = ws + (int64_t)m * RP + cv;
                        bytes = 16;
                    } else if (m <= -2) {
                        src = xin + (int64_t)(-2 - m) * RP + cv;
                        bytes = 16;
                    }
                }
                mr_cp16(Xs + sb * (MR_KC * RP) + row * RP + cv, src, bytes);
            }
        }
        mr_cp_commit();
    };

    for (int rt0 = 0; rt0 < nrows; rt0 += MR_MT) {
        float acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
        int q0 = 0, c00 = 0;  // the chunk multiplied next, then the two in flight behind it
        int q1 = 0, c01 = 0;
        advance(q1, c01);
        int q2 = q1, c02 = c01;
        advance(q2, c02);
        issue(q0, c00, rt0, 0);
        issue(q1, c01, rt0, 1);
        // row group tyr of k-part kp: rows rt0 + 4 tyr .. + 3, columns kp kn .. + kn of each chunk
        const int S = mr_kparts(nrows - rt0), G = 16 / S, kn = MR_KC / S;
        const int tyr = ty % G, kp = ty / G;
        const bool active = rt0 + tyr * 4 < nrows;
        int sb = 0;
        while (q0 < np) {
            mr_cp_wait<1>();   // this thread's copies of chunk q0 have landed
            __syncthreads();   // everyone's have; the buffer of the previous chunk is free
            issue(q2, c02, rt0, sb == 0 ? MR_NSA - 1 : sb - 1);
            if (active) {
                const float *Ab = As + sb * (MR_KC * MR_MT);
                const float *Xb = Xs + sb * (MR_KC * RP);
#pragma unroll 8
                for (int kk = 0; kk < kn; ++kk) {
                    const int k = kp * kn + kk;
                    float a4[4], x4[4];
                    mr_get4(a4, Ab + k * MR_MT + tyr * 4);
                    mr_get4(x4, Xb + k * RP + tx * 4);
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] += a4[i] * x4[j];
                }
            }
            q0 = q1;
            c00 = c01;
            q1 = q2;
            c01 = c02;
            advance(q2, c02);
            sb = sb + 1 == MR_NSA ? 0 : sb + 1;
        }
        mr_cp_wait<0>();
        if (S > 1) {  // k-parts 1 .. S-1 add into part 0 through the staging buffers
            __syncthreads();  // every group is done with the last chunk's buffer
            if (kp > 0 && active) {
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) As[(((kp - 1) * G + tyr) * 4 + i) * RP + tx * 4 + j] = acc[i][j];
            }
            __syncthreads();
            if (kp == 0 && active) {
                for (int p = 1; p < S; ++p)
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] += As[(((p - 1) * G + tyr) * 4 + i) * RP + tx * 4 + j];
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = rt0 + tyr * 4 + i;
            if (kp > 0 || r >= nrows) continue;
            const int64_t d = (dst + r) * RP + tx * 4;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float v = acc[i][j];
                const float prev = (flags & T_ACCUM) ? ws[d + j] : 0.f;
                if (flags & T_SCATTER) yout[d + j] = (YT)((flags & T_ACCUM) ? prev + v : v);
                else if (flags & T_ATOMIC) atomicAdd(ws + d + j, v);
                else if (flags & T_ACCUM) ws[d + j] = prev + v;
                else ws[d + j] = v;
            }
        }
        __syncthreads();
    }
    __syncthreads();
}

// Targets [t0, t1) of one phase: a CTA takes t0 + blockIdx.x first, then
// claims the next unstarted target from the phase's counter (zero at launch),
// so CTAs that finish early take over the remaining work.
template <class T, int RP, bool DF, class YT>
__device__ __forceinline__ void mr_phase(char *smem, int64_t t0, int64_t t1, int32_t *ctr,
                                         const int64_t *__restrict__ roff, const int64_t *__restrict__ blob,
                                         const T *__restrict__ A, T *ws, const T *__restrict__ xin, YT *yout) {
    __shared__ int64_t s_next;
    int64_t t = t0 + blockIdx.x;
    while (t < t1) {
        if constexpr (std::is_same<T, float>::value && !DF)
            mr_target_async<RP, YT>(smem, t, roff, blob, A, ws, xin, yout);
        else
            mr_target<T, RP, DF, YT>(smem, t, roff, blob, A, ws, xin, yout);
        if (threadIdx.x == 0) s_next = t0 + gridDim.x + atomicAdd(ctr, 1);
        __syncthreads();
        t = s_next;
    }
}

template <class T, int RP, bool DF, class YT>
__global__ void __launch_bounds__(4 * RP)
    mr_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob, int64_t t0, int64_t t1,
              int32_t *ctr, const T *__restrict__ A, T *ws, const T *__restrict__ xin, YT *yout) {
    extern __shared__ __align__(16) char mr_smem[];
    mr_phase<T, RP, DF, YT>(mr_smem, t0, t1, ctr, roff, blob, A, ws, xin, yout);
}

template <class T, int RP, bool DF, class YT>
__global__ void __launch_bounds__(4 * RP)
    mr_coop_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob,
                   const int64_t *__restrict__ pstart, int nphase, int32_t *ctr, const T *__restrict__ A,
                   T *ws, const T *__restrict__ xin, YT *yout, unsigned *bar, int32_t *err) {
    extern __shared__ __align__(16) char mr_smem[];
    for (int p = 0; p < nphase; ++p) {
        mr_phase<T, RP, DF, YT>(mr_smem, pstart[p], pstart[p + 1], ctr + p, roff, blob, A, ws, xin, yout);
        if (p + 1 < nphase) grid_barrier(bar, gridDim.x, err);
    }
}

static int mr_num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// Dataflow form of mr_coop_kernel: no grid barriers. Targets are claimed in
// their stored order (a topological order: every producer of a target
// precedes it), first blockIdx.x, then from a global counter; a CTA waits
// until its target's producer count rem[t] reaches zero (bounded spin: on
// timeout it sets *err = 3 and proceeds, so the kernel always ends), runs it,
// and decrements the counts of its consumers cidx[coff[t] .. coff[t+1]).
// The launch is cooperative, so every CTA is resident: a waiting target's
// producers have all been claimed by running CTAs. Workspace reads are as in
// the barrier launch (gathered sources by cp.async.cg from L2 or by plain
// loads, an accumulating target's own rows by plain loads); the dependencies
// order every writer of a row before its readers, and each producer fences
// its writes before releasing its consumers.
template <class T, int RP, bool DF, class YT>
__global__ void __launch_bounds__(4 * RP)
    mr_flow_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob, int64_t nt, int32_t *ctr,
                   int32_t *rem, const int64_t *__restrict__ coff, const int32_t *__restrict__ cidx,
                   const T *__restrict__ A, T *ws, const T *__restrict__ xin, YT *yout, int32_t *err) {
    extern __shared__ __align__(16) char mr_smem[];
    __shared__ int64_t s_next;
    int64_t t = blockIdx.x;
    while (t < nt) {
        if (threadIdx.x == 0) {
            long long it = 0;
            while (*((volatile int32_t *)(rem + t)) > 0) {
                if (++it > (1LL << 20)) {  // about 0.1 s
                    atomicExch(err, 3);
                    break;
                }
                __nanosleep(64);
            }
            __threadfence();
        }
        __syncthreads();
        if constexpr (std::is_same<T, float>::value && !DF)
            mr_target_async<RP, YT>(mr_smem, t, roff, blob, A, ws, xin, yout);  // ends with a barrier
        else
            mr_target<T, RP, DF, YT>(mr_smem, t, roff, blob, A, ws, xin, yout);  // ends with a barrier
        if (threadIdx.x < 32) {
            __threadfence();  // this CTA's results are visible before its consumers are released
            for (int64_t e = coff[t] + threadIdx.x; e < coff[t + 1]; e += 32) atomicSub(rem + cidx[e], 1);
            if (threadIdx.x == 0) s_next = gridDim.x + atomicAdd(ctr, 1);
        }
        __syncthreads();
        t = s_next;
    }
}

template <class T, int RP, bool DF, class YT>
static cudaError_t mr_flow_launch(const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr, int32_t *rem,
                                  const int64_t *coff, const int32_t *cidx, const T *A, T *ws, const T *xin,
                                  YT *yout, int32_t *err, cudaStream_t st) {
    using Lay = MrLayout<T, RP>;
    constexpr size_t SMEM = (std::is_same<T, float>::value && !DF) ? Lay::smem_async : Lay::smem;
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaFuncSetAttribute(mr_flow_kernel<T, RP, DF, YT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SMEM) != cudaSuccess)
            return cudaErrorInvalidValue;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mr_flow_kernel<T, RP, DF, YT>, Lay::NT, SMEM);
        if (per_sm <= 0) return cudaErrorCooperativeLaunchTooLarge;
    }
    const int grid = mr_num_sms() * per_sm;
    void *args[] = {(void *)&roff, (void *)&blob, (void *)&nt, (void *)&ctr, (void *)&rem, (void *)&coff,
                    (void *)&cidx, (void *)&A, (void *)&ws, (void *)&xin, (void *)&yout, (void *)&err};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)mr_flow_kernel<T, RP, DF, YT>, dim3(grid), dim3(Lay::NT),
                                                args, SMEM, st);
    count_launch();
    return e;
}
template <class T, bool DF, class YT>
static cudaError_t mr_flow_dispatch(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr,
                                    int32_t *rem, const int64_t *coff, const int32_t *cidx, const T *A, T *ws,
                                    const T *xin, YT *yout, int32_t *err, cudaStream_t st) {
    switch (rp) {
    case 16: return mr_flow_launch<T, 16, DF, YT>(roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
    case 32: return mr_flow_launch<T, 32, DF, YT>(roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
    case 64: return mr_flow_launch<T, 64, DF, YT>(roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
    default: return cudaErrorInvalidValue;
    }
}
cudaError_t launch_mr_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr, int32_t *rem,
                               const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const float *xin,
                               double *yout, int32_t *err, cudaStream_t st) {
    return mr_flow_dispatch<float, false>(rp, roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
}
cudaError_t launch_mr_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr, int32_t *rem,
                               const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const float *xin,
                               float *yout, int32_t *err, cudaStream_t st) {
    return mr_flow_dispatch<float, false>(rp, roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
}
cudaError_t launch_mr_f64_flow(int rp, bool df, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr,
                               int32_t *rem, const int64_t *coff, const int32_t *cidx, const double *A, double *ws,
                               const double *xin, double *yout, int32_t *err, cudaStream_t st) {
    if (df) return mr_flow_dispatch<double, true>(rp, roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
    return mr_flow_dispatch<double, false>(rp, roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
}

template <class T, int RP, bool DF, class YT>
static cudaError_t mr_launch_t(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                               const MrPhases *phased, int32_t *ctr, const T *A, T *ws, const T *xin,
                               YT *yout, unsigned *bar, int32_t *err, cudaStream_t st) {
    using Lay = MrLayout<T, RP>;
    constexpr size_t SMEM = (std::is_same<T, float>::value && !DF) ? Lay::smem_async : Lay::smem;
    static int per_sm_coop = 0, per_sm = 0;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(mr_coop_kernel<T, RP, DF, YT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)SMEM);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(mr_kernel<T, RP, DF, YT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int nsm = mr_num_sms();
    if (phased) {
        if (per_sm == 0) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mr_kernel<T, RP, DF, YT>, Lay::NT, SMEM);
            if (per_sm <= 0) per_sm = 1;
        }
        for (int p = 0; p < phased->n; ++p) {
            const int64_t t0 = phased->t0[p], t1 = phased->t1[p];
            if (t1 <= t0) continue;
            const int64_t cap = (int64_t)nsm * per_sm;
            const int grid = (int)(t1 - t0 < cap ? t1 - t0 : cap);
            mr_kernel<T, RP, DF, YT><<<grid, Lay::NT, SMEM, st>>>(roff, blob, t0, t1, ctr + p, A, ws, xin, yout);
            count_launch();
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    if (per_sm_coop == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_coop, mr_coop_kernel<T, RP, DF, YT>, Lay::NT, SMEM);
        if (per_sm_coop <= 0) return cudaErrorCooperativeLaunchTooLarge;
    }
    const int grid = nsm * per_sm_coop;
    void *args[] = {(void *)&roff, (void *)&blob, (void *)&pstart, (void *)&nphase, (void *)&ctr, (void *)&A,
                    (void *)&ws,   (void *)&xin,  (void *)&yout,   (void *)&bar,    (void *)&err};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)mr_coop_kernel<T, RP, DF, YT>, dim3(grid), dim3(Lay::NT), args,
                                                SMEM, st);
    count_launch();
    return e;
}

template <class T, bool DF = false, class YT = double>
static cudaError_t mr_dispatch(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                               const MrPhases *phased, int32_t *ctr, const T *A, T *ws, const T *xin,
                               YT *yout, unsigned *bar, int32_t *err, cudaStream_t st) {
    switch (rp) {
    case 16: return mr_launch_t<T, 16, DF, YT>(roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
    case 32: return mr_launch_t<T, 32, DF, YT>(roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
    case 64: return mr_launch_t<T, 64, DF, YT>(roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_mr_f64(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                          const MrPhases *phased, int32_t *ctr, const double *A, double *ws, const double *xin, double *yout,
                          unsigned *bar, int32_t *err, cudaStream_t st) {
    return mr_dispatch<double>(rp, roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
}
cudaError_t launch_mr_df64(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                           const MrPhases *phased, int32_t *ctr, const double *A, double *ws, const double *xin, double *yout,
                           unsigned *bar, int32_t *err, cudaStream_t st) {
    return mr_dispatch<double, true>(rp, roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
}
cudaError_t launch_mr_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                          const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin, double *yout,
                          unsigned *bar, int32_t *err, cudaStream_t st) {
    return mr_dispatch<float>(rp, roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
}
cudaError_t launch_mr_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                          const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin, float *yout,
                          unsigned *bar, int32_t *err, cudaStream_t st) {
    return mr_dispatch<float, false, float>(rp, roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err,
                                            st);
}

// b[i] = (hi, lo) FP32 pair of a[i] (df_split_fast), for the double-FP32 product
__global__ void mr_split_kernel(const double *__restrict__ a, float2 *__restrict__ b, int64_t n) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        b[e] = df_split_fast(a[e]);
}
cudaError_t launch_mr_split(const double *a, void *b, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    mr_split_kernel<<<1216, 256, 0, st>>>(a, reinterpret_cast<float2 *>(b), n);
    count_launch();
    return cudaGetLastError();
}

// Calibration vectors of the FP32 product's error (interleaved, rp columns,
// column index c0 + e % rp): even columns pseudo-random in [-1, 1) (splitmix64
// of the element index), odd columns smooth, cos(pi * k * (t + 0.5) / n).
__global__ void mr_calib_fill_kernel(double *__restrict__ z, int64_t n, int rp, int c0) {
    const int64_t tot = n * rp;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = e / rp;
        const int c = c0 + (int)(e % rp);
        double v;
        if (c % 2 == 0) {
            uint64_t x = (uint64_t)t * 64u + (uint64_t)c + 0x9E3779B97F4A7C15ull;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            x ^= x >> 31;
            v = 2.0 * ((double)(x >> 11) * 0x1.0p-53) - 1.0;
        } else {
            v = cospi((double)(c / 2 + 1) * ((double)t + 0.5) / (double)n);
        }
        z[e] = v;
    }
}
cudaError_t launch_calib_fill(double *z, int64_t n, int rp, int c0, cudaStream_t st) {
    mr_calib_fill_kernel<<<1216, 256, 0, st>>>(z, n, rp, c0);
    count_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------ pack / unpack ---
// xi[t*rp + c] = x[perm[t] + c*ldx] for c < nrhs, 0 for the padding columns
__global__ void mr_pack_kernel(const double *__restrict__ x, int64_t ldx, double *__restrict__ xi,
                               const int32_t *__restrict__ perm, int64_t n, int nrhs, int rp) {
    const int64_t tot = n * rp;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = e / rp;
        const int c = (int)(e % rp);
        xi[e] = c < nrhs ? x[(perm ? (int64_t)perm[t] : t) + (int64_t)c * ldx] : 0.0;
    }
}
__global__ void mr_unpack_kernel(const double *__restrict__ yi, double *__restrict__ y, int64_t ldy,
                                 const int32_t *__restrict__ perm, int64_t n, int nrhs, int rp) {
    const int64_t tot = n * rp;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = e / rp;
        const int c = (int)(e % rp);
        if (c < nrhs) y[(perm ? (int64_t)perm[t] : t) + (int64_t)c * ldy] = yi[e];
    }
}
template <class T>
__global__ void mr_widen_kernel(const T *__restrict__ a, double *__restrict__ b, int64_t n) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        b[e] = (double)a[e];
}
cudaError_t launch_mr_pack(const double *x, int64_t ldx, double *xi, const int32_t *perm, int64_t n, int nrhs,
                           int rp, cudaStream_t st) {
    mr_pack_kernel<<<1216, 256, 0, st>>>(x, ldx, xi, perm, n, nrhs, rp);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_mr_unpack(const double *yi, double *y, int64_t ldy, const int32_t *perm, int64_t n, int nrhs,
                             int rp, cudaStream_t st) {
    mr_unpack_kernel<<<1216, 256, 0, st>>>(yi, y, ldy, perm, n, nrhs, rp);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_mr_widen_f64(const double *a, double *b, int64_t n, cudaStream_t st) {
    mr_widen_kernel<double><<<1216, 256, 0, st>>>(a, b, n);
    count_launch();
    return cudaGetLastError();
}
cudaError_t launch_mr_widen_f32(const float *a, double *b, int64_t n, cudaStream_t st) {
    mr_widen_kernel<float><<<1216, 256, 0, st>>>(a, b, n);
    count_launch();
    return cudaGetLastError();
}

}  // namespace h2w
