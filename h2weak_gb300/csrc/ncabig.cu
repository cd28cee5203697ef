// The NCA pivot search for large blocks on many SMs at once (sm_103a).
//
// The reference's ACA (1D/codes/aca.hpp:296-446) is sequential in its
// pivots, and one CTA per block (nca_kernel) leaves a block of tens of
// thousands of rows and columns on a single SM. Here the CTAs of one
// cooperative launch form G groups; a group works on one large block at a
// time, its CTAs striding over the block's columns (residual rows) and rows
// (residual columns), with a bounded group barrier after each pass. Every
// entry and residual is computed by one thread in the reference's operation
// order (separately rounded multiply and subtract), the argmax keeps the
// lowest index among equal magnitudes, and every CTA of the group reduces the
// per-CTA partials in the same CTA order, so all CTAs agree on every pivot
// and on the stopping test without further communication.
//
// No rank limit is built in: the residual updates stream the coefficients of
// the kept terms through a fixed shared-memory chunk (the subtraction order
// stays the pivot order), and a block whose rank reaches the capacity of its
// scratch (rcap terms of U and V) stops and reports -rank, so that the host
// runs it again with more scratch (the search is deterministic: the same
// pivots come out, the earlier ones unchanged).
#include <climits>

#include "dfmath.cuh"
#include "entry.cuh"

namespace h2w {

constexpr int NG_THREADS = 256;
constexpr int NG_COEF = 1024;  // coefficients of kept terms staged per chunk (8 KB)

struct NgPart {             // per-CTA partials of one pass
    double v, s;            // best |value| (argmax), sum of squares
    int32_t i, pad;
};

// Group barrier: ctr[0] arrivals, ctr[1] generation; bounded spin sets *err.
__device__ __forceinline__ void ng_barrier(unsigned *ctr, unsigned members, int32_t *err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = ctr + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(ctr, 1u);
        if (arrived == members - 1) {
            atomicExch(ctr, 0u);
            __threadfence();
            atomicAdd(ctr + 1, 1u);
        } else {
            long long it = 0;
            while (*vgen == gen) {
                if (++it > (1LL << 26)) {
                    atomicExch(err, 1);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

template <class M>
__device__ __forceinline__ bool ng_better(M a, int ia, M b, int ib) { return a > b || (a == b && ia < ib); }

// CTA-local argmax / sum, then written as this CTA's partial
__device__ void ng_cta_part(double v, int i, double s, NgPart *out, double *shv, int *shi, double *shs) {
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, i, o);
        if (ng_better(ov, oi, v, i)) { v = ov; i = oi; }
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { shv[w] = v; shi[w] = i; shs[w] = s; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bv = shv[0], ss = shs[0];
        int bi = shi[0];
        for (int q = 1; q < NG_THREADS / 32; ++q) {
            if (ng_better(shv[q], shi[q], bv, bi)) { bv = shv[q]; bi = shi[q]; }
            ss += shs[q];
        }
        *out = {bv, ss, bi, 0};
    }
    __syncthreads();
}
// the group's result from its members' partials, in member order
__device__ void ng_group(const NgPart *part, int g, int G, int S, double &v, int &i, double &s) {
    v = -1.0;
    i = INT_MAX;
    s = 0.0;
    for (int k = 0; k < S; ++k) {
        const NgPart p = part[g + k * G];
        if (ng_better(p.v, p.i, v, i)) { v = p.v; i = p.i; }
        s += p.s;
    }
}
__device__ __forceinline__ bool ng_bit(const uint32_t *m, int i) { return (m[i >> 5] >> (i & 31)) & 1u; }

// Scratch element types of the group search. double: the reference's FP64
// operations in its order (bitwise its residuals for equal entries). float2:
// double-FP32 pairs (hi + lo, about 2^-48 relative; TwoSum / TwoProduct
// error-free transformations) on the FP32 pipes, for the kernels whose
// entries already differ from the reference's in the last bit (they use log):
// GB300 runs FP64 at 1/64 of the FP32 rate, and the residual updates, a
// product and a subtraction per kept term and entry, are the search's work.
// The squares and the stopping test's dots only need FP32 there.
// What the pair entries of the kernels built on log need: log(R^2) times
// scale for R^2 >= thr (the log table in shared memory).
struct NgEnt {
    const DfLogTab *tab;
    Df scale;
    float thr;
};

template <class E> struct NgOps;
template <> struct NgOps<double> {
    using Acc = double;
    using Mag = double;
    static constexpr bool kFuse = false;
    static __device__ __forceinline__ double from(double d) { return d; }
    static __device__ __forceinline__ double mag(double e) { return fabs(e); }
    static __device__ __forceinline__ double entry(const KParams &kp, int i, int j, const NgEnt &) {
        return kentry(kp, i, j);
    }
    static __device__ __forceinline__ double submul(double v, double c, double x) {
        return __dsub_rn(v, __dmul_rn(c, x));
    }
    static __device__ __forceinline__ double inv(double p) { return p; }  // divided exactly below
    static __device__ __forceinline__ double div(double c, double p) { return __ddiv_rn(c, p); }
    static __device__ __forceinline__ double sq(double e) { return e * e; }
    static __device__ __forceinline__ double dot(double a, double b) { return a * b; }
};
template <> struct NgOps<float2> {
    using Acc = float;
    using Mag = float;  // |hi| orders the pairs as its FP64 value would
    static constexpr bool kFuse = true;
    static __device__ __forceinline__ float2 from(double d) {
        const float h = __double2float_rn(d);
        return make_float2(h, __double2float_rn(d - (double)h));
    }
    static __device__ __forceinline__ float mag(float2 e) { return fabsf(e.x); }
    // The entry as a pair: the coordinate differences in FP64 (as the
    // reference forms them), split into pairs with integer operations, R^2
    // and the pair logarithm on the FP32 pipes, times the kernel's constant;
    // the diagonal, and pairs closer than the kernel's log range, from the
    // FP64 entry.
    static __device__ __forceinline__ float2 entry(const KParams &kp, int i, int j, const NgEnt &c) {
        if (i == j) return from(kp.diag);
        const double *a = kp.pts + (size_t)i * kp.dim, *b = kp.pts + (size_t)j * kp.dim;
        float2 d = df_split_fast(__dsub_rn(a[0], b[0]));
        Df r2 = df_sqr(Df{d.x, d.y});
        if (kp.dim >= 2) {
            d = df_split_fast(__dsub_rn(a[1], b[1]));
            r2 = df_add(r2, df_sqr(Df{d.x, d.y}));
        }
        if (kp.dim == 3) {
            d = df_split_fast(__dsub_rn(a[2], b[2]));
            r2 = df_add(r2, df_sqr(Df{d.x, d.y}));
        }
        r2 = df_fast(r2.h, r2.l);
        if (!(r2.h >= c.thr)) return from(kentry(kp, i, j));
        const Df v = df_mul(df_log(r2, c.tab), c.scale);
        return make_float2(v.h, v.l);
    }
    // renormalised pair of a + b (TwoSum of the high parts, the lows added)
    static __device__ __forceinline__ float2 add(float ah, float al, float bh, float bl) {
        const float s = __fadd_rn(ah, bh), bb = __fsub_rn(s, ah);
        const float e = __fadd_rn(__fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb)), __fadd_rn(al, bl));
        const float h = __fadd_rn(s, e);
        return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
    }
    static __device__ __forceinline__ float2 mul(float2 a, float2 b) {
        const float p = __fmul_rn(a.x, b.x);
        float e = __fmaf_rn(a.x, b.x, -p);
        e = __fmaf_rn(a.x, b.y, e);
        e = __fmaf_rn(a.y, b.x, e);
        const float h = __fadd_rn(p, e);
        return make_float2(h, __fsub_rn(e, __fsub_rn(h, p)));
    }
    static __device__ __forceinline__ float2 submul(float2 v, float2 c, float2 x) {
        const float p = __fmul_rn(c.x, x.x);
        float e = __fmaf_rn(c.x, x.x, -p);
        e = __fmaf_rn(c.x, x.y, e);
        e = __fmaf_rn(c.y, x.x, e);
        return add(v.x, v.y, -p, -e);
    }
    static __device__ __forceinline__ float2 inv(float2 p) { return from(1.0 / ((double)p.x + (double)p.y)); }
    static __device__ __forceinline__ float2 div(float2 c, float2 ip) { return mul(c, ip); }
    static __device__ __forceinline__ float sq(float2 e) { return e.x * e.x; }
    static __device__ __forceinline__ float dot(float2 a, float2 b) { return a.x * b.x; }
};

// Subtracts the kept terms l0..l1-1 (coefficients in shared memory) from the
// residual entries a (column base[0]) and b (base[off], when hb), in pivot
// order; NG_UNROLL terms are loaded before their subtractions.
constexpr int NG_UNROLL = 8;
template <class Op, class E>
__device__ __forceinline__ void ng_sub_terms(E &a, E &b, bool hb, const E *__restrict__ base, size_t ld, int off,
                                             const E *coef, int l0, int l1) {
    int l = l0;
    for (; l + NG_UNROLL <= l1; l += NG_UNROLL) {
        E xa[NG_UNROLL], xb[NG_UNROLL];
#pragma unroll
        for (int k = 0; k < NG_UNROLL; ++k) {
            xa[k] = base[(size_t)(l + k) * ld];
            xb[k] = hb ? base[(size_t)(l + k) * ld + off] : xa[k];
        }
#pragma unroll
        for (int k = 0; k < NG_UNROLL; ++k) {
            const E c = coef[l + k - l0];
            a = Op::submul(a, c, xa[k]);
            b = Op::submul(b, c, xb[k]);
        }
    }
    for (; l < l1; ++l) {
        const E c = coef[l - l0];
        a = Op::submul(a, c, base[(size_t)l * ld]);
        if (hb) b = Op::submul(b, c, base[(size_t)l * ld + off]);
    }
}
// Sum over the 32 lanes of each of d[0..7]: the lanes with (lane & 3) == 0
// return the sum of d[lane >> 2] (a butterfly that halves the values at
// each of the first three steps: 9 shuffles for 8 sums).
__device__ __forceinline__ float ng_reduce8(const float (&d)[8], int lane) {
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    float e[4], f[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float send = b4 ? d[i] : d[i + 4], keep = b4 ? d[i + 4] : d[i];
        e[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float send = b3 ? e[i] : e[i + 2], keep = b3 ? e[i + 2] : e[i];
        f[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    const float send = b2 ? f[0] : f[1], keep = b2 ? f[1] : f[0];
    float g = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    g += __shfl_xor_sync(0xffffffffu, g, 2);
    g += __shfl_xor_sync(0xffffffffu, g, 1);
    return g;
}

// ng_sub_terms for a whole warp (every lane calls it; ha / hb mark the
// lane's two entries), which also sums, per kept term l, <term l, newest
// term> over the warp's entries into wrow[l - l0] (pa, pb: the newest term's
// values at the two entries, zero where absent). Same residual operations in
// the same order as ng_sub_terms.
template <class Op, class E>
__device__ __forceinline__ void ng_sub_terms_dots(E &a, E &b, bool ha, bool hb, const E *__restrict__ base, size_t ld,
                                                  int off, const E *coef, int l0, int l1, E pa, E pb, float *wrow,
                                                  int lane) {
    const E z = Op::from(0.0);
    int l = l0;
    for (; l + NG_UNROLL <= l1; l += NG_UNROLL) {
        E xa[NG_UNROLL], xb[NG_UNROLL];
#pragma unroll
        for (int k = 0; k < NG_UNROLL; ++k) {
            xa[k] = ha ? base[(size_t)(l + k) * ld] : z;
            xb[k] = hb ? base[(size_t)(l + k) * ld + off] : z;
        }
        float d[NG_UNROLL];
#pragma unroll
        for (int k = 0; k < NG_UNROLL; ++k) {
            const E c = coef[l + k - l0];
            a = Op::submul(a, c, xa[k]);
            b = Op::submul(b, c, xb[k]);
            d[k] = Op::dot(xa[k], pa) + Op::dot(xb[k], pb);
        }
        const float g = ng_reduce8(d, lane);
        if ((lane & 3) == 0) wrow[l - l0 + (lane >> 2)] += g;
    }
    for (; l < l1; ++l) {
        const E c = coef[l - l0];
        const E x1 = ha ? base[(size_t)l * ld] : z, x2 = hb ? base[(size_t)l * ld + off] : z;
        a = Op::submul(a, c, x1);
        b = Op::submul(b, c, x2);
        float d = Op::dot(x1, pa) + Op::dot(x2, pb);
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (lane == 0) wrow[l - l0] += d;
    }
}

// The CTA's fused sums of nl kept terms: the warps' rows added in warp
// order, written to out[0], out[2], ... (every thread calls it).
__device__ __forceinline__ void ng_wpart_out(const float *wpart, int nl, double *out) {
    __syncthreads();
    for (int q = threadIdx.x; q < nl; q += NG_THREADS) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < NG_THREADS / 32; ++w) s += wpart[w * NG_COEF + q];
        out[2 * q] = (double)s;
    }
}

// normS after the newest kept term (rank terms, norms nu, nv): 2 |<U_l, u>
// <V_l, v>| per term from the members' partial dots summed in member order,
// the terms split over the group's CTAs; then every CTA sums them in the
// same fixed order (the same normS everywhere).
__device__ __forceinline__ double ng_norms(const double *dots, double *gterm, int dcap, int g, int G, int S, int gi,
                                           int rank, double nu, double nv, double normS, double *shs, unsigned *bar,
                                           int32_t *err) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int l = gi * NG_THREADS + tid; l < rank; l += S * NG_THREADS) {
        double du = 0.0, dv = 0.0;
        for (int k = 0; k < S; ++k) {
            const double *dk = dots + (size_t)(g + k * G) * 2 * dcap;
            du += dk[2 * l];
            dv += dk[2 * l + 1];
        }
        gterm[l] = 2.0 * fabs(du * dv);
    }
    ng_barrier(bar, S, err);
    double part = 0.0;
    for (int l = tid; l < rank; l += NG_THREADS) part += gterm[l];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) shs[warp] = part;
    __syncthreads();
    double ns = normS * normS + (nu * nv) * (nu * nv);
    for (int q = 0; q < NG_THREADS / 32; ++q) ns += shs[q];
    __syncthreads();
    return sqrt(ns);
}

// The last chunk's step for residual-column entry t: scaled by the pivot,
// stored, its square summed, the row-pivot candidate updated.
template <class Op, class E>
__device__ __forceinline__ void ng_col_final(E c, int t, E piv, int ri, const uint32_t *rm, E *Ur,
                                             typename Op::Acc &us, typename Op::Mag &u0, int &j0) {
    const E u = Op::div(c, piv);
    Ur[t] = u;
    us += Op::sq(u);
    if (t != ri && !ng_bit(rm, t)) {
        const typename Op::Mag a = Op::mag(c);
        if (ng_better(a, t, u0, j0)) { u0 = a; j0 = t; }
    }
}

// One lane's share of <a, b> over a CTA's chunks of NG_THREADS entries
// (first entry t0, chunks cstride apart), summed in entry order; the loads of
// a full chunk are issued before its products.
template <class Op, class E>
__device__ __forceinline__ void ng_dot_part(const E *__restrict__ a, const E *__restrict__ b, int n, int t0,
                                            int cstride, typename Op::Acc &d) {
    constexpr int K = NG_THREADS / 32;
    for (; t0 < n; t0 += cstride) {
        if (t0 + 32 * (K - 1) < n) {
            E xa[K], xb[K];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                xa[k] = a[t0 + 32 * k];
                xb[k] = b[t0 + 32 * k];
            }
#pragma unroll
            for (int k = 0; k < K; ++k) d += Op::dot(xa[k], xb[k]);
        } else {
            for (int t = t0; t < n; t += 32) d += Op::dot(a[t], b[t]);
        }
    }
}

template <class E>
__global__ void __launch_bounds__(NG_THREADS, 2)
    nca_group_kernel(const NcaProb *__restrict__ probs, const int64_t *__restrict__ moff, int nprob, int G,
                     const int32_t *__restrict__ idx, KParams kp, double tol, E *__restrict__ scr,
                     uint32_t *__restrict__ masks, int32_t *__restrict__ rank_out, int32_t *__restrict__ prow,
                     int32_t *__restrict__ pcol, int32_t *status, unsigned *bars, int32_t *err, NgPart *prow_part,
                     NgPart *pcol_part, double *dots, int dcap, const DfLogTab *__restrict__ logtab) {
    using Op = NgOps<E>;
    using Acc = typename Op::Acc;
    __shared__ E ng_coef[NG_COEF];
    __shared__ double shv[32], shs[32];
    __shared__ int shi[32];
    __shared__ float ng_wpart[Op::kFuse ? (NG_THREADS / 32) * NG_COEF : 1];  // per-warp fused sums
    __shared__ DfLogTab ng_tab[Op::kFuse ? 128 : 1];
    using Mag = typename Op::Mag;
    NgEnt ent{ng_tab, Df{0.f, 0.f}, 0.f};
    if (Op::kFuse) {
        for (int q = threadIdx.x; q < 128; q += NG_THREADS) ng_tab[q] = logtab[q];
        // log(R) = log(R^2) / 2 (1D), c2d log(R^2) (2D), log(R) / log(a) for R >= a = 1e-4 (3D)
        const double sc = kp.dim == 1 ? 0.5 : kp.dim == 2 ? kp.c2d : 0.5 / kp.loga;
        const float2 sp = NgOps<float2>::from(sc);
        ent.scale = Df{sp.x, sp.y};
        ent.thr = kp.dim == 3 ? 1.0001e-8f : 1e-30f;
        __syncthreads();
    }
    const int g = blockIdx.x % G, gi = blockIdx.x / G;
    const int S = (gridDim.x - g + G - 1) / G;  // members of group g
    unsigned *bar = bars + 2 * g;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int cstride = S * NG_THREADS;
    const double tiny = 1e-36;
    double *gterm = dots + (size_t)gridDim.x * 2 * dcap + (size_t)g * dcap;  // the group's normS terms
    for (int b = g; b < nprob; b += G) {
        const NcaProb pb = probs[b];
        const int n1 = pb.n1, n2 = pb.n2, rcap = pb.rcap;
        const int32_t *I = idx + pb.ri, *J = idx + pb.ci;
        E *U = scr + pb.u, *V = scr + pb.v;
        uint32_t *rm = masks + moff[b], *cm = rm + (n1 + 31) / 32;
        for (int q = gi * NG_THREADS + tid; q < (n1 + 31) / 32 + (n2 + 31) / 32; q += cstride) rm[q] = 0u;
        if (gi == 0 && tid == 0) rank_out[b] = 0;
        ng_barrier(bar, S, err);
        const int mn = n1 < n2 ? n1 : n2;
        if (mn == 0 || rcap == 0) continue;
        // first pivot row: the first row whose largest |entry| exceeds 1e-36
        int ri = -1, ci = -1;
        double bv, ss;
        int bi;
        for (int l = 0; l < n1 && ri < 0; ++l) {
            double v0 = -1.0;
            int i0 = INT_MAX;
            for (int s2 = gi * NG_THREADS + tid; s2 < n2; s2 += cstride) {
                const double v = kentry(kp, I[l], J[s2]);
                V[s2] = Op::from(v);
                const double a = fabs(v);
                if (ng_better(a, s2, v0, i0)) { v0 = a; i0 = s2; }
            }
            ng_cta_part(v0, i0, 0.0, prow_part + blockIdx.x, shv, shi, shs);
            ng_barrier(bar, S, err);
            ng_group(prow_part, g, G, S, bv, bi, ss);
            if (bv > tiny) { ri = l; ci = bi; }
            ng_barrier(bar, S, err);  // the partials are read before the next row overwrites them
        }
        if (ri < 0) continue;
        const E piv0 = Op::inv(V[ci]);
        // first column; the first row's squares
        {
            double v0 = -1.0;
            Acc us = 0, vs = 0;
            int i0 = INT_MAX;
            for (int t = gi * NG_THREADS + tid; t < n1; t += cstride) {
                const double c = kentry(kp, I[t], J[ci]);
                const E u = Op::div(Op::from(c), piv0);
                U[t] = u;
                us += Op::sq(u);
                if (t != ri) {
                    const double a = fabs(c);
                    if (ng_better(a, t, v0, i0)) { v0 = a; i0 = t; }
                }
            }
            for (int s2 = gi * NG_THREADS + tid; s2 < n2; s2 += cstride) vs += Op::sq(V[s2]);
            ng_cta_part(v0, i0, (double)us, pcol_part + blockIdx.x, shv, shi, shs);
            ng_cta_part(-1.0, INT_MAX, (double)vs, prow_part + blockIdx.x, shv, shi, shs);
        }
        ng_barrier(bar, S, err);
        double nu, nv;
        {
            double a;
            int nri;
            ng_group(pcol_part, g, G, S, a, nri, nu);
            nu = sqrt(nu);
            double dummy;
            int di;
            ng_group(prow_part, g, G, S, dummy, di, nv);
            nv = sqrt(nv);
            if (gi == 0 && tid == 0) {
                prow[pb.piv] = ri;
                pcol[pb.piv] = ci;
                rm[ri >> 5] |= 1u << (ri & 31);
                cm[ci >> 5] |= 1u << (ci & 31);
            }
            ri = nri;
        }
        int rank = 1;
        double normS = 0.0;
        bool over = false;
        // pend: the newest term's normS terms are not summed yet. The
        // double-FP32 search sums them inside the next pivot's two residual
        // passes, which read every kept term anyway, and drops that pivot
        // when the stopping test then says stop (the same pivots, one
        // traversal of the kept terms per pivot instead of two); the FP64
        // search, and a next pivot that cannot start, sum them in a pass of
        // their own.
        constexpr bool kFuse = Op::kFuse;
        bool pend = false;
        float *wrow = ng_wpart + (kFuse ? warp * NG_COEF : 0);
        double *dme = dots + (size_t)blockIdx.x * 2 * dcap;
        ng_barrier(bar, S, err);
        for (;;) {
            if (!pend && !(nu * nv > tol * normS)) break;
            if (rank >= mn) break;
            if (pend && (!kFuse || rank >= rcap || ri < 0 || ri >= n1)) {
                // this CTA's partial dots of every kept u, v with the newest
                // ones (the newest included), one warp per term, over the
                // CTA's rows and columns in a fixed order
                const E *Up = U + (size_t)(rank - 1) * n1, *Vp = V + (size_t)(rank - 1) * n2;
                for (int l = warp; l < rank; l += NG_THREADS / 32) {
                    const E *Ul = U + (size_t)l * n1, *Vl = V + (size_t)l * n2;
                    Acc du = 0, dv = 0;
                    ng_dot_part<Op, E>(Ul, Up, n1, gi * NG_THREADS + lane, cstride, du);
                    ng_dot_part<Op, E>(Vl, Vp, n2, gi * NG_THREADS + lane, cstride, dv);
                    for (int o = 16; o > 0; o >>= 1) {
                        du += __shfl_xor_sync(0xffffffffu, du, o);
                        dv += __shfl_xor_sync(0xffffffffu, dv, o);
                    }
                    if (lane == 0) {
                        dme[2 * l] = (double)du;
                        dme[2 * l + 1] = (double)dv;
                    }
                }
                ng_barrier(bar, S, err);
                normS = ng_norms(dots, gterm, dcap, g, G, S, gi, rank, nu, nv, normS, shs, bar, err);
                pend = false;
                ng_barrier(bar, S, err);  // the terms are read before the next step overwrites them
                continue;
            }
            if (rank >= rcap) {
                over = true;
                break;
            }
            if (ri < 0 || ri >= n1) {
                if (gi == 0 && tid == 0) atomicOr(status, 2);
                break;
            }
            const bool fuse = kFuse && pend;
            // residual row ri over this CTA's columns (kept terms subtracted in
            // pivot order, chunk by chunk); column pivot. The loop over column
            // pairs runs warp-uniform (the fused sums reduce across lanes).
            E *Vr = V + (size_t)rank * n2;
            const E *Vp = Vr - n2;
            Mag v0 = -1;
            Acc vs = 0;
            int i0 = INT_MAX;
            for (int l0 = 0; l0 < rank; l0 += NG_COEF) {
                const int l1 = rank - l0 < NG_COEF ? rank : l0 + NG_COEF;
                const bool last = l1 == rank;
                __syncthreads();
                for (int l = l0 + tid; l < l1; l += NG_THREADS) ng_coef[l - l0] = U[(size_t)l * n1 + ri];
                if (fuse)
                    for (int q = lane; q < NG_COEF; q += 32) wrow[q] = 0.f;
                __syncthreads();
                // two columns per thread and NG_UNROLL kept terms loaded ahead of
                // their subtractions: the loads of a term do not wait on the
                // previous subtraction (same operations, same order per entry)
                for (int sb = gi * NG_THREADS + warp * 32; sb < n2; sb += 2 * cstride) {
                    const int s2 = sb + lane, s2b = s2 + cstride;
                    const bool ha = s2 < n2, hb = s2b < n2;
                    E va = Op::from(0.0), vb = Op::from(0.0);
                    if (ha) va = l0 == 0 ? Op::entry(kp, I[ri], J[s2], ent) : Vr[s2];
                    if (hb) vb = l0 == 0 ? Op::entry(kp, I[ri], J[s2b], ent) : Vr[s2b];
                    if (fuse) {
                        const E pa = ha ? Vp[s2] : Op::from(0.0), pv = hb ? Vp[s2b] : Op::from(0.0);
                        ng_sub_terms_dots<Op, E>(va, vb, ha, hb, V + (ha ? s2 : 0), (size_t)n2, cstride, ng_coef, l0,
                                                 l1, pa, pv, wrow, lane);
                    } else if (ha) {
                        ng_sub_terms<Op, E>(va, vb, hb, V + s2, (size_t)n2, cstride, ng_coef, l0, l1);
                    }
                    if (!ha) continue;
                    Vr[s2] = va;
                    if (hb) Vr[s2b] = vb;
                    if (last) {
                        vs += Op::sq(va);
                        if (!ng_bit(cm, s2)) {
                            const Mag a = Op::mag(va);
                            if (ng_better(a, s2, v0, i0)) { v0 = a; i0 = s2; }
                        }
                        if (hb) {
                            vs += Op::sq(vb);
                            if (!ng_bit(cm, s2b)) {
                                const Mag a = Op::mag(vb);
                                if (ng_better(a, s2b, v0, i0)) { v0 = a; i0 = s2b; }
                            }
                        }
                    }
                }
                if (fuse) ng_wpart_out(ng_wpart, l1 - l0, dme + 2 * l0 + 1);
            }
            ng_cta_part((double)v0, i0, (double)vs, prow_part + blockIdx.x, shv, shi, shs);
            ng_barrier(bar, S, err);
            ng_group(prow_part, g, G, S, bv, bi, ss);
            if (bi < 0 || bi >= n2) {
                if (gi == 0 && tid == 0) atomicOr(status, 2);
                break;
            }
            ci = bi;
            const double cnv = sqrt(ss);
            const E piv = Op::inv(Vr[ci]);
            // residual column ci over this CTA's rows; next row pivot. The
            // unscaled residual is kept in Ur across chunks, scaled by the
            // pivot after the last one.
            E *Ur = U + (size_t)rank * n1;
            const E *Up = Ur - n1;
            Mag u0 = -1;
            Acc us = 0;
            int j0 = INT_MAX;
            for (int l0 = 0; l0 < rank; l0 += NG_COEF) {
                const int l1 = rank - l0 < NG_COEF ? rank : l0 + NG_COEF;
                const bool last = l1 == rank;
                __syncthreads();
                for (int l = l0 + tid; l < l1; l += NG_THREADS) ng_coef[l - l0] = V[(size_t)l * n2 + ci];
                if (fuse)
                    for (int q = lane; q < NG_COEF; q += 32) wrow[q] = 0.f;
                __syncthreads();
                for (int tbase = gi * NG_THREADS + warp * 32; tbase < n1; tbase += 2 * cstride) {
                    const int t = tbase + lane, tb = t + cstride;
                    const bool ha = t < n1, hb = tb < n1;
                    E ca = Op::from(0.0), cb = Op::from(0.0);
                    if (ha) ca = l0 == 0 ? Op::entry(kp, I[t], J[ci], ent) : Ur[t];
                    if (hb) cb = l0 == 0 ? Op::entry(kp, I[tb], J[ci], ent) : Ur[tb];
                    if (fuse) {
                        const E pa = ha ? Up[t] : Op::from(0.0), pv = hb ? Up[tb] : Op::from(0.0);
                        ng_sub_terms_dots<Op, E>(ca, cb, ha, hb, U + (ha ? t : 0), (size_t)n1, cstride, ng_coef, l0,
                                                 l1, pa, pv, wrow, lane);
                    } else if (ha) {
                        ng_sub_terms<Op, E>(ca, cb, hb, U + t, (size_t)n1, cstride, ng_coef, l0, l1);
                    }
                    if (!ha) continue;
                    if (!last) {
                        Ur[t] = ca;
                        if (hb) Ur[tb] = cb;
                        continue;
                    }
                    ng_col_final<Op, E>(ca, t, piv, ri, rm, Ur, us, u0, j0);
                    if (hb) ng_col_final<Op, E>(cb, tb, piv, ri, rm, Ur, us, u0, j0);
                }
                if (fuse) ng_wpart_out(ng_wpart, l1 - l0, dme + 2 * l0);
            }
            ng_cta_part((double)u0, j0, (double)us, pcol_part + blockIdx.x, shv, shi, shs);
            ng_barrier(bar, S, err);
            int nri;
            ng_group(pcol_part, g, G, S, bv, nri, ss);
            const double cnu = sqrt(ss);
            if (fuse) {
                // the newest kept term's normS terms, then its stopping test:
                // on stop the pivot just searched is dropped
                normS = ng_norms(dots, gterm, dcap, g, G, S, gi, rank, nu, nv, normS, shs, bar, err);
                pend = false;
                if (!(nu * nv > tol * normS)) break;
            }
            if (cnu < 1e-36 || cnv < 1e-36) break;
            if (gi == 0 && tid == 0) {
                prow[pb.piv + rank] = ri;
                pcol[pb.piv + rank] = ci;
                rm[ri >> 5] |= 1u << (ri & 31);
                cm[ci >> 5] |= 1u << (ci & 31);
            }
            ++rank;
            nu = cnu;
            nv = cnv;
            ri = nri;
            pend = true;
        }
        // an overflowing block reports -rank: the host runs it again with more scratch
        if (gi == 0 && tid == 0) rank_out[b] = over ? -rank : rank;
        ng_barrier(bar, S, err);
    }
}

static int ng_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

int nca_group_grid(int dcap, bool df) {
    (void)dcap;  // shared memory no longer depends on the rank
    int per_sm = 0;
    if (df) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nca_group_kernel<float2>, NG_THREADS, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nca_group_kernel<double>, NG_THREADS, 0);
    return per_sm > 0 ? ng_sms() * per_sm : 0;
}

cudaError_t launch_nca_group(const NcaProb *probs, const int64_t *moff, int nprob, int G, int grid,
                             const int32_t *idx, const KParams &kp, double tol, double *scr, uint32_t *masks,
                             int32_t *rank, int32_t *prow, int32_t *pcol, int32_t *status, unsigned *bars,
                             int32_t *err, void *prow_part, void *pcol_part, double *dots, int dcap, bool df,
                             const void *logtab, cudaStream_t st) {
    if (nprob <= 0) return cudaSuccess;
    NgPart *pr = reinterpret_cast<NgPart *>(prow_part), *pc = reinterpret_cast<NgPart *>(pcol_part);
    const DfLogTab *tab = reinterpret_cast<const DfLogTab *>(logtab);
    void *args[] = {(void *)&probs, (void *)&moff, (void *)&nprob, (void *)&G,    (void *)&idx,  (void *)&kp,
                    (void *)&tol,   (void *)&scr,  (void *)&masks, (void *)&rank, (void *)&prow, (void *)&pcol,
                    (void *)&status, (void *)&bars, (void *)&err, (void *)&pr,   (void *)&pc,   (void *)&dots,
                    (void *)&dcap,  (void *)&tab};
    const void *fn = df ? (const void *)nca_group_kernel<float2> : (const void *)nca_group_kernel<double>;
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(NG_THREADS), args, 0, st);
    count_launch();
    return e;
}

size_t nca_group_part_bytes() { return sizeof(NgPart); }

}  // namespace h2w
