// Tensor-core form of the FP32 multi-vector product (sm_103a, tcgen05).
//
// Same packed target records, phases and dynamic target claiming as the
// FP32 FMA kernel in multi.cu: a target is a small GEMM, (rows <= 64) x RP =
// sum over its panels of A_p (rows x w_p) X_p (w_p x RP). Here the GEMM runs
// on the 5th-generation tensor cores:
//
//  * Operands are split for TF32 arithmetic, a = hi + lo with hi = tf32(a)
//    (round to nearest) and lo = a - hi (exact in FP32). One M = 128 A tile
//    holds hi in rows 0-63 and lo in rows 64-127, so the two MMAs per K step,
//    against X_hi and X_lo, form all four products hi*hi, hi*lo, lo*hi,
//    lo*lo with no padded rows; the epilogue adds row r and row r + 64.
//    Accuracy is that of an FP32 product (a few 2^-22 relative per term).
//  * Staging: 32 operator columns per chunk, loaded by all 256 threads with
//    coalesced loads (panel columns and gathered source rows), split, and
//    written as 16-byte units into K-major, no-swizzle canonical layouts
//    (8-row x 16-byte core matrices; 8-row groups 1040 bytes apart so that
//    the 16-byte stores of eight consecutive rows hit distinct banks).
//  * One elected thread issues tcgen05.mma (kind::tf32, M 128, N RP, K 8)
//    from shared-memory descriptors into an FP32 accumulator in tensor
//    memory and commits each chunk to that stage's mbarrier; the next chunk
//    is loaded and staged into the other stage meanwhile.
//  * Epilogue: four warps read the accumulator rows with tcgen05.ld, pass
//    them through shared memory, and all threads write the result rows with
//    the target's write mode (overwrite / accumulate / atomic / scatter).
//
// Every mbarrier wait is bounded: a wait that runs out sets *err (code 2)
// and the CTA carries on without waiting, so the kernel always ends; tensor
// memory is allocated once per CTA and freed before the kernel returns.
#include "kernels.cuh"
#include "sync.cuh"

namespace h2w {
namespace {

constexpr int TC_NT = 256;     // threads per CTA
constexpr int TC_KC = 32;      // operator columns per chunk
constexpr int TC_NS = 4;       // staging buffers (shared memory)
constexpr int TC_GROUP = 1040; // bytes between 8-row groups of a staged tile

template <int RP> struct TcLayout {
    static constexpr int a_bytes = 16 * TC_GROUP;       // 128 rows: hi 0-63, lo 64-127
    static constexpr int b_bytes = RP / 8 * TC_GROUP;   // RP rows
    static constexpr int stage = a_bytes + 2 * b_bytes; // A, X_hi, X_lo
    static constexpr int map_off = BRG_REC_WORDS * 8;
    static constexpr int stage_off = map_off + 4 * MR_XS_ELEMS;
    static constexpr int bar_off = stage_off + TC_NS * stage;
    static constexpr int smem = bar_off + 8 * TC_NS + 16;
    static constexpr int xrow = RP + 4;                 // epilogue exchange row (floats)
    static constexpr int nbq = (8 * RP + TC_NT - 1) / TC_NT;  // X quads per thread per chunk
    static constexpr uint32_t tmem_cols = RP < 32 ? 32 : RP;
    // instruction descriptor: D F32, A and B TF32, both K-major, N = RP, M = 128
    static constexpr uint32_t idesc =
        (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(RP >> 3) << 17) | ((128u >> 4) << 24);
    static_assert(RP % 16 == 0 && RP <= 64, "N");
    static_assert(2 * 64 * xrow * 4 <= TC_NS * stage, "epilogue exchange fits the staging buffers");
    static_assert(smem <= 227 * 1024, "one CTA per SM");
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t tf32_hi(float a) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(a));
    return r;
}
// shared-memory matrix descriptor: start, leading (K-direction) and stride
// (8-row group) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3fff) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(TC_GROUP >> 4) << 32) |
           (1ull << 46);
}
// byte offset of (row r, column quad kq) in a staged tile
__device__ __forceinline__ int tc_off(int r, int kq) { return (r >> 3) * TC_GROUP + kq * 128 + (r & 7) * 16; }

__device__ __forceinline__ void tc_st4(char *p, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(smem_u32(p)), "r"(a), "r"(b), "r"(c), "r"(d));
}
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
                 "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Pipeline state, uniform across the CTA: parity of the next wait and
// commits not yet waited, one bit per staging buffer.
struct TcPipe {
    uint32_t parity, pending;
    bool failed;
};
// One lane per warp polls (bounded) and shares the outcome with its warp.
__device__ __forceinline__ void tc_wait(TcPipe &pp, uint64_t *bars, int s, int32_t *err) {
    if (!((pp.pending >> s) & 1u)) return;
    pp.pending &= ~(1u << s);
    const uint32_t par = (pp.parity >> s) & 1u;
    pp.parity ^= 1u << s;
    if (pp.failed) return;
    uint32_t done = 0;
    if ((threadIdx.x & 31) == 0) {
        for (int it = 0; it < (1 << 24) && !done; ++it) {
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                : "=r"(done)
                : "r"(smem_u32(bars + s)), "r"(par)
                : "memory");
        }
    }
    done = __shfl_sync(0xffffffffu, done, 0);
    if (!done) {
        pp.failed = true;
        if ((threadIdx.x & 31) == 0) atomicExch(err, 2);
    }
}

template <int RP, class YT>
__device__ __forceinline__ void tc_target(char *smem, uint32_t tmem, TcPipe &pp, int64_t t,
                                          const int64_t *__restrict__ roff, const int64_t *__restrict__ blob,
                                          const float *__restrict__ A, float *ws, const float *__restrict__ xin,
                                          YT *yout, int32_t *err) {
    using L = TcLayout<RP>;
    int64_t *rec = reinterpret_cast<int64_t *>(smem);
    int32_t *map = reinterpret_cast<int32_t *>(smem + L::map_off);
    char *stg = smem + L::stage_off;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::bar_off);
    const int tid = threadIdx.x, warp = tid / 32;

    const int64_t o = roff[t];
    const int nw = (int)(roff[t + 1] - o);
    for (int q = tid; q < nw; q += TC_NT) rec[q] = blob[o + q];
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
    for (int e = tid; e < xend; e += TC_NT) map[e] = -1;
    __syncthreads();
    for (int s = 0; s < ns; ++s) {
        const int64_t src = seg[2 * s], w1 = seg[2 * s + 1];
        const int len = (int)(w1 & 0xffffffff), code = (int)(w1 >> 32);
        const int xo = code >> 1;
        const bool g = code & 1;
        for (int i = tid; i < len; i += TC_NT) map[xo + i] = g ? -(2 + (int)(src + i)) : (int)(src + i);
    }
    __syncthreads();

    // chunk registers: A quads (row m, columns 4kq..4kq+3), X quads (vector n,
    // columns 4kq..4kq+3). Four sets: the loads of chunks i+1 .. i+4 are in
    // flight while chunk i is multiplied (one CTA per SM holds tensor memory,
    // so the latency is hidden inside the CTA).
    struct Regs {
        float a[2][4], x[L::nbq][4];
    };
    Regs R0, R1, R2, R3;
    auto width = [&](int q) { return (int)(pan[3 * q + 1] >> 32); };
    auto advance = [&](int &q, int &c0) {
        if (q >= np) return;
        c0 += TC_KC;
        if (c0 >= width(q)) {
            ++q;
            c0 = 0;
        }
    };
    // chunk (panel q, columns c0 .. c0+31) of rows rt0 .. rt0+63 into registers
    auto load = [&](Regs &R, int q, int c0, int rt0) {
        const int64_t pa = pan[3 * q];
        const int lda = (int)(pan[3 * q + 1] & 0xffffffff), w = (int)(pan[3 * q + 1] >> 32);
        const int xoff = (int)pan[3 * q + 2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int qi = tid + TC_NT * u, m = qi & 63, kq = qi >> 6;
            const int r = rt0 + m;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = c0 + 4 * kq + j;
                R.a[u][j] = (c < w && r < nrows) ? A[pa + (int64_t)c * lda + r] : 0.f;
            }
        }
#pragma unroll
        for (int u = 0; u < L::nbq; ++u) {
            const int qi = tid + TC_NT * u, n = qi % RP, kq = qi / RP;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = c0 + 4 * kq + j;
                float v = 0.f;
                if (qi < 8 * RP && c < w) {
                    const int m = map[xoff + c];
                    if (m >= 0) v = ws[(int64_t)m * RP + n];
                    else if (m <= -2) v = xin[(int64_t)(-2 - m) * RP + n];
                }
                R.x[u][j] = v;
            }
        }
    };
    auto store = [&](const Regs &R, int s) {
        char *As = stg + s * L::stage, *Bh = As + L::a_bytes, *Bl = Bh + L::b_bytes;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int qi = tid + TC_NT * u, m = qi & 63, kq = qi >> 6;
            uint32_t h[4], l[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                h[j] = tf32_hi(R.a[u][j]);
                l[j] = __float_as_uint(R.a[u][j] - __uint_as_float(h[j]));
            }
            tc_st4(As + tc_off(m, kq), h[0], h[1], h[2], h[3]);
            tc_st4(As + tc_off(m + 64, kq), l[0], l[1], l[2], l[3]);
        }
#pragma unroll
        for (int u = 0; u < L::nbq; ++u) {
            const int qi = tid + TC_NT * u, n = qi % RP, kq = qi / RP;
            if (qi < 8 * RP) {
                uint32_t h[4], l[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    h[j] = tf32_hi(R.x[u][j]);
                    l[j] = __float_as_uint(R.x[u][j] - __uint_as_float(h[j]));
                }
                tc_st4(Bh + tc_off(n, kq), h[0], h[1], h[2], h[3]);
                tc_st4(Bl + tc_off(n, kq), l[0], l[1], l[2], l[3]);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    };
    // MMAs of the chunk in buffer s into the accumulator (the first one of a
    // row tile overwrites it), committed to that buffer's mbarrier
    auto mma = [&](int s, bool first) {
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(stg + s * L::stage);
            const uint32_t bh0 = a0 + L::a_bytes, bl0 = bh0 + L::b_bytes;
#pragma unroll
            for (int ks = 0; ks < TC_KC / 8; ++ks) {
                const uint64_t da = tc_desc(a0 + 256 * ks);
                tc_mma(tmem, da, tc_desc(bh0 + 256 * ks), L::idesc, (first && ks == 0) ? 0u : 1u);
                tc_mma(tmem, da, tc_desc(bl0 + 256 * ks), L::idesc, 1u);
            }
            tc_commit(bars + s);
        }
        pp.pending |= 1u << s;
    };

    for (int rt0 = 0; rt0 < nrows; rt0 += 64) {
        if (np > 0) {
            // cursors of chunks i+1 .. i+4 (q == np: past the end)
            int q1 = 0, c1 = 0;
            advance(q1, c1);
            int q2 = q1, c2 = c1;
            advance(q2, c2);
            int q3 = q2, c3 = c2;
            advance(q3, c3);
            int q4 = q3, c4 = c3;
            advance(q4, c4);
            load(R0, 0, 0, rt0);
            if (q1 < np) load(R1, q1, c1, rt0);
            if (q2 < np) load(R2, q2, c2, rt0);
            if (q3 < np) load(R3, q3, c3, rt0);
            tc_wait(pp, bars, 0, err);
            store(R0, 0);
            __syncthreads();
            int s = 0;
            bool first = true;
            // one chunk: multiply chunk i (buffer s), load chunk i+4 into the
            // registers chunk i came from, stage chunk i+1
            auto step = [&](Regs &Rload, const Regs &Rstore) {
                mma(s, first);
                first = false;
                if (q1 >= np) return false;
                if (q4 < np) load(Rload, q4, c4, rt0);
                s = s + 1 == TC_NS ? 0 : s + 1;
                tc_wait(pp, bars, s, err);
                store(Rstore, s);
                __syncthreads();
                q1 = q2; c1 = c2;
                q2 = q3; c2 = c3;
                q3 = q4; c3 = c4;
                advance(q4, c4);
                return true;
            };
            while (step(R0, R1) && step(R1, R2) && step(R2, R3) && step(R3, R0)) {
            }
            for (int b = 0; b < TC_NS; ++b) tc_wait(pp, bars, b, err);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        // epilogue: accumulator rows (lanes) 0-63 = hi part, 64-127 = lo part
        float *hb = reinterpret_cast<float *>(stg), *lb = hb + 64 * L::xrow;
        if (np > 0 && warp < 4) {
            const int row = 32 * warp + (tid & 31);
            float *dstrow = row < 64 ? hb + row * L::xrow : lb + (row - 64) * L::xrow;
#pragma unroll
            for (int cb = 0; cb < RP; cb += 16) {
                uint32_t v[16];
                const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)cb;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(ta));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 16; j += 4)
                    *reinterpret_cast<float4 *>(dstrow + cb + j) =
                        make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]), __uint_as_float(v[j + 2]),
                                    __uint_as_float(v[j + 3]));
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        const int nr = nrows - rt0 < 64 ? nrows - rt0 : 64;
        for (int e = tid; e < nr * (RP / 4); e += TC_NT) {
            const int r = e / (RP / 4), n4 = (e % (RP / 4)) * 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (np > 0) {
                const float4 h = *reinterpret_cast<const float4 *>(hb + r * L::xrow + n4);
                const float4 l = *reinterpret_cast<const float4 *>(lb + r * L::xrow + n4);
                v = make_float4(h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w);
            }
            const float vv[4] = {v.x, v.y, v.z, v.w};
            const int64_t d = (dst + rt0 + r) * RP + n4;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (flags & T_SCATTER) yout[d + j] = (YT)((flags & T_ACCUM) ? ws[d + j] + vv[j] : vv[j]);
                else if (flags & T_ATOMIC) atomicAdd(ws + d + j, vv[j]);
                else if (flags & T_ACCUM) ws[d + j] += vv[j];
                else ws[d + j] = vv[j];
            }
        }
        __syncthreads();
    }
}

template <int RP, class YT>
__device__ __forceinline__ void tc_phase(char *smem, uint32_t tmem, TcPipe &pp, int64_t t0, int64_t t1,
                                         int32_t *ctr, const int64_t *__restrict__ roff,
                                         const int64_t *__restrict__ blob, const float *__restrict__ A, float *ws,
                                         const float *__restrict__ xin, YT *yout, int32_t *err) {
    __shared__ int64_t s_next;
    int64_t t = t0 + blockIdx.x;
    while (t < t1) {
        tc_target<RP, YT>(smem, tmem, pp, t, roff, blob, A, ws, xin, yout, err);
        if (threadIdx.x == 0) s_next = t0 + gridDim.x + atomicAdd(ctr, 1);
        __syncthreads();
        t = s_next;
    }
}

// mbarriers and tensor memory for one CTA
template <int RP>
__device__ __forceinline__ uint32_t tc_setup(char *smem) {
    using L = TcLayout<RP>;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L::bar_off);
    uint32_t *slot = reinterpret_cast<uint32_t *>(smem + L::bar_off + 8 * TC_NS);
    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_NS; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + s)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x / 32 == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(L::tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return *slot;
}
template <int RP>
__device__ __forceinline__ void tc_teardown(uint32_t tmem) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (threadIdx.x / 32 == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TcLayout<RP>::tmem_cols));
}

template <int RP, class YT>
__global__ void __launch_bounds__(TC_NT, 1)
    mrt_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob, int64_t t0, int64_t t1, int32_t *ctr,
               const float *__restrict__ A, float *ws, const float *__restrict__ xin, YT *yout, int32_t *err) {
    extern __shared__ __align__(1024) char tc_smem[];
    const uint32_t tmem = tc_setup<RP>(tc_smem);
    TcPipe pp{0u, 0u, false};
    tc_phase<RP, YT>(tc_smem, tmem, pp, t0, t1, ctr, roff, blob, A, ws, xin, yout, err);
    tc_teardown<RP>(tmem);
}

template <int RP, class YT>
__global__ void __launch_bounds__(TC_NT, 1)
    mrt_coop_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob,
                    const int64_t *__restrict__ pstart, int nphase, int32_t *ctr, const float *__restrict__ A,
                    float *ws, const float *__restrict__ xin, YT *yout, unsigned *bar, int32_t *err) {
    extern __shared__ __align__(1024) char tc_smem[];
    const uint32_t tmem = tc_setup<RP>(tc_smem);
    TcPipe pp{0u, 0u, false};
    for (int p = 0; p < nphase; ++p) {
        tc_phase<RP, YT>(tc_smem, tmem, pp, pstart[p], pstart[p + 1], ctr + p, roff, blob, A, ws, xin, yout, err);
        if (p + 1 < nphase) grid_barrier(bar, gridDim.x, err);
    }
    tc_teardown<RP>(tmem);
}

int tc_num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int RP, class YT>
cudaError_t mrt_launch(const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                       const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin, YT *yout,
                       unsigned *bar, int32_t *err, cudaStream_t st) {
    using L = TcLayout<RP>;
    static int per_sm_coop = 0, per_sm = 0;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(mrt_coop_kernel<RP, YT>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::smem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(mrt_kernel<RP, YT>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::smem);
        if (e != cudaSuccess) return e;
        // all of the unified L1 / shared memory as shared memory: two CTAs per SM
        cudaFuncSetAttribute(mrt_coop_kernel<RP, YT>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaFuncSetAttribute(mrt_kernel<RP, YT>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        attr = true;
    }
    const int nsm = tc_num_sms();
    if (phased) {
        if (per_sm == 0) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mrt_kernel<RP, YT>, TC_NT, L::smem);
            if (per_sm <= 0) per_sm = 1;
        }
        for (int p = 0; p < phased->n; ++p) {
            const int64_t t0 = phased->t0[p], t1 = phased->t1[p];
            if (t1 <= t0) continue;
            const int64_t cap = (int64_t)nsm * per_sm;
            const int grid = (int)(t1 - t0 < cap ? t1 - t0 : cap);
            mrt_kernel<RP, YT><<<grid, TC_NT, L::smem, st>>>(roff, blob, t0, t1, ctr + p, A, ws, xin, yout, err);
            count_launch();
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    if (per_sm_coop == 0) {
        // CTAs per SM from the kernel's registers and shared memory (the
        // cooperative launch itself checks co-residency: a grid that does not
        // fit is refused with cudaErrorCooperativeLaunchTooLarge, and one CTA
        // fewer per SM is tried)
        cudaFuncAttributes fa{};
        int dev = 0, smem_sm = 0, regs_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
        if (cudaFuncGetAttributes(&fa, mrt_coop_kernel<RP, YT>) != cudaSuccess) return cudaErrorInvalidValue;
        const int per_block_smem = L::smem + (int)fa.sharedSizeBytes + 1024;
        const int per_block_regs = ((fa.numRegs + 7) / 8 * 8) * TC_NT;
        int n = per_block_smem > 0 ? smem_sm / per_block_smem : 1;
        if (per_block_regs > 0 && regs_sm / per_block_regs < n) n = regs_sm / per_block_regs;
        per_sm_coop = n < 1 ? 1 : (n > 4 ? 4 : n);
    }
    void *args[] = {(void *)&roff, (void *)&blob, (void *)&pstart, (void *)&nphase, (void *)&ctr, (void *)&A,
                    (void *)&ws,   (void *)&xin,  (void *)&yout,   (void *)&bar,    (void *)&err};
    while (true) {
        const int grid = nsm * per_sm_coop;
        cudaError_t e = cudaLaunchCooperativeKernel((const void *)mrt_coop_kernel<RP, YT>, dim3(grid), dim3(TC_NT), args,
                                                    L::smem, st);
        if (e == cudaErrorCooperativeLaunchTooLarge && per_sm_coop > 1) {
            cudaGetLastError();
            --per_sm_coop;
            continue;
        }
        count_launch();
        return e;
    }
}

}  // namespace

template <class YT>
static cudaError_t mrt_dispatch(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                                const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin,
                                YT *yout, unsigned *bar, int32_t *err, cudaStream_t st) {
    switch (rp) {
    case 16: return mrt_launch<16, YT>(roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
    case 32: return mrt_launch<32, YT>(roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
    case 64: return mrt_launch<64, YT>(roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
    default: return cudaErrorInvalidValue;
    }
}
cudaError_t launch_mrt_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                           const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin,
                           double *yout, unsigned *bar, int32_t *err, cudaStream_t st) {
    return mrt_dispatch(rp, roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
}
cudaError_t launch_mrt_f32(int rp, const int64_t *roff, const int64_t *blob, const int64_t *pstart, int nphase,
                           const MrPhases *phased, int32_t *ctr, const float *A, float *ws, const float *xin,
                           float *yout, unsigned *bar, int32_t *err, cudaStream_t st) {
    return mrt_dispatch(rp, roff, blob, pstart, nphase, phased, ctr, A, ws, xin, yout, bar, err, st);
}

}  // namespace h2w
