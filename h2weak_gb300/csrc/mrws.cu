// Warp-specialised FP32 multi-vector product on the dataflow launch (sm_103a).
//
// The same packed target records, dependency counts and claim order as
// mr_flow_kernel in multi.cu; the work of a CTA is split by role:
//
//  * one producer warp claims targets, reads their records (plain loads from
//    L1/L2), waits for each target's producer count, and streams its chunks
//    (32 operator columns x the tile's rows, and the 32 gathered source rows
//    of RP vectors) into a ring of MW_NS shared-memory stages with bulk
//    asynchronous copies (cp.async.bulk, completing on the stage's "full"
//    mbarrier): one copy per operator chunk, one per run of consecutive
//    source rows;
//  * 4 RP consumer threads (8 warps at RP = 64) multiply each stage as it
//    lands (4 rows x 4 vectors per thread; a tile of at most 32 or 16 rows
//    splits the stage's columns over the otherwise idle row groups, whose
//    partial sums meet in shared memory), free it on its "empty" mbarrier,
//    write the tile's rows with the target's write mode after its last
//    chunk, and the last warp done with a target releases its consumers.
//    The consumer warps never wait on one another at a barrier: their
//    hand-offs are shared-memory counters with bounded waits.
//
// The producer runs up to MW_NS chunks ahead, across target boundaries, so
// the record reads, dependency waits and copy latency of the next target
// overlap the current target's multiply, epilogue and release.
//
// Copies: the kernel reads a slice-contiguous copy of the FP32 operator
// (each target's panel slice stored on its own at leading dimension
// pad4(rows), launch_slice_copy_f32), so a chunk is one copy of
// 4 * pad4(rows) * 32 bytes at a 16-byte aligned address. Given any other
// layout it falls back to one copy per column (tiles of a target of more
// than 64 rows) or, for panels off the 16-byte rule, to the producer's own
// stores, as it does for gathered columns without a source. Rows past a
// tile's last row and columns past a chunk's width are never used: a row's
// result reads only its own operator row, and the consumers' column loop
// stops at the chunk width.
//
// Every wait is bounded: a dependency wait that runs out sets *err = 3, an
// mbarrier wait *err = 4, and the thread carries on, so the kernel always
// ends. The launch is cooperative (every CTA resident), as the dependency
// waits require.
#include "kernels.cuh"

namespace h2w {
namespace {

constexpr int MW_KC = 32;  // operator columns per chunk
constexpr int MW_MT = 64;  // result rows per tile
constexpr int MW_NS = 3;   // shared-memory stages

// one stage's chunk: t < 0 ends the stream; last bit 0 marks the tile's last
// chunk, bit 1 the target's last tile
struct MwMeta {
    int64_t dst;
    int32_t nrows, flags, rt0, kw, t, last, astride, pad;  // astride: floats between staged operator columns
};

template <int RP> struct MwLayout {
    static constexpr int CN = 4 * RP;  // consumer threads: 16 row groups x RP/4 vector groups
    static constexpr int NT = CN + 32;
    static constexpr size_t a_bytes = (size_t)4 * MW_KC * MW_MT;
    static constexpr size_t stage = a_bytes + (size_t)4 * MW_KC * RP;
    static constexpr size_t map_off = MW_NS * stage;
    static constexpr size_t red_off = map_off + (size_t)4 * MR_XS_ELEMS;  // k-part partials of a short tile
    static constexpr size_t bar_off = red_off + (size_t)4 * 48 * RP;
    static constexpr size_t meta_off = bar_off + (size_t)16 * MW_NS;
    // int32 words: [0] set by a wait that ran out, [1] split-K partial writers
    // done, [2] partial readers done, [4 .. 11] consumer warps done with the
    // target of sequence number i (mod 8)
    static constexpr size_t fail_off = meta_off + sizeof(MwMeta) * MW_NS;
    static constexpr size_t smem = fail_off + 48;
};

__device__ __forceinline__ uint32_t mw_sa(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mw_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mw_sa(b)) : "memory");
}
__device__ __forceinline__ void mw_arrive_tx(uint64_t *b, uint32_t tx) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mw_sa(b)), "r"(tx) : "memory");
}
__device__ __forceinline__ void mw_bulk(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     mw_sa(dst)),
                 "l"(src), "r"(bytes), "r"(mw_sa(b))
                 : "memory");
}
// bounded wait of this thread for the mbarrier phase of the given parity;
// after any wait of the CTA ran out (*fail set), waits return at once
__device__ __forceinline__ void mw_wait(uint64_t *b, uint32_t par, volatile int32_t *fail, int32_t *err) {
    uint32_t done = 0;
    for (int it = 0; it < (1 << 20) && !done && !*fail; ++it)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done)
                     : "r"(mw_sa(b)), "r"(par)
                     : "memory");
    if (!done && !*fail) {
        *fail = 1;
        atomicExch(err, 4);
    }
}
// bounded wait of a warp's lane 0 until the shared counter reaches want
__device__ __forceinline__ void mw_until(volatile int32_t *c, int32_t want, volatile int32_t *fail, int32_t *err) {
    if ((threadIdx.x & 31) == 0) {
        long long it = 0;
        while (*c - want < 0 && !*fail) {
            if (++it > (1LL << 22)) {
                *fail = 1;
                atomicExch(err, 4);
                break;
            }
        }
        __threadfence_block();
    }
    __syncwarp();
}
// log2 of the k-parts of a tile of `rows` rows: the idle row groups of a
// short tile take a share of each chunk's columns (parts stay warp-uniform:
// at most 2 for RP 16)
template <int RP> __device__ __forceinline__ int mw_kparts_log2(int rows) {
    return rows > 32 ? 0 : ((rows > 16 || RP == 16) ? 1 : 2);
}

template <int RP>
__device__ __forceinline__ void mw_produce(char *sm, const int64_t *__restrict__ roff,
                                           const int64_t *__restrict__ blob, int64_t nt, int32_t *ctr,
                                           const int32_t *rem, const float *__restrict__ A, const float *ws,
                                           const float *__restrict__ xin, int32_t *err) {
    using Lay = MwLayout<RP>;
    const int lane = threadIdx.x & 31;
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + Lay::bar_off), *empty = full + MW_NS;
    MwMeta *meta = reinterpret_cast<MwMeta *>(sm + Lay::meta_off);
    int32_t *map = reinterpret_cast<int32_t *>(sm + Lay::map_off);
    volatile int32_t *fail = reinterpret_cast<volatile int32_t *>(sm + Lay::fail_off);
    uint32_t g = 0;  // chunks sent: stage g % MW_NS, its fill number g / MW_NS
    auto acquire = [&]() -> int {
        const int s = (int)(g % MW_NS);
        const uint32_t n = g / MW_NS;
        if (n > 0) mw_wait(empty + s, (n - 1) & 1u, fail, err);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        return s;
    };
    int64_t t = blockIdx.x;
    while (t < nt) {
        const int64_t o = roff[t];
        const int64_t dst = blob[o], w1 = blob[o + 1], w2 = blob[o + 2];
        const int nrows = (int)(w1 & 0xffffffff), flags = (int)(w1 >> 32);
        const int np = (int)(w2 & 0xffffffff), ns = (int)(w2 >> 32);
        const int64_t *pan = blob + o + 3;
        const int64_t *seg = pan + 3 * np;
        int xend = 0, nch = 0;
        for (int q = 0; q < np; ++q) {
            const int w = (int)(pan[3 * q + 1] >> 32);
            xend = max(xend, (int)pan[3 * q + 2] + w);
            nch += (w + MW_KC - 1) / MW_KC;
        }
        // source map of the gathered columns (this warp's own table)
        for (int e = lane; e < xend; e += 32) map[e] = -1;
        __syncwarp();
        for (int s = 0; s < ns; ++s) {
            const int64_t src = seg[2 * s], sw = seg[2 * s + 1];
            const int len = (int)(sw & 0xffffffff), code = (int)(sw >> 32);
            const int xo = code >> 1;
            const bool gi = code & 1;
            for (int i = lane; i < len; i += 32) map[xo + i] = gi ? -(2 + (int)(src + i)) : (int)(src + i);
        }
        // the target's producers have written its workspace rows
        if (lane == 0) {
            long long it = 0;
            while (*((volatile const int32_t *)(rem + t)) > 0) {
                if (++it > (1LL << 20)) {
                    atomicExch(err, 3);
                    break;
                }
                __nanosleep(64);
            }
        }
        __syncwarp();
        __threadfence();
        asm volatile("fence.proxy.async.global;" ::: "memory");  // the copies read what generic stores wrote
        for (int rt0 = 0; rt0 < nrows; rt0 += MW_MT) {
            const int rows_t = min(MW_MT, nrows - rt0);
            const uint32_t abytes = 4u * (uint32_t)((rows_t + 3) & ~3);
            const int last_tile = rt0 + MW_MT >= nrows ? 2 : 0;
            int ci = 0;  // chunk of this tile
            for (int q = 0; q <= np; ++q) {
                // q == np: a tile without columns still sends one empty chunk (its epilogue writes zeros)
                if (q == np && nch > 0) break;
                const int64_t pa = q < np ? pan[3 * q] : 0;
                const int lda = q < np ? (int)(pan[3 * q + 1] & 0xffffffff) : 0;
                const int w = q < np ? (int)(pan[3 * q + 1] >> 32) : 0;
                const int xoff = q < np ? (int)pan[3 * q + 2] : 0;
                const bool vec = ((pa & 3) == 0) && ((lda & 3) == 0);
                // a single-tile target whose panel is stored at its own padded height
                // has each chunk's columns in one contiguous block
                const bool whole = vec && rt0 == 0 && lda == (int)(abytes / 4);
                for (int c0 = 0; c0 < w || (q == np && c0 == 0); c0 += MW_KC) {
                    const int kw = min(MW_KC, w - c0);
                    const int s = acquire();
                    float *As = reinterpret_cast<float *>(sm + s * Lay::stage);
                    float *Xs = As + MW_KC * MW_MT;
                    const float *asrc = nullptr, *xsrc = nullptr;
                    uint32_t abytes_l = 0, xbytes_l = 0;
                    if (whole) {
                        if (lane == 0 && kw > 0) {
                            asrc = A + pa + (int64_t)c0 * lda;
                            abytes_l = 4u * (uint32_t)lda * (uint32_t)kw;
                        }
                    } else if (lane < kw) {
                        const float *p = A + pa + (int64_t)(c0 + lane) * lda + rt0;
                        if (vec) {
                            asrc = p;
                            abytes_l = abytes;
                        } else {
                            for (int r = 0; r < rows_t; ++r) As[lane * MW_MT + r] = p[r];
                        }
                    }
                    // source rows: runs of consecutive workspace (or input) rows go as one copy
                    const int m = lane < kw ? map[xoff + c0 + lane] : -1;
                    const int kind = m >= 0 ? 1 : (m <= -2 ? 2 : 0);
                    const int64_t idx = m >= 0 ? (int64_t)m : (int64_t)(-2 - m);
                    const int pkind = __shfl_up_sync(0xffffffffu, kind, 1);
                    const int64_t pidx = __shfl_up_sync(0xffffffffu, idx, 1);
                    const bool start = kind != 0 && !(lane > 0 && pkind == kind && pidx + 1 == idx);
                    const unsigned brk = __ballot_sync(0xffffffffu, start || kind == 0);
                    if (start) {
                        const unsigned after = brk & ~((2u << lane) - 1u);  // 2u << 31 wraps to 0: no lanes after
                        const int end = min(kw, after ? __ffs(after) - 1 : 32);
                        xsrc = (kind == 1 ? ws : xin) + idx * RP;
                        xbytes_l = 4u * RP * (uint32_t)(end - lane);
                    } else if (kind == 0 && lane < kw) {
                        for (int j = 0; j < RP; ++j) Xs[lane * RP + j] = 0.f;
                    }
                    uint32_t tx = abytes_l + xbytes_l;
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) tx += __shfl_xor_sync(0xffffffffu, tx, off);
                    ++ci;
                    if (lane == 0) {
                        MwMeta mm;
                        mm.dst = dst;
                        mm.nrows = nrows;
                        mm.flags = flags;
                        mm.rt0 = rt0;
                        mm.kw = max(kw, 0);
                        mm.t = (int32_t)t;
                        mm.last = (ci >= nch ? 1 : 0) | (ci >= nch ? last_tile : 0);
                        mm.astride = whole ? lda : MW_MT;
                        meta[s] = mm;
                    }
                    __syncwarp();  // this stage's own stores precede the arrival
                    if (lane == 0) mw_arrive_tx(full + s, tx);
                    __syncwarp();
                    if (asrc) mw_bulk(whole ? As : As + lane * MW_MT, asrc, abytes_l, full + s);
                    if (xsrc) mw_bulk(Xs + lane * RP, xsrc, xbytes_l, full + s);
                    ++g;
                }
            }
        }
        int64_t nx = 0;
        if (lane == 0) nx = gridDim.x + atomicAdd(ctr, 1);
        t = __shfl_sync(0xffffffffu, nx, 0);
    }
    const int s = acquire();
    if (lane == 0) {
        meta[s].t = -1;
        mw_arrive(full + s);
    }
}

template <int RP, class YT>
__device__ __forceinline__ void mw_consume(char *sm, const int64_t *__restrict__ coff,
                                           const int32_t *__restrict__ cidx, int32_t *rem, float *ws, YT *yout,
                                           int32_t *err) {
    using Lay = MwLayout<RP>;
    constexpr int CN = Lay::CN, NWARP = CN / 32;
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + Lay::bar_off), *empty = full + MW_NS;
    const MwMeta *meta = reinterpret_cast<const MwMeta *>(sm + Lay::meta_off);
    float *red = reinterpret_cast<float *>(sm + Lay::red_off);
    volatile int32_t *fail = reinterpret_cast<volatile int32_t *>(sm + Lay::fail_off);
    int32_t *wr = reinterpret_cast<int32_t *>(sm + Lay::fail_off) + 1, *rd = wr + 1, *done = wr + 3;
    const int tid = threadIdx.x, lane = tid & 31;
    const int ty = tid / (RP / 4), tx = tid % (RP / 4);
    int32_t wr_want = 0, rd_want = 0;  // partial writers / readers of all short tiles so far (every warp counts alike)
    uint32_t seq = 0;                  // targets completed
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (uint32_t g = 0;; ++g) {
        const int s = (int)(g % MW_NS);
        mw_wait(full + s, (g / MW_NS) & 1u, fail, err);
        const MwMeta m = meta[s];
        if (m.t < 0) break;
        const float *As = reinterpret_cast<const float *>(sm + s * Lay::stage);
        const float *Xs = As + MW_KC * MW_MT;
        const int ls = mw_kparts_log2<RP>(min(MW_MT, m.nrows - m.rt0)), S = 1 << ls, G = 16 >> ls;
        const int tyr = ty & (G - 1), kp = ty >> (4 - ls);
        const int kn = (m.kw + S - 1) >> ls, k0 = kp * kn, k1 = min(m.kw, k0 + kn);
        const bool active = m.rt0 + tyr * 4 < m.nrows;
        auto term = [&](int k) {
            const float4 a = *reinterpret_cast<const float4 *>(As + k * m.astride + tyr * 4);
            const float4 x = *reinterpret_cast<const float4 *>(Xs + k * RP + tx * 4);
            const float a4[4] = {a.x, a.y, a.z, a.w}, x4[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = __fmaf_rn(a4[i], x4[j], acc[i][j]);
        };
        if (active) {
            if (k1 - k0 == MW_KC) {  // a full chunk of a tall tile: compile-time trip count
#pragma unroll 8
                for (int k = 0; k < MW_KC; ++k) term(k);
            } else {
#pragma unroll 4
                for (int k = k0; k < k1; ++k) term(k);
            }
        }
        __syncwarp();
        if (lane == 0) mw_arrive(empty + s);
        if (!(m.last & 1)) continue;
        if (S > 1) {  // k-parts 1 .. S-1 add into part 0 through shared memory
            const int nr = RP >> (3 + ls), nw = NWARP - nr;  // warps of part 0, of the other parts
            if (kp > 0) {
                mw_until(rd, rd_want, fail, err);  // the previous short tile's partials are read
                if (active) {
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            red[(((kp - 1) * G + tyr) * 4 + i) * RP + tx * 4 + j] = acc[i][j];
                }
                __syncwarp();
                if (lane == 0) {
                    __threadfence_block();
                    atomicAdd(wr, 1);
                }
            } else {
                mw_until(wr, wr_want + nw, fail, err);  // this tile's partials are written
                if (active) {
                    for (int p = 1; p < S; ++p)
#pragma unroll
                        for (int i = 0; i < 4; ++i)
#pragma unroll
                            for (int j = 0; j < 4; ++j)
                                acc[i][j] += red[(((p - 1) * G + tyr) * 4 + i) * RP + tx * 4 + j];
                }
                __syncwarp();
                if (lane == 0) atomicAdd(rd, 1);
            }
            wr_want += nw;
            rd_want += nr;
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = m.rt0 + tyr * 4 + i;
            if (kp == 0 && r < m.nrows) {
                const int64_t d = (m.dst + r) * RP + tx * 4;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float v = acc[i][j];
                    const float prev = (m.flags & T_ACCUM) ? ws[d + j] : 0.f;
                    if (m.flags & T_SCATTER) yout[d + j] = (YT)((m.flags & T_ACCUM) ? prev + v : v);
                    else if (m.flags & T_ATOMIC) atomicAdd(ws + d + j, v);
                    else if (m.flags & T_ACCUM) ws[d + j] = prev + v;
                    else ws[d + j] = v;
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
        }
        if (m.last & 2) {
            // the last consumer warp done with the target releases its consumers (a
            // warp runs at most MW_NS stages, so targets, ahead of the slowest one)
            __syncwarp();
            int last = 0;
            if (lane == 0) {
                __threadfence();
                last = atomicAdd(done + (seq & 7), 1) == NWARP - 1;
                if (last) atomicExch(done + (seq & 7), 0);
            }
            last = __shfl_sync(0xffffffffu, last, 0);
            if (last) {
                __threadfence();
                for (int64_t e = coff[m.t] + lane; e < coff[m.t + 1]; e += 32) atomicSub(rem + cidx[e], 1);
            }
            ++seq;
        }
    }
}

template <int RP, class YT>
__global__ void __launch_bounds__(MwLayout<RP>::NT, 3)
    mw_flow_kernel(const int64_t *__restrict__ roff, const int64_t *__restrict__ blob, int64_t nt, int32_t *ctr,
                   int32_t *rem, const int64_t *__restrict__ coff, const int32_t *__restrict__ cidx,
                   const float *__restrict__ A, float *ws, const float *__restrict__ xin, YT *yout, int32_t *err) {
    using Lay = MwLayout<RP>;
    extern __shared__ __align__(128) char mw_smem[];
    uint64_t *full = reinterpret_cast<uint64_t *>(mw_smem + Lay::bar_off);
    if (threadIdx.x == 0) {
        for (int s = 0; s < MW_NS; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mw_sa(full + s)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mw_sa(full + MW_NS + s)), "r"(Lay::CN / 32));
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int i = 0; i < 12; ++i) reinterpret_cast<int32_t *>(mw_smem + Lay::fail_off)[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x >= Lay::CN) mw_produce<RP>(mw_smem, roff, blob, nt, ctr, rem, A, ws, xin, err);
    else mw_consume<RP, YT>(mw_smem, coff, cidx, rem, ws, yout, err);
}

int mw_num_sms() {
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
cudaError_t mw_launch(const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr, int32_t *rem,
                      const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const float *xin, YT *yout,
                      int32_t *err, cudaStream_t st) {
    using Lay = MwLayout<RP>;
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaFuncSetAttribute(mw_flow_kernel<RP, YT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)Lay::smem) != cudaSuccess)
            return cudaErrorInvalidValue;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mw_flow_kernel<RP, YT>, Lay::NT, Lay::smem);
        if (per_sm <= 0) return cudaErrorCooperativeLaunchTooLarge;
    }
    const int grid = mw_num_sms() * per_sm;
    void *args[] = {(void *)&roff, (void *)&blob, (void *)&nt, (void *)&ctr, (void *)&rem, (void *)&coff,
                    (void *)&cidx, (void *)&A, (void *)&ws, (void *)&xin, (void *)&yout, (void *)&err};
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)mw_flow_kernel<RP, YT>, dim3(grid), dim3(Lay::NT), args,
                                                Lay::smem, st);
    count_launch();
    return e;
}

template <class YT>
cudaError_t mw_dispatch(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr, int32_t *rem,
                        const int64_t *coff, const int32_t *cidx, const float *A, float *ws, const float *xin,
                        YT *yout, int32_t *err, cudaStream_t st) {
    switch (rp) {
    case 16: return mw_launch<16, YT>(roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
    case 32: return mw_launch<32, YT>(roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
    case 64: return mw_launch<64, YT>(roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

// one CTA per slice
__global__ void slice_copy_kernel(const float *__restrict__ src, const int64_t *__restrict__ sl, float *dst) {
    const int64_t *d = sl + 6 * (int64_t)blockIdx.x;
    const int64_t a = d[0], lda = d[1], rows = d[2], w = d[3], o = d[4], ld = d[5];
    for (int64_t e = threadIdx.x; e < ld * w; e += blockDim.x) {
        const int64_t c = e / ld, r = e - c * ld;
        dst[o + e] = r < rows ? src[a + c * lda + r] : 0.f;
    }
}
cudaError_t launch_slice_copy_f32(const float *src, const int64_t *slices, int64_t n, float *dst, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > (int64_t)INT32_MAX) return cudaErrorInvalidValue;
    slice_copy_kernel<<<(unsigned)n, 256, 0, st>>>(src, slices, dst);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_mw_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr,
                               int32_t *rem, const int64_t *coff, const int32_t *cidx, const float *A, float *ws,
                               const float *xin, double *yout, int32_t *err, cudaStream_t st) {
    return mw_dispatch<double>(rp, roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
}
cudaError_t launch_mw_f32_flow(int rp, const int64_t *roff, const int64_t *blob, int64_t nt, int32_t *ctr,
                               int32_t *rem, const int64_t *coff, const int32_t *cidx, const float *A, float *ws,
                               const float *xin, float *yout, int32_t *err, cudaStream_t st) {
    return mw_dispatch<float>(rp, roff, blob, nt, ctr, rem, coff, cidx, A, ws, xin, yout, err, st);
}

}  // namespace h2w
