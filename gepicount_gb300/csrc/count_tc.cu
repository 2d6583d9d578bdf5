// tcgen05 pair-count kernel: the per-class plane Gram on the 5th-generation
// tensor cores (FP8 e4m3 operands, FP32 accumulators in tensor memory), exact,
// with the fused scoring epilogue of the other counting kernels.
//
// A set genotype bit becomes the e4m3 value 2^-6 (byte 0x08); products are
// 2^-12 and FP32 sums of them are exact, so count = accumulator * 4096.  The
// bit-planes stay packed (1 bit per sample) in HBM and L2; CUDA cores expand
// them on chip, using the nibble-transposed word layout (decode.cu): the four
// bytes of samples 4t..4t+3 of a word w are ((w >> t) << 3) & 0x08080808.
//
// Tile: 40 A SNPs x 32 B SNPs.  MMA M = 128 TMEM lanes: lane quarter q holds A
// SNPs 10q..10q+9, lane 3i+p of the quarter = plane p of SNP i (lanes 30, 31
// zero).  MMA N = 96: B row 3j+q = plane q of B SNP j.  K = 32 samples per
// tcgen05.mma, 8 per 256-sample pipeline chunk (one barrier wait and one
// commit per 8 MMAs: the issuing thread's wait and commit latency is then
// hidden behind the 512 tensor cycles of the chunk).
//
// Tensor memory (512 columns, one CTA per SM): two accumulator buffers of
// 192 columns (class 0 at +0, class 1 at +96) and two A stages of 64 columns
// (256 fp8 per lane).  Shared memory: two B stages of 96 rows x 256 bytes in
// the SWIZZLE_NONE K-major core-matrix layout (8 rows x 16 B cores, k-group
// stride 128 B, row-group stride 2048 B).
//
// Warp roles (17 warps, persistent CTA striding over the tile list):
//   producers  two groups, warps 0-3 and 8-11, take alternate chunks (one
//              stage each); in a chunk each warp writes A for its TMEM lane
//              quarter by tcgen05.st and 6 of the 768 B words by st.shared
//   epilogue   warps 4-7 and 12-15 (two per lane quarter, each half of the B
//              SNPs): drain an accumulator buffer per tile (tcgen05.ld),
//              exchange the three A planes of a SNP through shared memory and
//              score every SNP pair (score_tests)
//   MMA        warp 16, one thread: 8 x tcgen05.mma per chunk, commits
// mbarriers: full[s] (4 producer warps) / empty[s] (tcgen05.commit) per stage,
// dfull[b] (commit) / dempty[b] (8 epilogue warps) per accumulator buffer.
// Every wait is bounded by a clock budget; on expiry the kernel records an
// error, drains its own MMAs, frees its tensor memory and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "device.cuh"

namespace gepi {

constexpr int kTcASnps = 40;
constexpr int kTcBSnps = 32;
constexpr int kTcN = 3 * kTcBSnps;                 // 96
constexpr int kTcChunkWords = 8;                   // 256 samples per stage (8 MMAs)
constexpr int kTcStages = 2;
constexpr int kTcLbo = 128;                        // k-group stride (bytes)
constexpr int kTcSbo = kTcChunkWords * 2 * kTcLbo;   // 8-row group stride: 2,048 bytes
constexpr int kTcBStageBytes = (kTcN / 8) * kTcSbo;  // 24,576
constexpr int kTcXStride = 49;                     // epilogue exchange row pitch (floats)
constexpr int kTcThreads = 17 * 32;
constexpr int kTcMmaWarp = 16;
constexpr int kTcEpiWarps = 8;
constexpr uint32_t kTcCols = 512;
constexpr uint32_t kTcDCols = 2 * kTcN;            // one accumulator buffer
constexpr uint32_t kTcACol = 2 * kTcDCols;         // 384: first A stage
constexpr uint32_t kTcAStageCols = kTcChunkWords * 8;  // 64 columns (256 fp8 per lane)
constexpr uint32_t kTcIdesc =
    (1u << 4) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);  // f32 += e4m3*e4m3
constexpr size_t kTcSmemUsed =
    kTcStages * (size_t)kTcBStageBytes + (size_t)kTcEpiWarps * 32 * kTcXStride * 4;
constexpr size_t kTcSmem = 116 * 1024;             // > half an SM: one CTA (and TMEM owner) per SM
constexpr long long kTcWaitCycles = 4000000000ll;  // ~2 s at 2 GHz
static_assert(kTcSmemUsed <= kTcSmem, "smem layout");

__device__ __forceinline__ uint32_t su32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(su32(b))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return done != 0;
}

// Warp-uniform bounded wait: lane 0 polls, the verdict is broadcast.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t *b, uint32_t parity,
                                               volatile int *abort_flag, int *err, int code);

// Bounded wait; false when the CTA aborts or the clock budget runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile int *abort_flag,
                                          int *err, int code) {
    if (mbar_try(b, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(b, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > kTcWaitCycles) {
            *abort_flag = 1;
            atomicCAS(err, 0, code);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ bool mbar_wait_warp(uint64_t *b, uint32_t parity,
                                               volatile int *abort_flag, int *err, int code) {
    int ok = 0;
    if ((threadIdx.x & 31) == 0) ok = mbar_wait(b, parity, abort_flag, err, code) ? 1 : 0;
    return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ uint64_t tc_bdesc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(kTcLbo >> 4) << 16) |
           ((uint64_t)(kTcSbo >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
        "r"(a), "l"(bdesc), "r"(kTcIdesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint64_t *b) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(b))
        : "memory");
}

// 32 samples (one nibble-transposed word) -> 8 registers of 4 e4m3 bytes.
__device__ __forceinline__ void expand_word(uint32_t w, uint32_t *o) {
    constexpr uint32_t M = 0x08080808u;
    o[0] = (w << 3) & M;
    o[1] = (w << 2) & M;
    o[2] = (w << 1) & M;
    o[3] = w & M;
    o[4] = (w >> 1) & M;
    o[5] = (w >> 2) & M;
    o[6] = (w >> 3) & M;
    o[7] = (w >> 4) & M;
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
        "%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
        "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
        "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),
        "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]),
        "r"(r[29]), "r"(r[30]), "r"(r[31])
        : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr)
        : "memory");
}

template <bool DUMP>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_tile_kernel(const uint32_t *__restrict__ planes, int Wp, int W0,
                   const int2 *__restrict__ tiles, int ntiles, int a0, int a1, int b0, int b1,
                   ScanCtx ctx, uint32_t *__restrict__ dump, int *err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ uint64_t full_bar[kTcStages], empty_bar[kTcStages], dfull_bar[2], dempty_bar[2],
        fin_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nchunks = Wp / kTcChunkWords;
    const int csplit = W0 / kTcChunkWords;  // chunks of class 0

    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&full_bar[s], 4);
            mbar_init(&empty_bar[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&dfull_bar[b], 1);
            mbar_init(&dempty_bar[b], kTcEpiWarps);
        }
        mbar_init(&fin_bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(&tmem_slot)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmem_slot;
    volatile int *vabort = &abort_flag;

    if (warp < 4 || (warp >= 8 && warp < 12)) {
        // ---------------- producers ----------------
        const int q = warp & 3;             // TMEM lane quarter
        const int grp = warp >= 8;          // producer group: chunks of parity grp
        const int u = q * 32 + lane;        // 0..127 within the group
        const int ai = 10 * q + lane / 3, ap = lane % 3;
        const bool arow = lane < 30;
        constexpr int kBW = kTcN * kTcChunkWords / 128;  // B words per thread: 6
        int bn[kBW], bw[kBW];
#pragma unroll
        for (int m = 0; m < kBW; ++m) {
            const int wi = u + 128 * m;     // consecutive lanes: consecutive B rows
            bn[m] = wi % kTcN;
            bw[m] = wi / kTcN;
        }
        // The CTA's (tile, chunk) sequence is walked flat; this group takes
        // every other chunk and loads its next chunk ahead.
        const int my_tiles = blockIdx.x < (unsigned)ntiles
                                 ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                                 : 0;
        const int total = my_tiles * nchunks;
        struct Words {
            uint4 a0, a1;
            uint32_t b[kBW];
        };
        auto load = [&](int idx, Words &w) {
            w.a0 = w.a1 = make_uint4(0, 0, 0, 0);
#pragma unroll
            for (int m = 0; m < kBW; ++m) w.b[m] = 0;
            if (idx >= total) return;
            const int k = idx / nchunks, c = idx - k * nchunks;
            const int2 tl = tiles[blockIdx.x + k * gridDim.x];
            const int sa = a0 + tl.x * kTcASnps + ai;
            if (arow && sa < a1) {
                const uint4 *g = reinterpret_cast<const uint4 *>(planes + ((size_t)sa * 3 + ap) * Wp +
                                                                 kTcChunkWords * c);
                w.a0 = __ldg(g);
                w.a1 = __ldg(g + 1);
            }
            const int sb0 = b0 + tl.y * kTcBSnps;
#pragma unroll
            for (int m = 0; m < kBW; ++m) {
                const int sb = sb0 + bn[m] / 3;
                if (sb < b1)
                    w.b[m] = __ldg(planes + ((size_t)sb * 3 + bn[m] % 3) * Wp + kTcChunkWords * c + bw[m]);
            }
        };
        Words cur, nxt;
        load(grp, cur);
        for (int idx = grp; idx < total; idx += 2) {
            load(idx + 2, nxt);
            const uint32_t gc = (uint32_t)idx;
            const uint32_t s = gc % kTcStages;
            if (!mbar_wait_warp(&empty_bar[s], ((gc / kTcStages) & 1) ^ 1, vabort, err, 1)) break;
            tc_fence_after();
            const uint32_t ta = tbase + ((uint32_t)(32 * q) << 16) + kTcACol + s * kTcAStageCols;
            {
                uint32_t r[32];
                expand_word(cur.a0.x, r);
                expand_word(cur.a0.y, r + 8);
                expand_word(cur.a0.z, r + 16);
                expand_word(cur.a0.w, r + 24);
                tmem_st32(ta, r);
            }
            {
                uint32_t r[32];
                expand_word(cur.a1.x, r);
                expand_word(cur.a1.y, r + 8);
                expand_word(cur.a1.z, r + 16);
                expand_word(cur.a1.w, r + 24);
                tmem_st32(ta + 32, r);
            }
            unsigned char *stage = tc_smem + (size_t)s * kTcBStageBytes;
#pragma unroll
            for (int m = 0; m < kBW; ++m) {
                uint32_t o[8];
                expand_word(cur.b[m], o);
                unsigned char *st = stage + (bn[m] >> 3) * kTcSbo + (2 * bw[m]) * kTcLbo + (bn[m] & 7) * 16;
                *reinterpret_cast<uint4 *>(st) = make_uint4(o[0], o[1], o[2], o[3]);
                *reinterpret_cast<uint4 *>(st + kTcLbo) = make_uint4(o[4], o[5], o[6], o[7]);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&full_bar[s]);
            cur = nxt;
            if (__any_sync(0xffffffffu, *vabort != 0)) break;
        }
    } else if (warp == kTcMmaWarp) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint64_t bdesc[kTcStages];
#pragma unroll
            for (int st = 0; st < kTcStages; ++st)
                bdesc[st] = tc_bdesc(su32(tc_smem + (size_t)st * kTcBStageBytes));
            uint32_t gc = 0, lt = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++lt) {
                const uint32_t b = lt & 1;
                if (!mbar_wait(&dempty_bar[b], ((lt >> 1) & 1) ^ 1, vabort, err, 2)) break;
                tc_fence_after();
                const uint32_t dbuf = tbase + b * kTcDCols;
                for (int c = 0; c < nchunks; ++c, ++gc) {
                    const uint32_t s = gc % kTcStages;
                    if (!mbar_wait(&full_bar[s], (gc / kTcStages) & 1, vabort, err, 3)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = dbuf + (c < csplit ? 0u : (uint32_t)kTcN);
                    const uint32_t acc0 = (c == 0 || c == csplit) ? 0u : 1u;
                    const uint32_t a = tbase + kTcACol + s * kTcAStageCols;
                    const uint64_t bd = bdesc[s];
                    // k-group pair kk starts 2*kk*LBO = 256 B further: +16 in the address field
#pragma unroll
                    for (int kk = 0; kk < kTcChunkWords; ++kk)
                        tc_mma(d, a + kk * 8, bd + (uint64_t)(16 * kk), kk == 0 ? acc0 : 1u);
                    tc_commit(&empty_bar[s]);
                }
                if (!ok) break;
                tc_commit(&dfull_bar[b]);
            }
            // drain every MMA this thread issued before tensor memory is freed
            tc_commit(&fin_bar);
            const long long t0 = clock64();
            while (!mbar_try(&fin_bar, 0) && clock64() - t0 < kTcWaitCycles) {
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue (warps 4-7, 12-15) ----------------
        const int q = warp & 3;
        const int eh = warp >= 12;  // which half of the B SNPs
        const int ew = q + 4 * eh;  // 0..7
        float *xb = reinterpret_cast<float *>(tc_smem + kTcStages * (size_t)kTcBStageBytes) +
                    (size_t)ew * 32 * kTcXStride;
        const int i = lane / 3, p = lane % 3;
        const float theta = DUMP ? 0.f : ctx.st->theta;
        const float lp_thr = DUMP ? 0.f : ctx.st->lp_thr;
        uint32_t lt = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
            const uint32_t b = lt & 1;
            if (!mbar_wait_warp(&dfull_bar[b], (lt >> 1) & 1, vabort, err, 4)) break;
            tc_fence_after();
            const int2 tl = tiles[t];
            const int sA = a0 + tl.x * kTcASnps + 10 * q + i;
            const int sB0 = b0 + tl.y * kTcBSnps;
            const uint32_t tq = tbase + ((uint32_t)(32 * q) << 16) + b * kTcDCols;
            for (int g8 = 2 * eh; g8 < 2 * eh + 2; ++g8) {
                uint32_t v0[24], v1[24];
                tmem_ld16(tq + 24 * g8, *reinterpret_cast<uint32_t(*)[16]>(v0));
                tmem_ld8(tq + 24 * g8 + 16, *reinterpret_cast<uint32_t(*)[8]>(v0 + 16));
                tmem_ld16(tq + kTcN + 24 * g8, *reinterpret_cast<uint32_t(*)[16]>(v1));
                tmem_ld8(tq + kTcN + 24 * g8 + 16, *reinterpret_cast<uint32_t(*)[8]>(v1 + 16));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (g8 == 2 * eh + 1) {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&dempty_bar[b]);
                }
                if (DUMP) {
                    if (lane < 30 && sA < a1) {
#pragma unroll
                        for (int jl = 0; jl < 8; ++jl) {
                            const int sBt = sB0 + 8 * g8 + jl;
                            if (sBt >= b1) continue;
                            uint32_t *o = dump + ((size_t)(sA - a0) * (b1 - b0) + (sBt - b0)) * 18;
#pragma unroll
                            for (int qq = 0; qq < 3; ++qq) {
                                o[p * 3 + qq] = (uint32_t)(__uint_as_float(v0[3 * jl + qq]) * 4096.f);
                                o[9 + p * 3 + qq] = (uint32_t)(__uint_as_float(v1[3 * jl + qq]) * 4096.f);
                            }
                        }
                    }
                    continue;
                }
                float *row = xb + lane * kTcXStride;
#pragma unroll
                for (int k = 0; k < 24; ++k) {
                    row[k] = __uint_as_float(v0[k]) * 4096.f;
                    row[24 + k] = __uint_as_float(v1[k]) * 4096.f;
                }
                __syncwarp();
                if (lane < 30 && sA < a1) {
                    for (int jl = p; jl < 8; jl += 3) {
                        const int sBt = sB0 + 8 * g8 + jl;
                        if (sBt >= b1 || sBt > sA) continue;
                        float G[18];
#pragma unroll
                        for (int pp = 0; pp < 3; ++pp)
#pragma unroll
                            for (int qq = 0; qq < 3; ++qq) {
                                G[pp * 3 + qq] = xb[(3 * i + pp) * kTcXStride + 3 * jl + qq];
                                G[9 + pp * 3 + qq] = xb[(3 * i + pp) * kTcXStride + 24 + 3 * jl + qq];
                            }
                        score_tests(ctx, G, G + 9, sA, sBt, theta, lp_thr);
                    }
                }
                __syncwarp();
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTcCols)
                     : "memory");
    }
}

cudaError_t launch_tc_tiles(const uint32_t *planes, int Wp, int W0, const int2 *tiles, int ntiles,
                            int a0, int a1, int b0, int b1, const ScanCtx &ctx, uint32_t *dump,
                            int *err, int num_sms, cudaStream_t stream) {
    if (ntiles <= 0) return cudaSuccess;
    if ((Wp % kTcChunkWords) || (W0 % kTcChunkWords)) return cudaErrorInvalidValue;
    const int grid = ntiles < num_sms ? ntiles : num_sms;
    cudaError_t e;
    if (dump) {
        e = cudaFuncSetAttribute(tc_tile_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTcSmem);
        if (e != cudaSuccess) return e;
        tc_tile_kernel<true><<<grid, kTcThreads, kTcSmem, stream>>>(planes, Wp, W0, tiles, ntiles, a0,
                                                                    a1, b0, b1, ctx, dump, err);
    } else {
        e = cudaFuncSetAttribute(tc_tile_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTcSmem);
        if (e != cudaSuccess) return e;
        tc_tile_kernel<false><<<grid, kTcThreads, kTcSmem, stream>>>(planes, Wp, W0, tiles, ntiles,
                                                                     a0, a1, b0, b1, ctx, nullptr, err);
    }
    return cudaGetLastError();
}

int tc_tile_a_snps() { return kTcASnps; }
int tc_tile_b_snps() { return kTcBSnps; }

}  // namespace gepi
