// Plain popcount pair-count kernel with the fused scoring epilogue.
//
// Replaces k1_count / k1_count_sm + k1_entropy / k1_fisherpv
// (src/kernels/kernel1.cu:60-284, entropyD.cu:31-50, fisher_d.cu:290-311).
// The reference spends 12 popcounts per 64-bit word per allele-row pair (48
// per SNP pair); here one SNP pair costs 9 AND+POPC per 32-bit word per class
// (the 3x3 Gram of planes {A-row, a-row, valid}), from which all 4 row pairs x
// 5 functions follow exactly (device.cuh).
//
// CTA = TA x 32 SNP tile (A side x B side; TA = 32 or 64), 8 TA threads as
// 16 x TA/2, each thread a 2 x 2 SNP-pair micro-tile (A SNPs ty, ty + TA/2; B
// SNPs tx, tx+16).  K is streamed in chunks of KC words (32 KC samples; KC =
// 16 or 32) through a 3-stage cp.async pipeline; shared rows are padded to
// KC + 4 words (16-byte aligned rows for cp.async); 64-bit reads of the A
// operand broadcast.  The shapes are the autotuner's popcount variants: a
// taller tile reads each B tile once for twice the A SNPs, a shorter stage
// needs half the shared memory.
// Bound: integer POPC issue rate (16 lanes/clk/SM).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "device.cuh"
#include "tile_common.cuh"

namespace gepi {

// Two consecutive words (h = word pair index in the chunk) of one class.
template <int TA, int KC, int CLS>
__device__ __forceinline__ void popc_step(const uint32_t *__restrict__ sA,
                                          const uint32_t *__restrict__ sB, int ty, int tx, int h,
                                          uint32_t (&acc)[2][2][2][9]) {
    constexpr int S = PopcGeom<TA, KC>::kStride;
    uint2 a[2][3], b[2][3];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int p = 0; p < 3; ++p)
            a[i][p] = *reinterpret_cast<const uint2 *>(sA + ((ty + (TA / 2) * i) * 3 + p) * S + 2 * h);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            b[j][q] = *reinterpret_cast<const uint2 *>(sB + ((tx + 16 * j) * 3 + q) * S + 2 * h);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    acc[CLS][i][j][p * 3 + q] +=
                        __popc(a[i][p].x & b[j][q].x) + __popc(a[i][p].y & b[j][q].y);
}

// tiles[blockIdx.x] = (A tile, B tile) of the SNP ranges [a0,a1) x [b0,b1);
// A tiles hold TA SNPs, B tiles 32; K streamed KC words per stage.
// DUMP: write the 18 Gram counts of every (s, t) in range to dump instead of
// scoring (verification entry point).
template <int TA, int KC, bool DUMP>
__device__ __forceinline__ void popc_tile(uint32_t *smem, const int2 tile,
                                          const uint32_t *__restrict__ planes, int Wp, int W0,
                                          int a0, int a1, int b0, int b1, const ScanCtx &ctx,
                                          uint32_t *__restrict__ dump) {
    using G = PopcGeom<TA, KC>;
    const int sA0 = a0 + tile.x * TA, sB0 = b0 + tile.y * kTileBSnps;
    const int nAr = 3 * min(TA, a1 - sA0), nBr = 3 * min(kTileBSnps, b1 - sB0);
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int nchunks = (Wp + KC - 1) / KC;
    const uint32_t *gA = planes + (size_t)sA0 * 3 * Wp;
    const uint32_t *gB = planes + (size_t)sB0 * 3 * Wp;

    uint32_t acc[2][2][2][9];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int k = 0; k < 9; ++k) acc[c][i][j][k] = 0u;

#pragma unroll
    for (int s = 0; s < G::kStages - 1; ++s) {
        if (s < nchunks) load_tile_stage<TA, KC>(smem, planes, gA, gB, nAr, nBr, Wp, s, s, tid);
        cp_async_commit();
    }
    for (int chunk = 0; chunk < nchunks; ++chunk) {
        cp_async_wait<G::kStages - 2>();
        __syncthreads();
        const int nxt = chunk + G::kStages - 1;
        if (nxt < nchunks)
            load_tile_stage<TA, KC>(smem, planes, gA, gB, nAr, nBr, Wp, nxt, nxt % G::kStages, tid);
        cp_async_commit();
        const int stage = chunk % G::kStages;
        const uint32_t *sA = smem + (size_t)stage * G::kStageWords;
        const uint32_t *sB = sA + G::kARows * G::kStride;
        // words [chunk*KC, W0) are class 0; W0 is a multiple of 8 words.
        int hsplit = (W0 - chunk * KC) / 2;
        hsplit = hsplit < 0 ? 0 : (hsplit > KC / 2 ? KC / 2 : hsplit);
#pragma unroll 2
        for (int h = 0; h < hsplit; ++h) popc_step<TA, KC, 0>(sA, sB, ty, tx, h, acc);
#pragma unroll 2
        for (int h = hsplit; h < KC / 2; ++h) popc_step<TA, KC, 1>(sA, sB, ty, tx, h, acc);
    }

    if (DUMP) {
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int s = sA0 + ty + (TA / 2) * i, t = sB0 + tx + 16 * j;
                if (s >= a1 || t >= b1) continue;
                uint32_t *o = dump + ((size_t)(s - a0) * (b1 - b0) + (t - b0)) * 18;
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    o[k] = acc[0][i][j][k];
                    o[9 + k] = acc[1][i][j][k];
                }
            }
        return;
    }
    // Epilogue: park the counts in shared memory (as exact floats) so the
    // scoring runs per pair with a bounded register footprint.
    cp_async_wait<0>();
    __syncthreads();
    float *sG = reinterpret_cast<float *>(smem) + (size_t)tid * 72;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                sG[(i * 2 + j) * 18 + k] = (float)acc[0][i][j][k];
                sG[(i * 2 + j) * 18 + 9 + k] = (float)acc[1][i][j][k];
            }
    const float theta = ctx.st->theta;
    const float lp_thr = ctx.st->lp_thr;
    // Fisher: tests that pass the bounds are queued (a shared atomic), and the
    // exact sums run on all the CTA's threads once scoring is done -- not on the
    // one or two lanes of a warp whose tests passed.  A full queue evaluates in
    // place.
    uint32_t *fq = nullptr;
    if (ctx.objective != 0 && !ctx.pend) {
        fq = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(smem) + G::kCountBytes);
        if (tid == 0) *fq = 0u;
        __syncthreads();
    }
#pragma unroll 1
    for (int ij = 0; ij < 4; ++ij) {
        const int i = ij >> 1, j = ij & 1;
        const int s = sA0 + ty + (TA / 2) * i, t = sB0 + tx + 16 * j;
        if (s >= a1 || t >= b1 || t > s) continue;
        score_pair(ctx, sG + ij * 18, s, t, theta, lp_thr, fq, G::kFisherQCap);
    }
    if (fq) {
        __syncthreads();
        const uint32_t n = min(*fq, (uint32_t)G::kFisherQCap);
        const int4 *qa = reinterpret_cast<const int4 *>(fq + 4);
        const int2 *qb = reinterpret_cast<const int2 *>(qa + G::kFisherQCap);
        for (uint32_t e = tid; e < n; e += G::kThreads) {
            const int4 a = qa[e];
            const int2 b = qb[e];
            exact_test(ctx, a.x, a.y >> 3, a.y & 7, a.z, a.w, b.x, b.y);
        }
    }
}

template <int TA, int KC, bool DUMP>
__global__ void __launch_bounds__(PopcGeom<TA, KC>::kThreads, PopcGeom<TA, KC>::kMinBlocks)
    popc_tile_kernel(const uint32_t *__restrict__ planes, int Wp, int W0,
                     const int2 *__restrict__ tiles, int a0, int a1, int b0, int b1, ScanCtx ctx,
                     uint32_t *__restrict__ dump) {
    extern __shared__ __align__(16) uint32_t smem[];
    popc_tile<TA, KC, DUMP>(smem, tiles[blockIdx.x], planes, Wp, W0, a0, a1, b0, b1, ctx, dump);
}

// Batched engine: persistent CTAs claim tiles of many requests' work list
// (WorkQueue) with an atomic counter; each tile is scored into its request's
// candidate buffer with its request's tables and threshold.
template <int TA, int KC>
__global__ void __launch_bounds__(PopcGeom<TA, KC>::kThreads, PopcGeom<TA, KC>::kMinBlocks)
    popc_batch_kernel(const ReqDesc *__restrict__ reqs, WorkQueue *q) {
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ int4 cur;
    for (;;) {
        if (threadIdx.x == 0) cur = resolve_work(reqs, q, (int)atomicAdd(&q->next, 1u));
        __syncthreads();
        const int4 d = cur;
        if (d.x < 0) break;
        const ReqDesc &R = reqs[d.x];
        popc_tile<TA, KC, false>(smem, make_int2(d.y, d.z), R.planes, R.Wp, R.W0, R.a0, R.a1, R.b0,
                                 R.b1, R.ctx, nullptr);
        __syncthreads();  // shared memory and `cur` are reused by the next tile
    }
}

template <int TA, int KC>
static cudaError_t launch_popc_shape(const uint32_t *planes, int Wp, int W0, const int2 *tiles,
                                     int ntiles, int a0, int a1, int b0, int b1,
                                     const ScanCtx &ctx, uint32_t *dump, cudaStream_t stream) {
    using G = PopcGeom<TA, KC>;
    // The shared-memory opt-in above 48 KB is a property of the current
    // device's context, so it is set on every launch (a cheap host call) rather
    // than cached once per process: a process that scans on several GPUs, or
    // from several host threads, gets it on each device.
    auto kern = dump ? popc_tile_kernel<TA, KC, true> : popc_tile_kernel<TA, KC, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)G::kSmem);
    if (e != cudaSuccess) return e;
    kern<<<ntiles, G::kThreads, G::kSmem, stream>>>(planes, Wp, W0, tiles, a0, a1, b0, b1, ctx, dump);
    return cudaGetLastError();
}

// setup: the shared-memory opt-in and the occupancy query only (outside any
// stream capture); the engine does it before it captures a step graph.  The
// persistent grid (CTAs the GPU holds at once) is kept per device.
template <int TA, int KC>
static cudaError_t launch_popc_batch_shape(const ReqDesc *reqs, WorkQueue *q, int num_sms,
                                           bool setup, cudaStream_t stream) {
    using G = PopcGeom<TA, KC>;
    static std::atomic<int> resident[64];
    auto kern = popc_batch_kernel<TA, KC>;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (setup) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::kSmem);
        if (e != cudaSuccess) return e;
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::kThreads, G::kSmem) !=
                cudaSuccess ||
            per_sm <= 0) {
            (void)cudaGetLastError();
            per_sm = 1;
        }
        if (dev < 64) resident[dev].store(per_sm);
        return cudaSuccess;
    }
    const int per_sm = dev < 64 ? std::max(1, resident[dev].load()) : 1;
    kern<<<num_sms * per_sm, G::kThreads, G::kSmem, stream>>>(reqs, q);
    return cudaGetLastError();
}

cudaError_t launch_popc_batch(int ta, int kc, const ReqDesc *reqs, WorkQueue *q, int num_sms,
                              cudaStream_t stream, bool setup) {
    if (ta == 32 && kc == 32) return launch_popc_batch_shape<32, 32>(reqs, q, num_sms, setup, stream);
    if (ta == 32 && kc == 16) return launch_popc_batch_shape<32, 16>(reqs, q, num_sms, setup, stream);
    if (ta == 64 && kc == 32) return launch_popc_batch_shape<64, 32>(reqs, q, num_sms, setup, stream);
    if (ta == 64 && kc == 16) return launch_popc_batch_shape<64, 16>(reqs, q, num_sms, setup, stream);
    return cudaErrorInvalidValue;
}

cudaError_t launch_popc_tiles(int ta, int kc, const uint32_t *planes, int Wp, int W0,
                              const int2 *tiles, int ntiles, int a0, int a1, int b0, int b1,
                              const ScanCtx &ctx, uint32_t *dump, cudaStream_t stream) {
    if (ntiles <= 0) return cudaSuccess;
    if (ta == 32 && kc == 32)
        return launch_popc_shape<32, 32>(planes, Wp, W0, tiles, ntiles, a0, a1, b0, b1, ctx, dump, stream);
    if (ta == 32 && kc == 16)
        return launch_popc_shape<32, 16>(planes, Wp, W0, tiles, ntiles, a0, a1, b0, b1, ctx, dump, stream);
    if (ta == 64 && kc == 32)
        return launch_popc_shape<64, 32>(planes, Wp, W0, tiles, ntiles, a0, a1, b0, b1, ctx, dump, stream);
    if (ta == 64 && kc == 16)
        return launch_popc_shape<64, 16>(planes, Wp, W0, tiles, ntiles, a0, a1, b0, b1, ctx, dump, stream);
    return cudaErrorInvalidValue;
}

}  // namespace gepi
