// Plain popcount pair-count kernel with the fused scoring epilogue.
//
// Replaces k1_count / k1_count_sm + k1_entropy / k1_fisherpv
// (src/kernels/kernel1.cu:60-284, entropyD.cu:31-50, fisher_d.cu:290-311).
// The reference spends 12 popcounts per 64-bit word per allele-row pair (48
// per SNP pair); here one SNP pair costs 9 AND+POPC per 32-bit word per class
// (the 3x3 Gram of planes {A-row, a-row, valid}), from which all 4 row pairs x
// 5 functions follow exactly (device.cuh).
//
// CTA = 32 x 32 SNP tile (A side x B side), 256 threads as 16 x 16, each
// thread a 2 x 2 SNP-pair micro-tile (A SNPs ty, ty+16; B SNPs tx, tx+16).
// K is streamed in chunks of 32 words (1024 samples) through a 3-stage
// cp.async pipeline; shared rows are padded to 36 words (16-byte aligned rows for
// cp.async); 64-bit reads of the A operand broadcast.
// Bound: integer POPC issue rate (16 lanes/clk/SM).
#include <cuda_runtime.h>

#include <cstdint>

#include "device.cuh"
#include "tile_common.cuh"

namespace gepi {

constexpr int kPopcTile = kTileSnps;
constexpr int kPopcKC = kTileKC;
constexpr int kPopcStride = kTileStride;
constexpr int kPopcRows = kTileRows;
constexpr int kPopcStages = kTileStages;
constexpr int kPopcThreads = 256;
constexpr size_t kPopcSmem = kTileSmem;

// Two consecutive words (h = word pair index in the chunk) of one class.
template <int CLS>
__device__ __forceinline__ void popc_step(const uint32_t *__restrict__ sA,
                                          const uint32_t *__restrict__ sB, int ty, int tx, int h,
                                          uint32_t (&acc)[2][2][2][9]) {
    uint2 a[2][3], b[2][3];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int p = 0; p < 3; ++p)
            a[i][p] = *reinterpret_cast<const uint2 *>(sA + ((ty + 16 * i) * 3 + p) * kPopcStride + 2 * h);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            b[j][q] = *reinterpret_cast<const uint2 *>(sB + ((tx + 16 * j) * 3 + q) * kPopcStride + 2 * h);
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

// tiles[blockIdx.x] = (A tile, B tile) of the SNP ranges [a0,a1) x [b0,b1).
// DUMP: write the 18 Gram counts of every (s, t) in range to dump instead of
// scoring (verification entry point).
template <bool DUMP>
__global__ void __launch_bounds__(kPopcThreads, 2)
    popc_tile_kernel(const uint32_t *__restrict__ planes, int Wp, int W0,
                     const int2 *__restrict__ tiles, int a0, int a1, int b0, int b1, ScanCtx ctx,
                     uint32_t *__restrict__ dump) {
    extern __shared__ __align__(16) uint32_t smem[];
    const int2 tile = tiles[blockIdx.x];
    const int sA0 = a0 + tile.x * kPopcTile, sB0 = b0 + tile.y * kPopcTile;
    const int nAr = 3 * min(kPopcTile, a1 - sA0), nBr = 3 * min(kPopcTile, b1 - sB0);
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int nchunks = (Wp + kPopcKC - 1) / kPopcKC;
    const uint32_t *gA = planes + (size_t)sA0 * 3 * Wp;
    const uint32_t *gB = planes + (size_t)sB0 * 3 * Wp;

    auto load_stage = [&](int chunk, int stage) {
        load_tile_stage<kPopcThreads>(smem, planes, gA, gB, nAr, nBr, Wp, chunk, stage, tid);
    };

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
    for (int s = 0; s < kPopcStages - 1; ++s) {
        if (s < nchunks) load_stage(s, s);
        cp_async_commit();
    }
    for (int chunk = 0; chunk < nchunks; ++chunk) {
        cp_async_wait<kPopcStages - 2>();
        __syncthreads();
        const int nxt = chunk + kPopcStages - 1;
        if (nxt < nchunks) load_stage(nxt, nxt % kPopcStages);
        cp_async_commit();
        const int stage = chunk % kPopcStages;
        const uint32_t *sA = smem + (size_t)stage * 2 * kPopcRows * kPopcStride;
        const uint32_t *sB = sA + kPopcRows * kPopcStride;
        // words [chunk*KC, W0) are class 0; W0 is a multiple of 4 words.
        int hsplit = (W0 - chunk * kPopcKC) / 2;
        hsplit = hsplit < 0 ? 0 : (hsplit > kPopcKC / 2 ? kPopcKC / 2 : hsplit);
#pragma unroll 2
        for (int h = 0; h < hsplit; ++h) popc_step<0>(sA, sB, ty, tx, h, acc);
#pragma unroll 2
        for (int h = hsplit; h < kPopcKC / 2; ++h) popc_step<1>(sA, sB, ty, tx, h, acc);
    }

    if (DUMP) {
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int s = sA0 + ty + 16 * i, t = sB0 + tx + 16 * j;
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
#pragma unroll 1
    for (int ij = 0; ij < 4; ++ij) {
        const int i = ij >> 1, j = ij & 1;
        const int s = sA0 + ty + 16 * i, t = sB0 + tx + 16 * j;
        if (s >= a1 || t >= b1 || t > s) continue;
        score_pair(ctx, sG + ij * 18, s, t, theta, lp_thr);
    }
}

cudaError_t launch_popc_tiles(const uint32_t *planes, int Wp, int W0, const int2 *tiles,
                              int ntiles, int a0, int a1, int b0, int b1, const ScanCtx &ctx,
                              uint32_t *dump, cudaStream_t stream) {
    if (ntiles <= 0) return cudaSuccess;
    // The shared-memory opt-in above 48 KB is a property of the current
    // device's context, so it is set on every launch (a cheap host call) rather
    // than cached once per process: a process that scans on several GPUs, or
    // from several host threads, gets it on each device.
    if (dump) {
        cudaError_t e = cudaFuncSetAttribute(popc_tile_kernel<true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kPopcSmem);
        if (e != cudaSuccess) return e;
        popc_tile_kernel<true><<<ntiles, kPopcThreads, kPopcSmem, stream>>>(
            planes, Wp, W0, tiles, a0, a1, b0, b1, ctx, dump);
    } else {
        cudaError_t e = cudaFuncSetAttribute(popc_tile_kernel<false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kPopcSmem);
        if (e != cudaSuccess) return e;
        popc_tile_kernel<false><<<ntiles, kPopcThreads, kPopcSmem, stream>>>(
            planes, Wp, W0, tiles, a0, a1, b0, b1, ctx, nullptr);
    }
    return cudaGetLastError();
}

int popc_tile_snps() { return kPopcTile; }

}  // namespace gepi
