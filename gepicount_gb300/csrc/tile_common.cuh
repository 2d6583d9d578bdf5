// Shared pieces of the tile-pair counting kernels: tile geometry of the
// shared-memory operand stages and the cp.async helpers.
//
// A CTA handles one 32 x 32 SNP tile pair.  Each operand stage holds the 96
// plane rows (3 per SNP, row 3s+p) of its 32 SNPs for 32 words (1,024
// samples), rows padded to a 36-word pitch (16-byte aligned for cp.async).
#pragma once

#include <cstdint>

namespace gepi {

constexpr int kTileSnps = 32;
constexpr int kTileKC = 32;                  // words per K chunk
constexpr int kTileStride = kTileKC + 4;     // padded smem row pitch (words)
constexpr int kTileRows = kTileSnps * 3;     // plane rows per operand
constexpr int kTileStages = 3;
constexpr size_t kTileStageWords = (size_t)2 * kTileRows * kTileStride;
constexpr size_t kTileSmem = (size_t)kTileStages * kTileStageWords * 4;

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src, int src_bytes) {
    unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem_src),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Issue the cp.async copies of K chunk `chunk` of both operands into `stage`.
// Rows past the range (row >= nAr / nBr) and words past Wp are zero-filled.
template <int NTHREADS>
__device__ __forceinline__ void load_tile_stage(uint32_t *smem, const uint32_t *planes,
                                                const uint32_t *gA, const uint32_t *gB, int nAr,
                                                int nBr, int Wp, int chunk, int stage, int tid) {
    uint32_t *sA = smem + (size_t)stage * kTileStageWords;
    uint32_t *sB = sA + kTileRows * kTileStride;
    const int wbase = chunk * kTileKC;
    constexpr int per_op = kTileRows * (kTileKC / 4);
#pragma unroll
    for (int c = tid; c < 2 * per_op; c += NTHREADS) {
        const int op = c >= per_op;
        const int rem = c - op * per_op;
        const int row = rem >> 3, q = rem & 7;
        const int w = wbase + 4 * q;
        const bool ok = (row < (op ? nBr : nAr)) && (w < Wp);
        const uint32_t *g = (op ? gB : gA) + (size_t)row * Wp + w;
        uint32_t *d = (op ? sB : sA) + row * kTileStride + 4 * q;
        cp_async16(d, ok ? g : planes, ok ? 16 : 0);
    }
}

}  // namespace gepi
