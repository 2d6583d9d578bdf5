// Shared pieces of the tile-pair popcount kernels: tile geometry of the
// shared-memory operand stages and the cp.async helpers.
//
// A CTA handles one TA x 32 SNP tile pair.  Each operand stage holds the plane
// rows (3 per SNP, row 3s+p) of its SNPs for KC words (32 KC samples), rows
// padded to a KC + 4 word pitch (16-byte aligned for cp.async, and the A reads
// of a half warp spread over the banks).
#pragma once

#include <cstddef>
#include <cstdint>

namespace gepi {

constexpr int kTileBSnps = 32;  // B SNPs of every popcount tile

template <int TA, int KC>
struct PopcGeom {
    static_assert(TA == 32 || TA == 64, "A SNPs per tile");
    static_assert(KC % 8 == 0 && KC >= 8, "words per stage: whole 16-byte copies, even split");
    static constexpr int kThreads = 8 * TA;            // 16 x TA/2 threads, 2 x 2 SNP pairs each
    static constexpr int kStride = KC + 4;             // padded smem row pitch (words)
    static constexpr int kARows = 3 * TA;
    static constexpr int kBRows = 3 * kTileBSnps;
    static constexpr int kStages = 3;
    static constexpr size_t kStageWords = (size_t)(kARows + kBRows) * kStride;
    static constexpr size_t kPipeBytes = (size_t)kStages * kStageWords * 4;
    static constexpr size_t kCountBytes = (size_t)kThreads * 72 * 4;  // 72 counts per thread
    // Fisher tests that passed the bounds, queued for the whole CTA to
    // evaluate (a count, then int4 {rA, rB * 8 + f, w, x} and int2 {y, z}).
    static constexpr int kFisherQCap = kThreads;
    static constexpr size_t kEpiBytes = kCountBytes + 16 + (size_t)kFisherQCap * 24;
    static constexpr size_t kSmem = kPipeBytes > kEpiBytes ? kPipeBytes : kEpiBytes;
    static constexpr int kMinBlocks = TA == 32 ? 2 : 1;  // 128 registers per thread
};

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
template <int TA, int KC>
__device__ __forceinline__ void load_tile_stage(uint32_t *smem, const uint32_t *planes,
                                                const uint32_t *gA, const uint32_t *gB, int nAr,
                                                int nBr, int Wp, int chunk, int stage, int tid) {
    using G = PopcGeom<TA, KC>;
    uint32_t *sA = smem + (size_t)stage * G::kStageWords;
    uint32_t *sB = sA + G::kARows * G::kStride;
    const int wbase = chunk * KC;
    constexpr int kPieces = KC / 4;  // 16-byte pieces per row
    constexpr int kA = G::kARows * kPieces;
    constexpr int kAll = kA + G::kBRows * kPieces;
#pragma unroll
    for (int c = tid; c < kAll; c += G::kThreads) {
        const int op = c >= kA;
        const int rem = c - op * kA;
        const int row = rem / kPieces, q = rem % kPieces;
        const int w = wbase + 4 * q;
        const bool ok = (row < (op ? nBr : nAr)) && (w < Wp);
        const uint32_t *g = (op ? gB : gA) + (size_t)row * Wp + w;
        uint32_t *d = (op ? sB : sA) + row * G::kStride + 4 * q;
        cp_async16(d, ok ? g : planes, ok ? 16 : 0);
    }
}

}  // namespace gepi
