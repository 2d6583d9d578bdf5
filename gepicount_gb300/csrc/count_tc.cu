// tcgen05 pair-count kernel: the per-class plane Gram on the 5th-generation
// tensor cores (packed FP4 E2M1 operands with unit block scales, FP32
// accumulators in tensor memory), exact, with the fused scoring epilogue of the
// other counting kernels.
//
// A set genotype bit becomes the E2M1 value 1.0 (nibble 0x2) and a clear bit
// 0; the UE8M0 block scales are all 1.0 (byte 0x7F), so every product is 0 or
// 1 and the FP32 accumulator holds the count exactly (below 2^24).  The
// bit-planes stay packed (1 bit per sample) in HBM and L2; CUDA cores expand
// them on chip, four E2M1 words per plane word: word t of the expansion takes
// bits t, t+4, ..., t+28 into nibbles 0..7.  The sample order inside K is the
// same for both operands, so the dot product is popcount(a & b).
//
// Tile: 80 A SNPs x 64 B SNPs, computed by a CTA pair (a cluster of two CTAs
// on two SMs) with tcgen05.mma.cta_group::2, M = 256: CTA r holds A SNPs
// 40r..40r+39 of the tile in its tensor memory and B SNPs 32r..32r+31 in its
// shared memory, and receives the 40 x 64 accumulator of its own A SNPs.  Each
// SM thus expands its 40 A SNPs and half of the 64 B SNPs (216 rows per chunk;
// 312 for a 40 x 64 tile on one SM).  Lane quarter q of a CTA holds A SNPs
// 10q..10q+9 of its half, lane 3i+p of the quarter = plane p of SNP i (lanes
// 30, 31 zero).  MMA N = 192: B row 3j+q = plane q of B SNP j (the even CTA's
// shared memory holds rows 0..95, the odd CTA's rows 96..191).  K = 64 samples
// per tcgen05.mma (kind::mxf4, scale_vec::2X); a pipeline chunk is up to 384
// samples of one class (6 MMAs, one barrier wait and one commit).
//
// Operand layout in HBM (built once per plane set by tc_relayout_kernel): the
// plane words cut into 12-word (384-sample) blocks, block-major --
// blk[(b * rows_pad + row) * 12 + w] -- with class 0 in blocks [0, n0) and
// class 1 in [n0, n0 + n1), a short last block of a class zero-filled and
// rows_pad - 3 * n_snps zero rows at the end.  A chunk of a CTA's half tile is
// then two contiguous runs (120 A rows x 48 B, 96 B rows x 48 B) that the
// bulk-copy engine (cp.async.bulk) lands in a shared-memory ring; producer
// warps expand them, A into tensor memory (tcgen05.st), B into shared memory;
// one thread of the even CTA issues the pair's MMAs.  No thread waits on
// global memory.
//
// Tensor memory (512 columns, one CTA per SM, allocated for the pair): one
// accumulator of 384 columns (class 0 at +0, class 1 at +192), two A stages of
// 48 columns (384 E2M1 per lane) and 32 columns of scale factors (all 0x7F).
// The accumulator's class halves ping-pong: the scoring warps copy a tile's
// class-0 half out as soon as its MMAs are done and hand it back while class 1
// accumulates, so the next tile's MMAs start without draining the tensor pipe.
// Shared memory: two B stages of 96 rows x 192 bytes in the SWIZZLE_NONE
// K-major core-matrix layout (8 rows x 16 B cores, k-group stride 128 B,
// row-group stride 1536 B), the packed ring (4 slots) and the scoring warps'
// exchange rows.
//
// Warp roles (18 warps per CTA, the pair striding over the tile list):
//   MMA        warp 0 of the even CTA, one thread: up to 6 x tcgen05.mma per
//              chunk, commits (multicast to both CTAs' barriers)
//   TMA        warp 1, one thread: two bulk copies per chunk
//   producers  warps 2-9 share every chunk: the warp of lane quarter q and half
//              h expands words 6h..6h+5 of packed A row 30q+lane (lane < 30);
//              the first six also expand six words of one of the 96 B rows
//              (thread t: row t % 96, words 6 (t / 96) ..); stages alternate
//              between chunks
//   epilogue   warps 10-17 (two per lane quarter, each 32 B SNPs): copy their
//              part of each class half of the accumulator (tcgen05.ld) to
//              shared memory as 16-bit counts and hand it back, then bound
//              every SNP pair per row pair (one chi^2 bound covers a row
//              pair's five tests, for either objective; lane = B SNP, one A
//              SNP per round); the rare lane whose bound passes runs the
//              per-test bounds and the out-of-line refinement
// mbarriers: pfull[j] (copy transaction bytes) / pempty[j] (8 producer warps)
// per ring slot of each CTA; full[s] (even CTA: 16 producer warps of the pair)
// / empty[s] (commit, both CTAs) per stage; dfull[c] (commit, both CTAs) /
// dempty[c] (even CTA: 16 epilogue warps of the pair) per class half c of the
// accumulator: the scoring warps copy class 0 out while class 1 accumulates.
// Every wait is bounded by a clock budget; on expiry the kernel records an
// error, drains its own MMAs and copies, meets its peer at the final cluster
// barrier, frees its tensor memory and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>

#include "device.cuh"

namespace gepi {

constexpr int kTcASnps = 40;                       // A SNPs per CTA
constexpr int kTcPairASnps = 2 * kTcASnps;         // A SNPs per tile (CTA pair): 80
constexpr int kTcBSnps = 64;
constexpr int kTcARows = 3 * kTcASnps;             // 120
constexpr int kTcN = 3 * kTcBSnps;                 // 192
constexpr int kTcBRows = kTcN / 2;                 // B rows per CTA: 96
constexpr int kTcChunkWords = 12;                  // 384 samples per chunk (6 MMAs of K = 64)
constexpr int kTcHalfWords = kTcChunkWords / 2;    // words of a row per producer thread
constexpr int kTcStages = 2;                       // A/B operand stages
constexpr int kTcPStages = 4;                      // packed ring depth
constexpr int kTcLbo = 128;                        // k-group stride (bytes)
constexpr int kTcSbo = kTcChunkWords * kTcLbo;     // 8-row group stride: 1,536 bytes
constexpr int kTcBStageBytes = (kTcBRows / 8) * kTcSbo;   // 18,432
constexpr int kTcPABytes = kTcARows * kTcChunkWords * 4;  // 5,760
constexpr int kTcPBBytes = kTcBRows * kTcChunkWords * 4;  // 4,608
constexpr int kTcPStageBytes = kTcPABytes + kTcPBBytes;   // 10,368
constexpr int kTcMaxClass = 65535;                 // class sizes the 16-bit exchange holds
constexpr int kTcEpiWarps = 8;                     // scoring warps: two per lane quarter
constexpr int kTcProducerWarps = 8;
constexpr int kTcThreads = (2 + kTcProducerWarps + kTcEpiWarps) * 32;
constexpr int kTcBWarps = 2 * kTcBRows / 32;       // the first 6 producer warps also expand B
// The issuing warps come first: the schedulers favour lower-numbered (older)
// warps, and the single MMA thread is on every chunk's critical path.
constexpr int kTcMmaWarp = 0;
constexpr int kTcTmaWarp = 1;
constexpr int kTcProdWarp0 = 2;                    // producer warps 2-9
constexpr int kTcEpiWarp0 = kTcProdWarp0 + kTcProducerWarps;  // epilogue warps 10-17
constexpr int kTcEpiGroups = kTcBSnps / 8 / (kTcEpiWarps / 4);  // groups of 8 B SNPs a warp scores: 4
constexpr int kTcXPitch = 48 * kTcEpiGroups + 2;   // exchange row pitch (16-bit counts): 97 words
constexpr uint32_t kTcCols = 512;
constexpr uint32_t kTcDCols = 2 * kTcN;            // the accumulator (both classes): 384
constexpr uint32_t kTcACol = kTcDCols;             // 384: first A stage
constexpr uint32_t kTcAStageCols = kTcChunkWords * 4;  // 48 columns (384 E2M1 per lane)
constexpr uint32_t kTcSfCol = kTcACol + kTcStages * kTcAStageCols;  // 480: scale factors
constexpr uint32_t kTcIdesc = (1u << 7) | (1u << 10)           // A, B = E2M1
                              | ((uint32_t)(kTcN >> 3) << 17)  // N
                              | (1u << 23)                     // scales UE8M0
                              | ((uint32_t)(256 >> 4) << 24);  // M (the pair)
constexpr size_t kTcPOff = kTcStages * (size_t)kTcBStageBytes;               // packed ring
constexpr size_t kTcXOff = kTcPOff + kTcPStages * (size_t)kTcPStageBytes;    // exchange rows
// Fisher: each scoring warp queues the tests that pass its bounds (16 bytes
// each) and evaluates them 32 at a time, one per lane
constexpr int kTcQCap = 64;
constexpr size_t kTcQOff = (kTcXOff + (size_t)kTcEpiWarps * 32 * kTcXPitch * 2 + 15) / 16 * 16;
constexpr size_t kTcSmem = kTcQOff + (size_t)kTcEpiWarps * kTcQCap * 16;
static_assert(kTcSfCol + 32 <= kTcCols, "tensor memory budget");
static_assert(kTcBWarps * 32 == 2 * kTcBRows && kTcBWarps <= kTcProducerWarps, "B pieces");
static_assert(kTcHalfWords == 4 || kTcHalfWords == 6,
              "a producer thread stores 16 or 24 tensor-memory columns");
// Clock budget of every wait on another role's progress (~2 s at 2 GHz).  The
// kernel takes it as an argument: the library passes this value.  Waits for
// this CTA's own copies and MMAs on the way out (mbar_drain) always use the
// full budget, so nothing lands in a CTA's memory after it has exited.
//
// Timeout test (GEPI_DEBUG_STALL=<cycles>, tests only): the producers of both
// CTAs withhold their arrivals on the first chunk's full barrier -- a flag
// that nothing else sets -- and every wait gives up after <cycles>.  The MMA
// thread's wait for that stage then runs out, the CTA pair takes the abort
// path (drain, final cluster barrier, tensor-memory free) and the host reads
// GEPI_ERR_TIMEOUT; nothing faults and the context stays usable.
constexpr long long kTcWaitCycles = 4000000000ll;
static_assert(kTcPStageBytes % 128 == 0 && kTcPABytes % 128 == 0 && kTcPOff % 128 == 0,
              "TMA destinations 128-byte aligned");
static_assert(kTcSmem > 114 * 1024 && kTcSmem <= 227 * 1024,
              "more than half an SM: one CTA (and tensor-memory owner) per SM");

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

// A waiting thread may sleep in try_wait until the phase completes, for at
// most kTcSuspendNs; spinning warps would take issue slots from the producers.
constexpr uint32_t kTcSuspendNs = 20000;

__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(su32(b)), "r"(parity), "r"(kTcSuspendNs)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes)
                 : "memory");
}

// Bulk copy of `bytes` contiguous bytes into shared memory, completion on mbarrier `b`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            su32(dst)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(su32(b))
        : "memory");
}

// Bounded wait; false when the CTA aborts or the clock budget runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, volatile int *abort_flag,
                                          int *err, int code, long long budget) {
    if (mbar_try(b, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try(b, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > budget) {
            *abort_flag = 1;
            atomicCAS(err, 0, code);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Address of `b` (this CTA's shared memory) in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t cluster_addr(const void *b, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(su32(b)), "r"(rank));
    return r;
}

// One arrival per warp on a barrier given by its cluster address (possibly in
// the peer CTA).  Default (CTA-scope) semantics: what the arrival publishes is
// tensor-memory and async-proxy work, ordered by the tcgen05 thread-sync fences
// and the shared-to-async proxy fence around it; a cluster-scope release would
// add a memory barrier per chunk.
__device__ __forceinline__ void mbar_arrive_warp_cl(uint32_t caddr) {
    asm volatile(
        "{\n .reg .pred p;\n elect.sync _|p, 0xffffffff;\n"
        " @p mbarrier.arrive.shared::cluster.b64 _, [%0];\n}\n" ::"r"(caddr)
        : "memory");
}

// Every thread of both CTAs of the pair.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Warp-wide bounded wait: every lane polls the same barrier (a lane-0 poll
// plus a broadcast costs a reconvergence per wait).  The warp decides as one:
// it enters the wait converged, and in every iteration all its lanes execute
// the same try_wait on the same barrier word, read the same clock (one
// counter read per warp) and the same abort flag in the same instructions, so
// every branch of the loop is uniform and the lanes leave together with the
// same result -- the .sync.aligned tcgen05.st/ld and elect.sync that follow
// see the whole warp.  An explicit vote after the wait measured 7% slower on
// the 100,000 x 10,000 scan (238 against 224 ms), a __syncwarp and a shared
// flag read 14%.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t *b, uint32_t parity,
                                               volatile int *abort_flag, int *err, int code,
                                               long long budget) {
    return mbar_wait(b, parity, abort_flag, err, code, budget);
}

// One arrival per warp, by a lane elected in-line (predicated, no branch).
__device__ __forceinline__ void mbar_arrive_warp(uint64_t *b) {
    asm volatile(
        "{\n .reg .pred p;\n elect.sync _|p, 0xffffffff;\n"
        " @p mbarrier.arrive.shared::cta.b64 _, [%0];\n}\n" ::"r"(su32(b))
        : "memory");
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

// One MMA of the pair (issued by the even CTA): D rows of CTA r = its own A
// (tensor memory at `a`), B = both CTAs' stages at the same shared address.
__device__ __forceinline__ void tc_mma2(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t sf,
                                        uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %5, 0;\n"
        " tcgen05.mma.cta_group::2.kind::mxf4.block_scale.scale_vec::2X [%0], [%1], %2, %3, [%4], "
        "[%4], p;\n}\n" ::"r"(d),
        "r"(a), "l"(bdesc), "r"(kTcIdesc), "r"(sf), "r"(acc));
}

// Completion of the pair's MMAs issued so far arrives on barrier `b` (same
// offset) in both CTAs.
__device__ __forceinline__ void tc_commit2_both(uint64_t *b) {
    asm volatile(
        "{\n .reg .b16 m;\n mov.b16 m, 3;\n"
        " tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
        "[%0], m;\n}\n" ::"r"(su32(b))
        : "memory");
}

// ... on this CTA's barrier `b` only.
__device__ __forceinline__ void tc_commit2(uint64_t *b) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(b))
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *b) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(b))
        : "memory");
}

// 32 samples (one plane word) -> 4 registers of 8 E2M1 nibbles (1.0 or 0).
__device__ __forceinline__ void expand_word(uint32_t w, uint32_t *o) {
    constexpr uint32_t M = 0x22222222u;
    o[0] = (w << 1) & M;
    o[1] = w & M;
    o[2] = (w >> 1) & M;
    o[3] = (w >> 2) & M;
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t *r) {
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

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t *r) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16};" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
        "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
        "r"(r[15])
        : "memory");
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t *r) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
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

// Bounded wait used on the way out: ignores the abort flag (the copies or MMAs
// it waits for are this CTA's own and must land before the CTA exits).
__device__ __forceinline__ void mbar_drain(uint64_t *b, uint32_t parity) {
    if (mbar_try(b, parity)) return;
    const long long t0 = clock64();
    while (!mbar_try(b, parity) && clock64() - t0 < kTcWaitCycles) {
    }
}

// Stage-1 bounds of the 20 tests of an SNP pair (row pairs (2s+i, 2t+j), five
// functions each) as a bit mask, bit 5 * (2i + j) + f.  Same bounds as
// score_tests; the tests that pass are refined one by one out of line, which
// keeps the epilogue's code small (its warps share the instruction cache with
// the producers).
// Stage-1 bounds of the five tests of every row pair in `rp` (bit 2i+j) as a
// bit mask, bit 5 * (2i + j) + f.  Same bounds as score_tests; the tests that
// pass are refined one by one out of line.
template <int OBJ>
__device__ __forceinline__ uint32_t tc_stage1(const ScanCtx &ctx, const float *G0, const float *G1,
                                              uint32_t rp, float theta, float lp_thr) {
    const float y = G0[8], z = G1[8];
    const float m = y + z, yz = y * z;
    uint32_t mask = 0;
    // unrolled: constant indices keep the counts in registers
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        if (!((rp >> r) & 1u)) continue;
        const int i = r >> 1, j = r & 1;
        float on0[5], on1[5];
        {
            const float n11 = G0[i * 3 + j], rr = G0[i * 3 + 2], c = G0[6 + j];
            const float n10 = rr - n11, n01 = c - n11;
            on0[0] = n11; on0[1] = n01; on0[2] = n10; on0[3] = y - rr - c + n11; on0[4] = n10 + n01;
        }
        {
            const float n11 = G1[i * 3 + j], rr = G1[i * 3 + 2], c = G1[6 + j];
            const float n10 = rr - n11, n01 = c - n11;
            on1[0] = n11; on1[1] = n01; on1[2] = n10; on1[3] = z - rr - c + n11; on1[4] = n10 + n01;
        }
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            const float w = on0[f], x = on1[f];
            bool pass;
            if (OBJ == 0) {
                const float xx = w + x;
                const float Q = xx * (m - xx) * yz;
                const float wz = w * z, xy = x * y;
                const float D = fabsf(wz - xy) + (wz + xy) * 2.384185791015625e-07f;  // 2^-22
                pass = D * D >= theta * Q;
            } else {
                const int iw = (int)w, ix = (int)x, iy = (int)y, iz = (int)z;
                const float *L = ctx.lf32;
                const float lp = __ldg(L + (iw + ix)) + __ldg(L + (iy + iz - iw - ix)) +
                                 __ldg(L + iy) + __ldg(L + iz) - __ldg(L + (iy + iz)) -
                                 __ldg(L + iw) - __ldg(L + (iy - iw)) - __ldg(L + ix) -
                                 __ldg(L + (iz - ix));
                pass = lp <= lp_thr;
            }
            mask |= (uint32_t)pass << (5 * r + f);
        }
    }
    return mask;
}

// Stages 2 and 3 of one test that passed stage 1: for entropy the FP32
// estimate of m*I with its error margin (as in score_tests), then the exact key.
template <int OBJ>
static __device__ __noinline__ void tc_refine(const ScanCtx &ctx, int rA, int rB, int f, int w,
                                              int x, int y, int z) {
    if (OBJ == 0) {
        const float fw = (float)w, fx = (float)x, fy = (float)y, fz = (float)z;
        const float m = fy + fz, xx = fw + fx;
        const float Tm = tlog2f(m), Ty = tlog2f(fy), Tz = tlog2f(fz);
        const float a = tlog2f(fw), b = tlog2f(fy - fw), c = tlog2f(fx), d = tlog2f(fz - fx);
        const float e = tlog2f(xx), g = tlog2f(m - xx);
        const float est = ((Tm + a) + (b + c)) + d - (e + g) - (Ty + Tz);
        const float tm = ctx.st->tau_f * m;
        const float mag = Tm + a + b + c + d + e + g + Ty + Tz + fabsf(tm);
        if (est + (2e-6f * mag + 1e-3f) < tm) return;
    }
    exact_test(ctx, rA, rB, f, w, x, y, z);
}

// Two 16-bit counts as floats: 2^23 + v has v in its low mantissa bits (an
// ALU or each and one packed FMA-pipe subtract, exact, instead of two
// conversion-unit instructions).
__device__ __forceinline__ float2 u16f2(uint16_t a, uint16_t b) {
    return __fadd2_rn(make_float2(__uint_as_float(0x4B000000u | (uint32_t)a),
                                  __uint_as_float(0x4B000000u | (uint32_t)b)),
                      make_float2(-8388608.0f, -8388608.0f));
}

// Two accumulator counts (FP32 bit patterns of exact integers below 2^16) as
// one word of two 16-bit counts, lo | hi << 16: adding 2^23 puts each count in
// the low mantissa bits (exact, so the rounding mode does not matter), and one
// byte permute takes the two low halves -- one packed FMA-pipe add and one
// ALU instruction instead of two conversion-unit instructions, a shift and an
// or.
__device__ __forceinline__ uint32_t pack_counts(uint32_t lo, uint32_t hi) {
    const float2 ab = __fadd2_rn(make_float2(__uint_as_float(lo), __uint_as_float(hi)),
                                 make_float2(8388608.0f, 8388608.0f));
    return __byte_perm(__float_as_uint(ab.x), __float_as_uint(ab.y), 0x5410);
}

// Cells of row pair (2s+ri, 2t+rj) in one class's 3 x 3 Gram G -- n11 and the
// two margins -- selected in registers: a runtime index into G would place all
// of G in local memory, stored on every round.
__device__ __forceinline__ void gram_cells(const float *G, int ri, int rj, int &n11, int &r, int &c) {
    n11 = (int)(ri ? (rj ? G[4] : G[3]) : (rj ? G[1] : G[0]));
    r = (int)(ri ? G[5] : G[2]);
    c = (int)(rj ? G[7] : G[6]);
}

// Count of function f (AND, NAND, ANDN, NANDN, XOR) from n11 and the margins.
__device__ __forceinline__ int fun_count(int n11, int r, int c, int tot, int f) {
    switch (f) {
    case 0: return n11;
    case 1: return c - n11;
    case 2: return r - n11;
    case 3: return tot - r - c + n11;
    default: return r + c - 2 * n11;
    }
}

// Chunk c of a tile: class 0 owns chunks [0, n0) over words [0, W0), class 1
// chunks [n0, n0 + n1) over words [W0, Wp); the last chunk of a class may be
// short (its box reaches into the next class or past the row, which the MMAs
// of the chunk do not read).
struct ChunkMap {
    int n0, nchunks, W0, W1;
    __device__ __forceinline__ int start(int c) const {
        return c < n0 ? kTcChunkWords * c : W0 + kTcChunkWords * (c - n0);
    }
    __device__ __forceinline__ int mmas(int c) const {  // K = 64 samples = 2 words per MMA
        const int rem = c < n0 ? W0 - kTcChunkWords * c : W1 - kTcChunkWords * (c - n0);
        return (rem < kTcChunkWords ? rem : kTcChunkWords) >> 1;
    }
};

// ---- the roles, shared by the single-request and the batched kernel --------

// Barriers and wait policy of one CTA.  budget: clock budget of waits on other
// roles (kTcWaitCycles; a test lowers it).
struct TcSync {
    uint64_t *pfull, *pempty, *full, *empty, *dfull, *dempty;
    volatile int *abort_flag;
    int *err;
    long long budget;
};

// A producer lane's fixed geometry: lane quarter q, A words HW h .. of packed
// A row 30 q + lane (lanes 30, 31 re-read row 30q+29 and clear it), and for
// the first six producer warps a B piece (row u = t % 96, words HW hb ..;
// consecutive lanes on consecutive rows: conflict-free 16-byte stores).
struct TcProducer {
    static constexpr int HW = kTcHalfWords;
    int h, u, hb, arow_off;
    bool arow, has_b;
    uint32_t ta0;
    unsigned char *bst0;

    __device__ __forceinline__ TcProducer(unsigned char *smem, uint32_t tbase, int warp, int lane) {
        const int q = warp & 3;  // TMEM lane quarter
        h = (warp - kTcProdWarp0) >> 2;
        arow = lane < 30;
        arow_off = (30 * q + (arow ? lane : 29)) * (kTcChunkWords * 4);
        ta0 = tbase + ((uint32_t)(32 * q) << 16) + kTcACol + 4 * HW * h;
        has_b = warp - kTcProdWarp0 < kTcBWarps;
        const int t8 = 32 * (warp - kTcProdWarp0) + lane;
        u = t8 % kTcBRows;
        hb = t8 / kTcBRows;
        bst0 = smem + (u >> 3) * kTcSbo + (HW * hb) * kTcLbo + (u & 7) * 16;
    }

    // Global chunk idx: packed ring slot idx % kTcPStages -> stage idx %
    // kTcStages (A into tensor memory, B into shared memory), then one arrival
    // per warp on the pair's full barrier (none when `withhold`).  false: the
    // CTA aborts.
    __device__ __forceinline__ bool chunk(unsigned char *smem, const TcSync &S, int idx,
                                          bool withhold) const {
        const uint32_t j = (uint32_t)idx % kTcPStages, s = (uint32_t)idx % kTcStages;
        if (!mbar_wait_warp(&S.pfull[j], ((uint32_t)idx / kTcPStages) & 1, S.abort_flag, S.err, 5,
                            S.budget))
            return false;
        const unsigned char *pk = smem + kTcPOff + (size_t)j * kTcPStageBytes;
        // every lane loads: no divergence
        uint2 pa[HW / 2], pb[HW / 2];
        {
            const uint2 *r = reinterpret_cast<const uint2 *>(pk + 4 * HW * h + arow_off);
#pragma unroll
            for (int m = 0; m < HW / 2; ++m) {
                pa[m] = r[m];
                pa[m].x = arow ? pa[m].x : 0u;
                pa[m].y = arow ? pa[m].y : 0u;
            }
        }
        if (has_b) {
            const uint2 *r =
                reinterpret_cast<const uint2 *>(pk + kTcPABytes + u * (kTcChunkWords * 4) + 4 * HW * hb);
#pragma unroll
            for (int m = 0; m < HW / 2; ++m) pb[m] = r[m];
        }
        __syncwarp();
        mbar_arrive_warp(&S.pempty[j]);
        // expand into registers before waiting for the stage: the wait is on the
        // MMAs kTcStages chunks back, and only the stores follow it
        uint32_t r[4 * HW], o[4 * HW];
#pragma unroll
        for (int m = 0; m < HW / 2; ++m) {
            expand_word(pa[m].x, r + 8 * m);
            expand_word(pa[m].y, r + 8 * m + 4);
        }
        if (has_b) {
#pragma unroll
            for (int m = 0; m < HW / 2; ++m) {
                expand_word(pb[m].x, o + 8 * m);
                expand_word(pb[m].y, o + 8 * m + 4);
            }
        }
        if (!mbar_wait_warp(&S.empty[s], (((uint32_t)idx / kTcStages) & 1) ^ 1, S.abort_flag, S.err, 1,
                            S.budget))
            return false;
        tc_fence_after();
        tmem_st16(ta0 + s * kTcAStageCols, r);
        if constexpr (HW == 6) tmem_st8(ta0 + s * kTcAStageCols + 16, r + 16);
        if (has_b) {
            unsigned char *bst = bst0 + (size_t)s * kTcBStageBytes;
#pragma unroll
            for (int m = 0; m < HW; ++m)
                *reinterpret_cast<uint4 *>(bst + m * kTcLbo) =
                    make_uint4(o[4 * m], o[4 * m + 1], o[4 * m + 2], o[4 * m + 3]);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncwarp();
        if (!withhold) mbar_arrive_warp_cl(cluster_addr(&S.full[s], 0));
        return true;
    }
};

// The copy issuer's chunk: waits for ring slot idx % kTcPStages to be free and
// lands chunk c of the tile's packed A rows (from arow) and B rows (from brow).
__device__ __forceinline__ bool tc_copy_chunk(unsigned char *smem, const TcSync &S, int idx,
                                              const uint32_t *blk, int rows_pad, int c, size_t arow,
                                              size_t brow, bool wait_free = true) {
    const uint32_t j = (uint32_t)idx % kTcPStages;
    if (wait_free && !mbar_wait(&S.pempty[j], (((uint32_t)idx / kTcPStages) & 1) ^ 1, S.abort_flag,
                                S.err, 6, S.budget))
        return false;
    unsigned char *pk = smem + kTcPOff + (size_t)j * kTcPStageBytes;
    const uint32_t *base = blk + (size_t)c * rows_pad * kTcChunkWords;
    mbar_expect_tx(&S.pfull[j], kTcPStageBytes);
    bulk_load(pk, base + arow * kTcChunkWords, kTcPABytes, &S.pfull[j]);
    bulk_load(pk + kTcPABytes, base + brow * kTcChunkWords, kTcPBBytes, &S.pfull[j]);
    return true;
}

// Every copy the issuer made (`issued` chunks) lands before the CTA exits.
__device__ __forceinline__ void tc_copy_drain(const TcSync &S, int issued) {
    for (int idx = issued > kTcPStages ? issued - kTcPStages : 0; idx < issued; ++idx)
        mbar_drain(&S.pfull[idx % kTcPStages], ((uint32_t)idx / kTcPStages) & 1);
}


// A scoring warp's fixed geometry: lane quarter q, B SNPs 32 eh .. 32 eh + 31
// of the tile, its exchange rows (16-bit counts, row = TMEM lane: plane p of A
// SNP i at row 3i + p, laid out [class][B plane qq][B SNP jl] so that the 32
// lanes reading one plane pair of 32 B SNPs hit 16 consecutive words; odd word
// pitch, so the copy-out is conflict-free too).
struct TcScorer {
    static constexpr int kB = 8 * kTcEpiGroups;  // B SNPs of the warp: 32
    int eh, aoff;
    uint16_t *xh;
    uint4 *qb;  // Fisher: this warp's queue of tests for exact evaluation
    uint32_t tq;
    __device__ __forceinline__ TcScorer(unsigned char *smem, uint32_t tbase, int warp, uint32_t rank) {
        const int q = warp & 3;
        const int ew = warp - kTcEpiWarp0;
        eh = ew >> 2;
        xh = reinterpret_cast<uint16_t *>(smem + kTcXOff) + (size_t)ew * 32 * kTcXPitch;
        qb = reinterpret_cast<uint4 *>(smem + kTcQOff) + (size_t)ew * kTcQCap;
        aoff = kTcASnps * (int)rank + 10 * q;  // this warp's first A SNP in the tile
        tq = tbase + ((uint32_t)(32 * q) << 16) + 3 * kB * eh;
    }

    // Local tile lt (A tile tx, B tile ty of ranges [a0,a1) x [b0,b1)): copy
    // each class half out as soon as its MMAs are done and hand it back (the
    // tensor pipe goes on with the other half, then the next tile), then bound
    // every SNP pair per row pair: lane = B SNP, one A SNP per round; the rare
    // lane whose bound passes runs the per-test bounds and the out-of-line
    // refinement on the counts it holds.  false: the CTA aborts.
    template <bool DUMP, int OBJ>
    __device__ __forceinline__ bool tile(const TcSync &S, int lane, uint32_t lt, int tx, int ty,
                                         int a0, int a1, int b0, int b1, const ScanCtx &ctx,
                                         float theta, float lp_thr, uint32_t *dump) const {
        const int sAq = a0 + tx * kTcPairASnps + aoff;  // A SNP 0 of the lane quarter
        const int sB0 = b0 + ty * kTcBSnps + kB * eh;
        for (int cls = 0; cls < 2; ++cls) {
            if (!mbar_wait_warp(&S.dfull[cls], lt & 1, S.abort_flag, S.err, 4, S.budget)) return false;
            tc_fence_after();
            uint32_t *rw = reinterpret_cast<uint32_t *>(xh + lane * kTcXPitch) + cls * (3 * kB / 2);
#pragma unroll
            for (int gl = 0; gl < kTcEpiGroups; ++gl) {
                uint32_t v[24];  // column 3 jl' + qq of B SNPs 8 gl + jl'
                tmem_ld16(tq + cls * kTcN + 24 * gl, *reinterpret_cast<uint32_t(*)[16]>(v));
                tmem_ld8(tq + cls * kTcN + 24 * gl + 16, *reinterpret_cast<uint32_t(*)[8]>(v + 16));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int qq = 0; qq < 3; ++qq)
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        rw[qq * (kB / 2) + 4 * gl + m] =
                            pack_counts(v[6 * m + qq], v[6 * m + 3 + qq]);
            }
            tc_fence_before();
            __syncwarp();
            mbar_arrive_warp_cl(cluster_addr(&S.dempty[cls], 0));
        }
        __syncwarp();
        if constexpr (DUMP) {
            const int i = lane / 3, p = lane % 3, sA = sAq + i;
            if (lane < 30 && sA < a1) {
                const uint16_t *xr = xh + lane * kTcXPitch;
                for (int jb = 0; jb < kB; ++jb) {
                    const int sBt = sB0 + jb;
                    if (sBt >= b1) continue;
                    uint32_t *o = dump + ((size_t)(sA - a0) * (b1 - b0) + (sBt - b0)) * 18;
#pragma unroll
                    for (int qq = 0; qq < 3; ++qq) {
                        o[p * 3 + qq] = xr[qq * kB + jb];
                        o[9 + p * 3 + qq] = xr[3 * kB + qq * kB + jb];
                    }
                }
            }
            __syncwarp();
            return true;
        }
        const int sBt = sB0 + lane;
        int fill = 0;  // Fisher queue entries (warp-uniform)
        // Fisher: the queued tests, one per lane, then the queue is empty
        auto drain = [&]() {
            __syncwarp();
            for (int i = lane; i < fill; i += 32) {
                const uint4 e = qb[i];
                exact_test(ctx, (int)e.x, (int)(e.y >> 3), (int)(e.y & 7u), (int)(e.z & 0xFFFFu),
                           (int)(e.z >> 16), (int)(e.w & 0xFFFFu), (int)(e.w >> 16));
            }
            __syncwarp();
            fill = 0;
        };
        for (int r = 0; r < 10; ++r) {
            const int sA = sAq + r;
            float G[18];
            uint32_t mask = 0;
            if (sA < a1 && sBt < b1 && sBt <= sA) {
                const uint16_t *xr = xh + 3 * r * kTcXPitch + lane;
#pragma unroll
                for (int pp = 0; pp < 3; ++pp)
#pragma unroll
                    for (int qq = 0; qq < 3; ++qq) {
                        const float2 g2 = u16f2(xr[pp * kTcXPitch + qq * kB],
                                               xr[pp * kTcXPitch + 3 * kB + qq * kB]);  // class 0, 1
                        G[pp * 3 + qq] = g2.x;
                        G[9 + pp * 3 + qq] = g2.y;
                    }
                const uint32_t rp = rowpair_bounds(G, G + 9, sA == sBt, OBJ, theta, lp_thr);
                if (rp) mask = tc_stage1<OBJ>(ctx, G, G + 9, rp, theta, lp_thr);
            }
            // Fisher: the tests that passed go to the launch's pending list, for
            // a launch across the GPU to evaluate (a test past its capacity is
            // evaluated here); without one (batched engine), to the warp's
            // queue, whose exact tail sums then run 32 at a time, one per lane,
            // instead of on the one or two lanes whose tests passed -- a round
            // with more than the queue holds evaluates in place
            bool queue = false;
            int pos = 0;
            uint32_t gpos = 0;
            if constexpr (OBJ == 1) {
                const int n = __popc(mask);
                int incl = n;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 31);
                if (ctx.pend) {
                    if (total > 0) {
                        uint32_t base = 0;
                        if (lane == 31) base = atomicAdd(&ctx.pend->n, (uint32_t)total);
                        gpos = __shfl_sync(0xffffffffu, base, 31) + (uint32_t)(incl - n);
                    }
                } else {
                    if (total > 0 && fill + total > kTcQCap) drain();
                    queue = total > 0 && total <= kTcQCap;
                    pos = fill + incl - n;
                    if (queue) fill += total;
                }
            }
            while (mask) {
                const int bit = __ffs(mask) - 1;
                mask &= mask - 1;
                const int rpi = bit / 5, f = bit - 5 * rpi, ri = rpi >> 1, rj = rpi & 1;
                const int y = (int)G[8], z = (int)G[17];
                int n11, rr, cc;
                gram_cells(G, ri, rj, n11, rr, cc);
                const int w = fun_count(n11, rr, cc, y, f);
                gram_cells(G + 9, ri, rj, n11, rr, cc);
                const int x = fun_count(n11, rr, cc, z, f);
                const uint4 e = make_uint4((uint32_t)(2 * sA + ri), (uint32_t)(2 * sBt + rj) << 3 | (uint32_t)f,
                                           (uint32_t)w | (uint32_t)x << 16, (uint32_t)y | (uint32_t)z << 16);
                if (OBJ == 1 && ctx.pend && gpos < ctx.pend->cap) {
                    ctx.pend->ent[gpos] = e;
                    if (ctx.pend->tag) ctx.pend->tag[gpos] = ctx.pend_req;
                    ++gpos;
                } else if (queue)
                    qb[pos++] = e;
                else
                    tc_refine<OBJ>(ctx, 2 * sA + ri, 2 * sBt + rj, f, w, x, y, z);
            }
        }
        if constexpr (OBJ == 1) {
            if (fill > 0) drain();
        }
        __syncwarp();
        return true;
    }
};

// Common prologue of both kernels: barriers (and the batched kernel's ring
// barriers, `ring_bar`, `nring` of them), tensor memory for the pair.
__device__ __forceinline__ void tc_prologue(const TcSync &S, uint64_t *fin_bar, uint64_t *ring_bar,
                                            int nring, uint32_t *tmem_slot, int *abort_flag, int tid,
                                            int warp) {
    if (tid == 0) {
        for (int j = 0; j < kTcPStages; ++j) {
            mbar_init(&S.pfull[j], 1);
            mbar_init(&S.pempty[j], kTcProducerWarps);
        }
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&S.full[s], 2 * kTcProducerWarps);  // both CTAs' producers (even CTA's)
            mbar_init(&S.empty[s], 1);
        }
        for (int cls = 0; cls < 2; ++cls) {  // the accumulator's class halves
            mbar_init(&S.dfull[cls], 1);
            mbar_init(&S.dempty[cls], 2 * kTcEpiWarps);  // both CTAs' epilogues (even CTA's)
        }
        mbar_init(fin_bar, 1);
        for (int j = 0; j < nring; ++j) mbar_init(&ring_bar[j], 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        // one warp of each CTA of the pair, collectively
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(tmem_slot)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    }
}

__device__ __forceinline__ void tc_scales(uint32_t tbase, int warp) {
    if (warp < 4) {
        // unit block scales (UE8M0 1.0) over all lanes of the scale-factor columns
        uint32_t r[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) r[k] = 0x7F7F7F7Fu;
        tmem_st32(tbase + ((uint32_t)(32 * warp) << 16) + kTcSfCol, r);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
}

// Common epilogue: the pair's MMAs have drained (the even CTA's issuer waited
// for them) and no thread arrives on the peer's barriers any more once both
// CTAs pass the cluster barrier; then the pair's tensor memory is freed.
__device__ __forceinline__ void tc_teardown(uint32_t tbase, int warp) {
    tc_fence_before();
    __syncthreads();
    cluster_sync_all();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTcCols)
                     : "memory");
    }
}

// The single-request kernel (gepi_scan, gepi_scan_range, gepi_pair_counts).
// Its roles are written out in line rather than through the role structs the
// batched kernel shares: the same code behind those structs measured 8%
// slower on the 100,000 x 10,000 scan (242 against 224 ms).
// TEST: the wait budget and the withheld first arrival of the timeout test
// (GEPI_DEBUG_STALL) are kernel arguments; the library's instances compile
// them out.
template <bool DUMP, int OBJ, bool TEST>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kTcThreads, 1)
    tc_tile_kernel(const uint32_t *__restrict__ blk, int rows_pad, int Wp, int W0,
                   const int2 *__restrict__ tiles, int ntiles, int a0, int a1, int b0, int b1,
                   ScanCtx ctx, uint32_t *__restrict__ dump, int *err, long long wait_cycles,
                   int stall) {
    const long long budget = TEST ? wait_cycles : kTcWaitCycles;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ uint64_t pfull_bar[kTcPStages], pempty_bar[kTcPStages], full_bar[kTcStages],
        empty_bar[kTcStages], dfull_bar[2], dempty_bar[2], fin_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t rank = cluster_rank();  // 0: the CTA that issues the pair's MMAs
    int pair, npairs;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(pair));
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(npairs));
    ChunkMap cm;
    cm.W0 = W0;
    cm.W1 = Wp - W0;
    cm.n0 = (W0 + kTcChunkWords - 1) / kTcChunkWords;
    cm.nchunks = cm.n0 + (cm.W1 + kTcChunkWords - 1) / kTcChunkWords;
    const int nchunks = cm.nchunks;
    const int my_tiles = pair < ntiles ? (ntiles - pair + npairs - 1) / npairs : 0;
    const int total = my_tiles * nchunks;  // the pair's (tile, chunk) sequence, walked flat

    if (tid == 0) {
        for (int j = 0; j < kTcPStages; ++j) {
            mbar_init(&pfull_bar[j], 1);
            mbar_init(&pempty_bar[j], kTcProducerWarps);
        }
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&full_bar[s], 2 * kTcProducerWarps);  // both CTAs' producers (even CTA's)
            mbar_init(&empty_bar[s], 1);
        }
        for (int cls = 0; cls < 2; ++cls) {  // the accumulator's class halves
            mbar_init(&dfull_bar[cls], 1);
            mbar_init(&dempty_bar[cls], 2 * kTcEpiWarps);  // both CTAs' epilogues (even CTA's)
        }
        mbar_init(&fin_bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        // one warp of each CTA of the pair, collectively
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(&tmem_slot)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmem_slot;
    volatile int *vabort = &abort_flag;
    if (warp < 4) {
        // unit block scales (UE8M0 1.0) over all lanes of the scale-factor columns
        uint32_t r[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) r[k] = 0x7F7F7F7Fu;
        tmem_st32(tbase + ((uint32_t)(32 * warp) << 16) + kTcSfCol, r);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    // both CTAs' barriers are initialised and scale factors written before any
    // arrival from the peer or any MMA
    cluster_sync_all();
    tc_fence_after();

    if (warp >= kTcProdWarp0 && warp < kTcEpiWarp0) {
        // ---------------- producers ----------------
        constexpr int HW = kTcHalfWords;
        const int q = warp & 3;             // TMEM lane quarter
        const int h = (warp - kTcProdWarp0) >> 2;  // words HW h .. HW h + HW - 1 of each A row
        const bool arow = lane < 30;
        const int arow_off = (30 * q + (arow ? lane : 29)) * (kTcChunkWords * 4);
        const uint32_t ta0 = tbase + ((uint32_t)(32 * q) << 16) + kTcACol + 4 * HW * h;
        // B piece of the first six producer warps: row u = t % 96, words HW hb ..
        // HW hb + HW - 1 (consecutive lanes on consecutive rows: conflict-free
        // 16-byte stores)
        const bool has_b = warp - kTcProdWarp0 < kTcBWarps;
        const int t8 = 32 * (warp - kTcProdWarp0) + lane;
        const int u = t8 % kTcBRows, hb = t8 / kTcBRows;
        unsigned char *bst0 = tc_smem + (u >> 3) * kTcSbo + (HW * hb) * kTcLbo + (u & 7) * 16;
        for (int idx = 0; idx < total; ++idx) {
            const uint32_t j = (uint32_t)idx % kTcPStages, s = (uint32_t)idx % kTcStages;
            if (!mbar_wait_warp(&pfull_bar[j], ((uint32_t)idx / kTcPStages) & 1, vabort, err, 5, budget))
                break;
            const unsigned char *pk = tc_smem + kTcPOff + (size_t)j * kTcPStageBytes;
            // every lane loads (lanes 30, 31 re-read row 30q+29 and clear it): no divergence
            uint2 pa[HW / 2], pb[HW / 2];
            {
                const uint2 *r = reinterpret_cast<const uint2 *>(pk + 4 * HW * h + arow_off);
#pragma unroll
                for (int m = 0; m < HW / 2; ++m) {
                    pa[m] = r[m];
                    pa[m].x = arow ? pa[m].x : 0u;
                    pa[m].y = arow ? pa[m].y : 0u;
                }
            }
            if (has_b) {
                const uint2 *r = reinterpret_cast<const uint2 *>(pk + kTcPABytes +
                                                                 u * (kTcChunkWords * 4) + 4 * HW * hb);
#pragma unroll
                for (int m = 0; m < HW / 2; ++m) pb[m] = r[m];
            }
            __syncwarp();
            mbar_arrive_warp(&pempty_bar[j]);
            // expand into registers before waiting for the stage: the wait is
            // on the MMAs kTcStages chunks back, and only the stores follow it
            uint32_t r[4 * HW], o[4 * HW];
#pragma unroll
            for (int m = 0; m < HW / 2; ++m) {
                expand_word(pa[m].x, r + 8 * m);
                expand_word(pa[m].y, r + 8 * m + 4);
            }
            if (has_b) {
#pragma unroll
                for (int m = 0; m < HW / 2; ++m) {
                    expand_word(pb[m].x, o + 8 * m);
                    expand_word(pb[m].y, o + 8 * m + 4);
                }
            }
            if (!mbar_wait_warp(&empty_bar[s], (((uint32_t)idx / kTcStages) & 1) ^ 1, vabort, err, 1,
                                budget))
                break;
            tc_fence_after();
            tmem_st16(ta0 + s * kTcAStageCols, r);
            if constexpr (HW == 6) tmem_st8(ta0 + s * kTcAStageCols + 16, r + 16);
            if (has_b) {
                unsigned char *bst = bst0 + (size_t)s * kTcBStageBytes;
#pragma unroll
                for (int m = 0; m < HW; ++m)
                    *reinterpret_cast<uint4 *>(bst + m * kTcLbo) =
                        make_uint4(o[4 * m], o[4 * m + 1], o[4 * m + 2], o[4 * m + 3]);
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_fence_before();
            __syncwarp();
            if (!(TEST && stall && idx == 0)) mbar_arrive_warp_cl(cluster_addr(&full_bar[s], 0));
        }
    } else if (warp == kTcTmaWarp) {
        // ---------------- bulk-copy issuer ----------------
        if (lane == 0) {
            int issued = 0;
            int2 tl = make_int2(0, 0), tl_next = make_int2(0, 0);
            if (my_tiles > 0) tl_next = tiles[pair];
            int k = -1, c = nchunks;
            for (int idx = 0; idx < total; ++idx) {
                if (++c >= nchunks) {
                    c = 0;
                    ++k;
                    tl = tl_next;
                    if (k + 1 < my_tiles) tl_next = tiles[pair + (k + 1) * npairs];
                }
                const uint32_t j = (uint32_t)idx % kTcPStages;
                if (!mbar_wait(&pempty_bar[j], (((uint32_t)idx / kTcPStages) & 1) ^ 1, vabort, err, 6,
                               budget))
                    break;
                unsigned char *pk = tc_smem + kTcPOff + (size_t)j * kTcPStageBytes;
                const uint32_t *base = blk + (size_t)c * rows_pad * kTcChunkWords;
                const size_t arow = (size_t)3 * (a0 + tl.x * kTcPairASnps + kTcASnps * (int)rank);
                const size_t brow = (size_t)3 * (b0 + tl.y * kTcBSnps) + kTcBRows * rank;
                mbar_expect_tx(&pfull_bar[j], kTcPStageBytes);
                bulk_load(pk, base + arow * kTcChunkWords, kTcPABytes, &pfull_bar[j]);
                bulk_load(pk + kTcPABytes, base + brow * kTcChunkWords, kTcPBBytes, &pfull_bar[j]);
                issued = idx + 1;
            }
            // every copy this thread issued lands before the CTA exits
            for (int idx = issued > kTcPStages ? issued - kTcPStages : 0; idx < issued; ++idx)
                mbar_drain(&pfull_bar[idx % kTcPStages], ((uint32_t)idx / kTcPStages) & 1);
        }
        __syncwarp();
    } else if (warp == kTcMmaWarp) {
        // ---------------- MMA issuer (even CTA) ----------------
        if (rank == 0 && lane == 0) {
            // stage s's descriptor: the start-address field (address >> 4) moves by
            // s * kTcBStageBytes >> 4 (no per-stage array: a runtime-indexed one
            // would live in local memory, one load per chunk on the issue path)
            const uint64_t bdesc0 = tc_bdesc(su32(tc_smem));
            const uint32_t sf = tbase + kTcSfCol;
            uint32_t gc = 0, lt = 0;
            bool ok = true;
            for (int t = pair; t < ntiles && ok; t += npairs, ++lt) {
                for (int c = 0; c < nchunks; ++c, ++gc) {
                    const int cls = c < cm.n0 ? 0 : 1;
                    if (c == 0 || c == cm.n0) {
                        // both CTAs' epilogues have copied this class half of the
                        // previous tile's accumulator out (while the other half was
                        // being accumulated): the tensor pipe never drains between tiles
                        if (!mbar_wait(&dempty_bar[cls], (lt & 1) ^ 1, vabort, err, 2, budget)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
                    const uint32_t s = gc % kTcStages;
                    const int nm = cm.mmas(c);
                    const uint32_t d = tbase + (uint32_t)(cls * kTcN);
                    const uint32_t acc0 = (c == 0 || c == cm.n0) ? 0u : 1u;
                    const uint32_t a = tbase + kTcACol + s * kTcAStageCols;
                    const uint64_t bd = bdesc0 + (uint64_t)((s * (uint32_t)kTcBStageBytes) >> 4);
                    if (!mbar_wait(&full_bar[s], (gc / kTcStages) & 1, vabort, err, 3, budget)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    // MMA kk reads A columns 8kk.. and the k-group pair 2kk (256 B further
                    // each: +16 in the descriptor's address field)
#pragma unroll
                    for (int kk = 0; kk < kTcChunkWords / 2; ++kk)
                        if (kk < nm) tc_mma2(d, a + kk * 8, bd + (uint64_t)(16 * kk), sf, kk == 0 ? acc0 : 1u);
                    tc_commit2_both(&empty_bar[s]);
                    if (c == cm.n0 - 1 || c == nchunks - 1) tc_commit2_both(&dfull_bar[cls]);
                }
            }
            // drain every MMA this thread issued before either CTA frees tensor memory
            tc_commit2(&fin_bar);
            mbar_drain(&fin_bar, 0);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue (warps 10-17) ----------------
        const TcSync S{pfull_bar, pempty_bar, full_bar, empty_bar, dfull_bar, dempty_bar,
                       vabort,    err,        budget};
        const TcScorer E(tc_smem, tbase, warp, rank);
        const float theta = DUMP ? 0.f : ctx.st->theta;
        const float lp_thr = DUMP ? 0.f : ctx.st->lp_thr;
        uint32_t lt = 0;
        for (int t = pair; t < ntiles; t += npairs, ++lt) {
            const int2 tl = tiles[t];
            if (!E.template tile<DUMP, OBJ>(S, lane, lt, tl.x, tl.y, a0, a1, b0, b1, ctx, theta, lp_thr,
                                            dump))
                break;
        }
    }

    tc_fence_before();
    __syncthreads();
    // the pair's MMAs have drained (the even CTA's issuer waited for them) and
    // no thread arrives on the peer's barriers any more
    cluster_sync_all();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTcCols)
                     : "memory");
    }
}


// ---- batched kernel: one launch over the tiles of many requests ------------
//
// The tiles of every request of an engine step form one work list (runs of
// consecutive tiles of a request's list, WorkRange); CTA pairs claim tiles
// from it with an atomic counter, so pairs that drew cheap tiles (few samples)
// take more of them.  The copy issuer of the even CTA claims: it resolves the
// claimed index to (request, A tile, B tile), writes it into slot k % kTcRing
// of a ring in both CTAs' shared memory and arrives on that slot's barrier in
// both (release at cluster scope for the peer); every other role reads tile k
// from the ring after waiting on the barrier (acquire at cluster scope in the
// odd CTA).  A request index < 0 ends the pair's work.
//
// Slots are reused without an "empty" barrier because the claimer cannot get
// kTcRing tiles ahead of the slowest reader: publishing tile K (writing its
// ring slot) waits for the packed-ring slot of K's first chunk, so the even
// CTA's producers have loaded
// chunk g - 4 (g = K's first chunk), hence waited for the MMAs of chunk g - 7,
// which the MMA thread issued only after both CTAs' producers finished chunk
// g - 7 and both CTAs' scoring warps released the accumulator of the tile
// before it.  Every tile has at least two chunks (one per class), so all
// readers have read the slots of tiles <= K - 5; K - kTcRing = K - 8 is older.
constexpr int kTcRing = 8;

__device__ __forceinline__ bool mbar_try_cluster(uint64_t *b, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(su32(b)), "r"(parity), "r"(kTcSuspendNs)
        : "memory");
    return done != 0;
}

// Bounded wait for ring slot `slot` of tile k (the odd CTA acquires at cluster
// scope: the claimer in the even CTA wrote it).
__device__ __forceinline__ bool ring_wait(uint64_t *b, uint32_t parity, uint32_t rank,
                                          const TcSync &S) {
    if (rank == 0) return mbar_wait(b, parity, S.abort_flag, S.err, 7, S.budget);
    if (mbar_try_cluster(b, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_cluster(b, parity)) {
        if (*S.abort_flag) return false;
        if (clock64() - t0 > S.budget) {
            *S.abort_flag = 1;
            atomicCAS(S.err, 0, 7);
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ ChunkMap chunk_map(int W0, int Wp) {
    ChunkMap cm;
    cm.W0 = W0;
    cm.W1 = Wp - W0;
    cm.n0 = (W0 + kTcChunkWords - 1) / kTcChunkWords;
    cm.nchunks = cm.n0 + (cm.W1 + kTcChunkWords - 1) / kTcChunkWords;
    return cm;
}

template <int OBJ, bool TEST>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kTcThreads, 1)
    tc_batch_kernel(const ReqDesc *__restrict__ reqs, WorkQueue *q, long long wait_cycles, int stall) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ uint64_t pfull_bar[kTcPStages], pempty_bar[kTcPStages], full_bar[kTcStages],
        empty_bar[kTcStages], dfull_bar[2], dempty_bar[2], fin_bar, ring_bar[kTcRing];
    __shared__ int4 ring[kTcRing];
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t rank = cluster_rank();
    TcSync S{pfull_bar, pempty_bar, full_bar, empty_bar, dfull_bar, dempty_bar, &abort_flag, &q->err,
             TEST ? wait_cycles : kTcWaitCycles};
    tc_prologue(S, &fin_bar, ring_bar, kTcRing, &tmem_slot, &abort_flag, tid, warp);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmem_slot;
    tc_scales(tbase, warp);
    tc_fence_before();
    __syncthreads();
    cluster_sync_all();
    tc_fence_after();

    // tile k of this pair from the ring (all lanes of a warp read the same slot)
    auto next_tile = [&](int k, int4 &d) -> bool {
        const int slot = k % kTcRing;
        if (!ring_wait(&ring_bar[slot], ((uint32_t)k / kTcRing) & 1, rank, S)) return false;
        const volatile int *v = reinterpret_cast<const volatile int *>(&ring[slot]);
        d = make_int4(v[0], v[1], v[2], v[3]);
        return d.x >= 0;
    };

    if (warp >= kTcProdWarp0 && warp < kTcEpiWarp0) {
        const TcProducer P(tc_smem, tbase, warp, lane);
        int idx = 0;
        bool ok = true;
        int4 d;
        for (int k = 0; ok && next_tile(k, d); ++k) {
            const ReqDesc &R = reqs[d.x];
            const int nch = chunk_map(R.W0, R.Wp).nchunks;
            for (int c = 0; c < nch && ok; ++c, ++idx) ok = P.chunk(tc_smem, S, idx, TEST && stall && idx == 0);
        }
    } else if (warp == kTcTmaWarp) {
        if (lane == 0) {
            int idx = 0, issued = 0;
            const uint32_t peer_ring = cluster_addr(ring, 1), peer_bar = cluster_addr(ring_bar, 1);
            // The even CTA claims tile k + 1 (atomic and work-list search) right
            // after issuing tile k's first copy, so their latency overlaps the
            // tile's copies; it is published -- as before -- only once the
            // packed-ring slot of its first chunk is free.
            int4 claimed = make_int4(-1, 0, 0, 0);
            bool have_claim = false;
            for (int k = 0;; ++k) {
                const int slot = k % kTcRing;
                int4 d;
                if (rank == 0) {
                    // publish only once the packed-ring slot of the tile's first chunk is free
                    const uint32_t j = (uint32_t)idx % kTcPStages;
                    if (!mbar_wait(&S.pempty[j], (((uint32_t)idx / kTcPStages) & 1) ^ 1, S.abort_flag,
                                   S.err, 6, S.budget))
                        break;
                    if (have_claim) {
                        d = claimed;
                    } else {
                        const int t = (int)atomicAdd(&q->next, 1u);
                        d = resolve_work(reqs, q, t);
                    }
                    have_claim = false;
                    ring[slot] = d;
                    asm volatile("st.shared::cluster.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(
                                     peer_ring + (uint32_t)(slot * sizeof(int4))),
                                 "r"(d.x), "r"(d.y), "r"(d.z), "r"(d.w)
                                 : "memory");
                    mbar_arrive(&ring_bar[slot]);
                    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(
                                     peer_bar + (uint32_t)(slot * sizeof(uint64_t)))
                                 : "memory");
                    if (d.x < 0) break;
                } else if (!next_tile(k, d)) {
                    break;
                }
                const ReqDesc &R = reqs[d.x];
                const ChunkMap cm = chunk_map(R.W0, R.Wp);
                const size_t arow = (size_t)3 * (R.a0 + d.y * kTcPairASnps + kTcASnps * (int)rank);
                const size_t brow = (size_t)3 * (R.b0 + d.z * kTcBSnps) + kTcBRows * rank;
                bool ok = true;
                for (int c = 0; c < cm.nchunks; ++c, ++idx) {
                    // the even CTA waited for its first chunk's slot before publishing
                    ok = tc_copy_chunk(tc_smem, S, idx, R.blk, R.rows_pad, c, arow, brow,
                                       !(rank == 0 && c == 0));
                    if (!ok) break;
                    issued = idx + 1;
                    if (rank == 0 && c == 0) {
                        const int t = (int)atomicAdd(&q->next, 1u);
                        claimed = resolve_work(reqs, q, t);
                        have_claim = true;
                    }
                }
                if (!ok) break;
            }
            tc_copy_drain(S, issued);
        }
        __syncwarp();
    } else if (warp == kTcMmaWarp) {
        if (rank == 0 && lane == 0) {
            // The single-request kernel's issuer loop, on this kernel's own
            // barrier arrays: the issuer is on every chunk's critical path, and
            // the same loop written against the TcSync pointers measured 7 %
            // slower.
            const uint64_t bdesc0 = tc_bdesc(su32(tc_smem));
            const uint32_t sf = tbase + kTcSfCol;
            volatile int *vabort = &abort_flag;
            int *err = &q->err;
            const long long budget = S.budget;
            uint32_t gc = 0, lt = 0;
            bool ok = true;
            int4 tk;
            for (int k = 0; ok && next_tile(k, tk); ++k, ++lt) {
                const ReqDesc &R = reqs[tk.x];
                const ChunkMap cm = chunk_map(R.W0, R.Wp);
                const int nchunks = cm.nchunks;
                for (int c = 0; c < nchunks; ++c, ++gc) {
                    const int cls = c < cm.n0 ? 0 : 1;
                    if (c == 0 || c == cm.n0) {
                        // both CTAs' epilogues have copied this class half of the
                        // previous tile's accumulator out
                        if (!mbar_wait(&dempty_bar[cls], (lt & 1) ^ 1, vabort, err, 2, budget)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
                    const uint32_t s = gc % kTcStages;
                    const int nm = cm.mmas(c);
                    const uint32_t d = tbase + (uint32_t)(cls * kTcN);
                    const uint32_t acc0 = (c == 0 || c == cm.n0) ? 0u : 1u;
                    const uint32_t a = tbase + kTcACol + s * kTcAStageCols;
                    const uint64_t bd = bdesc0 + (uint64_t)((s * (uint32_t)kTcBStageBytes) >> 4);
                    if (!mbar_wait(&full_bar[s], (gc / kTcStages) & 1, vabort, err, 3, budget)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
#pragma unroll
                    for (int kk = 0; kk < kTcChunkWords / 2; ++kk)
                        if (kk < nm) tc_mma2(d, a + kk * 8, bd + (uint64_t)(16 * kk), sf, kk == 0 ? acc0 : 1u);
                    tc_commit2_both(&empty_bar[s]);
                    if (c == cm.n0 - 1 || c == nchunks - 1) tc_commit2_both(&dfull_bar[cls]);
                }
            }
            // drain every MMA this thread issued before either CTA frees tensor memory
            tc_commit2(&fin_bar);
            mbar_drain(&fin_bar, 0);
        }
        __syncwarp();
    } else {
        const TcScorer E(tc_smem, tbase, warp, rank);
        uint32_t lt = 0;
        int4 d;
        for (int k = 0; next_tile(k, d); ++k, ++lt) {
            const ReqDesc &R = reqs[d.x];
            const ScanCtx ctx = R.ctx;
            const float theta = ctx.st->theta, lp_thr = ctx.st->lp_thr;
            if (!E.template tile<false, OBJ>(S, lane, lt, d.y, d.z, R.a0, R.a1, R.b0, R.b1, ctx, theta,
                                             lp_thr, nullptr))
                break;
        }
    }
    tc_teardown(tbase, warp);
}

// Block-major operand layout (see the file comment).
__global__ void tc_relayout_kernel(const uint32_t *__restrict__ planes, int Wp, int W0, int nrows,
                                   int rows_pad, int n0, int nblk, uint32_t *__restrict__ blk) {
    const size_t total = (size_t)nblk * rows_pad * kTcChunkWords;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int w = (int)(i % kTcChunkWords);
        const size_t br = i / kTcChunkWords;
        const int row = (int)(br % rows_pad), b = (int)(br / rows_pad);
        const int start = b < n0 ? kTcChunkWords * b : W0 + kTcChunkWords * (b - n0);
        const int end = b < n0 ? W0 : Wp;
        uint32_t v = 0;
        if (row < nrows && start + w < end) v = planes[(size_t)row * Wp + start + w];
        blk[i] = v;
    }
}

void tc_block_shape(int n_snps, int Wp, int W0, int *rows_pad, int *nblk) {
    const int n0 = (W0 + kTcChunkWords - 1) / kTcChunkWords;
    const int n1 = (Wp - W0 + kTcChunkWords - 1) / kTcChunkWords;
    // a copy from any SNP's first row (A: up to 80 SNPs on, 120 rows; B: 192 rows) stays inside
    *rows_pad = 3 * n_snps + std::max(3 * kTcPairASnps, kTcN);
    *nblk = n0 + n1;
}

size_t tc_block_words(int n_snps, int Wp, int W0) {
    int rows_pad, nblk;
    tc_block_shape(n_snps, Wp, W0, &rows_pad, &nblk);
    return (size_t)nblk * rows_pad * kTcChunkWords;
}

cudaError_t launch_tc_relayout(const uint32_t *planes, int Wp, int W0, int n_snps, uint32_t *blk,
                               int num_sms, cudaStream_t stream) {
    int rows_pad, nblk;
    tc_block_shape(n_snps, Wp, W0, &rows_pad, &nblk);
    const int n0 = (W0 + kTcChunkWords - 1) / kTcChunkWords;
    tc_relayout_kernel<<<num_sms * 8, 256, 0, stream>>>(planes, Wp, W0, 3 * n_snps, rows_pad, n0,
                                                         nblk, blk);
    return cudaGetLastError();
}

// Pairs of CTAs the GPU holds at once (each pair on two SMs of one GPC): the
// persistent grid, asked of the occupancy calculator once per device.
template <class K>
static cudaError_t resident_pairs(K kern, int num_sms, cudaStream_t stream, int *out) {
    static std::atomic<int> resident[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int pairs = dev < 64 ? resident[dev].load() : 0;
    if (pairs <= 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2 * (num_sms / 2));
        cfg.blockDim = dim3(kTcThreads);
        cfg.dynamicSmemBytes = kTcSmem;
        cfg.stream = stream;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, (const void *)kern, &cfg) != cudaSuccess || nc <= 0) {
            (void)cudaGetLastError();
            nc = num_sms / 2;
        }
        pairs = std::min(nc, num_sms / 2);
        if (dev < 64) resident[dev].store(pairs);
    }
    *out = pairs;
    return cudaSuccess;
}

// The timeout test's settings (GEPI_DEBUG_STALL=<cycles>): true when set.
static bool debug_stall(long long *wait_cycles) {
    *wait_cycles = kTcWaitCycles;
    if (const char *w = std::getenv("GEPI_DEBUG_STALL")) {
        const long long v = std::atoll(w);
        if (v > 0) {
            *wait_cycles = std::min(v, kTcWaitCycles);
            return true;
        }
    }
    return false;
}

template <bool DUMP, int OBJ, bool TEST>
static cudaError_t launch_tc_pairs(const uint32_t *blk, int rows_pad, int Wp, int W0,
                                   const int2 *tiles, int ntiles, int a0, int a1, int b0, int b1,
                                   const ScanCtx &ctx, uint32_t *dump, int *err, int num_sms,
                                   long long wait_cycles, cudaStream_t stream) {
    auto kern = tc_tile_kernel<DUMP, OBJ, TEST>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    if (e != cudaSuccess) return e;
    int pairs = 0;
    if ((e = resident_pairs(kern, num_sms, stream, &pairs)) != cudaSuccess) return e;
    pairs = std::max(1, std::min(pairs, ntiles));
    kern<<<2 * pairs, kTcThreads, kTcSmem, stream>>>(blk, rows_pad, Wp, W0, tiles, ntiles, a0, a1,
                                                    b0, b1, ctx, dump, err, wait_cycles, TEST ? 1 : 0);
    return cudaGetLastError();
}

__device__ __forceinline__ void pending_test(const ScanCtx &ctx, uint4 e) {
    exact_test(ctx, (int)e.x, (int)(e.y >> 3), (int)(e.y & 7u), (int)(e.z & 0xFFFFu),
               (int)(e.z >> 16), (int)(e.w & 0xFFFFu), (int)(e.w >> 16));
}

// The Fisher tests a counting launch left in ctx.pend (the first min(count,
// cap); any beyond were evaluated in the launch), one per thread.
__global__ void __launch_bounds__(256) fisher_pending_kernel(ScanCtx ctx) {
    const PendList &L = *ctx.pend;
    const uint32_t n = min(L.n, L.cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        pending_test(ctx, L.ent[i]);
}

// The same for a batched engine step: one list for all its requests, each
// entry evaluated with its own request's tables, threshold and buffer.
__global__ void __launch_bounds__(256)
    fisher_pending_batch_kernel(const ReqDesc *__restrict__ reqs, const PendList *list) {
    const PendList &L = *list;
    const uint32_t n = min(L.n, L.cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // a local copy, as every other caller of exact_test passes one
        const ScanCtx ctx = reqs[L.tag[i]].ctx;
        pending_test(ctx, L.ent[i]);
    }
}

cudaError_t launch_fisher_pending(const ScanCtx &ctx, int num_sms, cudaStream_t stream) {
    fisher_pending_kernel<<<num_sms * 4, 256, 0, stream>>>(ctx);
    return cudaGetLastError();
}

cudaError_t launch_fisher_pending_batch(const ReqDesc *reqs, const PendList *list, int num_sms,
                                        cudaStream_t stream) {
    fisher_pending_batch_kernel<<<num_sms * 4, 256, 0, stream>>>(reqs, list);
    return cudaGetLastError();
}

cudaError_t launch_tc_tiles(const uint32_t *blk, int n_snps, int Wp, int W0, const int2 *tiles,
                            int ntiles, int a0, int a1, int b0, int b1, const ScanCtx &ctx,
                            uint32_t *dump, int *err, int num_sms, cudaStream_t stream) {
    if (ntiles <= 0) return cudaSuccess;
    // whole K = 64 MMAs per class, 16-byte aligned copies, counts that fit the
    // scoring warps' 16-bit exchange
    if ((W0 & 1) || (Wp & 1) || W0 <= 0 || Wp <= W0 || (reinterpret_cast<uintptr_t>(blk) & 15) ||
        32 * W0 > kTcMaxClass + 31 + 32 || 32 * (Wp - W0) > kTcMaxClass + 31 + 32)
        return cudaErrorInvalidValue;
    int rows_pad, nblk;
    tc_block_shape(n_snps, Wp, W0, &rows_pad, &nblk);
    long long wc = 0;
    const bool test = debug_stall(&wc);
    if (dump)
        return test ? launch_tc_pairs<true, 0, true>(blk, rows_pad, Wp, W0, tiles, ntiles, a0, a1, b0,
                                                     b1, ctx, dump, err, num_sms, wc, stream)
                    : launch_tc_pairs<true, 0, false>(blk, rows_pad, Wp, W0, tiles, ntiles, a0, a1, b0,
                                                      b1, ctx, dump, err, num_sms, wc, stream);
    if (ctx.objective == 0)
        return test ? launch_tc_pairs<false, 0, true>(blk, rows_pad, Wp, W0, tiles, ntiles, a0, a1,
                                                      b0, b1, ctx, nullptr, err, num_sms, wc, stream)
                    : launch_tc_pairs<false, 0, false>(blk, rows_pad, Wp, W0, tiles, ntiles, a0, a1,
                                                       b0, b1, ctx, nullptr, err, num_sms, wc, stream);
    return launch_tc_pairs<false, 1, false>(blk, rows_pad, Wp, W0, tiles, ntiles, a0, a1, b0, b1, ctx,
                                            nullptr, err, num_sms, wc, stream);
}

// setup: the shared-memory opt-in and the occupancy query only (outside any
// stream capture); the engine does it before it captures a step graph.
template <int OBJ, bool TEST>
static cudaError_t launch_tc_batch_obj(const ReqDesc *reqs, WorkQueue *q, int num_sms,
                                       long long wait_cycles, bool setup, cudaStream_t stream) {
    auto kern = tc_batch_kernel<OBJ, TEST>;
    int pairs = 0;
    if (setup) {
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
        if (e == cudaSuccess) e = resident_pairs(kern, num_sms, stream, &pairs);
        return e;
    }
    cudaError_t e = resident_pairs(kern, num_sms, stream, &pairs);
    if (e != cudaSuccess) return e;
    kern<<<2 * std::max(1, pairs), kTcThreads, kTcSmem, stream>>>(reqs, q, wait_cycles, TEST ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_tc_batch(const ReqDesc *reqs, WorkQueue *q, int objective, int num_sms,
                            cudaStream_t stream, bool setup) {
    long long wc = 0;
    const bool test = debug_stall(&wc);
    if (objective == 0)
        return test ? launch_tc_batch_obj<0, true>(reqs, q, num_sms, wc, setup, stream)
                    : launch_tc_batch_obj<0, false>(reqs, q, num_sms, wc, setup, stream);
    return launch_tc_batch_obj<1, false>(reqs, q, num_sms, wc, setup, stream);
}

bool tc_debug_stall() {
    long long wc = 0;
    return debug_stall(&wc);
}

bool tc_shape_ok(int Wp, int W0) {
    return !((W0 & 1) || (Wp & 1) || W0 <= 0 || Wp <= W0 || 32 * W0 > kTcMaxClass + 31 + 32 ||
             32 * (Wp - W0) > kTcMaxClass + 31 + 32);
}

int tc_rows_pad(int n_snps) {
    int rows_pad = 0, nblk = 0;
    tc_block_shape(n_snps, 2, 0, &rows_pad, &nblk);
    return rows_pad;
}

// Dense block-scaled FP4 MMA rates of this GPU, the roofline denominator of the
// tensor-core counting kernel: one CTA per SM issues `iters` back-to-back
// M=128 x N=256 x K=64 MMAs (A in tensor memory, B in shared memory, unit
// scales) and waits for them once.  Three exact encodings of 0/1 operands are
// probed (PTX tcgen05.mma block_scale forms):
//   kind 0: kind::mxf4,     scale_vec::2X, UE8M0 scales (the counting kernel's)
//   kind 1: kind::mxf4nvf4, scale_vec::2X, UE8M0 scales
//   kind 2: kind::mxf4nvf4, scale_vec::4X, UE4M3 scales
// A and B are E2M1 in every kind; all scale factors are 1.0 (UE8M0 0x7F, UE4M3
// 0x38), so the products are the same 0/1 values.
constexpr int kTcPeakKinds = 3;
template <int KIND>
__host__ __device__ constexpr uint32_t tc_peak_idesc() {
    return (1u << 7) | (1u << 10) | ((uint32_t)(256 >> 3) << 17) | (KIND == 2 ? 0u : (1u << 23)) |
           ((uint32_t)(128 >> 4) << 24);
}
constexpr int kTcPeakSmem = 120 * 1024;  // one CTA per SM

template <int KIND>
__device__ __forceinline__ void tc_peak_mma(uint32_t d, uint32_t a, uint64_t bd, uint32_t sf,
                                            uint32_t acc) {
    if constexpr (KIND == 0)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %5, 0;\n"
            " tcgen05.mma.cta_group::1.kind::mxf4.block_scale.scale_vec::2X [%0], [%1], %2, %3, "
            "[%4], [%4], p;\n}\n" ::"r"(d),
            "r"(a), "l"(bd), "r"(tc_peak_idesc<KIND>()), "r"(sf), "r"(acc));
    else if constexpr (KIND == 1)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %5, 0;\n"
            " tcgen05.mma.cta_group::1.kind::mxf4nvf4.block_scale.scale_vec::2X [%0], [%1], %2, %3, "
            "[%4], [%4], p;\n}\n" ::"r"(d),
            "r"(a), "l"(bd), "r"(tc_peak_idesc<KIND>()), "r"(sf), "r"(acc));
    else
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %5, 0;\n"
            " tcgen05.mma.cta_group::1.kind::mxf4nvf4.block_scale.scale_vec::4X [%0], [%1], %2, %3, "
            "[%4], [%4], p;\n}\n" ::"r"(d),
            "r"(a), "l"(bd), "r"(tc_peak_idesc<KIND>()), "r"(sf), "r"(acc));
}

template <int KIND>
__global__ void __launch_bounds__(128, 1) tc_peak_kernel(int iters, int *err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ uint64_t done_bar;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 8192 / 4; i += blockDim.x)
        reinterpret_cast<uint32_t *>(tc_smem)[i] = 0x22222222u;  // E2M1 1.0
    if (tid == 0) {
        mbar_init(&done_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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
    {
        const uint32_t one = KIND == 2 ? 0x38383838u : 0x7F7F7F7Fu;  // unit scales
        uint32_t r[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) r[k] = one;
        tmem_st32(tbase + ((uint32_t)(32 * warp) << 16) + kTcSfCol, r);
#pragma unroll
        for (int k = 0; k < 32; ++k) r[k] = 0x22222222u;
        tmem_st32(tbase + ((uint32_t)(32 * warp) << 16) + 256, r);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
        tc_fence_after();
        // 256 B rows x 32 B (one K = 64 block): core matrices 128 B apart along K,
        // 8-row groups 256 B apart
        const uint64_t bd = (uint64_t)((su32(tc_smem) & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) |
                            ((uint64_t)(256 >> 4) << 32) | (1ull << 46);
        const uint32_t sf = tbase + kTcSfCol;
        for (int i = 0; i < iters; ++i) tc_peak_mma<KIND>(tbase, tbase + 256, bd, sf, i > 0 ? 1u : 0u);
        tc_commit(&done_bar);
        const long long t0 = clock64();
        while (!mbar_try(&done_bar, 0)) {
            if (clock64() - t0 > kTcWaitCycles) {
                atomicExch(err, 7);
                break;
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

// Best of `reps` timed launches of probe `kind`; TFLOP/s counting 2 per
// multiply-accumulate.
cudaError_t tc_measure_peak(int num_sms, int reps, int kind, double *tflops, int *err,
                            cudaStream_t stream) {
    if (kind < 0 || kind >= kTcPeakKinds) return cudaErrorInvalidValue;
    auto kern = kind == 0 ? tc_peak_kernel<0> : kind == 1 ? tc_peak_kernel<1> : tc_peak_kernel<2>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kTcPeakSmem);
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess) return e;
    if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return e;
    }
    const int iters = 16384;
    double best = 0.0;
    for (int r = 0; r < reps + 1 && e == cudaSuccess; ++r) {
        cudaEventRecord(e0, stream);
        kern<<<num_sms, 128, kTcPeakSmem, stream>>>(iters, err);
        cudaEventRecord(e1, stream);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        float ms = 0.f;
        if (e == cudaSuccess && r > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f) {
            const double flop = 2.0 * num_sms * (double)iters * 128.0 * 256.0 * 64.0;
            best = std::max(best, flop / (ms * 1e-3) / 1e12);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return e;
}

int tc_max_class() { return kTcMaxClass; }

}  // namespace gepi
