// Host-side internals shared by the plane-set code (scan.cu) and the scan
// engine (engine.cu): kernel launchers, the plane-set handle, helpers.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "common.h"
#include "device.cuh"

namespace gepi {

cudaError_t launch_decode_bed(const uint8_t *bed_payload, size_t bps, int n_snps,
                              const int32_t *perm, int Wp, uint32_t *planes, cudaStream_t stream);
cudaError_t launch_marginal(const uint32_t *planes, int n_snps, int Wp, int W0, float *score,
                            int num_sms, cudaStream_t stream);
cudaError_t launch_decode_rows(const uint64_t *bits, const uint64_t *valid, int nw, int n_snps,
                               const int32_t *perm, int Wp, uint32_t *planes,
                               cudaStream_t stream, int num_sms);
// Popcount kernel of tile height ta (32 or 64 A SNPs; B tiles hold 32) and kc
// plane words per pipeline stage (16 or 32).
cudaError_t launch_popc_tiles(int ta, int kc, const uint32_t *planes, int Wp, int W0,
                              const int2 *tiles, int ntiles, int a0, int a1, int b0, int b1,
                              const ScanCtx &ctx, uint32_t *dump, cudaStream_t stream);
// Exact evaluation of the Fisher tests a counting launch left in ctx.pend.
cudaError_t launch_fisher_pending(const ScanCtx &ctx, int num_sms, cudaStream_t stream);
// The same for a batched engine step's shared list (entries tagged by request).
cudaError_t launch_fisher_pending_batch(const ReqDesc *reqs, const PendList *list, int num_sms,
                                        cudaStream_t stream);
cudaError_t launch_tc_tiles(const uint32_t *blk, int n_snps, int Wp, int W0, const int2 *tiles,
                            int ntiles, int a0, int a1, int b0, int b1, const ScanCtx &ctx,
                            uint32_t *dump, int *err, int num_sms, cudaStream_t stream);
cudaError_t launch_tc_relayout(const uint32_t *planes, int Wp, int W0, int n_snps, uint32_t *blk,
                               int num_sms, cudaStream_t stream);
// Batched engine: one persistent launch over the work list `q` of many
// requests (reqs), tiles claimed with an atomic counter.  Tensor cores: every
// request of one objective; popcount: every request of one (ta, kc) variant.
// setup = true: only the kernel's shared-memory opt-in and occupancy query,
// done once outside any stream capture before a launch is captured.
cudaError_t launch_tc_batch(const ReqDesc *reqs, WorkQueue *q, int objective, int num_sms,
                            cudaStream_t stream, bool setup = false);
cudaError_t launch_popc_batch(int ta, int kc, const ReqDesc *reqs, WorkQueue *q, int num_sms,
                              cudaStream_t stream, bool setup = false);
bool tc_shape_ok(int Wp, int W0);  // class widths the tensor-core kernel takes
bool tc_debug_stall();             // the timeout test's setting (GEPI_DEBUG_STALL) is on
int fisher_fp64_walks();           // GEPI_DEBUG_FISHER_FP64: Fisher walks in FP64 at any N
int tc_rows_pad(int n_snps);       // rows of the block-major operand copy
size_t tc_block_words(int n_snps, int Wp, int W0);
cudaError_t tc_measure_peak(int num_sms, int reps, int kind, double *tflops, int *err,
                            cudaStream_t stream);
int tc_max_class();  // samples per class the tensor-core kernel takes
cudaError_t run_select_compact(Cand *in, Cand *out, ScanState *st, void *sel, uint32_t cap,
                               uint32_t k, int n_override, uint32_t n_compact, int objective,
                               float lp_margin, int num_sms, cudaStream_t stream);
size_t sel_state_bytes();
constexpr int kSelectLaunches = 20;  // init + 8 x (histogram, pick) + apply + compact + count
// The selects of every request of an engine step, decided on the device
// (20 launches whatever the number of requests).
cudaError_t run_select_batch(SelJob *jobs, int njobs, int num_sms, cudaStream_t stream);

// Counting variants: a counting kernel with its tile shape and plane words per
// pipeline stage.  Every variant gives the same results bit for bit; the
// autotuner times them per plane-set shape (replacing the reference's
// --block-sizes / --max-grid-area, gEpiCount.cpp:135-141, misc1.cu:35-89).
// Ids are 1-based and stable (gepi_count_variant_name).
struct CountVariant {
    int id;
    int method;  // GEPI_METHOD_POPC or GEPI_METHOD_TENSOR
    int ta, tb;  // SNPs per tile, A x B
    int words;   // plane words (32 samples each) per pipeline stage
    const char *name;
};
constexpr int kNumVariants = 4;
constexpr int kVariantPopcDefault = 1;  // GEPI_METHOD_POPC
constexpr int kVariantTensor = 4;       // GEPI_METHOD_TENSOR
const CountVariant *count_variant(int id);  // nullptr outside [1, kNumVariants]
// One counting launch of variant v over tiles[0, ntiles).
cudaError_t launch_count(const CountVariant &v, const gepi_planes *pl, const int2 *tiles,
                         int ntiles, int a0, int a1, int b0, int b1, const ScanCtx &ctx,
                         uint32_t *dump, int *err, cudaStream_t stream);

// Candidates a scan lets accumulate before a device select raises its
// threshold: 16 k (at least 64 Ki), at most half the buffer.  Raising the
// threshold early keeps the bound passes -- and the exact scoring they cost --
// for the few tests near the final top-k; the results do not depend on it.
// A tiles per band of a tile list (build_tiles): bands of about 320 A SNPs
// whatever the tile height.
inline int tile_band(int TA) { return std::max(1, 320 / TA); }

inline uint32_t select_budget(uint32_t cap, int k) {
    const uint64_t want = std::max<uint64_t>(65536u, 16ull * (uint64_t)k);
    return (uint32_t)std::min<uint64_t>(cap / 2, want);
}
// Tests in a scan's first batch: half the select budget (Fisher: 64 Ki).
// The threshold is raised to the k-th best candidate after every batch that
// leaves more than this many: a stale threshold lets every later test above it
// through the bounds and into the candidate buffer (one global atomic each),
// which costs far more than the select.
inline uint32_t select_trigger(uint32_t budget, int k) {
    return (uint32_t)std::min<uint64_t>(budget, std::max<uint64_t>(1024u, 2ull * (uint64_t)k));
}
inline double pilot_tests(int objective, uint32_t budget) {
    return objective == GEPI_ENTROPY ? budget / 2.0 : 1.0 * (1 << 16);
}

struct DeviceGuard {
    int prev = -1;
    bool ok = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

template <class T>
void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// Plane-set memory (planes, operand blocks, candidate buffers, staging) comes
// from one stream-ordered pool per device that keeps freed memory for reuse
// (scan.cu): building plane sets over and over (one per cohort, request or
// step) then costs no cudaMalloc / cudaFree of hundreds of MB each time.
cudaError_t pool_alloc(int device, void **p, size_t bytes, cudaStream_t s);
template <class T>
cudaError_t pool_alloc(int device, T **p, size_t bytes, cudaStream_t s) {
    return pool_alloc(device, reinterpret_cast<void **>(p), bytes, s);
}
template <class T>
void pool_free(T *&p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
}


// Plane-set helpers (scan.cu).
gepi_status pl_check_mem(size_t bytes, const char *what);
}  // namespace gepi

// The plane-set handle of the C ABI.
struct gepi_planes {
    uint64_t serial = 0;  // unique per plane set in the process (keys cached tile orders)
    int device = 0, num_sms = 0;
    int auto_variant = 0;  // AUTO's counting variant for this plane set (0 = not tuned yet)
    float tune_ms[gepi::kNumVariants + 1] = {};  // autotuner timing of variant v (0: untimed)
    int n_snps = 0, S0 = 0, S1 = 0, W0 = 0, W1 = 0, Wp = 0;
    uint32_t *d_planes = nullptr;
    uint32_t *d_tc_blocks = nullptr;  // block-major copy for the tensor-core kernel (lazy)
    std::vector<float> marginal;      // per-SNP marginal phi^2 (lazy; orders scan tiles)
    cudaStream_t stream = nullptr;
    uint64_t *d_T = nullptr;
    int F = 0;
    double *d_lf = nullptr;
    float *d_lf32 = nullptr;
    float lf_max = 0.f;
    gepi::Cand *d_cand[2] = {nullptr, nullptr};
    uint32_t cap = 0;
    // Fisher pending list of the scans (lazy): its PendList header, then the entries
    gepi::PendList *d_pend = nullptr;
    gepi::ScanState *d_state = nullptr;
    gepi::ScanState *h_state = nullptr;
    void *d_sel = nullptr;
    int2 *d_tiles = nullptr;
    size_t tiles_cap = 0;
    // the scan tile list d_tiles holds (ranges, tile shape, hot-first order);
    // any other upload of d_tiles clears tiles_valid
    bool tiles_valid = false;
    std::array<int64_t, 7> tiles_key{};
    size_t tiles_n = 0;
    std::vector<cudaEvent_t> ev;  // timing events, reused across scans
    gepi_scan_stats stats{};
    std::vector<double> last_values;  // FP64 objective of the last ranked list (gepi_last_scan_values)
};


namespace gepi {

gepi_status pl_ensure_tables(gepi_planes *pl);
gepi_status pl_ensure_tc_blocks(gepi_planes *pl);
// Counting variant of a request (method, optional variant id; AUTO tunes once per plane set).
gepi_status pl_resolve_variant(gepi_planes *pl, int m, int variant, const CountVariant **out);
// The tile list of a triangle scan: bands of about 320 A SNPs, and with `hot`
// the tiles of the strongest marginal SNPs first (large lists only).
gepi_status pl_scan_tiles(gepi_planes *pl, int a0, int a1, int b0, int b1, int TA, int TB, bool hot,
                          std::vector<int2> &out);
void pl_build_tiles(int a0, int a1, int b0, int b1, int TA, int TB, bool triangle, int band,
                    std::vector<int2> &out);

}  // namespace gepi
