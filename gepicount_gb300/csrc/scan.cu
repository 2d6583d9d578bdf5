// Scan orchestration and the C ABI (include/gepi.h).
//
// Replaces launch_process_gpu_1 (src/kernels/kernel1.cu:295-505): instead of
// square batches of 4096 x 4096 allele rows with a full device sort, a host
// D2H of every count and a host merge per batch, the scan walks a list of
// 32 x 32 SNP tile pairs (lower triangle of the SNP-pair matrix, or the
// rectangle of a range request) in a few adaptive batches.  Each batch is one
// launch of the counting kernel with the fused epilogue; between batches a
// device radix select raises the ranking threshold and compacts the candidate
// buffer.  Only the final survivors (about k records) cross PCIe/C2C.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"
#include "tables.h"

namespace gepi {

static thread_local std::string g_last_error;

gepi_status set_error(gepi_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}
void clear_error() { g_last_error.clear(); }

}  // namespace gepi

using namespace gepi;

namespace {

// Bytes the pool keeps after frees (kPoolKeep at most).
constexpr uint64_t kPoolKeep = 8ull << 30;

cudaMemPool_t device_pool(int device) {
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    std::lock_guard<std::mutex> lk(mu);
    auto it = pools.find(device);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    uint64_t keep = kPoolKeep;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[device] = p;
    return p;
}

// Memory the pool holds unused (counts as free).
size_t pool_idle_bytes(int device) {
    cudaMemPool_t p = device_pool(device);
    uint64_t res = 0, used = 0;
    if (!p || cudaMemPoolGetAttribute(p, cudaMemPoolAttrReservedMemCurrent, &res) != cudaSuccess ||
        cudaMemPoolGetAttribute(p, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess)
        return 0;
    return res > used ? (size_t)(res - used) : 0;
}

gepi_status check_mem(size_t bytes, const char *what) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return GEPI_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) fr += pool_idle_bytes(dev);
    if (bytes + (64u << 20) > fr)
        return set_error(GEPI_ERR_OOM, std::string(what) + ": needs " + std::to_string(bytes >> 20) +
                                           " MiB, " + std::to_string(fr >> 20) + " MiB free");
    return GEPI_OK;
}

// Class-sorted permutation: slot -> source sample (-1 = pad).
void build_perm(const std::vector<int> &cls0, const std::vector<int> &cls1, int W0, int Wp,
                std::vector<int32_t> &perm) {
    perm.assign((size_t)Wp * 32, -1);
    for (size_t j = 0; j < cls0.size(); ++j) perm[j] = cls0[j];
    for (size_t j = 0; j < cls1.size(); ++j) perm[(size_t)W0 * 32 + j] = cls1[j];
}

gepi_status planes_alloc(gepi_planes *pl, int device, int n_snps, int S0, int S1) {
    pl->device = device;
    pl->n_snps = n_snps;
    pl->S0 = S0;
    pl->S1 = S1;
    // every class gets at least one padded block, so an empty class still has
    // (all-zero) words for the counting kernels to sum
    pl->W0 = std::max(1, (S0 + kClassPadSamples - 1) / kClassPadSamples) * (kClassPadSamples / 32);
    pl->W1 = std::max(1, (S1 + kClassPadSamples - 1) / kClassPadSamples) * (kClassPadSamples / 32);
    pl->Wp = pl->W0 + pl->W1;
    GEPI_CUDA(cudaDeviceGetAttribute(&pl->num_sms, cudaDevAttrMultiProcessorCount, device));
    GEPI_CUDA(cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking));
    size_t bytes = (size_t)n_snps * 3 * pl->Wp * 4;
    GEPI_TRY(check_mem(bytes, "genotype planes"));
    GEPI_CUDA(pool_alloc(device, &pl->d_planes, bytes, pl->stream));
    return GEPI_OK;
}

void planes_free(gepi_planes *pl) {
    if (!pl) return;
    DeviceGuard g(pl->device);
    if (pl->stream) {
        pool_free(pl->d_planes, pl->stream);
        pool_free(pl->d_tc_blocks, pl->stream);
        pool_free(pl->d_cand[0], pl->stream);
        pool_free(pl->d_cand[1], pl->stream);
        pool_free(pl->d_pend, pl->stream);
        pool_free(pl->d_T, pl->stream);
        pool_free(pl->d_lf, pl->stream);
        pool_free(pl->d_lf32, pl->stream);
        pool_free(pl->d_state, pl->stream);
        pool_free(pl->d_sel, pl->stream);
        pool_free(pl->d_tiles, pl->stream);
        cudaStreamSynchronize(pl->stream);
    }
    if (pl->h_state) cudaFreeHost(pl->h_state);
    pl->h_state = nullptr;
    for (cudaEvent_t e : pl->ev) cudaEventDestroy(e);
    pl->ev.clear();
    if (pl->stream) cudaStreamDestroy(pl->stream);
    pl->stream = nullptr;
}

// The scoring tables of a sample count (the fixed-point T(n) table takes
// milliseconds to build), kept for the process: plane sets of one cohort size
// -- one per step of an end-to-end loop, or many cohorts of one study -- build
// them once.  At most kTableCacheBytes are kept; a full cache starts over.
struct ScoreTables {
    int F = 0;
    std::vector<uint64_t> T;
    std::vector<double> lf;
    std::vector<float> lf32;
};
constexpr size_t kTableCacheBytes = 64ull << 20;

std::shared_ptr<const ScoreTables> score_tables(int64_t nmax) {
    static std::mutex mu;
    static std::map<int64_t, std::shared_ptr<const ScoreTables>> cache;
    static size_t bytes = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(nmax);
        if (it != cache.end()) return it->second;
    }
    auto t = std::make_shared<ScoreTables>();
    t->F = tfix_bits(nmax);
    build_tfix(nmax, t->F, t->T);
    build_lfact(nmax, t->lf, t->lf32);
    const size_t b = t->T.size() * 8 + t->lf.size() * 8 + t->lf32.size() * 4;
    std::lock_guard<std::mutex> lk(mu);
    if (bytes + b > kTableCacheBytes) {
        cache.clear();
        bytes = 0;
    }
    if (cache.emplace(nmax, t).second) bytes += b;
    return t;
}

gepi_status ensure_tables(gepi_planes *pl) {
    if (pl->d_T) return GEPI_OK;
    const int64_t nmax = (int64_t)pl->S0 + pl->S1;
    const std::shared_ptr<const ScoreTables> t = score_tables(nmax);
    pl->F = t->F;
    pl->lf_max = (float)t->lf.back();
    GEPI_CUDA(pool_alloc(pl->device, &pl->d_T, t->T.size() * 8, pl->stream));
    GEPI_CUDA(pool_alloc(pl->device, &pl->d_lf, t->lf.size() * 8, pl->stream));
    GEPI_CUDA(pool_alloc(pl->device, &pl->d_lf32, t->lf32.size() * 4, pl->stream));
    GEPI_CUDA(cudaMemcpyAsync(pl->d_T, t->T.data(), t->T.size() * 8, cudaMemcpyHostToDevice, pl->stream));
    GEPI_CUDA(cudaMemcpyAsync(pl->d_lf, t->lf.data(), t->lf.size() * 8, cudaMemcpyHostToDevice,
                              pl->stream));
    GEPI_CUDA(cudaMemcpyAsync(pl->d_lf32, t->lf32.data(), t->lf32.size() * 4, cudaMemcpyHostToDevice,
                              pl->stream));
    GEPI_CUDA(cudaStreamSynchronize(pl->stream));  // `t` may leave the cache once this returns
    return GEPI_OK;
}

gepi_status ensure_scan_buffers(gepi_planes *pl, int k) {
    uint64_t want = std::max<uint64_t>(1u << 22, ((uint64_t)k * 8 + 1023) & ~1023ull);
    // GEPI_DEBUG_CAP shrinks the candidate buffer (>= 4k entries) so tests can
    // drive the overflow / retry path on small inputs.
    if (const char *e = std::getenv("GEPI_DEBUG_CAP")) {
        long long v = std::atoll(e);
        if (v > 0) want = std::max<uint64_t>((uint64_t)v, 4ull * (uint64_t)k);
        if (pl->cap != want) {
            pool_free(pl->d_cand[0], pl->stream);
            pool_free(pl->d_cand[1], pl->stream);
            pl->cap = 0;
        }
    }
    if (want > (1ull << 31)) return set_error(GEPI_ERR_LIMIT, "topmost too large");
    if (pl->cap < want) {
        pool_free(pl->d_cand[0], pl->stream);
        pool_free(pl->d_cand[1], pl->stream);
        GEPI_TRY(check_mem(2 * want * sizeof(Cand), "candidate buffers"));
        GEPI_CUDA(pool_alloc(pl->device, &pl->d_cand[0], want * sizeof(Cand), pl->stream));
        GEPI_CUDA(pool_alloc(pl->device, &pl->d_cand[1], want * sizeof(Cand), pl->stream));
        pl->cap = (uint32_t)want;
    }
    if (!pl->d_state) GEPI_CUDA(pool_alloc(pl->device, &pl->d_state, sizeof(ScanState), pl->stream));
    if (!pl->h_state) GEPI_CUDA(cudaMallocHost(&pl->h_state, sizeof(ScanState)));
    if (!pl->d_sel) GEPI_CUDA(pool_alloc(pl->device, &pl->d_sel, sel_state_bytes(), pl->stream));
    return GEPI_OK;
}

gepi_status upload_tiles(gepi_planes *pl, const std::vector<int2> &tiles) {
    pl->tiles_valid = false;
    if (tiles.size() > pl->tiles_cap) {
        pool_free(pl->d_tiles, pl->stream);
        GEPI_CUDA(pool_alloc(pl->device, &pl->d_tiles, tiles.size() * sizeof(int2), pl->stream));
        pl->tiles_cap = tiles.size();
    }
    if (!tiles.empty())
        GEPI_CUDA(cudaMemcpyAsync(pl->d_tiles, tiles.data(), tiles.size() * sizeof(int2),
                                  cudaMemcpyHostToDevice, pl->stream));
    return GEPI_OK;
}

// Tile pairs (A tile i of TA SNPs, B tile j of TB SNPs) of [a0,a1) x [b0,b1)
// holding at least one (s, t) with t <= s (all pairs when !triangle).  The
// list runs in bands of `band` A tiles: within a band every B tile is visited
// once for all the band's A tiles, so concurrently running CTAs share B tiles
// in L2 and each B tile is fetched from HBM about once per band.
// The tensor-core kernel reads the planes in 384-sample blocks, block-major;
// the copy is made on first use and kept with the plane set.
gepi_status ensure_tc_blocks(gepi_planes *pl) {
    if (pl->d_tc_blocks) return GEPI_OK;
    const size_t bytes = tc_block_words(pl->n_snps, pl->Wp, pl->W0) * 4;
    GEPI_TRY(check_mem(bytes, "tensor-core operand blocks"));
    GEPI_CUDA(pool_alloc(pl->device, &pl->d_tc_blocks, bytes, pl->stream));
    GEPI_CUDA(launch_tc_relayout(pl->d_planes, pl->Wp, pl->W0, pl->n_snps, pl->d_tc_blocks,
                                 pl->num_sms, pl->stream));
    return GEPI_OK;
}

void build_tiles(int a0, int a1, int b0, int b1, int TA, int TB, bool triangle, int band,
                 std::vector<int2> &out) {
    out.clear();
    const int nat = (a1 - a0 + TA - 1) / TA, nbt = (b1 - b0 + TB - 1) / TB;
    if (band < 1) band = 1;
    for (int i0 = 0; i0 < nat; i0 += band) {
        const int i1 = std::min(nat, i0 + band);
        for (int j = 0; j < nbt; ++j) {
            const int tmin = b0 + j * TB;
            bool any = false;
            for (int i = i0; i < i1; ++i) {
                const int smax = std::min(a0 + i * TA + TA - 1, a1 - 1);
                if (triangle && tmin > smax) continue;
                out.push_back(make_int2(i, j));
                any = true;
            }
            if (triangle && !any) break;
        }
    }
}

uint64_t next_serial() {
    static std::atomic<uint64_t> n{0};
    return ++n;
}

// Per-SNP marginal association (computed once per plane set).
gepi_status ensure_marginal(gepi_planes *pl) {
    if (!pl->marginal.empty() || pl->n_snps <= 0) return GEPI_OK;
    float *d = nullptr;
    GEPI_CUDA(pool_alloc(pl->device, &d, sizeof(float) * (size_t)pl->n_snps, pl->stream));
    std::vector<float> h((size_t)pl->n_snps);
    cudaError_t e = launch_marginal(pl->d_planes, pl->n_snps, pl->Wp, pl->W0, d, pl->num_sms, pl->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), d, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, pl->stream);
    pool_free(d, pl->stream);  // stream-ordered: no device-wide synchronization
    if (e == cudaSuccess) e = cudaStreamSynchronize(pl->stream);
    GEPI_CUDA(e);
    pl->marginal.swap(h);
    return GEPI_OK;
}

// Tiles holding a pair of one of the kHotSnps SNPs with the strongest marginal
// association go first: tests of such pairs tend to rank high (a function of
// two rows follows the stronger row), so the threshold reaches close to its
// final value within a few percent of the tiles and the bounds reject most of
// the rest.  The hot A tiles run B-tile-major (each B tile fetched once for
// all of them), then the hot B tiles, then every other tile in band order.
// The ranked result does not depend on the order.
constexpr int kHotSnps = 16;
constexpr size_t kHotMinTiles = 4096;  // smaller scans keep the band order
constexpr uint32_t kPendCap = 1u << 18;  // Fisher pending tests per launch (4 MB)

// The triangle scan's tile list in that order, generated directly: counted,
// sized once and written through a pointer (no sort, no partition).  Empty hot
// sets give the plain band order of build_tiles.  One thread: the fill is
// bound by the stores, and a thread team would keep spinning beside the
// scan's host loop.
void scan_tile_order(int a0, int a1, int b0, int b1, int TA, int TB, int band,
                     const std::vector<int> &hot_a, const std::vector<int> &hot_b,
                     std::vector<int2> &out) {
    const int nat = (a1 - a0 + TA - 1) / TA, nbt = (b1 - b0 + TB - 1) / TB;
    if (nat <= 0 || nbt <= 0) {
        out.clear();
        return;
    }
    if (band < 1) band = 1;
    // B tiles j < jend[i] pair with A tile i (t <= s somewhere in the tile)
    std::vector<int> jend((size_t)nat);
    size_t total = 0;
    for (int i = 0; i < nat; ++i) {
        const int smax = std::min(a0 + i * TA + TA - 1, a1 - 1);
        const int e = smax < b0 ? 0 : (smax - b0) / TB + 1;
        jend[(size_t)i] = std::min(nbt, e);
        total += (size_t)jend[(size_t)i];
    }
    // grown only when too small (a reused buffer is then not cleared: every
    // entry kept is written below), shrunk to the tiles written at the end
    if (out.size() < total) out.resize(total);
    int2 *w = out.data();
    std::vector<char> isa((size_t)nat, 0), isb((size_t)nbt, 0);
    for (int i : hot_a) isa[(size_t)i] = 1;
    for (int j : hot_b) isb[(size_t)j] = 1;
    for (int j = 0; j < nbt; ++j)
        for (int i : hot_a)
            if (j < jend[(size_t)i]) *w++ = make_int2(i, j);
    for (int i = 0; i < nat; ++i)
        if (!isa[(size_t)i])
            for (int j : hot_b)
                if (j < jend[(size_t)i]) *w++ = make_int2(i, j);
    for (int i0 = 0; i0 < nat; i0 += band) {
        const int i1 = std::min(nat, i0 + band);
        bool any_hot = false;
        for (int i = i0; i < i1; ++i) any_hot |= isa[(size_t)i] != 0;
        // jend grows with i: below the band's first A tile's end, every A tile of
        // a band without hot rows pairs with B tile j
        const int jmin = any_hot ? 0 : jend[(size_t)i0], jmax = jend[(size_t)(i1 - 1)];
        for (int j = 0; j < jmin; ++j) {
            if (isb[(size_t)j]) continue;
            for (int i = i0; i < i1; ++i) *w++ = make_int2(i, j);
        }
        for (int j = jmin; j < jmax; ++j) {
            if (isb[(size_t)j]) continue;
            for (int i = i0; i < i1; ++i)
                if (!isa[(size_t)i] && j < jend[(size_t)i]) *w++ = make_int2(i, j);
        }
    }
    out.resize((size_t)(w - out.data()));
}

// The A and B tiles of the kHotSnps strongest marginal SNPs (ascending).
void hot_tiles(const std::vector<float> &score, int a0, int a1, int b0, int b1, int TA, int TB,
               std::vector<int> &hot_a, std::vector<int> &hot_b) {
    hot_a.clear();
    hot_b.clear();
    const int lo = std::min(a0, b0), hi = std::max(a1, b1);
    std::vector<int> idx;
    idx.reserve((size_t)(hi - lo));
    for (int snp = lo; snp < hi; ++snp)
        if (score[(size_t)snp] > 0.f) idx.push_back(snp);
    if (idx.empty()) return;
    const size_t P = std::min<size_t>(kHotSnps, idx.size());
    std::nth_element(idx.begin(), idx.begin() + (P - 1), idx.end(), [&](int x, int y) {
        return score[(size_t)x] != score[(size_t)y] ? score[(size_t)x] > score[(size_t)y] : x < y;
    });
    for (size_t q = 0; q < P; ++q) {
        const int snp = idx[q];
        if (snp >= a0 && snp < a1) hot_a.push_back((snp - a0) / TA);
        if (snp >= b0 && snp < b1) hot_b.push_back((snp - b0) / TB);
    }
    for (auto *v : {&hot_a, &hot_b}) {
        std::sort(v->begin(), v->end());
        v->erase(std::unique(v->begin(), v->end()), v->end());
    }
}

gepi_status ensure_events(gepi_planes *pl, size_t n) {
    while (pl->ev.size() < n) {
        cudaEvent_t e;
        GEPI_CUDA(cudaEventCreate(&e));
        pl->ev.push_back(e);
    }
    return GEPI_OK;
}

// Device time of one launch of counting variant `v` over the triangle of SNPs
// [0, n) with a threshold nothing passes (the steady state of a long scan,
// where the fused bounds reject almost every test).  The first launch warms up.
gepi_status time_count_kernel(gepi_planes *pl, const CountVariant &v, int n, float *ms) {
    if (v.method == GEPI_METHOD_TENSOR) GEPI_TRY(ensure_tc_blocks(pl));
    std::vector<int2> tiles;
    build_tiles(0, n, 0, n, v.ta, v.tb, true, tile_band(v.ta), tiles);
    GEPI_TRY(upload_tiles(pl, tiles));
    GEPI_TRY(ensure_events(pl, 4));
    ScanState st{};
    st.tau_key = ~0ull;
    st.theta = INFINITY;
    st.lp_thr = -INFINITY;
    st.tau_f = INFINITY;
    st.tau_val = INFINITY;
    *pl->h_state = st;
    GEPI_CUDA(cudaMemcpyAsync(pl->d_state, pl->h_state, sizeof(ScanState), cudaMemcpyHostToDevice,
                              pl->stream));
    ScanCtx ctx;
    ctx.T = pl->d_T;
    ctx.F = pl->F;
    ctx.lf = pl->d_lf;
    ctx.lf32 = pl->d_lf32;
    ctx.objective = GEPI_ENTROPY;
    ctx.fisher_fp64 = 0;
    ctx.pend = nullptr;
    ctx.pend_req = 0;
    ctx.cap = pl->cap;
    ctx.st = pl->d_state;
    ctx.cand = pl->d_cand[0];
    for (int rep = 0; rep < 2; ++rep) {
        GEPI_CUDA(cudaEventRecord(pl->ev[2], pl->stream));
        GEPI_CUDA(launch_count(v, pl, pl->d_tiles, (int)tiles.size(), 0, n, 0, n, ctx, nullptr,
                               &pl->d_state->kerr, pl->stream));
        GEPI_CUDA(cudaEventRecord(pl->ev[3], pl->stream));
    }
    GEPI_CUDA(cudaMemcpyAsync(pl->h_state, pl->d_state, sizeof(ScanState), cudaMemcpyDeviceToHost,
                              pl->stream));
    GEPI_CUDA(cudaStreamSynchronize(pl->stream));
    if (pl->h_state->kerr)
        return set_error(GEPI_ERR_TIMEOUT, "counting kernel gave up a bounded wait (code " +
                                               std::to_string(pl->h_state->kerr) + ")");
    GEPI_CUDA(cudaEventElapsedTime(ms, pl->ev[2], pl->ev[3]));
    return GEPI_OK;
}

// Counting variant of a request: `variant` > 0 names one (gepi_params.variant),
// else GEPI_METHOD_POPC and _TENSOR take their default variant and AUTO the
// tuned one.  AUTO is tuned once per plane set: every variant is timed on the
// leading triangle of up to 4,096 SNPs at the set's full sample width (sample
// count moves the crossover: the tensor-core kernel's fixed per-tile epilogue
// is amortised over the samples; tile height trades B-tile reuse against the
// ragged edge of small triangles) and the fastest is kept.  Plane sets of
// fewer than 256 SNPs use the default popcount variant without timing.
gepi_status resolve_variant(gepi_planes *pl, int m, int variant, const CountVariant **out) {
    // the tensor-core kernel hands counts to its scoring warps as 16-bit values
    const bool tc_ok = pl->S0 <= tc_max_class() && pl->S1 <= tc_max_class();
    auto tc_refused = [&]() {
        return set_error(GEPI_ERR_ARG, "the tensor-core counting kernel takes at most " +
                                           std::to_string(tc_max_class()) +
                                           " samples per class; use the popcount method");
    };
    if (variant != 0) {
        const CountVariant *v = count_variant(variant);
        if (!v) return set_error(GEPI_ERR_ARG, "unknown counting variant " + std::to_string(variant));
        if (v->method == GEPI_METHOD_TENSOR && !tc_ok) return tc_refused();
        *out = v;
        return GEPI_OK;
    }
    if (m == GEPI_METHOD_TENSOR && !tc_ok) return tc_refused();
    if (m == GEPI_METHOD_POPC || m == GEPI_METHOD_TENSOR) {
        *out = count_variant(m == GEPI_METHOD_POPC ? kVariantPopcDefault : kVariantTensor);
        return GEPI_OK;
    }
    if (!pl->auto_variant) {
        if (pl->n_snps < 256) {
            pl->auto_variant = kVariantPopcDefault;
        } else {
            // The timing depends only on the shape (class widths, tuning
            // triangle) and the device, so it is kept for the process: later
            // plane sets of the same shape reuse the first one's choice.
            static std::mutex mu;
            static std::map<std::array<int, 4>, std::array<float, kNumVariants + 1>> tuned;
            const int n = std::min(pl->n_snps, 4096);
            const std::array<int, 4> key{pl->device, pl->W0, pl->Wp, n};
            {
                std::lock_guard<std::mutex> lk(mu);
                auto it = tuned.find(key);
                if (it != tuned.end()) {
                    pl->auto_variant = (int)it->second[0];
                    for (int v = 1; v <= kNumVariants; ++v) pl->tune_ms[v] = it->second[v];
                }
            }
            if (!pl->auto_variant) {
                GEPI_TRY(ensure_tables(pl));
                GEPI_TRY(ensure_scan_buffers(pl, 1));
                std::array<float, kNumVariants + 1> row{};
                int best = 0;
                for (int v = 1; v <= kNumVariants; ++v) {
                    const CountVariant &cv = *count_variant(v);
                    if (cv.method == GEPI_METHOD_TENSOR && !tc_ok) continue;
                    float ms = 0.f;
                    GEPI_TRY(time_count_kernel(pl, cv, n, &ms));
                    row[v] = ms;
                    if (!best || ms < row[best]) best = v;
                }
                row[0] = (float)best;
                pl->auto_variant = best;
                for (int v = 1; v <= kNumVariants; ++v) pl->tune_ms[v] = row[v];
                std::lock_guard<std::mutex> lk(mu);
                tuned[key] = row;
            }
        }
    }
    *out = count_variant(pl->auto_variant);
    return GEPI_OK;
}

bool cand_better(const Cand &a, const Cand &b) {
    if (a.key != b.key) return a.key > b.key;
    if (a.rA != b.rA) return a.rA < b.rA;
    return a.rBfun < b.rBfun;
}

// Top-k of `count` candidates (ranked by the deterministic tie-break) into
// tops[0, k), zero-filling the rest.  `values` (optional) receives the double
// each `ent` is rounded from (0 for zero-filled slots).
void rank_candidates(std::vector<Cand> &host, gepi_result *tops, int k,
                     std::vector<double> *values = nullptr) {
    std::memset(tops, 0, sizeof(gepi_result) * (size_t)k);
    const size_t keep = std::min<size_t>(host.size(), (size_t)k);
    std::partial_sort(host.begin(), host.begin() + keep, host.end(), cand_better);
    if (values) values->assign((size_t)k, 0.0);
    for (size_t i = 0; i < keep; ++i) {
        const Cand &c = host[i];
        gepi_result &r = tops[i];
        r.sA = c.rA;
        r.sB = c.rBfun >> 3;
        r.fun = (char)(c.rBfun & 7);
        for (int j = 0; j < 4; ++j) r.n[j] = c.n[j];
        const double v = -value_of_key(c.key);
        r.ent = (float)v;
        if (values) (*values)[i] = v;
    }
}

// Progress reporting at tile-band ends (gepi_scan_progress).

struct Progress {
    gepi_progress_fn fn = nullptr;
    void *user = nullptr;
    int points = 0;
    bool with_tops = false;
    const std::vector<int2> *tiles = nullptr;
    int band = 1;         // A tiles per band of the tile list
    size_t next_end = 0;  // tile index (a band end) at which the next callback fires
    int next_point = 1;
    std::chrono::steady_clock::time_point t0;

    bool band_end(size_t t) const {
        const auto &T = *tiles;
        return t == 0 || t >= T.size() || T[t].x / band != T[t - 1].x / band;
    }
    // first band end at or after tile index `thr`
    size_t end_at_or_after(size_t thr) const {
        const size_t n = tiles->size();
        if (thr >= n) return n;
        if (thr == 0) thr = 1;
        while (thr < n && !band_end(thr)) ++thr;
        return thr;
    }
    size_t threshold(int point) const {
        return (size_t)std::ceil((double)point * (double)tiles->size() / (double)points);
    }
    void start(const std::vector<int2> &T, int band_tiles) {
        tiles = &T;
        band = band_tiles;
        t0 = std::chrono::steady_clock::now();
        next_point = 1;
        next_end = points > 0 ? end_at_or_after(threshold(1)) : end_at_or_after(1);
    }
    // after a callback at tile index t: the next firing point
    void advance(size_t t) {
        const size_t n = tiles->size();
        if (points > 0) {
            while (next_point <= points && end_at_or_after(threshold(next_point)) <= t) ++next_point;
            next_end = next_point <= points ? end_at_or_after(threshold(next_point)) : n + 1;
        } else {
            next_end = t < n ? end_at_or_after(t + 1) : n + 1;
        }
    }
};

gepi_status scan_impl(gepi_planes *pl, const gepi_params *par, int a0, int na, int b0, int nb,
                      gepi_result *tops, int k, Progress *prog = nullptr) {
    clear_error();
    if (!pl || !par || !tops || k <= 0) return set_error(GEPI_ERR_ARG, "gepi_scan: bad argument");
    if (par->objective != GEPI_ENTROPY && par->objective != GEPI_FISHER)
        return set_error(GEPI_ERR_ARG, "gepi_scan: unknown objective");
    if (par->method < GEPI_METHOD_AUTO || par->method > GEPI_METHOD_TENSOR)
        return set_error(GEPI_ERR_ARG, "gepi_scan: unknown method");
    if (a0 < 0 || b0 < 0 || na < 0 || nb < 0 || a0 + na > pl->n_snps || b0 + nb > pl->n_snps)
        return set_error(GEPI_ERR_ARG, "gepi_scan: SNP range outside the planes");
    DeviceGuard g(pl->device);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    GEPI_TRY(ensure_tables(pl));
    GEPI_TRY(ensure_scan_buffers(pl, k));
    std::memset(tops, 0, sizeof(gepi_result) * (size_t)k);
    pl->last_values.clear();

    const CountVariant *cv = nullptr;
    GEPI_TRY(resolve_variant(pl, par->method, par->variant, &cv));
    if (cv->method == GEPI_METHOD_TENSOR) GEPI_TRY(ensure_tc_blocks(pl));
    const int TA = cv->ta, TB = cv->tb;
    // kept per thread (a fresh 8 MB list per scan, config 3, costs page
    // faults); a scan started from a progress callback of another gets its own
    static thread_local std::vector<int2> tile_buf;
    static thread_local int depth = 0;
    struct Depth {
        int &d;
        ~Depth() { --d; }
    } nested{++depth};
    std::vector<int2> own;
    std::vector<int2> &tiles = depth == 1 ? tile_buf : own;
    // progress snapshots cover band prefixes, so they keep the band order (and
    // need the list on the host); other scans reuse the list already on the
    // device when the ranges and tile shape repeat
    const bool hot = !(prog && prog->fn);
    const std::array<int64_t, 7> tkey{a0, (int64_t)a0 + na, b0, (int64_t)b0 + nb, TA, TB, hot ? 1 : 0};
    size_t ntiles = 0;
    if (hot && pl->tiles_valid && pl->tiles_key == tkey) {
        ntiles = pl->tiles_n;
    } else {
        GEPI_TRY(pl_scan_tiles(pl, a0, a0 + na, b0, b0 + nb, TA, TB, hot, tiles));
        GEPI_TRY(upload_tiles(pl, tiles));
        ntiles = tiles.size();
        if (hot) {
            pl->tiles_valid = true;
            pl->tiles_key = tkey;
            pl->tiles_n = ntiles;
        }
    }
    GEPI_TRY(ensure_events(pl, 4));
    gepi_scan_stats &S = pl->stats;
    S = gepi_scan_stats{};
    S.method = cv->method;
    S.tile_snps = TA;
    S.variant = cv->id;
    S.tiles = ntiles;
    {
        // pairs (s, t), t < s, s in A, t in B; and SNPs in both ranges
        const int64_t ia0 = a0, ia1 = (int64_t)a0 + na, ib0 = b0, ib1 = (int64_t)b0 + nb;
        uint64_t pairs = 0;
        for (int64_t s = ia0; s < ia1; ++s) {
            const int64_t hi = std::min<int64_t>(s, ib1);
            if (hi > ib0) pairs += (uint64_t)(hi - ib0);
        }
        S.snp_pairs = pairs;
        const int64_t lo = std::max(ia0, ib0), hi = std::min(ia1, ib1);
        S.diag_snps = hi > lo ? (uint64_t)(hi - lo) : 0;
    }
    GEPI_CUDA(cudaEventRecord(pl->ev[0], pl->stream));
    if (prog && prog->fn) prog->start(tiles, tile_band(TA));
    else prog = nullptr;

    ScanState init{};
    init.tau_key = 0ull;
    init.theta = 0.f;
    init.lp_thr = INFINITY;
    init.tau_f = -INFINITY;
    init.tau_val = -INFINITY;
    *pl->h_state = init;
    GEPI_CUDA(cudaMemcpyAsync(pl->d_state, pl->h_state, sizeof(ScanState), cudaMemcpyHostToDevice,
                              pl->stream));

    const float lp_margin = 2e-6f * pl->lf_max + 1e-3f;
    int cur = 0;
    ScanCtx ctx;
    ctx.T = pl->d_T;
    ctx.F = pl->F;
    ctx.lf = pl->d_lf;
    ctx.lf32 = pl->d_lf32;
    ctx.objective = par->objective;
    ctx.fisher_fp64 = fisher_fp64_walks();
    ctx.cap = pl->cap;
    ctx.st = pl->d_state;
    ctx.pend = nullptr;
    ctx.pend_req = 0;
    if (par->objective == GEPI_FISHER && pl->S0 < 65536 && pl->S1 < 65536) {
        // The first batches hold one or a few tiles and, with no threshold
        // yet, up to all their tests reach the exact sum: on the few CTAs of
        // such a launch they would run nearly serially, so the counting kernel
        // leaves them to a launch across the GPU (entries hold 16-bit counts).
        const size_t bytes = 256 + (size_t)kPendCap * sizeof(uint4);
        if (!pl->d_pend) {
            GEPI_TRY(check_mem(bytes, "Fisher pending tests"));
            GEPI_CUDA(pool_alloc(pl->device, reinterpret_cast<void **>(&pl->d_pend), bytes,
                                 pl->stream));
        }
        PendList hdr{};
        hdr.ent = reinterpret_cast<uint4 *>(reinterpret_cast<char *>(pl->d_pend) + 256);
        hdr.cap = kPendCap;
        // GEPI_DEBUG_PEND_CAP shrinks the list so tests reach the in-launch
        // evaluation of the tests past its capacity
        if (const char *e = std::getenv("GEPI_DEBUG_PEND_CAP")) {
            const long long v = std::atoll(e);
            if (v > 0 && v < (long long)kPendCap) hdr.cap = (uint32_t)v;
        }
        // pageable source: staged before the call returns
        GEPI_CUDA(cudaMemcpyAsync(pl->d_pend, &hdr, sizeof hdr, cudaMemcpyHostToDevice, pl->stream));
        ctx.pend = pl->d_pend;
    }

    const double tests_per_tile = 20.0 * TA * TB;
    const uint32_t budget = select_budget(pl->cap, k);
    const uint32_t trigger = select_trigger(budget, k);
    size_t batch =
        (size_t)std::max(1.0, std::floor(pilot_tests(par->objective, budget) / tests_per_tile));
    size_t t = 0;
    uint32_t count = 0;
    int retries = 0;
    while (t < ntiles) {
        size_t nbt = std::min(batch, ntiles - t);
        // a snapshot needs exactly the tiles before its band end
        if (prog && prog->with_tops && t < prog->next_end) nbt = std::min(nbt, prog->next_end - t);
        ctx.cand = pl->d_cand[cur];
        GEPI_CUDA(cudaEventRecord(pl->ev[2], pl->stream));
        GEPI_CUDA(launch_count(*cv, pl, pl->d_tiles + t, (int)nbt, a0, a0 + na, b0, b0 + nb, ctx,
                               nullptr, &pl->d_state->kerr, pl->stream));
        GEPI_CUDA(cudaEventRecord(pl->ev[3], pl->stream));
        GEPI_CUDA(cudaMemcpyAsync(pl->h_state, pl->d_state, sizeof(ScanState),
                                  cudaMemcpyDeviceToHost, pl->stream));
        GEPI_CUDA(cudaStreamSynchronize(pl->stream));
        {
            float ms = 0.f;
            GEPI_CUDA(cudaEventElapsedTime(&ms, pl->ev[2], pl->ev[3]));
            S.count_ms += ms;
            S.max_count_ms = std::max<double>(S.max_count_ms, ms);
            S.count_launches += 1;
        }
        if (pl->h_state->kerr)
            return set_error(GEPI_ERR_TIMEOUT, "counting kernel gave up a bounded wait (code " +
                                                   std::to_string(pl->h_state->kerr) + ")");
        if (pl->h_state->overflow) {
            // Tighten with everything captured (a valid lower bound), drop this
            // batch's partial appends, retry it in halves.  Only more than
            // `cap` exactly tied candidates can keep overflowing a 1-tile batch.
            if (++retries > 64)
                return set_error(GEPI_ERR_LIMIT, "candidate buffer keeps overflowing (massive ties)");
            S.overflows += 1;
            S.other_launches += kSelectLaunches;
            GEPI_CUDA(run_select_compact(pl->d_cand[cur], pl->d_cand[cur ^ 1], pl->d_state,
                                         pl->d_sel, pl->cap, (uint32_t)k, (int)pl->cap, count,
                                         par->objective, lp_margin, pl->num_sms, pl->stream));
            cur ^= 1;
            GEPI_CUDA(cudaMemcpyAsync(pl->h_state, pl->d_state, sizeof(ScanState),
                                      cudaMemcpyDeviceToHost, pl->stream));
            GEPI_CUDA(cudaStreamSynchronize(pl->stream));
            count = pl->h_state->count;
            batch = std::max<size_t>(1, nbt / 2);
            if (par->verbose)
                std::fprintf(stderr, "gepi: candidate overflow, batch -> %zu tiles\n", batch);
            continue;
        }
        const uint32_t appended = pl->h_state->count - count;
        count = pl->h_state->count;
        t += nbt;
        retries = 0;
        S.batches += 1;
        if (count > trigger && t < ntiles) {
            S.other_launches += kSelectLaunches;
            GEPI_CUDA(run_select_compact(pl->d_cand[cur], pl->d_cand[cur ^ 1], pl->d_state,
                                         pl->d_sel, pl->cap, (uint32_t)k, -1, 0xFFFFFFFFu,
                                         par->objective, lp_margin, pl->num_sms, pl->stream));
            cur ^= 1;
            GEPI_CUDA(cudaMemcpyAsync(pl->h_state, pl->d_state, sizeof(ScanState),
                                      cudaMemcpyDeviceToHost, pl->stream));
            GEPI_CUDA(cudaStreamSynchronize(pl->stream));
            count = pl->h_state->count;
        }
        if (prog && t >= prog->next_end) {
            gepi_progress pr{};
            pr.elapsed_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - prog->t0).count();
            pr.tiles_done = t;
            pr.tiles_total = ntiles;
            // bands before the one in progress are complete
            const int band = prog->band;
            const int bands_done = t < ntiles ? tiles[t].x / band : (na + TA - 1) / TA;
            pr.snps_done = a0 + std::min(na, bands_done * band * TA);
            std::vector<gepi_result> snap;
            if (prog->with_tops) {
                std::vector<Cand> host(count);
                if (count)
                    GEPI_CUDA(cudaMemcpyAsync(host.data(), pl->d_cand[cur], (size_t)count * sizeof(Cand),
                                              cudaMemcpyDeviceToHost, pl->stream));
                GEPI_CUDA(cudaStreamSynchronize(pl->stream));
                snap.resize((size_t)k);
                rank_candidates(host, snap.data(), k);
                pr.tops = snap.data();
                pr.ntops = k;
            }
            prog->fn(prog->user, &pr);
            prog->advance(t);
        }
        // Next batch: as many tiles as the remaining budget allows at the
        // append rate just observed (an over-estimate once tau has risen),
        // growing at most 8x per step.
        const double rate = std::max(1.0, (double)appended) / (double)nbt;
        const double room = (double)budget - (double)count;
        double nb_next = room > 0 ? room / rate : 1.0;
        nb_next = std::min(nb_next, 8.0 * (double)nbt);
        batch = (size_t)std::max(1.0, nb_next);
        if (par->verbose)
            std::fprintf(stderr, "gepi: %zu/%zu tiles, %u candidates, next batch %zu\n", t, ntiles,
                         count, batch);
    }
    if (count > (uint32_t)k) {
        S.other_launches += kSelectLaunches;
        GEPI_CUDA(run_select_compact(pl->d_cand[cur], pl->d_cand[cur ^ 1], pl->d_state, pl->d_sel,
                                     pl->cap, (uint32_t)k, -1, 0xFFFFFFFFu, par->objective,
                                     lp_margin, pl->num_sms, pl->stream));
        cur ^= 1;
        GEPI_CUDA(cudaMemcpyAsync(pl->h_state, pl->d_state, sizeof(ScanState),
                                  cudaMemcpyDeviceToHost, pl->stream));
        GEPI_CUDA(cudaStreamSynchronize(pl->stream));
        count = pl->h_state->count;
    }
    GEPI_CUDA(cudaEventRecord(pl->ev[1], pl->stream));
    std::vector<Cand> host(count);
    if (count)
        GEPI_CUDA(cudaMemcpyAsync(host.data(), pl->d_cand[cur], (size_t)count * sizeof(Cand),
                                  cudaMemcpyDeviceToHost, pl->stream));
    GEPI_CUDA(cudaStreamSynchronize(pl->stream));
    {
        float ms = 0.f;
        GEPI_CUDA(cudaEventElapsedTime(&ms, pl->ev[0], pl->ev[1]));
        S.scan_ms = ms;
        S.candidates = count;
    }
    rank_candidates(host, tops, k, &pl->last_values);
    if (prog && prog->next_end <= ntiles) {  // the last band end: the scan is complete
        gepi_progress pr{};
        pr.elapsed_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - prog->t0).count();
        pr.tiles_done = pr.tiles_total = ntiles;
        pr.snps_done = a0 + na;
        if (prog->with_tops) {
            pr.tops = tops;
            pr.ntops = k;
        }
        prog->fn(prog->user, &pr);
    }
    return GEPI_OK;
}

}  // namespace

namespace gepi {

// GEPI_DEBUG_FISHER_FP64=1 runs the Fisher tail walks in FP64 at every
// sample count, as they run from 2^24 samples up, so tests reach that code on
// small inputs.
int fisher_fp64_walks() {
    const char *e = std::getenv("GEPI_DEBUG_FISHER_FP64");
    return e && std::atoi(e) != 0 ? 1 : 0;
}

cudaError_t pool_alloc(int device, void **ptr, size_t bytes, cudaStream_t s) {
    cudaMemPool_t p = device_pool(device);
    if (!p) return cudaErrorMemoryAllocation;
    return cudaMallocFromPoolAsync(ptr, bytes, p, s);
}


gepi_status pl_check_mem(size_t bytes, const char *what) { return check_mem(bytes, what); }
gepi_status pl_ensure_tables(gepi_planes *pl) { return ensure_tables(pl); }
gepi_status pl_ensure_tc_blocks(gepi_planes *pl) { return ensure_tc_blocks(pl); }
gepi_status pl_resolve_variant(gepi_planes *pl, int m, int variant, const CountVariant **out) {
    return resolve_variant(pl, m, variant, out);
}

// The counting variants (ids 1..kNumVariants, stable).
static const CountVariant kVariants[kNumVariants] = {
    {1, GEPI_METHOD_POPC, 32, 32, 32, "popc_32x32_w32"},
    {2, GEPI_METHOD_POPC, 32, 32, 16, "popc_32x32_w16"},
    {3, GEPI_METHOD_POPC, 64, 32, 32, "popc_64x32_w32"},
    {4, GEPI_METHOD_TENSOR, 80, 64, 12, "tensor_80x64_w12"},
};

const CountVariant *count_variant(int id) {
    return id >= 1 && id <= kNumVariants ? &kVariants[id - 1] : nullptr;
}

cudaError_t launch_count(const CountVariant &v, const gepi_planes *pl, const int2 *tiles,
                         int ntiles, int a0, int a1, int b0, int b1, const ScanCtx &ctx,
                         uint32_t *dump, int *err, cudaStream_t stream) {
    if (ctx.pend) {
        cudaError_t e = cudaMemsetAsync(&ctx.pend->n, 0, sizeof(uint32_t), stream);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e =
        v.method == GEPI_METHOD_TENSOR
            ? launch_tc_tiles(pl->d_tc_blocks, pl->n_snps, pl->Wp, pl->W0, tiles, ntiles, a0, a1, b0,
                              b1, ctx, dump, err, pl->num_sms, stream)
            : launch_popc_tiles(v.ta, v.words, pl->d_planes, pl->Wp, pl->W0, tiles, ntiles, a0, a1,
                                b0, b1, ctx, dump, stream);
    if (e == cudaSuccess && ctx.pend) e = launch_fisher_pending(ctx, pl->num_sms, stream);
    return e;
}
gepi_status pl_scan_tiles(gepi_planes *pl, int a0, int a1, int b0, int b1, int TA, int TB, bool hot,
                          std::vector<int2> &out) {
    std::vector<int> hot_a, hot_b;
    // at least about kHotMinTiles tiles in the triangle
    const double est = 0.5 * (double)(a1 - a0) * (double)(b1 - b0) / ((double)TA * TB);
    if (hot && est >= (double)kHotMinTiles) {
        GEPI_TRY(ensure_marginal(pl));
        hot_tiles(pl->marginal, a0, a1, b0, b1, TA, TB, hot_a, hot_b);
    }
    scan_tile_order(a0, a1, b0, b1, TA, TB, tile_band(TA), hot_a, hot_b, out);
    return GEPI_OK;
}

void pl_build_tiles(int a0, int a1, int b0, int b1, int TA, int TB, bool triangle, int band,
                    std::vector<int2> &out) {
    build_tiles(a0, a1, b0, b1, TA, TB, triangle, band, out);
}

}  // namespace gepi

extern "C" {

const char *gepi_status_string(gepi_status s) {
    switch (s) {
    case GEPI_OK: return "ok";
    case GEPI_ERR_ARG: return "invalid argument";
    case GEPI_ERR_IO: return "i/o error";
    case GEPI_ERR_FORMAT: return "format error";
    case GEPI_ERR_CUDA: return "CUDA error";
    case GEPI_ERR_OOM: return "out of device memory";
    case GEPI_ERR_NOCLASS: return "phenotype class 1 or 2 is empty";
    case GEPI_ERR_TIMEOUT: return "device wait timed out";
    case GEPI_ERR_UNSUPPORTED: return "unsupported";
    case GEPI_ERR_LIMIT: return "request beyond a documented limit";
    }
    return "unknown status";
}

const char *gepi_last_error(void) { return g_last_error.c_str(); }

int gepi_abi_version(void) { return GEPI_ABI_VERSION; }

gepi_status gepi_planes_from_bed(const uint8_t *bed, size_t bed_bytes, int n_bim_snps,
                                 int n_samples, const int32_t *phenotype, int device,
                                 gepi_planes **out) {
    clear_error();
    if (!bed || !phenotype || !out || n_bim_snps <= 0 || n_samples <= 0)
        return set_error(GEPI_ERR_ARG, "gepi_planes_from_bed: bad argument");
    *out = nullptr;
    const size_t bps = ((size_t)n_samples + 3) / 4;
    if (bed_bytes < 3 || bed[0] != 0x6c || bed[1] != 0x1b)
        return set_error(GEPI_ERR_FORMAT, ".bed: Incorrect Magic");
    if (bed_bytes != 3 + (size_t)n_bim_snps * bps)
        return set_error(GEPI_ERR_FORMAT, ".bed: size " + std::to_string(bed_bytes) +
                                              " different than expected " +
                                              std::to_string(3 + (size_t)n_bim_snps * bps));
    std::vector<int> c0, c1;
    for (int i = 0; i < n_samples; ++i) {
        if (phenotype[i] == 1) c0.push_back(i);
        else if (phenotype[i] == 2) c1.push_back(i);
    }
    if (c0.empty() || c1.empty()) return set_error(GEPI_ERR_NOCLASS, "Error in class mask data");
    DeviceGuard g(device);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    gepi_planes *pl = new gepi_planes();
    pl->serial = next_serial();
    gepi_status st = planes_alloc(pl, device, n_bim_snps, (int)c0.size(), (int)c1.size());
    uint8_t *d_bed = nullptr;
    int32_t *d_perm = nullptr;
    auto fail = [&](gepi_status s) {
        pool_free(d_bed, pl->stream);
        pool_free(d_perm, pl->stream);
        planes_free(pl);
        delete pl;
        return s;
    };
    if (st != GEPI_OK) return fail(st);
    std::vector<int32_t> perm;
    build_perm(c0, c1, pl->W0, pl->Wp, perm);
    // the whole file image is copied (with its 3-byte header) so that the
    // copy starts where the caller's buffer does, usually on a page boundary
    if ((st = check_mem(bed_bytes + perm.size() * 4, ".bed staging")) != GEPI_OK) return fail(st);
    if (pool_alloc(device, &d_bed, bed_bytes, pl->stream) != cudaSuccess ||
        pool_alloc(device, &d_perm, perm.size() * 4, pl->stream) != cudaSuccess)
        return fail(set_error(GEPI_ERR_OOM, ".bed staging allocation failed"));
    cudaError_t e = cudaMemcpyAsync(d_bed, bed, bed_bytes, cudaMemcpyHostToDevice, pl->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_perm, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice, pl->stream);
    if (e == cudaSuccess)
        e = launch_decode_bed(d_bed + 3, bps, n_bim_snps, d_perm, pl->Wp, pl->d_planes, pl->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(pl->stream);
    if (e != cudaSuccess)
        return fail(set_error(GEPI_ERR_CUDA, std::string("decode: ") + cudaGetErrorString(e)));
    pool_free(d_bed, pl->stream);
    pool_free(d_perm, pl->stream);
    *out = pl;
    return GEPI_OK;
}

gepi_status gepi_planes_from_rows(const uint64_t *bits, const uint64_t *valid, int n_rows,
                                  int n_words, const uint64_t *mask1, const uint64_t *mask2,
                                  int device, gepi_planes **out) {
    clear_error();
    if (!bits || !valid || !mask1 || !mask2 || !out || n_rows <= 0 || (n_rows & 1) || n_words <= 0)
        return set_error(GEPI_ERR_ARG, "gepi_planes_from_rows: bad argument");
    *out = nullptr;
    const int n_snps = n_rows / 2;
    for (int s = 0; s < n_snps; ++s)
        if (std::memcmp(valid + (size_t)(2 * s) * n_words, valid + (size_t)(2 * s + 1) * n_words,
                        (size_t)n_words * 8) != 0)
            return set_error(GEPI_ERR_FORMAT, "valid rows of allele pair " + std::to_string(s) +
                                                  " differ");
    std::vector<int> c0, c1;
    for (int i = 0; i < n_words * 64; ++i) {
        const uint64_t bit = 1ull << (i & 63);
        const bool in0 = mask1[i >> 6] & bit, in1 = mask2[i >> 6] & bit;
        if (in0 && in1) return set_error(GEPI_ERR_FORMAT, "sample in both class masks");
        if (in0) c0.push_back(i);
        if (in1) c1.push_back(i);
    }
    if (c0.empty() || c1.empty()) return set_error(GEPI_ERR_NOCLASS, "Error in class mask data");
    DeviceGuard g(device);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    gepi_planes *pl = new gepi_planes();
    pl->serial = next_serial();
    gepi_status st = planes_alloc(pl, device, n_snps, (int)c0.size(), (int)c1.size());
    uint64_t *d_bits = nullptr, *d_valid = nullptr;
    int32_t *d_perm = nullptr;
    auto fail = [&](gepi_status s) {
        pool_free(d_bits, pl->stream);
        pool_free(d_valid, pl->stream);
        pool_free(d_perm, pl->stream);
        planes_free(pl);
        delete pl;
        return s;
    };
    if (st != GEPI_OK) return fail(st);
    std::vector<int32_t> perm;
    build_perm(c0, c1, pl->W0, pl->Wp, perm);
    const size_t rb = (size_t)n_rows * n_words * 8;
    if ((st = check_mem(2 * rb + perm.size() * 4, "row staging")) != GEPI_OK) return fail(st);
    if (pool_alloc(device, &d_bits, rb, pl->stream) != cudaSuccess ||
        pool_alloc(device, &d_valid, rb, pl->stream) != cudaSuccess ||
        pool_alloc(device, &d_perm, perm.size() * 4, pl->stream) != cudaSuccess)
        return fail(set_error(GEPI_ERR_OOM, "row staging allocation failed"));
    cudaError_t e = cudaMemcpyAsync(d_bits, bits, rb, cudaMemcpyHostToDevice, pl->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_valid, valid, rb, cudaMemcpyHostToDevice, pl->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_perm, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice, pl->stream);
    if (e == cudaSuccess)
        e = launch_decode_rows(d_bits, d_valid, n_words, n_snps, d_perm, pl->Wp, pl->d_planes,
                               pl->stream, pl->num_sms);
    if (e == cudaSuccess) e = cudaStreamSynchronize(pl->stream);
    if (e != cudaSuccess)
        return fail(set_error(GEPI_ERR_CUDA, std::string("decode rows: ") + cudaGetErrorString(e)));
    pool_free(d_bits, pl->stream);
    pool_free(d_valid, pl->stream);
    pool_free(d_perm, pl->stream);
    *out = pl;
    return GEPI_OK;
}

void gepi_planes_destroy(gepi_planes *pl) {
    if (!pl) return;
    planes_free(pl);
    delete pl;
}

int gepi_planes_num_snps(const gepi_planes *pl) { return pl ? pl->n_snps : 0; }

gepi_status gepi_planes_class_sizes(const gepi_planes *pl, int *n0, int *n1) {
    if (!pl) return set_error(GEPI_ERR_ARG, "null planes");
    if (n0) *n0 = pl->S0;
    if (n1) *n1 = pl->S1;
    return GEPI_OK;
}

gepi_status gepi_scan(gepi_planes *pl, const gepi_params *par, gepi_result *tops, int k) {
    if (!pl) return set_error(GEPI_ERR_ARG, "null planes");
    return scan_impl(pl, par, 0, pl->n_snps, 0, pl->n_snps, tops, k);
}

gepi_status gepi_scan_range(gepi_planes *pl, const gepi_params *par, int a0, int na, int b0,
                            int nb, gepi_result *tops, int k) {
    return scan_impl(pl, par, a0, na, b0, nb, tops, k);
}

gepi_status gepi_shard_range(int32_t n_snps, int32_t n_shards, int32_t shard, int32_t *a0,
                             int32_t *na, int32_t *b0, int32_t *nb) {
    clear_error();
    if (n_snps < 0 || n_shards <= 0 || shard < 0 || shard >= n_shards || !a0 || !na || !b0 || !nb)
        return set_error(GEPI_ERR_ARG, "gepi_shard_range: bad argument");
    // rows [r_s, r_{s+1}) with r_s = n sqrt(s / S): pairs per shard ~ r_{s+1}^2 - r_s^2, even
    auto bound = [&](int s_) {
        if (s_ >= n_shards) return n_snps;
        return (int32_t)std::llround((double)n_snps * std::sqrt((double)s_ / (double)n_shards));
    };
    const int32_t r0 = bound(shard), r1 = std::max(r0, bound(shard + 1));
    *a0 = r0;
    *na = r1 - r0;
    *b0 = 0;
    *nb = r1;
    return GEPI_OK;
}

gepi_status gepi_merge_results(int32_t n_samples, int32_t objective,
                               const gepi_result *const *lists, const int32_t *lens,
                               int32_t n_lists, gepi_result *out, int32_t k) {
    clear_error();
    if (n_samples <= 0 || !lists || !lens || n_lists < 0 || !out || k <= 0)
        return set_error(GEPI_ERR_ARG, "gepi_merge_results: bad argument");
    if (objective != GEPI_ENTROPY && objective != GEPI_FISHER)
        return set_error(GEPI_ERR_ARG, "gepi_merge_results: unknown objective");
    // the scan's fixed-point table for this sample count, built once
    static std::mutex mu;
    static std::map<int32_t, std::pair<int, std::vector<uint64_t>>> tables;
    const std::pair<int, std::vector<uint64_t>> *tab = nullptr;
    if (objective == GEPI_ENTROPY) {
        std::lock_guard<std::mutex> lk(mu);
        auto it = tables.find(n_samples);
        if (it == tables.end()) {
            std::pair<int, std::vector<uint64_t>> t;
            t.first = tfix_bits(n_samples);
            build_tfix(n_samples, t.first, t.second);
            it = tables.emplace(n_samples, std::move(t)).first;
        }
        tab = &it->second;
    }
    std::vector<Cand> all;
    for (int32_t l = 0; l < n_lists; ++l) {
        if (lens[l] < 0 || (lens[l] > 0 && !lists[l]))
            return set_error(GEPI_ERR_ARG, "gepi_merge_results: bad list");
        for (int32_t i = 0; i < lens[l]; ++i) {
            const gepi_result &r = lists[l][i];
            const int w = r.n[0], x = r.n[1], y = r.n[2], z = r.n[3];
            // zero-filled slots and tests without association are not ranked
            if ((long long)w * z == (long long)x * y) continue;
            if (w < 0 || x < 0 || w > y || x > z || (int64_t)y + z > n_samples)
                return set_error(GEPI_ERR_ARG, "gepi_merge_results: counts inconsistent with n_samples");
            double value;
            if (objective == GEPI_ENTROPY) {
                // the exact key of the scan: the same integer sum, scaling and division
                const std::vector<uint64_t> &T = tab->second;
                const int m = y + z, xx = w + x;
                const uint64_t num = T[m] + T[w] + T[y - w] + T[x] + T[z - x] - T[xx] - T[m - xx] -
                                     T[y] - T[z];
                value = std::scalbn((double)(long long)num, -tab->first) / (double)m;
            } else {
                value = -fisher_lnp_host(w, y - w, x, z - x) * 0.43429448190325182765;
            }
            Cand c;
            c.key = key_of(value);
            c.rA = r.sA;
            c.rBfun = r.sB * 8 + (int)r.fun;
            for (int q = 0; q < 4; ++q) c.n[q] = r.n[q];
            all.push_back(c);
        }
    }
    rank_candidates(all, out, k);
    return GEPI_OK;
}

gepi_status gepi_scan_progress(gepi_planes *pl, const gepi_params *par, int a0, int na, int b0,
                               int nb, gepi_result *tops, int k, gepi_progress_fn fn, void *user,
                               int32_t points, int32_t with_tops) {
    Progress prog;
    prog.fn = fn;
    prog.user = user;
    prog.points = points;
    prog.with_tops = with_tops != 0;
    return scan_impl(pl, par, a0, na, b0, nb, tops, k, &prog);
}

gepi_status gepi_pair_counts(gepi_planes *pl, int method, int a0, int na, int b0, int nb,
                             uint32_t *out) {
    clear_error();
    if (!pl || !out || na <= 0 || nb <= 0 || a0 < 0 || b0 < 0 || a0 + na > pl->n_snps ||
        b0 + nb > pl->n_snps)
        return set_error(GEPI_ERR_ARG, "gepi_pair_counts: bad argument");
    int variant = 0;
    if (method >= GEPI_VARIANT(1)) {
        variant = method - GEPI_VARIANT(0);
        method = GEPI_METHOD_AUTO;
    }
    if (method < GEPI_METHOD_AUTO || method > GEPI_METHOD_TENSOR)
        return set_error(GEPI_ERR_ARG, "gepi_pair_counts: unknown method");
    DeviceGuard g(pl->device);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    const CountVariant *cv = nullptr;
    GEPI_TRY(resolve_variant(pl, method, variant, &cv));
    if (cv->method == GEPI_METHOD_TENSOR) GEPI_TRY(ensure_tc_blocks(pl));
    std::vector<int2> tiles;
    build_tiles(a0, a0 + na, b0, b0 + nb, cv->ta, cv->tb, false, 8, tiles);
    GEPI_TRY(upload_tiles(pl, tiles));
    const size_t bytes = (size_t)na * nb * 18 * 4;
    GEPI_TRY(check_mem(bytes, "pair counts"));
    uint32_t *d_out = nullptr;
    int *d_err = nullptr;
    GEPI_CUDA(cudaMalloc(&d_out, bytes + 256));
    d_err = reinterpret_cast<int *>(reinterpret_cast<char *>(d_out) + ((bytes + 255) & ~size_t(255)));
    ScanCtx ctx{};
    int herr = 0;
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), pl->stream);
    if (e == cudaSuccess)
        e = launch_count(*cv, pl, pl->d_tiles, (int)tiles.size(), a0, a0 + na, b0, b0 + nb, ctx, d_out,
                         d_err, pl->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, pl->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, pl->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(pl->stream);
    cudaFree(d_out);
    if (e != cudaSuccess)
        return set_error(GEPI_ERR_CUDA, std::string("pair counts: ") + cudaGetErrorString(e));
    if (herr)
        return set_error(GEPI_ERR_TIMEOUT, "counting kernel gave up a bounded wait (code " +
                                               std::to_string(herr) + ")");
    return GEPI_OK;
}

gepi_status gepi_planes_autotune(gepi_planes *pl, int32_t *method, float *popc_ms,
                                 float *tensor_ms) {
    clear_error();
    if (!pl) return set_error(GEPI_ERR_ARG, "gepi_planes_autotune: null planes");
    DeviceGuard g(pl->device);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    const CountVariant *cv = nullptr;
    GEPI_TRY(resolve_variant(pl, GEPI_METHOD_AUTO, 0, &cv));
    if (method) *method = cv->method;
    // the fastest timed variant of each kernel (0: not timed)
    float best[3] = {0.f, 0.f, 0.f};
    for (int v = 1; v <= kNumVariants; ++v) {
        const float ms = pl->tune_ms[v];
        const int m = count_variant(v)->method;
        if (ms > 0.f && (best[m] == 0.f || ms < best[m])) best[m] = ms;
    }
    if (popc_ms) *popc_ms = best[GEPI_METHOD_POPC];
    if (tensor_ms) *tensor_ms = best[GEPI_METHOD_TENSOR];
    return GEPI_OK;
}

gepi_status gepi_planes_autotune_variants(gepi_planes *pl, gepi_tune_report *out) {
    clear_error();
    if (!pl || !out) return set_error(GEPI_ERR_ARG, "gepi_planes_autotune_variants: bad argument");
    DeviceGuard g(pl->device);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    const CountVariant *cv = nullptr;
    GEPI_TRY(resolve_variant(pl, GEPI_METHOD_AUTO, 0, &cv));
    std::memset(out, 0, sizeof *out);
    out->variant = cv->id;
    out->n_variants = kNumVariants;
    for (int v = 1; v <= kNumVariants; ++v) out->ms[v - 1] = pl->tune_ms[v];
    return GEPI_OK;
}

const char *gepi_count_variant_name(int32_t variant) {
    const CountVariant *cv = count_variant(variant);
    return cv ? cv->name : "";
}

gepi_status gepi_count_variant_shape(int32_t variant, int32_t *method, int32_t *tile_a,
                                     int32_t *tile_b, int32_t *stage_words) {
    const CountVariant *cv = count_variant(variant);
    if (!cv) return set_error(GEPI_ERR_ARG, "unknown counting variant");
    if (method) *method = cv->method;
    if (tile_a) *tile_a = cv->ta;
    if (tile_b) *tile_b = cv->tb;
    if (stage_words) *stage_words = cv->words;
    return GEPI_OK;
}

gepi_status gepi_tensor_peak_tflops(int device, double *tflops) {
    return gepi_tensor_peak_probe(device, GEPI_PEAK_MXF4, tflops);
}

gepi_status gepi_tensor_peak_probe(int32_t device, int32_t kind, double *tflops) {
    clear_error();
    if (!tflops) return set_error(GEPI_ERR_ARG, "gepi_tensor_peak_probe: null output");
    if (kind < GEPI_PEAK_MXF4 || kind > GEPI_PEAK_MXF4NVF4_4X)
        return set_error(GEPI_ERR_ARG, "gepi_tensor_peak_probe: unknown kind");
    DeviceGuard g(device);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    int sms = 0;
    GEPI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    int *d_err = nullptr;
    GEPI_CUDA(cudaMalloc(&d_err, sizeof(int)));
    cudaError_t e = cudaMemset(d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = tc_measure_peak(sms, 3, kind, tflops, d_err, 0);
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_err);
    if (e != cudaSuccess) return set_error(GEPI_ERR_CUDA, std::string("tensor peak: ") + cudaGetErrorString(e));
    if (herr) return set_error(GEPI_ERR_TIMEOUT, "tensor peak kernel gave up its bounded wait");
    return GEPI_OK;
}

gepi_status gepi_last_scan_stats(const gepi_planes *pl, gepi_scan_stats *out) {
    if (!pl || !out) return set_error(GEPI_ERR_ARG, "gepi_last_scan_stats: bad argument");
    *out = pl->stats;
    return GEPI_OK;
}

gepi_status gepi_last_scan_values(const gepi_planes *pl, double *out, int32_t k) {
    if (!pl || !out || k <= 0) return set_error(GEPI_ERR_ARG, "gepi_last_scan_values: bad argument");
    if ((size_t)k > pl->last_values.size())
        return set_error(GEPI_ERR_ARG, "gepi_last_scan_values: k exceeds the last scan's list");
    std::memcpy(out, pl->last_values.data(), sizeof(double) * (size_t)k);
    return GEPI_OK;
}

gepi_status gepi_process_gpu_1(const uint64_t *bits, const uint64_t *valid, int n_rows,
                               int n_words, const uint64_t *mask1, const uint64_t *mask2,
                               gepi_result *tops, const gepi_params *par) {
    if (!par || !tops) return set_error(GEPI_ERR_ARG, "gepi_process_gpu_1: bad argument");
    gepi_planes *pl = nullptr;
    GEPI_TRY(gepi_planes_from_rows(bits, valid, n_rows, n_words, mask1, mask2, par->gpu_num, &pl));
    gepi_status s = gepi_scan(pl, par, tops, par->topmost);
    gepi_planes_destroy(pl);
    return s;
}

}  // extern "C"
