// Scan engine: runs many scan requests -- whole plane sets or SNP range x
// range blocks, on one or many plane sets (cohorts) of a device -- together,
// and the serving loop built on it.
//
// Replaces the reference's one-cohort-per-process batch loop
// (launch_process_gpu_1, src/kernels/kernel1.cu:387-483).  Each request walks
// its tile list in adaptive batches as a direct scan does, with the same
// exact thresholds, so its results are bit-identical to gepi_scan_range's.
// Requests progress independently and the host never waits on one request's
// device work while others could be launched: every device operation of a
// request (a counting batch, a threshold-raising radix select replayed from a
// CUDA graph, an overflow retry's compaction) ends in a completion event that
// the engine polls; when it fires, the request's next operation is issued at
// once.  Batches can be capped to a device-time quantum, and requests with
// little work left run on a high-priority stream, so short requests are not
// held behind long ones.  Tile lists depend only on the SNP ranges and tile
// shape and are cached on the device across requests.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"

namespace gepi {

namespace {

using Clock = std::chrono::steady_clock;

bool cand_better(const Cand &a, const Cand &b) {
    if (a.key != b.key) return a.key > b.key;
    if (a.rA != b.rA) return a.rA < b.rA;
    return a.rBfun < b.rBfun;
}

// Candidate-buffer capacity of a request, as for direct scans: 4 Mi records,
// more for large k; GEPI_DEBUG_CAP shrinks it (>= 4k) so tests can drive the
// overflow path.
uint64_t cand_cap(int k) {
    uint64_t want = std::max<uint64_t>(1u << 22, ((uint64_t)k * 8 + 1023) & ~1023ull);
    if (const char *e = std::getenv("GEPI_DEBUG_CAP")) {
        long long v = std::atoll(e);
        if (v > 0) want = std::max<uint64_t>((uint64_t)v, 4ull * (uint64_t)k);
    }
    return want;
}

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Requests whose remaining device work is estimated below this run on the
// high-priority stream.
constexpr double kShortMs = 50.0;
// Device bytes of cached tile lists kept when no request uses them.
constexpr size_t kTileCacheBytes = 1ull << 30;

}  // namespace

struct ScanRequest {
    gepi_planes *pl = nullptr;
    int a0 = 0, na = 0, b0 = 0, nb = 0;
    int k = 0, objective = 0, method = 0;
};

// Device tile list of one (SNP ranges, tile shape), shared by requests.
struct TileList {
    int2 *d = nullptr;
    size_t n = 0;
    int refs = 0;
    uint64_t stamp = 0;  // last use, for eviction
};
// (a0, a1, b0, b1, TA, TB, plane-set serial): the order puts the plane set's
// strongest marginal SNPs first, so lists are kept per plane set
using TileKey = std::array<int64_t, 7>;

// Device resources of one request, pooled by candidate capacity.
struct JobBuffers {
    Cand *cand[2] = {nullptr, nullptr};
    uint32_t cap = 0;
    ScanState *state = nullptr;
    ScanState *h_state = nullptr;  // pinned
    void *sel = nullptr;           // radix-select scratch
    cudaStream_t stream[2] = {nullptr, nullptr};  // normal, high priority
    // scan start, scan done, batch launch start / end, operation complete
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaGraphExec_t sel_graph[2] = {nullptr, nullptr};  // select+compact cand[c] -> cand[c^1]
    int sel_k = -1, sel_obj = -1;
    float sel_margin = 0.f;
};

// The device operation a request has in flight.
enum class Op { None, Batch, SelRetry, SelBudget, SelFinal };

struct Job {
    ScanRequest rq;
    gepi_result *tops = nullptr;
    std::vector<gepi_result> own_tops;  // serving: kept until gepi_server_wait
    uint64_t ticket = 0;
    size_t footprint = 0;
    bool finished = false;  // serving: results ready for the waiter
    bool tc = false;
    int TA = 0, TB = 0;
    TileList *tl = nullptr;
    size_t ntiles = 0, next = 0, batch = 1, inflight = 0, last_nbt = 0;
    uint32_t last_appended = 0;
    double ms_per_tile = 0.0;  // from the last batch (0: not measured yet)
    JobBuffers *buf = nullptr;
    cudaStream_t s = nullptr;  // stream of the request's last operation
    Op op = Op::None;
    int cur = 0;
    uint32_t count = 0, budget = 0;
    int retries = 0;
    float lp_margin = 0.f;
    bool started = false, done = false, final_selected = false;
    bool oldest = false;  // the oldest unfinished request (Policy::Oldest)
    gepi_status status = GEPI_OK;
    std::string error;
    gepi_scan_stats S{};
    Clock::time_point t_submit, t_admit, t_done;
};

// Which requests' launches go on the high-priority stream: those with little
// work left (shortest first), or the oldest unfinished request (first come,
// first served, with the others filling the SMs it leaves).
enum class Policy { ShortFirst, Oldest };

class Engine {
   public:
    // quantum_ms > 0 caps each batch at about that much device time.
    Engine(int device, double quantum_ms, Policy policy = Policy::ShortFirst)
        : device_(device), quantum_ms_(quantum_ms), policy_(policy) {}
    ~Engine();
    gepi_status init();
    // Method choice, plane-set tables and the device tile list: may run on
    // any thread (serialised internally).
    gepi_status prepare(Job &j);
    // Candidate buffers and the initial scan state: the polling thread.
    gepi_status admit(Job &j);
    // Issues the next operation of every idle request and completes those
    // whose operation has finished; returns how many completed or finished.
    int poll(std::vector<Job *> &active);
    // Returns a request's buffers (after its streams drain) and tile list.
    void release(Job &j);
    std::mutex run_mu;  // serialises gepi_scan_batch calls on the device

   private:
    gepi_status advance(Job &j);
    gepi_status complete(Job &j);
    gepi_status launch(Job &j);
    gepi_status select_async(Job &j, int n_override, uint32_t n_compact, Op op);
    gepi_status finish(Job &j);
    void size_next_batch(Job &j);
    void fail(Job &j, gepi_status st);

    int device_ = 0, num_sms_ = 0;
    double quantum_ms_ = 0.0;
    Policy policy_ = Policy::ShortFirst;
    int prio_lo_ = 0, prio_hi_ = 0;
    std::vector<std::unique_ptr<JobBuffers>> pool_;
    std::vector<JobBuffers *> free_;
    std::mutex prep_mu_, cache_mu_;
    cudaStream_t upload_ = nullptr;
    std::map<TileKey, TileList> tiles_;
    size_t tile_bytes_ = 0;
    uint64_t stamp_ = 0;
};

Engine::~Engine() {
    DeviceGuard g(device_);
    for (auto &b : pool_) {
        for (cudaStream_t s : b->stream)
            if (s) cudaStreamSynchronize(s);
        dfree(b->cand[0]);
        dfree(b->cand[1]);
        dfree(b->state);
        dfree(b->sel);
        if (b->h_state) cudaFreeHost(b->h_state);
        for (cudaEvent_t e : b->ev)
            if (e) cudaEventDestroy(e);
        for (cudaGraphExec_t x : b->sel_graph)
            if (x) cudaGraphExecDestroy(x);
        for (cudaStream_t s : b->stream)
            if (s) cudaStreamDestroy(s);
    }
    for (auto &kv : tiles_)
        if (kv.second.d) cudaFreeAsync(kv.second.d, upload_);
    if (upload_) {
        cudaStreamSynchronize(upload_);
        cudaStreamDestroy(upload_);
    }
}

gepi_status Engine::init() {
    DeviceGuard g(device_);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    GEPI_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_));
    GEPI_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo_, &prio_hi_));
    GEPI_CUDA(cudaStreamCreateWithFlags(&upload_, cudaStreamNonBlocking));
    return GEPI_OK;
}

gepi_status Engine::prepare(Job &j) {
    std::lock_guard<std::mutex> lk(prep_mu_);
    DeviceGuard g(device_);
    const ScanRequest &rq = j.rq;
    gepi_planes *pl = rq.pl;
    GEPI_TRY(pl_ensure_tables(pl));
    int method = 0;
    GEPI_TRY(pl_resolve_method(pl, rq.method, &method));
    j.tc = method == GEPI_METHOD_TENSOR;
    if (j.tc) GEPI_TRY(pl_ensure_tc_blocks(pl));
    GEPI_CUDA(cudaStreamSynchronize(pl->stream));  // decode, relayout, tables done
    j.TA = j.tc ? tc_tile_a_snps() : popc_tile_snps();
    j.TB = j.tc ? tc_tile_b_snps() : popc_tile_snps();

    const TileKey key{rq.a0, (int64_t)rq.a0 + rq.na, rq.b0, (int64_t)rq.b0 + rq.nb, j.TA, j.TB,
                      (int64_t)pl->serial};
    {
        std::lock_guard<std::mutex> ck(cache_mu_);
        auto it = tiles_.find(key);
        if (it != tiles_.end()) {
            it->second.refs += 1;
            it->second.stamp = ++stamp_;
            j.tl = &it->second;
        }
    }
    if (!j.tl) {
        // only this thread inserts (prep_mu_ held), so the key is still absent
        std::vector<int2> tiles;
        GEPI_TRY(pl_scan_tiles(pl, rq.a0, rq.a0 + rq.na, rq.b0, rq.b0 + rq.nb, j.TA, j.TB, true, tiles));
        TileList t;
        t.n = tiles.size();
        if (t.n) {
            const size_t bytes = t.n * sizeof(int2);
            GEPI_TRY(pl_check_mem(bytes, "tile list"));
            GEPI_CUDA(cudaMallocAsync((void **)&t.d, bytes, upload_));
            GEPI_CUDA(cudaMemcpyAsync(t.d, tiles.data(), bytes, cudaMemcpyHostToDevice, upload_));
            GEPI_CUDA(cudaStreamSynchronize(upload_));
        }
        std::lock_guard<std::mutex> ck(cache_mu_);
        t.refs = 1;
        t.stamp = ++stamp_;
        TileList &e = tiles_[key];
        e = t;
        j.tl = &e;
        tile_bytes_ += t.n * sizeof(int2);
        // evict unused lists, least recently used first, above the cache size
        while (tile_bytes_ > kTileCacheBytes) {
            auto victim = tiles_.end();
            for (auto it = tiles_.begin(); it != tiles_.end(); ++it)
                if (it->second.refs == 0 &&
                    (victim == tiles_.end() || it->second.stamp < victim->second.stamp))
                    victim = it;
            if (victim == tiles_.end()) break;
            tile_bytes_ -= victim->second.n * sizeof(int2);
            if (victim->second.d) cudaFreeAsync(victim->second.d, upload_);
            tiles_.erase(victim);
        }
    }
    j.ntiles = j.tl->n;
    j.S = gepi_scan_stats{};
    j.S.method = method;
    j.S.tile_snps = j.TA;
    j.S.tiles = j.ntiles;
    {
        // pairs (s, t), t < s, s in A, t in B; and SNPs in both ranges
        const int64_t ia0 = rq.a0, ia1 = (int64_t)rq.a0 + rq.na, ib0 = rq.b0,
                      ib1 = (int64_t)rq.b0 + rq.nb;
        uint64_t pairs = 0;
        for (int64_t s = ia0; s < ia1; ++s) {
            const int64_t hi = std::min<int64_t>(s, ib1);
            if (hi > ib0) pairs += (uint64_t)(hi - ib0);
        }
        j.S.snp_pairs = pairs;
        const int64_t lo = std::max(ia0, ib0), hi = std::min(ia1, ib1);
        j.S.diag_snps = hi > lo ? (uint64_t)(hi - lo) : 0;
    }
    return GEPI_OK;
}

gepi_status Engine::admit(Job &j) {
    DeviceGuard g(device_);
    const uint64_t cap = cand_cap(j.rq.k);
    if (cap > (1ull << 31)) return set_error(GEPI_ERR_LIMIT, "topmost too large");
    JobBuffers *b = nullptr;
    for (size_t i = 0; i < free_.size(); ++i)
        if (free_[i]->cap == cap) {
            b = free_[i];
            free_.erase(free_.begin() + i);
            break;
        }
    if (!b) {
        GEPI_TRY(pl_check_mem(2 * cap * sizeof(Cand), "candidate buffers"));
        auto nb = std::make_unique<JobBuffers>();
        nb->cap = (uint32_t)cap;
        // owned by the pool from here on, so the destructor frees a partial set
        b = nb.get();
        pool_.push_back(std::move(nb));
        GEPI_CUDA(cudaMalloc(&b->cand[0], cap * sizeof(Cand)));
        GEPI_CUDA(cudaMalloc(&b->cand[1], cap * sizeof(Cand)));
        GEPI_CUDA(cudaMalloc(&b->state, sizeof(ScanState)));
        GEPI_CUDA(cudaMalloc(&b->sel, sel_state_bytes()));
        GEPI_CUDA(cudaMallocHost(&b->h_state, sizeof(ScanState)));
        GEPI_CUDA(cudaStreamCreateWithPriority(&b->stream[0], cudaStreamNonBlocking, prio_lo_));
        GEPI_CUDA(cudaStreamCreateWithPriority(&b->stream[1], cudaStreamNonBlocking, prio_hi_));
        for (cudaEvent_t &e : b->ev) GEPI_CUDA(cudaEventCreate(&e));
    }
    j.buf = b;
    // the first batch goes on the high-priority stream (no rate measured yet),
    // so the state upload is ordered before it on that stream
    j.s = b->stream[1];
    ScanState init{};
    init.tau_key = 0ull;
    init.theta = 0.f;
    init.lp_thr = INFINITY;
    init.tau_f = -INFINITY;
    init.tau_val = -INFINITY;
    *b->h_state = init;  // the previous user's copies have drained (release)
    GEPI_CUDA(cudaMemcpyAsync(b->state, b->h_state, sizeof(ScanState), cudaMemcpyHostToDevice, j.s));

    // as in the direct scan: the same select budget and first batch
    const double tests_per_tile = 20.0 * j.TA * j.TB;
    j.budget = select_budget(b->cap, j.rq.k);
    j.batch = (size_t)std::max(1.0, std::floor(pilot_tests(j.rq.objective, j.budget) / tests_per_tile));
    j.lp_margin = 2e-6f * j.rq.pl->lf_max + 1e-3f;
    j.cur = 0;
    j.next = 0;
    j.count = 0;
    j.retries = 0;
    j.ms_per_tile = 0.0;
    j.op = Op::None;
    j.started = j.done = j.final_selected = false;
    j.t_admit = Clock::now();
    return GEPI_OK;
}

void Engine::release(Job &j) {
    DeviceGuard g(device_);
    if (j.buf) {
        for (cudaStream_t s : j.buf->stream) cudaStreamSynchronize(s);  // nothing in flight on reuse
        free_.push_back(j.buf);
        j.buf = nullptr;
    }
    if (j.tl) {
        std::lock_guard<std::mutex> ck(cache_mu_);
        j.tl->refs -= 1;
        j.tl = nullptr;
    }
}

void Engine::fail(Job &j, gepi_status st) {
    j.status = st;
    j.error = gepi_last_error();
    j.done = true;
    j.op = Op::None;
    j.t_done = Clock::now();
}

// Queues the next batch of `j`: counting launch, state read-back, completion
// event.  The policy picks the stream (high priority: a request with little
// work left, or the oldest request); every earlier operation of the request
// has completed, so changing streams between operations keeps its order.
gepi_status Engine::launch(Job &j) {
    JobBuffers *b = j.buf;
    gepi_planes *pl = j.rq.pl;
    const ScanRequest &r = j.rq;
    j.inflight = std::min(j.batch, j.ntiles - j.next);
    const bool high =
        policy_ == Policy::Oldest
            ? j.oldest
            : (j.ms_per_tile <= 0.0 || (double)(j.ntiles - j.next) * j.ms_per_tile < kShortMs);
    j.s = b->stream[high ? 1 : 0];
    ScanCtx ctx;
    ctx.T = pl->d_T;
    ctx.F = pl->F;
    ctx.lf = pl->d_lf;
    ctx.lf32 = pl->d_lf32;
    ctx.objective = r.objective;
    ctx.cap = b->cap;
    ctx.st = b->state;
    ctx.cand = b->cand[j.cur];
    if (!j.started) {
        GEPI_CUDA(cudaEventRecord(b->ev[0], j.s));
        j.started = true;
    }
    GEPI_CUDA(cudaEventRecord(b->ev[2], j.s));
    if (j.tc)
        GEPI_CUDA(launch_tc_tiles(pl->d_tc_blocks, pl->n_snps, pl->Wp, pl->W0, j.tl->d + j.next,
                                  (int)j.inflight, r.a0, r.a0 + r.na, r.b0, r.b0 + r.nb, ctx,
                                  nullptr, &b->state->kerr, num_sms_, j.s));
    else
        GEPI_CUDA(launch_popc_tiles(pl->d_planes, pl->Wp, pl->W0, j.tl->d + j.next,
                                    (int)j.inflight, r.a0, r.a0 + r.na, r.b0, r.b0 + r.nb, ctx,
                                    nullptr, j.s));
    GEPI_CUDA(cudaEventRecord(b->ev[3], j.s));
    GEPI_CUDA(cudaMemcpyAsync(b->h_state, b->state, sizeof(ScanState), cudaMemcpyDeviceToHost, j.s));
    GEPI_CUDA(cudaEventRecord(b->ev[4], j.s));
    j.op = Op::Batch;
    return GEPI_OK;
}

// Device radix select of the k-th best key, then compaction into the other
// buffer, state read-back and completion event.  The common form (all
// entries) replays a CUDA graph captured once per buffer orientation.
gepi_status Engine::select_async(Job &j, int n_override, uint32_t n_compact, Op op) {
    JobBuffers *b = j.buf;
    const int k = j.rq.k, obj = j.rq.objective;
    Cand *in = b->cand[j.cur], *out = b->cand[j.cur ^ 1];
    j.S.other_launches += kSelectLaunches;
    bool done = false;
    if (n_override < 0 && n_compact == 0xFFFFFFFFu) {
        if (b->sel_k != k || b->sel_obj != obj || b->sel_margin != j.lp_margin) {
            for (cudaGraphExec_t &x : b->sel_graph)
                if (x) {
                    cudaGraphExecDestroy(x);
                    x = nullptr;
                }
            b->sel_k = k;
            b->sel_obj = obj;
            b->sel_margin = j.lp_margin;
        }
        cudaGraphExec_t &x = b->sel_graph[j.cur];
        if (!x) {
            cudaGraph_t graph = nullptr;
            if (cudaStreamBeginCapture(j.s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                cudaError_t e = run_select_compact(in, out, b->state, b->sel, b->cap, (uint32_t)k,
                                                   -1, 0xFFFFFFFFu, obj, j.lp_margin, num_sms_, j.s);
                cudaError_t e2 = cudaStreamEndCapture(j.s, &graph);
                if (e == cudaSuccess && e2 == cudaSuccess && graph &&
                    cudaGraphInstantiate(&x, graph, 0) != cudaSuccess)
                    x = nullptr;
                if (graph) cudaGraphDestroy(graph);
                cudaGetLastError();  // a failed capture leaves the plain launches below
            }
        }
        if (x) {
            GEPI_CUDA(cudaGraphLaunch(x, j.s));
            done = true;
        }
    }
    if (!done)
        GEPI_CUDA(run_select_compact(in, out, b->state, b->sel, b->cap, (uint32_t)k, n_override,
                                     n_compact, obj, j.lp_margin, num_sms_, j.s));
    j.cur ^= 1;
    GEPI_CUDA(cudaMemcpyAsync(b->h_state, b->state, sizeof(ScanState), cudaMemcpyDeviceToHost, j.s));
    GEPI_CUDA(cudaEventRecord(b->ev[4], j.s));
    j.op = op;
    return GEPI_OK;
}

// Reads the surviving candidates back and writes the ranked top-k.
gepi_status Engine::finish(Job &j) {
    JobBuffers *b = j.buf;
    const uint32_t count = j.count;
    std::vector<Cand> host(count);
    GEPI_CUDA(cudaEventRecord(b->ev[1], j.s));
    if (count)  // pageable destination: returns when the copy is done
        GEPI_CUDA(cudaMemcpyAsync(host.data(), b->cand[j.cur], (size_t)count * sizeof(Cand),
                                  cudaMemcpyDeviceToHost, j.s));
    GEPI_CUDA(cudaEventSynchronize(b->ev[1]));
    float ms = 0.f;
    if (j.started) GEPI_CUDA(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
    j.S.scan_ms = ms;
    j.S.candidates = count;
    const int k = j.rq.k;
    std::memset(j.tops, 0, sizeof(gepi_result) * (size_t)k);
    const size_t keep = std::min<size_t>(host.size(), (size_t)k);
    std::partial_sort(host.begin(), host.begin() + keep, host.end(), cand_better);
    for (size_t i = 0; i < keep; ++i) {
        const Cand &c = host[i];
        gepi_result &r = j.tops[i];
        r.sA = c.rA;
        r.sB = c.rBfun >> 3;
        r.fun = (char)(c.rBfun & 7);
        for (int q = 0; q < 4; ++q) r.n[q] = c.n[q];
        r.ent = (float)(-value_of_key(c.key));
    }
    j.done = true;
    j.t_done = Clock::now();
    return GEPI_OK;
}

// Next batch: as many tiles as the remaining budget allows at the append
// rate just observed, growing at most 8x per step, and within the device-time
// quantum at the rate just measured (an over-estimate when other requests
// shared the SMs).
void Engine::size_next_batch(Job &j) {
    const double nbt = (double)std::max<size_t>(1, j.last_nbt);
    const double rate = std::max(1.0, (double)j.last_appended) / nbt;
    const double room = (double)j.budget - (double)j.count;
    double nb_next = room > 0 ? room / rate : 1.0;
    nb_next = std::min(nb_next, 8.0 * nbt);
    if (quantum_ms_ > 0.0 && j.ms_per_tile > 0.0)
        nb_next = std::min(nb_next, quantum_ms_ / j.ms_per_tile);
    j.batch = (size_t)std::max(1.0, nb_next);
}

// Issues the request's next operation (no operation in flight).
gepi_status Engine::advance(Job &j) {
    if (j.next >= j.ntiles) {
        if (j.count > (uint32_t)j.rq.k && !j.final_selected)
            return select_async(j, -1, 0xFFFFFFFFu, Op::SelFinal);
        return finish(j);
    }
    return launch(j);
}

// Consumes the result of the operation that just completed, then advances.
gepi_status Engine::complete(Job &j) {
    JobBuffers *b = j.buf;
    const Op op = j.op;
    j.op = Op::None;
    const ScanState st = *b->h_state;
    switch (op) {
    case Op::Batch: {
        float ms = 0.f;
        GEPI_CUDA(cudaEventElapsedTime(&ms, b->ev[2], b->ev[3]));
        j.S.count_ms += ms;
        j.S.max_count_ms = std::max<double>(j.S.max_count_ms, ms);
        j.S.count_launches += 1;
        if (st.kerr)
            return set_error(GEPI_ERR_TIMEOUT, "counting kernel gave up a bounded wait (code " +
                                                   std::to_string(st.kerr) + ")");
        const size_t nbt = j.inflight;
        if (nbt > 0 && ms > 0.f) j.ms_per_tile = (double)ms / (double)nbt;
        j.last_nbt = nbt;
        if (st.overflow) {
            // Tighten with everything captured (a valid lower bound), drop
            // this batch's partial appends, retry it in halves.  Only more
            // than `cap` exactly tied candidates keep overflowing 1 tile.
            if (++j.retries > 64)
                return set_error(GEPI_ERR_LIMIT, "candidate buffer keeps overflowing (massive ties)");
            j.S.overflows += 1;
            return select_async(j, (int)b->cap, j.count, Op::SelRetry);
        }
        j.last_appended = st.count - j.count;
        j.count = st.count;
        j.next += nbt;
        j.retries = 0;
        j.S.batches += 1;
        if (j.next < j.ntiles && j.count > select_trigger(j.budget, j.rq.k))
            return select_async(j, -1, 0xFFFFFFFFu, Op::SelBudget);
        if (j.next < j.ntiles) size_next_batch(j);
        return advance(j);
    }
    case Op::SelRetry:
        j.count = st.count;
        j.batch = std::max<size_t>(1, j.last_nbt / 2);
        return advance(j);
    case Op::SelBudget:
        j.count = st.count;
        size_next_batch(j);
        return advance(j);
    case Op::SelFinal:
        j.count = st.count;
        j.final_selected = true;
        return advance(j);
    case Op::None:
        break;
    }
    return advance(j);
}

int Engine::poll(std::vector<Job *> &active) {
    DeviceGuard g(device_);
    int progressed = 0;
    if (policy_ == Policy::Oldest) {
        Job *old = nullptr;
        for (Job *j : active) {
            j->oldest = false;
            if (!j->done && (!old || j->t_admit < old->t_admit)) old = j;
        }
        if (old) old->oldest = true;
    }
    for (Job *j : active) {
        if (j->done || j->op != Op::None) continue;
        gepi_status st = advance(*j);  // newly admitted, or an empty range
        if (st != GEPI_OK) fail(*j, st);
        if (j->done) ++progressed;
    }
    for (Job *j : active) {
        if (j->done || j->op == Op::None) continue;
        const cudaError_t q = cudaEventQuery(j->buf->ev[4]);
        if (q == cudaErrorNotReady) continue;
        gepi_status st = GEPI_OK;
        if (q != cudaSuccess) {
            cudaGetLastError();
            st = set_error(GEPI_ERR_CUDA, std::string("scan operation: ") + cudaGetErrorString(q));
        } else {
            st = complete(*j);
        }
        if (st != GEPI_OK) fail(*j, st);
        ++progressed;
    }
    return progressed;
}

// ---- the device engines used by gepi_scan_batch -----------------------------

namespace {

std::mutex g_engines_mu;
std::map<int, std::unique_ptr<Engine>> g_engines;  // one per device, kept until exit

gepi_status device_engine(int device, Engine **out) {
    std::lock_guard<std::mutex> lk(g_engines_mu);
    auto it = g_engines.find(device);
    if (it == g_engines.end()) {
        auto e = std::make_unique<Engine>(device, 0.0);
        GEPI_TRY(e->init());
        it = g_engines.emplace(device, std::move(e)).first;
    }
    *out = it->second.get();
    return GEPI_OK;
}

gepi_status check_request(const gepi_scan_req &r, ScanRequest *out) {
    if (!r.planes) return set_error(GEPI_ERR_ARG, "scan request: null planes");
    if (r.topmost <= 0) return set_error(GEPI_ERR_ARG, "scan request: topmost must be > 0");
    if (r.objective != GEPI_ENTROPY && r.objective != GEPI_FISHER)
        return set_error(GEPI_ERR_ARG, "scan request: unknown objective");
    if (r.method < GEPI_METHOD_AUTO || r.method > GEPI_METHOD_TENSOR)
        return set_error(GEPI_ERR_ARG, "scan request: unknown method");
    const int n = r.planes->n_snps;
    ScanRequest q;
    q.pl = r.planes;
    if (r.na < 0 || r.nb < 0) {
        q.a0 = 0;
        q.na = n;
        q.b0 = 0;
        q.nb = n;
    } else {
        if (r.a0 < 0 || r.b0 < 0 || (int64_t)r.a0 + r.na > n || (int64_t)r.b0 + r.nb > n)
            return set_error(GEPI_ERR_ARG, "scan request: SNP range outside the planes");
        q.a0 = r.a0;
        q.na = r.na;
        q.b0 = r.b0;
        q.nb = r.nb;
    }
    q.k = r.topmost;
    q.objective = r.objective;
    q.method = r.method;
    *out = q;
    return GEPI_OK;
}

// Device memory a request holds while admitted: two candidate buffers.
size_t request_footprint(int k) { return 2 * cand_cap(k) * sizeof(Cand) + sizeof(ScanState); }

void idle_wait() { std::this_thread::sleep_for(std::chrono::microseconds(20)); }

Policy env_policy(Policy dflt) {
    if (const char *e = std::getenv("GEPI_SERVE_POLICY")) {
        if (!std::strcmp(e, "oldest")) return Policy::Oldest;
        if (!std::strcmp(e, "short")) return Policy::ShortFirst;
    }
    return dflt;
}

double env_quantum_ms(double dflt) {
    if (const char *e = std::getenv("GEPI_QUANTUM_MS")) {
        const double v = std::atof(e);
        if (v >= 0.0) return v;
    }
    return dflt;
}

}  // namespace

}  // namespace gepi

using namespace gepi;

extern "C" {

gepi_status gepi_scan_batch(const gepi_scan_req *reqs, int32_t n, gepi_result *const *tops,
                            gepi_scan_stats *stats) {
    clear_error();
    if (!reqs || !tops || n <= 0) return set_error(GEPI_ERR_ARG, "gepi_scan_batch: bad argument");
    std::vector<Job> jobs((size_t)n);
    for (int i = 0; i < n; ++i) {
        GEPI_TRY(check_request(reqs[i], &jobs[i].rq));
        if (!tops[i]) return set_error(GEPI_ERR_ARG, "gepi_scan_batch: null result array");
        if (reqs[i].planes->device != reqs[0].planes->device)
            return set_error(GEPI_ERR_ARG, "gepi_scan_batch: requests on different devices");
        jobs[i].tops = tops[i];
    }
    Engine *eng = nullptr;
    GEPI_TRY(device_engine(reqs[0].planes->device, &eng));
    std::lock_guard<std::mutex> run_lock(eng->run_mu);
    std::vector<Job *> active;
    gepi_status st = GEPI_OK;
    for (Job &j : jobs) {
        st = eng->prepare(j);
        if (st == GEPI_OK) st = eng->admit(j);
        active.push_back(&j);
        if (st != GEPI_OK) break;
    }
    while (st == GEPI_OK) {
        bool any = false;
        for (Job *j : active) any |= !j->done;
        if (!any) break;
        if (eng->poll(active) == 0) idle_wait();
        for (Job *j : active)
            if (j->status != GEPI_OK) {
                st = set_error(j->status, j->error);
                break;
            }
    }
    for (int i = 0; i < n; ++i) {
        if (stats) stats[i] = jobs[i].S;
        eng->release(jobs[i]);
    }
    return st;
}

}  // extern "C"

// The serving loop's state (C ABI handle).
struct gepi_server {
    int device = 0;
    size_t budget = 0, used = 0;
    std::unique_ptr<gepi::Engine> engine;
    std::thread thread;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<gepi::Job *> pending;
    std::map<uint64_t, std::unique_ptr<gepi::Job>> jobs;
    uint64_t next_ticket = 1;
    bool stop = false;

    void run();
};

void gepi_server::run() {
    cudaSetDevice(device);
    std::vector<Job *> active, admitting;
    bool idle = false;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                // admission: FIFO while the footprint fits; the head always
                // gets in when nothing runs, so no request starves
                while (!pending.empty()) {
                    Job *j = pending.front();
                    if (!active.empty() && used + j->footprint > budget) break;
                    pending.pop_front();
                    used += j->footprint;
                    admitting.push_back(j);
                }
                if (!active.empty() || !admitting.empty()) break;
                if (stop) return;
                cv_work.wait(lk);
            }
            // nothing completed last time round: sleep briefly, waking on a submit
            if (idle && admitting.empty()) cv_work.wait_for(lk, std::chrono::microseconds(20));
        }
        for (Job *j : admitting) {
            gepi_status st = engine->admit(*j);
            if (st != GEPI_OK) {
                j->status = st;
                j->error = gepi_last_error();
                j->done = true;
                j->t_done = Clock::now();
            }
            active.push_back(j);
        }
        admitting.clear();
        idle = engine->poll(active) == 0;
        bool any = false;
        for (Job *j : active)
            if (j->done) {
                engine->release(*j);
                any = true;
            }
        if (!any) continue;
        std::lock_guard<std::mutex> lk(mu);
        for (Job *j : active)
            if (j->done) {
                used -= j->footprint;
                j->finished = true;
            }
        active.erase(std::remove_if(active.begin(), active.end(), [](Job *j) { return j->done; }),
                     active.end());
        idle = false;
        cv_done.notify_all();
    }
}

extern "C" {

gepi_status gepi_server_create(int32_t device, size_t hbm_budget_bytes, gepi_server **out) {
    clear_error();
    if (!out) return set_error(GEPI_ERR_ARG, "gepi_server_create: null output");
    *out = nullptr;
    auto srv = std::make_unique<gepi_server>();
    srv->device = device;
    srv->budget = hbm_budget_bytes ? hbm_budget_bytes : (16ull << 30);
    srv->engine =
        std::make_unique<Engine>(device, env_quantum_ms(4.0), env_policy(Policy::ShortFirst));
    GEPI_TRY(srv->engine->init());
    gepi_server *p = srv.get();
    p->thread = std::thread([p] { p->run(); });
    *out = srv.release();
    return GEPI_OK;
}

gepi_status gepi_server_submit(gepi_server *srv, const gepi_scan_req *req, uint64_t *ticket) {
    clear_error();
    if (!srv || !req || !ticket) return set_error(GEPI_ERR_ARG, "gepi_server_submit: bad argument");
    ScanRequest rq;
    GEPI_TRY(check_request(*req, &rq));
    if (rq.pl->device != srv->device)
        return set_error(GEPI_ERR_ARG, "gepi_server_submit: plane set on another device");
    auto j = std::make_unique<Job>();
    j->rq = rq;
    j->t_submit = Clock::now();
    j->own_tops.assign((size_t)rq.k, gepi_result{});
    j->tops = j->own_tops.data();
    j->footprint = request_footprint(rq.k);
    // method, tables and tile list on the caller's thread, off the loop
    gepi_status st = srv->engine->prepare(*j);
    if (st != GEPI_OK) {
        srv->engine->release(*j);
        return st;
    }
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        j->ticket = srv->next_ticket++;
        *ticket = j->ticket;
        srv->pending.push_back(j.get());
        srv->jobs[j->ticket] = std::move(j);
    }
    srv->cv_work.notify_one();
    return GEPI_OK;
}

gepi_status gepi_server_wait(gepi_server *srv, uint64_t ticket, gepi_result *tops,
                             gepi_request_info *info) {
    clear_error();
    if (!srv || !tops) return set_error(GEPI_ERR_ARG, "gepi_server_wait: bad argument");
    std::unique_ptr<Job> j;
    {
        std::unique_lock<std::mutex> lk(srv->mu);
        auto it = srv->jobs.find(ticket);
        if (it == srv->jobs.end()) return set_error(GEPI_ERR_ARG, "gepi_server_wait: unknown ticket");
        Job *p = it->second.get();
        srv->cv_done.wait(lk, [p] { return p->finished; });
        j = std::move(it->second);
        srv->jobs.erase(it);
    }
    if (info) {
        std::memset(info, 0, sizeof *info);
        const bool admitted = j->t_admit.time_since_epoch().count() != 0;
        info->queue_ms = admitted ? ms_between(j->t_submit, j->t_admit) : 0.0;
        info->latency_ms = ms_between(j->t_submit, j->t_done);
        info->device_ms = j->S.scan_ms;
        info->snp_pairs = j->S.snp_pairs;
        info->method = j->S.method;
    }
    if (j->status != GEPI_OK) return set_error(j->status, j->error);
    std::memcpy(tops, j->tops, sizeof(gepi_result) * (size_t)j->rq.k);
    return GEPI_OK;
}

void gepi_server_destroy(gepi_server *srv) {
    if (!srv) return;
    std::deque<Job *> dropped;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
        dropped.swap(srv->pending);
    }
    srv->cv_work.notify_all();
    if (srv->thread.joinable()) srv->thread.join();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        for (Job *j : dropped) {
            srv->engine->release(*j);
            j->status = GEPI_ERR_ARG;
            j->error = "server destroyed before the request was admitted";
            j->t_done = Clock::now();
            j->finished = true;
        }
    }
    srv->cv_done.notify_all();
    delete srv;
}

}  // extern "C"
