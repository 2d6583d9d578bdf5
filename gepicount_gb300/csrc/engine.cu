// Scan engine: runs many scan requests -- whole plane sets or SNP range x
// range blocks, on one or many plane sets (cohorts) of a device -- together,
// and the serving loop built on it.
//
// Replaces the reference's one-cohort-per-process batch loop
// (launch_process_gpu_1, src/kernels/kernel1.cu:387-483).  Each request walks
// its tile list in adaptive batches with the same exact thresholds as a direct
// scan, so its results are bit-identical to gepi_scan_range's.  The engine
// advances all requests in steps; one step is ONE CUDA graph replay:
//   * an upload of the step's descriptors (per request: its tables, this
//     step's candidate buffer and scan state, its slice of its tile list),
//   * one persistent counting launch per kernel group -- the tensor-core
//     kernel for every tensor-core request of an objective, the popcount
//     kernel of a variant for every popcount request of that variant -- whose
//     CTAs (pairs) claim tiles from the concatenated work list with an atomic
//     counter,
//   * one chain of 20 batched select launches over every request (the small
//     ones with gridDim.y = request, the histogram and compaction passes on
//     the whole grid walking the requests in turn), each request's select
//     decided on the device from its scan state exactly as the direct scan
//     decides it on the host,
//   * a read-back of every request's scan state.
// The graph is captured once per set of kernel groups and slot capacity and
// replayed with new descriptors every step.  Between steps the host sizes
// every request's next batch (append rate, select budget, optional
// device-time quantum), retires finished requests and admits new ones
// (serving), so requests arriving while others run join at the next step.
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
#include <functional>
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

// Device bytes of cached tile lists kept when no request uses them.
constexpr size_t kTileCacheBytes = 1ull << 30;

// Kernel groups of a step, in launch order: tensor cores (entropy, Fisher),
// then one per popcount variant.
constexpr int kGroups = 5;
// Fisher tests a step leaves for its pending-list launch (all requests; 80 MB
// with the request tags); past it they are evaluated in the counting launch
constexpr uint32_t kEnginePendCap = 1u << 22;
int group_of(const CountVariant &v, int objective) {
    if (v.method == GEPI_METHOD_TENSOR) return objective == GEPI_ENTROPY ? 0 : 1;
    return 1 + v.id;  // popcount variants 1..3 -> groups 2..4
}

}  // namespace

struct ScanRequest {
    gepi_planes *pl = nullptr;
    int a0 = 0, na = 0, b0 = 0, nb = 0;
    int k = 0, objective = 0, method = 0, variant = 0;
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

// Candidate buffers of one request, pooled by capacity.
struct JobBuffers {
    Cand *cand[2] = {nullptr, nullptr};
    uint32_t cap = 0;
};

struct Job {
    ScanRequest rq;
    gepi_result *tops = nullptr;
    std::vector<gepi_result> own_tops;  // serving: kept until gepi_server_wait
    uint64_t ticket = 0;
    size_t footprint = 0;
    bool finished = false;  // serving: results ready for the waiter
    const CountVariant *cv = nullptr;
    int group = 0;
    int TA = 0, TB = 0;
    double weight = 1.0;  // device cost of one tile relative to other requests'
    TileList *tl = nullptr;
    size_t ntiles = 0, next = 0, batch = 1, inflight = 0;
    JobBuffers *buf = nullptr;
    int slot = -1;
    int cur = 0;
    uint32_t count = 0, budget = 0, trigger = 0;
    int retries = 0;
    float lp_margin = 0.f;
    bool done = false, final_selected = false;
    gepi_status status = GEPI_OK;
    std::string error;
    gepi_scan_stats S{};
    Clock::time_point t_submit, t_admit, t_done;
};

// Which requests' tiles go first in a step and get the quantum first:
//  * ShortFirst: least work left first (shortest remaining time; the server's
//    default, the lowest tail latency measured on a mixed stream);
//  * Deadline: earliest deadline first, a request's deadline being its
//    submission time plus `slack` times its estimated device time alone
//    (tiles x measured ms per tile, plus about one millisecond): a long
//    request goes ahead of newer short ones once it has waited about slack x
//    its own time, so its latency approaches (1 + slack) x its time alone;
//  * Oldest: first come, first served.
enum class Policy { ShortFirst, Deadline, Oldest };

class Engine {
   public:
    // quantum_ms > 0 caps each step at about that much device time.
    Engine(int device, double quantum_ms, Policy policy = Policy::ShortFirst, double slack = 1.5)
        : device_(device), quantum_ms_(quantum_ms), policy_(policy), slack_(slack) {}
    ~Engine();
    gepi_status init();
    // Counting variant, plane-set tables and the device tile list: may run on
    // any thread (serialised internally).
    gepi_status prepare(Job &j);
    // Candidate buffers, a state slot and the initial scan state.
    gepi_status admit(Job &j);
    // One engine step over the active requests: finishes requests with no
    // tiles left, runs one batch of every other one (one graph replay) and
    // consumes the results.
    void step(std::vector<Job *> &active);
    // Returns a request's buffers, slot and tile list.
    void release(Job &j);
    std::mutex run_mu;  // serialises gepi_scan_batch calls on the device
    gepi_batch_stats counters{};  // launches since the last reset

   private:
    gepi_status ensure_slots(int need);
    cudaError_t ensure_pending();
    // setup = true: only the kernels' shared-memory opt-ins and occupancy
    // queries (outside any capture)
    cudaError_t enqueue_step(unsigned mask, bool setup = false);
    gepi_status launch_step(unsigned mask);
    gepi_status finish(std::vector<Job *> &jobs);
    void size_next_batch(Job &j, uint32_t appended, size_t nbt);
    void plan(std::vector<Job *> &run);

    int device_ = 0, num_sms_ = 0;
    double quantum_ms_ = 0.0;
    Policy policy_ = Policy::ShortFirst;
    double slack_ = 1.5;
    // stream_: the steps; upload_: tile lists; fin_: read-back of finished
    // requests' candidates while the next step runs
    cudaStream_t stream_ = nullptr, upload_ = nullptr, fin_ = nullptr;
    cudaEvent_t ev_[3] = {nullptr, nullptr, nullptr};  // step start, counting done, step done
    // per-slot device state: scan state, radix-select scratch
    int nslots_ = 0;
    ScanState *d_states_ = nullptr, *h_states_ = nullptr;
    unsigned char *d_sel_ = nullptr;
    std::vector<int> free_slots_;
    // step descriptors: pinned host image and its device copy, same layout
    // [WorkQueue x kGroups | ReqDesc x slots | SelJob x slots | WorkRange x slots x kGroups]
    size_t step_bytes_ = 0, off_reqs_ = 0, off_jobs_ = 0, off_ranges_ = 0;
    unsigned char *h_step_ = nullptr, *d_step_ = nullptr;
    WorkQueue *h_queues_ = nullptr;  // pinned: the launches' error codes, read back each step
    std::map<unsigned, cudaGraphExec_t> graphs_;
    // the steps' Fisher pending list (allocated with the first Fisher request):
    // fill counter, request tags, entries
    unsigned char *d_pend_buf_ = nullptr;
    PendList *d_pend_ = nullptr;  // its header, at the start of d_pend_buf_
    // estimated device ms per unit of tile weight, per kernel group
    double ms_per_weight_[kGroups] = {0, 0, 0, 0, 0};
    std::vector<std::unique_ptr<JobBuffers>> pool_;
    std::vector<JobBuffers *> free_;
    std::mutex prep_mu_, cache_mu_;
    std::map<TileKey, TileList> tiles_;
    size_t tile_bytes_ = 0;
    uint64_t stamp_ = 0;
};

Engine::~Engine() {
    DeviceGuard g(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second);
    for (auto &b : pool_) {
        dfree(b->cand[0]);
        dfree(b->cand[1]);
    }
    dfree(d_states_);
    dfree(d_sel_);
    dfree(d_step_);
    dfree(d_pend_buf_);
    if (h_states_) cudaFreeHost(h_states_);
    if (h_step_) cudaFreeHost(h_step_);
    if (h_queues_) cudaFreeHost(h_queues_);
    for (cudaEvent_t e : ev_)
        if (e) cudaEventDestroy(e);
    for (auto &kv : tiles_)
        if (kv.second.d) cudaFreeAsync(kv.second.d, upload_);
    if (upload_) {
        cudaStreamSynchronize(upload_);
        cudaStreamDestroy(upload_);
    }
    if (fin_) cudaStreamDestroy(fin_);
    if (stream_) cudaStreamDestroy(stream_);
}

gepi_status Engine::init() {
    DeviceGuard g(device_);
    if (!g.ok) return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    GEPI_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device_));
    GEPI_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    GEPI_CUDA(cudaStreamCreateWithFlags(&upload_, cudaStreamNonBlocking));
    GEPI_CUDA(cudaStreamCreateWithFlags(&fin_, cudaStreamNonBlocking));
    for (cudaEvent_t &e : ev_) GEPI_CUDA(cudaEventCreate(&e));
    GEPI_CUDA(cudaMallocHost(&h_queues_, sizeof(WorkQueue) * kGroups));
    return ensure_slots(16);
}

// Slot capacity (a power of two): per-slot scan states and select scratch, and
// the step descriptor buffers sized for that many requests.  Growing drops
// the captured graphs (their launch shapes depend on the capacity).
gepi_status Engine::ensure_slots(int need) {
    if (need <= nslots_) return GEPI_OK;
    int n = std::max(16, nslots_);
    while (n < need) n *= 2;
    GEPI_CUDA(cudaStreamSynchronize(stream_));
    for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
    ScanState *ds = nullptr, *hs = nullptr;
    unsigned char *dsel = nullptr, *hstep = nullptr, *dstep = nullptr;
    const size_t off_reqs = ((sizeof(WorkQueue) * kGroups + 255) / 256) * 256;
    const size_t off_jobs = off_reqs + ((sizeof(ReqDesc) * n + 255) / 256) * 256;
    const size_t off_ranges = off_jobs + ((sizeof(SelJob) * n + 255) / 256) * 256;
    const size_t bytes = off_ranges + sizeof(WorkRange) * (size_t)n * kGroups;
    cudaError_t e = cudaMalloc(&ds, sizeof(ScanState) * n);
    if (e == cudaSuccess) e = cudaMallocHost(&hs, sizeof(ScanState) * n);
    if (e == cudaSuccess) e = cudaMalloc(&dsel, sel_state_bytes() * n);
    if (e == cudaSuccess) e = cudaMallocHost(&hstep, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dstep, bytes);
    if (e == cudaSuccess && nslots_)  // keep the states of admitted requests
        e = cudaMemcpy(ds, d_states_, sizeof(ScanState) * nslots_, cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
        dfree(ds);
        dfree(dsel);
        dfree(dstep);
        if (hs) cudaFreeHost(hs);
        if (hstep) cudaFreeHost(hstep);
        return set_error(GEPI_ERR_CUDA, std::string("engine slots: ") + cudaGetErrorString(e));
    }
    std::memset(hstep, 0, bytes);
    std::memset(hs, 0, sizeof(ScanState) * n);
    if (nslots_) std::memcpy(hs, h_states_, sizeof(ScanState) * nslots_);
    dfree(d_states_);
    dfree(d_sel_);
    dfree(d_step_);
    if (h_states_) cudaFreeHost(h_states_);
    if (h_step_) cudaFreeHost(h_step_);
    d_states_ = ds;
    h_states_ = hs;
    d_sel_ = dsel;
    h_step_ = hstep;
    d_step_ = dstep;
    step_bytes_ = bytes;
    off_reqs_ = off_reqs;
    off_jobs_ = off_jobs;
    off_ranges_ = off_ranges;
    for (int s = n - 1; s >= nslots_; --s) free_slots_.push_back(s);
    std::sort(free_slots_.begin(), free_slots_.end(), std::greater<int>());
    nslots_ = n;
    return GEPI_OK;
}

// The Fisher pending list of the steps.  The step graphs bake in its address,
// so those captured before it existed (without its launches) are dropped.  A
// failure is not an error of the call: without the list the counting kernels
// evaluate the tests themselves.
cudaError_t Engine::ensure_pending() {
    if (d_pend_buf_) return cudaSuccess;
    const size_t tags = 256, ents = tags + (size_t)kEnginePendCap * 4;
    unsigned char *b = nullptr;
    cudaError_t e = cudaMalloc(&b, ents + (size_t)kEnginePendCap * sizeof(uint4));
    if (e != cudaSuccess) return e;
    PendList hdr{};
    hdr.ent = reinterpret_cast<uint4 *>(b + ents);
    hdr.tag = reinterpret_cast<uint32_t *>(b + tags);
    hdr.cap = kEnginePendCap;
    e = cudaMemcpy(b, &hdr, sizeof hdr, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) {
        cudaFree(b);
        return e;
    }
    for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
    d_pend_buf_ = b;
    d_pend_ = reinterpret_cast<PendList *>(b);
    return cudaSuccess;
}

// The device work of one step on the engine's stream: upload, the counting
// launches of the kernel groups in `mask` (bit g), the batched selects, the
// read-back.
cudaError_t Engine::enqueue_step(unsigned mask, bool setup) {
    WorkQueue *dq = reinterpret_cast<WorkQueue *>(d_step_);
    const ReqDesc *dreqs = reinterpret_cast<const ReqDesc *>(d_step_ + off_reqs_);
    SelJob *djobs = reinterpret_cast<SelJob *>(d_step_ + off_jobs_);
    // the timing events are recorded as graph nodes when captured (external
    // records), so the host can wait for and time every replay
    auto record = [&](cudaEvent_t ev) {
        return cudaEventRecordWithFlags(ev, stream_, cudaEventRecordExternal);
    };
    cudaError_t e = cudaSuccess;
    if (!setup) e = cudaMemcpyAsync(d_step_, h_step_, step_bytes_, cudaMemcpyHostToDevice, stream_);
    if (e == cudaSuccess && !setup) e = record(ev_[0]);
    if (e == cudaSuccess && !setup && d_pend_)
        e = cudaMemsetAsync(&d_pend_->n, 0, sizeof(uint32_t), stream_);
    for (int g = 0; g < kGroups && e == cudaSuccess; ++g) {
        if (!(mask & (1u << g))) continue;
        if (g < 2) {
            e = launch_tc_batch(dreqs, dq + g, g, num_sms_, stream_, setup);
        } else {
            const CountVariant *v = count_variant(g - 1);
            e = launch_popc_batch(v->ta, v->words, dreqs, dq + g, num_sms_, stream_, setup);
        }
    }
    if (setup) return e;
    if (e == cudaSuccess && d_pend_) e = launch_fisher_pending_batch(dreqs, d_pend_, num_sms_, stream_);
    if (e == cudaSuccess) e = record(ev_[1]);
    if (e == cudaSuccess) e = run_select_batch(djobs, nslots_, num_sms_, stream_);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_states_, d_states_, sizeof(ScanState) * nslots_, cudaMemcpyDeviceToHost,
                            stream_);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_queues_, d_step_, sizeof(WorkQueue) * kGroups, cudaMemcpyDeviceToHost,
                            stream_);
    if (e == cudaSuccess) e = record(ev_[2]);
    return e;
}

// Replays the step graph of `mask` (captured on first use; the timeout test's
// kernels are a graph of their own), or enqueues the same work directly if a
// capture is refused.
gepi_status Engine::launch_step(unsigned mask) {
    const unsigned key = mask | (tc_debug_stall() ? 1u << 16 : 0u);
    auto it = graphs_.find(key);
    if (it == graphs_.end()) {
        GEPI_CUDA(enqueue_step(mask, true));
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t x = nullptr;
        cudaError_t e = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t e1 = enqueue_step(mask);
            const cudaError_t e2 = cudaStreamEndCapture(stream_, &graph);
            e = e1 != cudaSuccess ? e1 : e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&x, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            GEPI_CUDA(enqueue_step(mask));
            return GEPI_OK;
        }
        it = graphs_.emplace(key, x).first;
    }
    GEPI_CUDA(cudaGraphLaunch(it->second, stream_));
    counters.graph_launches += 1;
    return GEPI_OK;
}

gepi_status Engine::prepare(Job &j) {
    std::lock_guard<std::mutex> lk(prep_mu_);
    DeviceGuard g(device_);
    const ScanRequest &rq = j.rq;
    gepi_planes *pl = rq.pl;
    GEPI_TRY(pl_ensure_tables(pl));
    GEPI_TRY(pl_resolve_variant(pl, rq.method, rq.variant, &j.cv));
    if (j.cv->method == GEPI_METHOD_TENSOR) GEPI_TRY(pl_ensure_tc_blocks(pl));
    GEPI_CUDA(cudaStreamSynchronize(pl->stream));  // decode, relayout, tables done
    j.TA = j.cv->ta;
    j.TB = j.cv->tb;
    j.group = group_of(*j.cv, rq.objective);
    // device cost of a tile: its pipeline stages (samples) times its SNP pairs
    const double w = (double)j.cv->words;
    j.weight = (std::ceil(pl->W0 / w) + std::ceil(pl->W1 / w)) * (double)j.TA * j.TB / 1024.0;

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
    j.S.method = j.cv->method;
    j.S.tile_snps = j.TA;
    j.S.variant = j.cv->id;
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
    if (free_slots_.empty()) GEPI_TRY(ensure_slots(nslots_ + 1));
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
    }
    j.buf = b;
    j.slot = free_slots_.back();
    free_slots_.pop_back();
    ScanState init{};
    init.tau_key = 0ull;
    init.theta = 0.f;
    init.lp_thr = INFINITY;
    init.tau_f = -INFINITY;
    init.tau_val = -INFINITY;
    // No step is in flight (admission happens between steps), so the slot of
    // the pinned read-back buffer is free; the upload is ordered before the
    // next step on the engine's stream, and that step's read-back -- which
    // overwrites the buffer -- after the upload.
    h_states_[j.slot] = init;
    GEPI_CUDA(cudaMemcpyAsync(d_states_ + j.slot, h_states_ + j.slot, sizeof(ScanState),
                              cudaMemcpyHostToDevice, stream_));

    // as in the direct scan: the same select budget, trigger and first batch
    const double tests_per_tile = 20.0 * j.TA * j.TB;
    j.budget = select_budget(b->cap, j.rq.k);
    j.trigger = select_trigger(j.budget, j.rq.k);
    j.batch = (size_t)std::max(1.0, std::floor(pilot_tests(j.rq.objective, j.budget) / tests_per_tile));
    j.lp_margin = 2e-6f * j.rq.pl->lf_max + 1e-3f;
    j.cur = 0;
    j.next = 0;
    j.count = 0;
    j.retries = 0;
    j.done = j.final_selected = false;
    j.t_admit = Clock::now();
    return GEPI_OK;
}

void Engine::release(Job &j) {
    DeviceGuard g(device_);
    if (j.buf) {
        free_.push_back(j.buf);
        j.buf = nullptr;
    }
    if (j.slot >= 0) {
        free_slots_.push_back(j.slot);
        j.slot = -1;
    }
    if (j.tl) {
        std::lock_guard<std::mutex> ck(cache_mu_);
        j.tl->refs -= 1;
        j.tl = nullptr;
    }
}

// Reads the surviving candidates of finished requests back and writes their
// ranked top-k.
gepi_status Engine::finish(std::vector<Job *> &jobs) {
    if (jobs.empty()) return GEPI_OK;
    std::vector<std::vector<Cand>> host(jobs.size());
    for (size_t i = 0; i < jobs.size(); ++i) {
        Job &j = *jobs[i];
        host[i].resize(j.count);
        // the request's last step has completed, and its buffers are not
        // part of the step that may be running on the engine's stream
        if (j.count)
            GEPI_CUDA(cudaMemcpyAsync(host[i].data(), j.buf->cand[j.cur], (size_t)j.count * sizeof(Cand),
                                      cudaMemcpyDeviceToHost, fin_));
    }
    GEPI_CUDA(cudaStreamSynchronize(fin_));
    for (size_t i = 0; i < jobs.size(); ++i) {
        Job &j = *jobs[i];
        const int k = j.rq.k;
        std::memset(j.tops, 0, sizeof(gepi_result) * (size_t)k);
        const size_t keep = std::min<size_t>(host[i].size(), (size_t)k);
        std::partial_sort(host[i].begin(), host[i].begin() + keep, host[i].end(), cand_better);
        for (size_t q = 0; q < keep; ++q) {
            const Cand &c = host[i][q];
            gepi_result &r = j.tops[q];
            r.sA = c.rA;
            r.sB = c.rBfun >> 3;
            r.fun = (char)(c.rBfun & 7);
            for (int t = 0; t < 4; ++t) r.n[t] = c.n[t];
            r.ent = (float)(-value_of_key(c.key));
        }
        j.S.candidates = j.count;
        j.done = true;
        j.t_done = Clock::now();
    }
    return GEPI_OK;
}

// Next batch: as many tiles as the remaining budget allows at the append
// rate just observed, growing at most 8x per step (the direct scan's rule).
void Engine::size_next_batch(Job &j, uint32_t appended, size_t nbt) {
    const double rate = std::max(1.0, (double)appended) / (double)std::max<size_t>(1, nbt);
    const double room = (double)j.budget - (double)j.count;
    double nb_next = room > 0 ? room / rate : 1.0;
    nb_next = std::min(nb_next, 8.0 * (double)std::max<size_t>(1, nbt));
    j.batch = (size_t)std::max(1.0, nb_next);
}

// This step's batch of every running request: its natural batch; under a
// device-time quantum the requests, in policy order, fill the quantum, each
// getting at least one tile.  The order is also the order of their tiles in
// the work lists, so the CTAs claim the first requests' tiles first.
void Engine::plan(std::vector<Job *> &run) {
    auto left = [&](const Job *j) {
        return (double)(j->ntiles - j->next) * j->weight * ms_per_weight_[j->group];
    };
    auto arrival = [](const Job *j) {  // submission (serving) or admission (batch)
        const Clock::time_point t = j->t_submit.time_since_epoch().count() ? j->t_submit : j->t_admit;
        return std::chrono::duration<double, std::milli>(t.time_since_epoch()).count();
    };
    if (policy_ == Policy::Oldest) {
        std::stable_sort(run.begin(), run.end(),
                         [&](const Job *a, const Job *b) { return arrival(a) < arrival(b); });
    } else if (policy_ == Policy::ShortFirst) {
        std::stable_sort(run.begin(), run.end(),
                         [&](const Job *a, const Job *b) { return left(a) < left(b); });
    } else {
        // estimated device time alone: every tile at the measured cost, plus
        // about one millisecond of fixed cost per request
        std::vector<std::pair<double, Job *>> key;
        key.reserve(run.size());
        for (Job *j : run) {
            const double alone = (double)j->ntiles * j->weight * ms_per_weight_[j->group] + 1.0;
            key.emplace_back(arrival(j) + slack_ * alone, j);
        }
        std::stable_sort(key.begin(), key.end(),
                         [](const auto &a, const auto &b) { return a.first < b.first; });
        for (size_t i = 0; i < run.size(); ++i) run[i] = key[i].second;
    }
    double room = quantum_ms_;
    for (Job *j : run) {
        size_t nbt = std::min(j->batch, j->ntiles - j->next);
        const double per_tile = j->weight * ms_per_weight_[j->group];
        if (quantum_ms_ > 0.0 && per_tile > 0.0 && nbt > 0) {
            const double fit = std::floor(std::max(0.0, room) / per_tile);
            nbt = std::max<size_t>(1, (size_t)std::min<double>((double)nbt, fit));
            room -= (double)nbt * per_tile;
        }
        j->inflight = nbt;
    }
}

void Engine::step(std::vector<Job *> &active) {
    DeviceGuard g(device_);
    const Clock::time_point t_step = Clock::now();
    // requests with every tile counted and no select pending finish; the rest
    // run a batch (possibly empty: only the final select is left)
    std::vector<Job *> fin, run;
    for (Job *j : active) {
        if (j->done) continue;
        if (j->next >= j->ntiles && (j->count <= (uint32_t)j->rq.k || j->final_selected))
            fin.push_back(j);
        else
            run.push_back(j);
    }
    auto fail_all = [&](std::vector<Job *> &js, gepi_status st) {
        for (Job *j : js) {
            j->status = st;
            j->error = gepi_last_error();
            j->done = true;
            j->t_done = Clock::now();
        }
    };
    // the finished requests' results are read back and ranked while the
    // step of the others runs
    auto finish_all = [&]() {
        if (fin.empty()) return;
        const gepi_status st = finish(fin);
        if (st != GEPI_OK) fail_all(fin, st);
    };
    if (run.empty()) {
        finish_all();
        counters.wall_ms += ms_between(t_step, Clock::now());
        return;
    }
    plan(run);
    for (Job *j : run) {
        if (j->rq.objective == GEPI_FISHER && !d_pend_buf_) {
            if (ensure_pending() != cudaSuccess) (void)cudaGetLastError();
            break;
        }
    }

    // the step's descriptors
    WorkQueue *hq = reinterpret_cast<WorkQueue *>(h_step_);
    ReqDesc *hreqs = reinterpret_cast<ReqDesc *>(h_step_ + off_reqs_);
    SelJob *hjobs = reinterpret_cast<SelJob *>(h_step_ + off_jobs_);
    WorkRange *hranges = reinterpret_cast<WorkRange *>(h_step_ + off_ranges_);
    const WorkRange *dranges = reinterpret_cast<const WorkRange *>(d_step_ + off_ranges_);
    for (int q = 0; q < kGroups; ++q) {
        hq[q] = WorkQueue{};
        hq[q].ranges = dranges + (size_t)q * nslots_;
    }
    for (int s = 0; s < nslots_; ++s) hjobs[s] = SelJob{};
    unsigned mask = 0;
    for (Job *j : run) {
        gepi_planes *pl = j->rq.pl;
        const int s = j->slot;
        ReqDesc &R = hreqs[s];
        R.planes = pl->d_planes;
        R.blk = pl->d_tc_blocks;
        R.tiles = j->tl->d;
        R.Wp = pl->Wp;
        R.W0 = pl->W0;
        R.rows_pad = j->cv->method == GEPI_METHOD_TENSOR ? tc_rows_pad(pl->n_snps) : 0;
        R.n_snps = pl->n_snps;
        R.a0 = j->rq.a0;
        R.a1 = j->rq.a0 + j->rq.na;
        R.b0 = j->rq.b0;
        R.b1 = j->rq.b0 + j->rq.nb;
        R.ctx.T = pl->d_T;
        R.ctx.F = pl->F;
        R.ctx.lf = pl->d_lf;
        R.ctx.lf32 = pl->d_lf32;
        R.ctx.objective = j->rq.objective;
        R.ctx.fisher_fp64 = fisher_fp64_walks();
        // Fisher: tests that pass the bounds go to the step's pending list
        // (entries hold 16-bit counts)
        const bool pend = j->rq.objective == GEPI_FISHER && d_pend_ && pl->S0 < 65536 &&
                          pl->S1 < 65536;
        R.ctx.pend = pend ? d_pend_ : nullptr;
        R.ctx.pend_req = (uint32_t)s;
        R.ctx.cand = j->buf->cand[j->cur];
        R.ctx.cap = j->buf->cap;
        R.ctx.st = d_states_ + s;
        const size_t nbt = j->inflight;
        if (nbt > 0) {
            WorkQueue &q = hq[j->group];
            WorkRange &r = hranges[(size_t)j->group * nslots_ + q.nranges];
            r.req = s;
            r.first = (int)j->next;
            r.start = q.ntiles;
            r.count = (int)nbt;
            q.ntiles += (int)nbt;
            q.nranges += 1;
            mask |= 1u << j->group;
        }
        SelJob &sj = hjobs[s];
        sj.in = j->buf->cand[j->cur];
        sj.out = j->buf->cand[j->cur ^ 1];
        sj.st = d_states_ + s;
        sj.sel = reinterpret_cast<SelState *>(d_sel_ + sel_state_bytes() * (size_t)s);
        sj.cap = j->buf->cap;
        sj.k = (uint32_t)j->rq.k;
        sj.trigger = j->trigger;
        sj.count_before = j->count;
        sj.final_batch = j->next + nbt >= j->ntiles ? 1 : 0;
        sj.objective = j->rq.objective;
        sj.lp_margin = j->lp_margin;
        sj.active = 1;
    }
    gepi_status st = launch_step(mask);
    finish_all();
    counters.steps += 1;
    // on any failure below, the step's device work finishes before the
    // requests -- and their buffers -- are released
    auto drain = [&]() {
        cudaStreamSynchronize(stream_);
        (void)cudaGetLastError();
    };
    counters.select_launches += kSelectLaunches;
    for (int q = 0; q < kGroups; ++q) counters.count_launches += (mask >> q) & 1u;
    if (st == GEPI_OK) {
        const cudaError_t e = cudaEventSynchronize(ev_[2]);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            st = set_error(GEPI_ERR_CUDA, std::string("engine step: ") + cudaGetErrorString(e));
        }
    }
    float count_ms = 0.f, step_ms = 0.f;
    if (st == GEPI_OK) {
        cudaEventElapsedTime(&count_ms, ev_[0], ev_[1]);
        cudaEventElapsedTime(&step_ms, ev_[0], ev_[2]);
        for (int q = 0; q < kGroups; ++q)
            if ((mask & (1u << q)) && h_queues_[q].err) {
                st = set_error(GEPI_ERR_TIMEOUT, "counting kernel gave up a bounded wait (code " +
                                                     std::to_string(h_queues_[q].err) + ")");
                break;
            }
    }
    if (st != GEPI_OK) {
        drain();
        fail_all(run, st);
        counters.wall_ms += ms_between(t_step, Clock::now());
        return;
    }
    counters.device_ms += step_ms;
    // Device cost per unit of tile weight, per group (for the quantum and the
    // deadlines).  A launch of few tiles leaves most SMs idle and its fixed
    // cost dominates, so its time over its weight overstates the cost of a
    // tile: such a step may only lower the estimate; steps of at least two
    // tiles per SM set it.
    {
        double w[kGroups] = {0, 0, 0, 0, 0};
        size_t nt[kGroups] = {0, 0, 0, 0, 0};
        for (Job *j : run) {
            w[j->group] += (double)j->inflight * j->weight;
            nt[j->group] += j->inflight;
        }
        double wsum = 0.0;
        size_t tsum = 0;
        for (int q = 0; q < kGroups; ++q) {
            wsum += w[q];
            tsum += nt[q];
        }
        if (wsum > 0.0 && count_ms > 0.f) {
            const double per = (double)count_ms / wsum;
            const bool full = tsum >= 2 * (size_t)num_sms_;
            for (int q = 0; q < kGroups; ++q) {
                if (w[q] <= 0.0) continue;
                double &e = ms_per_weight_[q];
                if (e <= 0.0)
                    e = per;
                else if (full)
                    e = 0.5 * (e + per);
                else if (per < e)
                    e = per;
            }
        }
    }
    for (Job *j : run) {
        const ScanState &ss = h_states_[j->slot];
        const size_t nbt = j->inflight;
        j->S.scan_ms += step_ms;
        j->S.other_launches += kSelectLaunches;
        if (nbt > 0) {
            j->S.count_ms += count_ms;
            j->S.max_count_ms = std::max<double>(j->S.max_count_ms, count_ms);
            j->S.count_launches += 1;
        }
        const uint32_t mode = ss.sel_mode;
        if (mode == 2) {
            // overflow: the select tightened with everything captured and kept
            // only the candidates from before the batch; retry it in halves
            j->cur ^= 1;
            j->count = ss.count;
            j->S.overflows += 1;
            if (++j->retries > 64) {
                j->status = set_error(GEPI_ERR_LIMIT, "candidate buffer keeps overflowing (massive ties)");
                j->error = gepi_last_error();
                j->done = true;
                j->t_done = Clock::now();
                continue;
            }
            j->batch = std::max<size_t>(1, nbt / 2);
            continue;
        }
        const uint32_t appended = ss.count_batch - j->count;
        if (mode == 1) j->cur ^= 1;
        j->count = ss.count;
        j->retries = 0;
        if (nbt > 0) {
            j->next += nbt;
            j->S.batches += 1;
        }
        if (j->next >= j->ntiles) {
            if (mode == 1) j->final_selected = true;
        } else {
            size_next_batch(*j, appended, nbt);
        }
    }
    counters.wall_ms += ms_between(t_step, Clock::now());
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
    if (r.variant != 0 && !count_variant(r.variant))
        return set_error(GEPI_ERR_ARG, "scan request: unknown counting variant");
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
    q.variant = r.variant;
    *out = q;
    return GEPI_OK;
}

// Device memory a request holds while admitted: two candidate buffers.
size_t request_footprint(int k) { return 2 * cand_cap(k) * sizeof(Cand) + sizeof(ScanState); }

Policy env_policy(Policy dflt) {
    if (const char *e = std::getenv("GEPI_SERVE_POLICY")) {
        if (!std::strcmp(e, "oldest")) return Policy::Oldest;
        if (!std::strcmp(e, "short")) return Policy::ShortFirst;
        if (!std::strcmp(e, "deadline")) return Policy::Deadline;
    }
    return dflt;
}

double env_slack(double dflt) {
    if (const char *e = std::getenv("GEPI_SERVE_SLACK")) {
        const double v = std::atof(e);
        if (v >= 0.0) return v;
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
    eng->counters = gepi_batch_stats{};
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
        eng->step(active);
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

gepi_status gepi_scan_batch_stats(int32_t device, gepi_batch_stats *out) {
    clear_error();
    if (!out) return set_error(GEPI_ERR_ARG, "gepi_scan_batch_stats: null output");
    Engine *eng = nullptr;
    GEPI_TRY(device_engine(device, &eng));
    std::lock_guard<std::mutex> run_lock(eng->run_mu);
    *out = eng->counters;
    return GEPI_OK;
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
    gepi_batch_stats stats{};  // the engine's counters, copied under mu between steps

    void run();
};

// Continuous batching: between two engine steps the loop admits queued
// requests (first in, first out, while their footprint fits the budget; the
// oldest always when nothing runs) and retires finished ones, so a request
// arriving while others run joins at the next step.
void gepi_server::run() {
    cudaSetDevice(device);
    std::vector<Job *> active, admitting;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(mu);
            stats = engine->counters;
            for (;;) {
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
        engine->step(active);
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
        std::make_unique<Engine>(device, env_quantum_ms(4.0), env_policy(Policy::ShortFirst),
                                 env_slack(1.5));
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
    // variant, tables and tile list on the caller's thread, off the loop
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

gepi_status gepi_server_stats(gepi_server *srv, gepi_batch_stats *out) {
    clear_error();
    if (!srv || !out) return set_error(GEPI_ERR_ARG, "gepi_server_stats: bad argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    *out = srv->stats;
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
