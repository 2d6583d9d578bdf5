// Device top-k machinery replacing the per-batch thrust::sort_by_key, the
// D2H of every count and the host streaming merge
// (src/kernels/kernel1.cu:448, misc1.cu:205-264).
//
// Counting kernels append every test whose exact key is >= tau_key to a
// candidate buffer.  When the buffer grows past its budget, a radix select
// finds the k-th largest key (8 passes of 8-bit digits), tau_key is raised to
// it and the buffer is compacted to keys >= tau_key (ties at the k-th place are
// kept).  Every test with key >= the final k-th key is therefore present at the
// end, and the host sorts the survivors by (key desc, rA, rB, fun).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "device.cuh"

namespace gepi {

struct SelState {
    unsigned long long prefix, mask;
    uint32_t krem;     // rank still to locate inside the current bucket (0 = no select)
    uint32_t n;        // entries examined
    uint32_t ncompact; // entries kept by compaction
    uint32_t pad;      // batched selects: the mode taken (0 none, 1 select, 2 overflow retry)
    uint32_t hist[256];
};

__global__ void sel_init_kernel(const ScanState *st, SelState *sel, uint32_t cap, uint32_t k,
                                int n_override) {
    if (threadIdx.x == 0) {
        uint32_t n = n_override >= 0 ? (uint32_t)n_override : st->count;
        if (n > cap) n = cap;
        sel->n = n;
        sel->krem = (n >= k && k > 0) ? k : 0u;
        sel->prefix = 0ull;
        sel->mask = 0ull;
        sel->ncompact = 0u;
    }
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sel->hist[i] = 0u;
}

__global__ void sel_hist_kernel(const Cand *__restrict__ cand, SelState *sel, int shift) {
    __shared__ uint32_t h[256];
    if (sel->krem == 0) return;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0u;
    __syncthreads();
    const uint32_t n = sel->n;
    const unsigned long long prefix = sel->prefix, mask = sel->mask;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned long long key = cand[i].key;
        if ((key & mask) == prefix) atomicAdd(&h[(key >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(&sel->hist[i], h[i]);
}

// One warp: walk buckets from the largest digit down to find the one holding
// the krem-th largest key, fix that digit, clear the histogram.
__device__ __forceinline__ void sel_pick(SelState *sel, int shift) {
    if (sel->krem == 0) return;
    const int lane = threadIdx.x;
    // lane L owns buckets 255-8L .. 248-8L (descending)
    uint32_t c[8], tot = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        c[j] = sel->hist[255 - 8 * lane - j];
        tot += c[j];
    }
    // exclusive prefix over lanes (descending bucket order)
    uint32_t incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t excl = incl - tot;
    const uint32_t k = sel->krem;
    const bool mine = excl < k && k <= incl;
    const unsigned ball = __ballot_sync(0xffffffffu, mine);
    const int owner = __ffs(ball) - 1;
    if (lane == owner) {
        uint32_t run = excl;
        int b = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (run + c[j] >= k) {
                b = 255 - 8 * lane - j;
                break;
            }
            run += c[j];
        }
        sel->krem = k - run;
        sel->prefix |= (unsigned long long)b << shift;
        sel->mask |= 255ull << shift;
    }
    __syncwarp();
    for (int i = lane; i < 256; i += 32) sel->hist[i] = 0u;
}

__global__ void sel_pick_kernel(SelState *sel, int shift) { sel_pick(sel, shift); }

// Raise tau_key to the selected key and derive the float bounds.
//   entropy: theta = (2^I - 1) * (1 - 2^-10), I the selected mutual information
//   Fisher : lp_thr = ln(p) + margin, p = 10^-v for the selected v = -log10 p
__device__ __forceinline__ void sel_apply(ScanState *st, const SelState *sel, int objective,
                                          float lp_margin) {
    if (sel->krem == 0) return;
    unsigned long long key = sel->prefix;
    if (key <= st->tau_key) return;
    st->tau_key = key;
    double v = value_of_key(key);
    st->tau_val = v;
    if (objective == 0) {
        st->tau_f = __double2float_rd(v);
        double th = (exp2(v) - 1.0) * (1.0 - 1.0 / 1024.0);
        st->theta = th > 0.0 ? __double2float_rd(th) : 0.0f;
    } else {
        double lp = -v * 2.302585092994045684 + (double)lp_margin;
        st->lp_thr = lp < 0.0 ? __double2float_ru(lp) : 0.0f;
    }
}

__global__ void sel_apply_kernel(ScanState *st, const SelState *sel, int objective,
                                 float lp_margin) {
    sel_apply(st, sel, objective, lp_margin);
}

__device__ __forceinline__ void compact_range(const Cand *__restrict__ in, Cand *__restrict__ out,
                                              const ScanState *st, SelState *sel,
                                              uint32_t n_limit) {
    const unsigned long long tau = st->tau_key;
    uint32_t n = sel->n;
    if (n > n_limit) n = n_limit;
    const int lane = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool keep = false;
        Cand c;
        if (i < n) {
            c = in[i];
            keep = c.key >= tau;
        }
        const unsigned ball = __ballot_sync(0xffffffffu, keep);
        uint32_t off = 0;
        if (lane == 0 && ball) off = atomicAdd(&sel->ncompact, (uint32_t)__popc(ball));
        off = __shfl_sync(0xffffffffu, off, 0);
        if (keep) out[off + __popc(ball & ((1u << lane) - 1u))] = c;
    }
}

__global__ void compact_kernel(const Cand *__restrict__ in, Cand *__restrict__ out,
                               const ScanState *st, SelState *sel, uint32_t n_limit) {
    compact_range(in, out, st, sel, n_limit);
}

__global__ void set_count_kernel(ScanState *st, const SelState *sel) {
    st->count = sel->ncompact;
    st->overflow = 0u;
}

// k-th largest key of the first min(count, cap) candidates (or n_override) ->
// tau_key, then compaction of the first n_compact candidates into `out`.
cudaError_t run_select_compact(Cand *in, Cand *out, ScanState *st, void *sel_raw, uint32_t cap,
                               uint32_t k, int n_override, uint32_t n_compact, int objective,
                               float lp_margin, int num_sms, cudaStream_t stream) {
    SelState *sel = static_cast<SelState *>(sel_raw);
    sel_init_kernel<<<1, 256, 0, stream>>>(st, sel, cap, k, n_override);
    const int grid = num_sms * 4;
    for (int shift = 56; shift >= 0; shift -= 8) {
        sel_hist_kernel<<<grid, 256, 0, stream>>>(in, sel, shift);
        sel_pick_kernel<<<1, 32, 0, stream>>>(sel, shift);
    }
    sel_apply_kernel<<<1, 1, 0, stream>>>(st, sel, objective, lp_margin);
    // compaction reads sel->n (= entries examined); limit to n_compact
    compact_kernel<<<grid, 256, 0, stream>>>(in, out, st, sel, n_compact);
    set_count_kernel<<<1, 1, 0, stream>>>(st, sel);
    return cudaGetLastError();
}

size_t sel_state_bytes() { return sizeof(SelState); }

// ---- batched selects: one chain of launches for every request of an engine
// step, replayed from a CUDA graph.  Each request's
// select is decided on the device from its scan state, exactly as the direct
// scan decides it on the host (scan.cu):
//   overflow in this batch             -> select over the first `cap` entries,
//                                         compaction of the `count_before`
//                                         entries captured before the batch
//                                         (the batch is retried in halves)
//   last batch and count > k, or
//   not last and count > trigger       -> select over all entries, compaction
//   otherwise                          -> nothing
// The mode taken is left in ScanState::sel_mode for the host.

// Slots without a request this step (active = 0) carry null state and
// scratch pointers: every batched kernel skips them before touching them.
__global__ void bsel_init_kernel(SelJob *jobs) {
    SelJob &j = jobs[blockIdx.y];
    if (!j.active) return;
    SelState *sel = j.sel;
    if (threadIdx.x == 0) {
        ScanState *st = j.st;
        const uint32_t count = st->count;
        int mode = 0;
        if (st->overflow) mode = 2;
        else if (j.final_batch ? count > j.k : count > j.trigger) mode = 1;
        uint32_t n = count > j.cap ? j.cap : count;
        sel->n = mode ? n : 0u;
        sel->krem = (mode && n >= j.k && j.k > 0) ? j.k : 0u;
        sel->prefix = 0ull;
        sel->mask = 0ull;
        sel->ncompact = 0u;
        sel->pad = (uint32_t)mode;
        st->sel_mode = (uint32_t)mode;
        st->count_batch = count;
    }
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sel->hist[i] = 0u;
}

// The histogram passes and the compaction run on a 1-D grid (4 CTAs per SM)
// that walks the slots in turn, so each request's pass gets the whole GPU
// whatever the slot capacity; the per-slot branches are uniform across a CTA
// (every thread reads the same descriptor and scratch words).
__global__ void bsel_hist_kernel(const SelJob *jobs, int njobs, int shift) {
    __shared__ uint32_t h[256];
    for (int q = 0; q < njobs; ++q) {
        const SelJob &j = jobs[q];
        if (!j.active) continue;
        SelState *sel = j.sel;
        if (sel->krem == 0) continue;
        for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0u;
        __syncthreads();
        const uint32_t n = sel->n;
        const unsigned long long prefix = sel->prefix, mask = sel->mask;
        const Cand *__restrict__ cand = j.in;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            unsigned long long key = cand[i].key;
            if ((key & mask) == prefix) atomicAdd(&h[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 256; i += blockDim.x)
            if (h[i]) atomicAdd(&sel->hist[i], h[i]);
        __syncthreads();  // h is cleared for the next slot
    }
}

__global__ void bsel_pick_kernel(const SelJob *jobs, int shift) {
    const SelJob &j = jobs[blockIdx.y];
    if (!j.active) return;
    sel_pick(j.sel, shift);
}

__global__ void bsel_apply_kernel(const SelJob *jobs) {
    const SelJob &j = jobs[blockIdx.y];
    if (!j.active) return;
    sel_apply(j.st, j.sel, j.objective, j.lp_margin);
}

__global__ void bcompact_kernel(const SelJob *jobs, int njobs) {
    for (int q = 0; q < njobs; ++q) {
        const SelJob &j = jobs[q];
        if (!j.active) continue;
        const int mode = (int)j.sel->pad;
        if (!mode) continue;
        compact_range(j.in, j.out, j.st, j.sel, mode == 2 ? j.count_before : 0xFFFFFFFFu);
    }
}

__global__ void bset_count_kernel(const SelJob *jobs) {
    const SelJob &j = jobs[blockIdx.y];
    if (!j.active || !j.sel->pad) return;
    j.st->count = j.sel->ncompact;
    j.st->overflow = 0u;
}

cudaError_t run_select_batch(SelJob *jobs, int njobs, int num_sms, cudaStream_t stream) {
    if (njobs <= 0) return cudaSuccess;
    const int grid = num_sms * 4;
    bsel_init_kernel<<<dim3(1, njobs), 256, 0, stream>>>(jobs);
    for (int shift = 56; shift >= 0; shift -= 8) {
        bsel_hist_kernel<<<grid, 256, 0, stream>>>(jobs, njobs, shift);
        bsel_pick_kernel<<<dim3(1, njobs), 32, 0, stream>>>(jobs, shift);
    }
    bsel_apply_kernel<<<dim3(1, njobs), 1, 0, stream>>>(jobs);
    bcompact_kernel<<<grid, 256, 0, stream>>>(jobs, njobs);
    bset_count_kernel<<<dim3(1, njobs), 1, 0, stream>>>(jobs);
    return cudaGetLastError();
}

}  // namespace gepi
