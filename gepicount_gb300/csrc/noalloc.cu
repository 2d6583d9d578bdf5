// gepi_process_gpu_1_noalloc: the process_gpu_1 scan for callers that cannot
// allocate device memory.
//
// Some hosts own every byte of GPU memory through their own pool or caching
// allocator (a framework plugin, a database operator, a process that must not
// grow its footprint after start-up) and forbid cudaMalloc/cudaFree from
// libraries they load.  This entry point serves them: the caller passes the
// same host inputs and host output as gepi_process_gpu_1, and every device
// buffer the scan needs -- uploaded rows, class permutation, genotype planes,
// scoring tables, tile list, candidate buffers, scan state, output records --
// is carved from ONE file-scope device array, g_noalloc_scratch, of
// kNoAllocScratchBytes (32 MiB).  Every GPU that loads the library holds that
// array until the process exits.  On success no cudaMalloc, cudaFree,
// cudaMallocHost, stream or event creation and no host heap allocation happen
// on this path: the class permutation and tile list are built by kernels, the
// log-factorial tables are computed on the host in fixed-size chunks on the
// stack (the same std::lgamma values gepi_process_gpu_1 uses, so both entry
// points give the same bits for either objective), the final ranking is done
// on the device, and only the k result records are copied back.  Error returns
// record their message in a std::string (heap); only the success path is
// allocation-free.
//
// Limits: the inputs, planes and tables must fit the array next to the
// candidate buffers (two buffers of kNoAllocCap = 65,536 records), and
// k <= kNoAllocCap / 4; larger requests return GEPI_ERR_LIMIT before any
// device work.  A Fisher scan also takes a pending list of tests for exact
// evaluation from the scratch left over (up to kNoAllocPendCap entries),
// and evaluates them in the counting launch when none is left.
//
// Device address: the host-side symbol g_noalloc_scratch is only a stand-in
// and must never be passed to a kernel.  Every call, with the caller's device
// made current, looks the array's device address up with
// cudaGetSymbolAddress (a cheap host call) and checks its return code, so a
// context torn down and rebuilt between calls (cudaDeviceReset) never leaves a
// stale address behind.
//
// Sharing: every call on a device uses the same array and finds the previous
// call's contents there; the call initialises everything it reads (scan state,
// select state, planes, tables, output records).  Calls that overlap on the
// same GPU (from several host threads) race on the array and must be
// serialised by the caller.  Work is issued on the legacy default stream and
// the call returns after it completes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "common.h"
#include "device.cuh"
#include "tables.h"

namespace gepi {

cudaError_t launch_decode_rows(const uint64_t *bits, const uint64_t *valid, int nw, int n_snps,
                               const int32_t *perm, int Wp, uint32_t *planes,
                               cudaStream_t stream, int num_sms);
cudaError_t launch_popc_tiles(int ta, int kc, const uint32_t *planes, int Wp, int W0,
                              const int2 *tiles, int ntiles, int a0, int a1, int b0, int b1,
                              const ScanCtx &ctx, uint32_t *dump, cudaStream_t stream);
int fisher_fp64_walks();
cudaError_t launch_fisher_pending(const ScanCtx &ctx, int num_sms, cudaStream_t stream);
cudaError_t run_select_compact(Cand *in, Cand *out, ScanState *st, void *sel, uint32_t cap,
                               uint32_t k, int n_override, uint32_t n_compact, int objective,
                               float lp_margin, int num_sms, cudaStream_t stream);
size_t sel_state_bytes();
// The popcount variant this entry point runs: 32 x 32 SNP tiles, 32 plane
// words per stage (the library's default popcount variant).
constexpr int kNoAllocTile = 32;
constexpr int kNoAllocStageWords = 32;

constexpr size_t kNoAllocScratchBytes = 32ull << 20;
constexpr uint32_t kNoAllocCap = 65536;
// Fisher pending list: at most this many entries, from scratch the request
// leaves free (a request never needs it to fit)
constexpr uint32_t kNoAllocPendCap = 1u << 18;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Device address of the scratch array on the current device `dev`.
gepi_status scratch_address(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kMaxDevices) return set_error(GEPI_ERR_ARG, "device ordinal out of range");
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return set_error(GEPI_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = static_cast<unsigned char *>(p);
    return GEPI_OK;
}

// Bump allocator over the scratch array (offsets only; nothing is allocated).
struct Carve {
    size_t used = 0;
    size_t take(size_t bytes) {
        size_t off = used;
        used += (bytes + 255) & ~size_t(255);
        return off;
    }
};

// Same integer log2 as the host table builder (tables.cpp): 64 fraction bits
// by repeated squaring of the Q1.63 mantissa, truncating each square.
__device__ uint64_t na_log2_fixed(uint64_t n, int F) {
    if (n <= 1) return 0;
    const int e = 63 - __clzll((long long)n);
    uint64_t x = n << (63 - e);
    uint64_t frac = 0;
    for (int i = 1; i <= 64; ++i) {
        const uint64_t hi = __umul64hi(x, x), lo = x * x;
        if (hi >> 63) {
            x = hi;
            frac |= 1ull << (64 - i);
        } else {
            x = (hi << 1) | (lo >> 63);
        }
    }
    const uint64_t r = (frac >> (64 - F)) + ((frac >> (63 - F)) & 1ull);
    return ((uint64_t)e << F) + r;
}

__global__ void na_tfix_kernel(uint64_t *T, int nmax, int F) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n <= nmax; n += gridDim.x * blockDim.x)
        T[n] = (uint64_t)n * na_log2_fixed((uint64_t)n, F);
}

// log(n!) for n in [0, nmax] as double and float, computed on the host with
// std::lgamma (the values build_lfact gives the allocating scan) in chunks of
// kLfChunk on the stack, each copied to the device synchronously.
constexpr int kLfChunk = 2048;
cudaError_t upload_lfact(double *lf, float *lf32, int nmax) {
    double hd[kLfChunk];
    float hf[kLfChunk];
    for (int n0 = 0; n0 <= nmax; n0 += kLfChunk) {
        const int cnt = std::min(kLfChunk, nmax + 1 - n0);
        for (int i = 0; i < cnt; ++i) {
            const double v = std::lgamma((double)(n0 + i) + 1.0);
            hd[i] = v;
            hf[i] = (float)v;
        }
        cudaError_t e = cudaMemcpy(lf + n0, hd, (size_t)cnt * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(lf32 + n0, hf, (size_t)cnt * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Class-sorted permutation from the two class masks (one block): slot j of
// class 0 is the j-th sample (in file order) of mask1, class 1 starts at
// word W0; every other slot is -1.
__global__ void na_perm_kernel(const uint64_t *m1, const uint64_t *m2, int nw, int W0, int Wp,
                               int32_t *perm) {
    __shared__ int base[2][1024];
    const int nslots = Wp * 32;
    for (int i = threadIdx.x; i < nslots; i += blockDim.x) perm[i] = -1;
    const int per = (nw + blockDim.x - 1) / blockDim.x;
    const int w0 = threadIdx.x * per, w1 = min(nw, w0 + per);
    int c0 = 0, c1 = 0;
    for (int w = w0; w < w1; ++w) {
        c0 += __popcll(m1[w]);
        c1 += __popcll(m2[w]);
    }
    base[0][threadIdx.x] = c0;
    base[1][threadIdx.x] = c1;
    __syncthreads();
    if (threadIdx.x == 0) {
        int a = 0, b = 0;
        for (int t = 0; t < (int)blockDim.x; ++t) {
            int va = base[0][t], vb = base[1][t];
            base[0][t] = a;
            base[1][t] = b;
            a += va;
            b += vb;
        }
    }
    __syncthreads();
    int s0 = base[0][threadIdx.x], s1 = W0 * 32 + base[1][threadIdx.x];
    for (int w = w0; w < w1; ++w) {
        uint64_t a = m1[w], b = m2[w];
        while (a) {
            const int bit = __ffsll((long long)a) - 1;
            perm[s0++] = w * 64 + bit;
            a &= a - 1;
        }
        while (b) {
            const int bit = __ffsll((long long)b) - 1;
            perm[s1++] = w * 64 + bit;
            b &= b - 1;
        }
    }
}

// Lower-triangle tile list (A tile i >= B tile j), row-major.
__global__ void na_tiles_kernel(int2 *tiles, int nt) {
    const long long total = (long long)nt * (nt + 1) / 2;
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < total;
         l += (long long)gridDim.x * blockDim.x) {
        int i = (int)((sqrt(8.0 * (double)l + 1.0) - 1.0) * 0.5);
        while ((long long)i * (i + 1) / 2 > l) --i;
        while ((long long)(i + 1) * (i + 2) / 2 <= l) ++i;
        tiles[l] = make_int2(i, (int)(l - (long long)i * (i + 1) / 2));
    }
}

__device__ __forceinline__ bool na_better(const Cand &a, const Cand &b) {
    if (a.key != b.key) return a.key > b.key;
    if (a.rA != b.rA) return a.rA < b.rA;
    return a.rBfun < b.rBfun;
}

// Final ranking on the device: the rank of each survivor is the number of
// survivors that beat it under (key desc, sA, sB, fun); ranks < k are written
// as result records, slots with no survivor are zeroed.  The survivors are the
// compacted candidates: at most k plus the tests tied with the k-th key, so
// the all-pairs count is about k^2 (2.7e8 comparisons at k = 16,384); only
// massive ties at the k-th key (up to the 65,536-record buffer) make it
// larger.
__global__ void na_rank_kernel(const Cand *cand, const ScanState *st, int k, gepi_result *out) {
    const uint32_t n = min(st->count, kNoAllocCap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x)
        if ((uint32_t)i >= n) {
            gepi_result z;
            memset(&z, 0, sizeof z);
            out[i] = z;
        }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Cand c = cand[i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < n; ++j) rank += na_better(cand[j], c) ? 1u : 0u;
        if (rank < (uint32_t)k) {
            gepi_result r;
            memset(&r, 0, sizeof r);
            r.sA = c.rA;
            r.sB = c.rBfun >> 3;
            r.fun = (char)(c.rBfun & 7);
            for (int q = 0; q < 4; ++q) r.n[q] = c.n[q];
            r.ent = (float)(-value_of_key(c.key));
            out[rank] = r;
        }
    }
}

}  // namespace
}  // namespace gepi

using namespace gepi;

extern "C" gepi_status gepi_process_gpu_1_noalloc(const uint64_t *bits, const uint64_t *valid,
                                                  int n_rows, int n_words, const uint64_t *mask1,
                                                  const uint64_t *mask2, gepi_result *tops,
                                                  const gepi_params *par) {
    clear_error();
    if (!bits || !valid || !mask1 || !mask2 || !tops || !par || n_rows <= 0 || (n_rows & 1) ||
        n_words <= 0)
        return set_error(GEPI_ERR_ARG, "gepi_process_gpu_1_noalloc: bad argument");
    const int k = par->topmost;
    if (k <= 0) return set_error(GEPI_ERR_ARG, "gepi_process_gpu_1_noalloc: topmost <= 0");
    if (par->objective != GEPI_ENTROPY && par->objective != GEPI_FISHER)
        return set_error(GEPI_ERR_ARG, "gepi_process_gpu_1_noalloc: unknown objective");
    if (par->method == GEPI_METHOD_TENSOR)
        return set_error(GEPI_ERR_UNSUPPORTED, "gepi_process_gpu_1_noalloc: popcount counting only");
    const int n_snps = n_rows / 2;
    for (int s = 0; s < n_snps; ++s)
        if (std::memcmp(valid + (size_t)(2 * s) * n_words, valid + (size_t)(2 * s + 1) * n_words,
                        (size_t)n_words * 8) != 0)
            return set_error(GEPI_ERR_FORMAT, "valid rows of an allele pair differ");
    int S0 = 0, S1 = 0;
    for (int w = 0; w < n_words; ++w) {
        if (mask1[w] & mask2[w]) return set_error(GEPI_ERR_FORMAT, "sample in both class masks");
        S0 += __builtin_popcountll(mask1[w]);
        S1 += __builtin_popcountll(mask2[w]);
    }
    if (S0 == 0 || S1 == 0) return set_error(GEPI_ERR_NOCLASS, "Error in class mask data");
    const int W0 = ((S0 + kClassPadSamples - 1) / kClassPadSamples) * (kClassPadSamples / 32);
    const int W1 = ((S1 + kClassPadSamples - 1) / kClassPadSamples) * (kClassPadSamples / 32);
    const int Wp = W0 + W1;
    const int nmax = S0 + S1;
    const int T = kNoAllocTile;
    const int nt = (n_snps + T - 1) / T;
    const long long ntiles = (long long)nt * (nt + 1) / 2;

    // Lay out the scratch array; reject requests that do not fit.
    Carve cv;
    const size_t o_state = cv.take(sizeof(ScanState));
    const size_t o_sel = cv.take(sel_state_bytes());
    const size_t o_cand0 = cv.take((size_t)kNoAllocCap * sizeof(Cand));
    const size_t o_cand1 = cv.take((size_t)kNoAllocCap * sizeof(Cand));
    const size_t o_out = cv.take((size_t)k * sizeof(gepi_result));
    const size_t o_m = cv.take(2 * (size_t)n_words * 8);
    const size_t o_bits = cv.take((size_t)n_rows * n_words * 8);
    const size_t o_valid = cv.take((size_t)n_rows * n_words * 8);
    const size_t o_perm = cv.take((size_t)Wp * 32 * 4);
    const size_t o_planes = cv.take((size_t)n_snps * 3 * Wp * 4);
    const size_t o_T = cv.take(((size_t)nmax + 1) * 8);
    const size_t o_lf = cv.take(((size_t)nmax + 1) * 8);
    const size_t o_lf32 = cv.take(((size_t)nmax + 1) * 4);
    const size_t o_tiles = cv.take((size_t)ntiles * sizeof(int2));
    if (k > (int)(kNoAllocCap / 4) || cv.used > kNoAllocScratchBytes)
        return set_error(GEPI_ERR_LIMIT,
                         "gepi_process_gpu_1_noalloc: needs " + std::to_string(cv.used) +
                             " bytes of scratch and k <= " + std::to_string(kNoAllocCap / 4) +
                             "; the fixed scratch array holds " +
                             std::to_string(kNoAllocScratchBytes) + " bytes");
    // Fisher: tests that pass the bounds are evaluated by a launch across the
    // GPU after each counting launch, from a pending list in the free scratch
    // (entries hold 16-bit counts); without room they run in the counting launch
    uint32_t pend_cap = 0;
    size_t o_pend = 0;
    if (par->objective == GEPI_FISHER && S0 < 65536 && S1 < 65536 &&
        cv.used + 256 + 4096 * sizeof(uint4) <= kNoAllocScratchBytes) {
        pend_cap = (uint32_t)std::min<size_t>(
            kNoAllocPendCap, (kNoAllocScratchBytes - cv.used - 256) / sizeof(uint4));
        o_pend = cv.take(256 + (size_t)pend_cap * sizeof(uint4));
    }

    int prev = -1;
    cudaGetDevice(&prev);
    if (cudaSetDevice(par->gpu_num) != cudaSuccess)
        return set_error(GEPI_ERR_CUDA, "cudaSetDevice failed");
    struct Restore {
        int d;
        ~Restore() {
            if (d >= 0) cudaSetDevice(d);
        }
    } restore{prev};
    unsigned char *base = nullptr;
    GEPI_TRY(scratch_address(par->gpu_num, &base));
    int num_sms = 0;
    GEPI_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, par->gpu_num));
    const cudaStream_t stream = 0;

    ScanState *d_state = reinterpret_cast<ScanState *>(base + o_state);
    void *d_sel = base + o_sel;
    Cand *d_cand[2] = {reinterpret_cast<Cand *>(base + o_cand0),
                       reinterpret_cast<Cand *>(base + o_cand1)};
    gepi_result *d_out = reinterpret_cast<gepi_result *>(base + o_out);
    uint64_t *d_m1 = reinterpret_cast<uint64_t *>(base + o_m), *d_m2 = d_m1 + n_words;
    uint64_t *d_bits = reinterpret_cast<uint64_t *>(base + o_bits);
    uint64_t *d_valid = reinterpret_cast<uint64_t *>(base + o_valid);
    int32_t *d_perm = reinterpret_cast<int32_t *>(base + o_perm);
    uint32_t *d_planes = reinterpret_cast<uint32_t *>(base + o_planes);
    uint64_t *d_T = reinterpret_cast<uint64_t *>(base + o_T);
    double *d_lf = reinterpret_cast<double *>(base + o_lf);
    float *d_lf32 = reinterpret_cast<float *>(base + o_lf32);
    int2 *d_tiles = reinterpret_cast<int2 *>(base + o_tiles);

    // Inputs, tables, permutation, planes, tile list.
    const size_t rb = (size_t)n_rows * n_words * 8;
    GEPI_CUDA(cudaMemcpy(d_bits, bits, rb, cudaMemcpyHostToDevice));
    GEPI_CUDA(cudaMemcpy(d_valid, valid, rb, cudaMemcpyHostToDevice));
    GEPI_CUDA(cudaMemcpy(d_m1, mask1, (size_t)n_words * 8, cudaMemcpyHostToDevice));
    GEPI_CUDA(cudaMemcpy(d_m2, mask2, (size_t)n_words * 8, cudaMemcpyHostToDevice));
    const int F = tfix_bits(nmax);
    na_tfix_kernel<<<num_sms, 256, 0, stream>>>(d_T, nmax, F);
    GEPI_CUDA(cudaGetLastError());
    GEPI_CUDA(upload_lfact(d_lf, d_lf32, nmax));
    na_perm_kernel<<<1, 1024, 0, stream>>>(d_m1, d_m2, n_words, W0, Wp, d_perm);
    GEPI_CUDA(cudaGetLastError());
    GEPI_CUDA(launch_decode_rows(d_bits, d_valid, n_words, n_snps, d_perm, Wp, d_planes, stream,
                                 num_sms));
    na_tiles_kernel<<<num_sms, 256, 0, stream>>>(d_tiles, nt);
    GEPI_CUDA(cudaGetLastError());

    ScanState st{};
    st.tau_key = 0ull;
    st.theta = 0.f;
    st.lp_thr = INFINITY;
    st.tau_f = -INFINITY;
    st.tau_val = -INFINITY;
    GEPI_CUDA(cudaMemcpy(d_state, &st, sizeof st, cudaMemcpyHostToDevice));

    ScanCtx ctx;
    ctx.T = d_T;
    ctx.F = F;
    ctx.lf = d_lf;
    ctx.lf32 = d_lf32;
    ctx.objective = par->objective;
    ctx.fisher_fp64 = fisher_fp64_walks();
    ctx.pend = nullptr;
    ctx.pend_req = 0;
    ctx.cap = kNoAllocCap;
    ctx.st = d_state;
    if (pend_cap) {
        PendList hdr{};
        hdr.ent = reinterpret_cast<uint4 *>(base + o_pend + 256);
        hdr.cap = pend_cap;
        GEPI_CUDA(cudaMemcpy(base + o_pend, &hdr, sizeof hdr, cudaMemcpyHostToDevice));
        ctx.pend = reinterpret_cast<PendList *>(base + o_pend);
    }
    const float lp_margin = 2e-6f * (float)std::lgamma((double)nmax + 1.0) + 1e-3f;

    // Adaptive batches over the tile list, as in the allocating scan.
    const double tests_per_tile = 20.0 * T * T;
    const uint32_t budget = kNoAllocCap / 2;
    const double pilot = par->objective == GEPI_ENTROPY ? kNoAllocCap / 4.0 : 4096.0;
    size_t batch = (size_t)std::max(1.0, std::floor(pilot / tests_per_tile));
    size_t t = 0;
    uint32_t count = 0;
    int cur = 0, retries = 0;
    while (t < (size_t)ntiles) {
        const size_t nbt = std::min(batch, (size_t)ntiles - t);
        ctx.cand = d_cand[cur];
        if (ctx.pend) GEPI_CUDA(cudaMemsetAsync(&ctx.pend->n, 0, sizeof(uint32_t), stream));
        GEPI_CUDA(launch_popc_tiles(kNoAllocTile, kNoAllocStageWords, d_planes, Wp, W0, d_tiles + t,
                                    (int)nbt, 0, n_snps, 0, n_snps,
                                    ctx, nullptr, stream));
        if (ctx.pend) GEPI_CUDA(launch_fisher_pending(ctx, num_sms, stream));
        GEPI_CUDA(cudaMemcpy(&st, d_state, sizeof st, cudaMemcpyDeviceToHost));
        if (st.overflow) {
            if (++retries > 64)
                return set_error(GEPI_ERR_LIMIT, "candidate buffer keeps overflowing (massive ties)");
            GEPI_CUDA(run_select_compact(d_cand[cur], d_cand[cur ^ 1], d_state, d_sel, kNoAllocCap,
                                         (uint32_t)k, (int)kNoAllocCap, count, par->objective,
                                         lp_margin, num_sms, stream));
            cur ^= 1;
            GEPI_CUDA(cudaMemcpy(&st, d_state, sizeof st, cudaMemcpyDeviceToHost));
            count = st.count;
            batch = std::max<size_t>(1, nbt / 2);
            if (par->verbose)
                std::fprintf(stderr, "gepi: candidate overflow, batch -> %zu tiles\n", batch);
            continue;
        }
        const uint32_t appended = st.count - count;
        count = st.count;
        t += nbt;
        retries = 0;
        if (count > budget && t < (size_t)ntiles) {
            GEPI_CUDA(run_select_compact(d_cand[cur], d_cand[cur ^ 1], d_state, d_sel, kNoAllocCap,
                                         (uint32_t)k, -1, 0xFFFFFFFFu, par->objective, lp_margin,
                                         num_sms, stream));
            cur ^= 1;
            GEPI_CUDA(cudaMemcpy(&st, d_state, sizeof st, cudaMemcpyDeviceToHost));
            count = st.count;
        }
        const double rate = std::max(1.0, (double)appended) / (double)nbt;
        const double room = (double)budget - (double)count;
        double nb_next = room > 0 ? room / rate : 1.0;
        nb_next = std::min(nb_next, 8.0 * (double)nbt);
        batch = (size_t)std::max(1.0, nb_next);
    }
    if (count > (uint32_t)k) {
        GEPI_CUDA(run_select_compact(d_cand[cur], d_cand[cur ^ 1], d_state, d_sel, kNoAllocCap,
                                     (uint32_t)k, -1, 0xFFFFFFFFu, par->objective, lp_margin,
                                     num_sms, stream));
        cur ^= 1;
    }
    na_rank_kernel<<<num_sms, 256, 0, stream>>>(d_cand[cur], d_state, k, d_out);
    GEPI_CUDA(cudaGetLastError());
    GEPI_CUDA(cudaMemcpy(tops, d_out, (size_t)k * sizeof(gepi_result), cudaMemcpyDeviceToHost));
    return GEPI_OK;
}
