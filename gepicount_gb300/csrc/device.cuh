// Device-side shared definitions: plane layout, scan state, candidate records
// and the fused scoring epilogue used by every counting kernel.
//
// Genotype planes (HBM, uint32 words): for .bim SNP s and plane p
//   p = 0 : carriers of the .bim column-5 allele (reference allele row 2s)
//   p = 1 : carriers of the .bim column-6 allele (reference allele row 2s+1)
//   p = 2 : valid (non-missing) call
// row (3s + p), words [0, W0) hold class-0 samples (phenotype 1) in file order,
// words [W0, W0+W1) class-1 samples (phenotype 2); each class is zero-padded
// to a multiple of 256 samples.  Row pitch Wp = W0 + W1 words (32 B multiple).
//
// For SNP pair (s, t) and class c the kernels produce the 9 Gram counts
// G[p*3+q] = popcount(plane_p(s) & plane_q(t)) over class-c words.  For allele
// rows rA = 2s+i, rB = 2t+j (bits a, b) the 2x2 table of the reference's
// binFunc (proc_gold.h:38-71) follows exactly:
//   n11 = G[i][j]; n10 = G[i][2]-n11; n01 = G[2][j]-n11;
//   n00 = G[2][2]-G[i][2]-G[2][j]+n11
//   on(AND)=n11, on(NAND ~a&b)=n01, on(ANDN a&~b)=n10, on(NANDN)=n00,
//   on(XOR)=n10+n01, valid = G[2][2].
#pragma once

#include <cstdint>

namespace gepi {

constexpr int kNumFuncs = 5;
constexpr int kClassPadSamples = 256;  // class blocks: whole 16-byte TMA steps and K = 64 MMAs

// Candidate record appended by the epilogue (32 bytes).
struct __align__(16) Cand {
    unsigned long long key;  // order-preserving image of the objective (larger = better)
    int32_t rA;              // allele row A (larger)
    int32_t rBfun;           // allele row B * 8 + function
    int32_t n[4];            // w, x, y, z
};
static_assert(sizeof(Cand) == 32, "Cand layout");

// Mutable scan state shared by the kernels of one scan (device memory).
struct ScanState {
    unsigned long long tau_key;  // append tests with key >= tau_key
    float theta;                 // entropy bound threshold (see score_tests)
    float lp_thr;                // Fisher bound: reject when log P(obs) > lp_thr (nats)
    uint32_t count;              // appended candidates (may exceed cap)
    uint32_t overflow;           // set when count went past cap
    float tau_f;                 // entropy: tau as mutual information in bits, rounded down
    int kerr;                    // non-zero: a counting kernel gave up a bounded wait
    double tau_val;              // tau as a value (I bits or -log10 p); -inf: none yet
    uint32_t sel_mode;           // batched engine: select run after the last batch
                                 // (0 none, 1 threshold select, 2 overflow retry)
    uint32_t count_batch;        // batched engine: count after the last batch, before its select
};

struct SelState;

// One request's select in a batched engine step (device memory; select.cu).
struct SelJob {
    Cand *in, *out;         // candidate buffer filled by the batch, and the other one
    ScanState *st;
    SelState *sel;          // radix-select scratch of the request
    uint32_t cap, k;
    uint32_t trigger;       // not the last batch: select when count > trigger
    uint32_t count_before;  // candidates before the batch (overflow: compaction limit)
    int32_t final_batch;    // the request's last batch: select when count > k
    int32_t objective;
    float lp_margin;
    int32_t active;         // 0: no batch this step
};

// A pending list of Fisher tests (device memory): entries {rA, rB * 8 + f,
// w | x << 16, y | z << 16}, the fill counter (may exceed cap), and -- in a
// list shared by a batched engine step's requests -- each entry's request.
struct PendList {
    uint4 *ent;
    uint32_t *tag;  // null for a single scan
    uint32_t n;
    uint32_t cap;
};

struct ScanCtx {
    const uint64_t *T;   // fixed-point n*log2(n) table, n in [0, Smax]
    int F;               // its fraction bits
    const double *lf;    // log(n!) table (Fisher exact path)
    const float *lf32;   // log(n!) as float (Fisher bound)
    int objective;       // 0 entropy, 1 Fisher
    int fisher_fp64;     // nonzero: Fisher tail walks in FP64 at every sample count
    // Fisher tests that passed the bounds are left in this list for a launch
    // across the GPU to evaluate after the counting launch; null: evaluated
    // inside the counting kernel.  pend_req: this request's tag in a list
    // shared by the requests of a batched engine step (its ReqDesc index).
    PendList *pend;
    uint32_t pend_req;
    Cand *cand;
    uint32_t cap;
    ScanState *st;
};

// ---- batched engine: one counting launch over the tiles of many requests ----

// A request of an engine step (device memory).
struct ReqDesc {
    const uint32_t *planes;  // plane layout (popcount kernels)
    const uint32_t *blk;     // block-major operand copy (tensor-core kernel)
    const int2 *tiles;       // the request's tile list
    int Wp, W0, rows_pad, n_snps;
    int a0, a1, b0, b1;      // SNP ranges
    ScanCtx ctx;             // tables, this step's candidate buffer, scan state
};
// A run of consecutive tiles of one request in a launch's work list.
struct WorkRange {
    int req;    // ReqDesc index
    int first;  // first tile, as an index into the request's tile list
    int start;  // position of the run's first tile in the work list
    int count;
};
// One launch's work list; CTAs claim indices with `next` (zeroed every step).
struct WorkQueue {
    unsigned int next;
    int ntiles;  // tiles in the list
    int nranges;
    int err;     // non-zero: the launch gave up a bounded wait
    const WorkRange *ranges;
};

#ifdef __CUDACC__
// Claimed work index t -> (request, A tile, B tile); (-1, 0, 0) past the end.
__device__ __forceinline__ int4 resolve_work(const ReqDesc *reqs, const WorkQueue *q, int t) {
    if (t >= q->ntiles) return make_int4(-1, 0, 0, 0);
    const WorkRange *rg = q->ranges;
    int lo = 0, hi = q->nranges - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (rg[mid].start <= t) lo = mid;
        else hi = mid - 1;
    }
    const WorkRange r = rg[lo];
    const int2 tl = reqs[r.req].tiles[r.first + (t - r.start)];
    return make_int4(r.req, tl.x, tl.y, 0);
}
#endif

// Order-preserving map double -> u64 (larger double -> larger key).
__host__ __device__ inline unsigned long long key_of(double v) {
    unsigned long long b;
#ifdef __CUDA_ARCH__
    b = (unsigned long long)__double_as_longlong(v);
#else
    __builtin_memcpy(&b, &v, 8);
#endif
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double value_of_key(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    double v;
#ifdef __CUDA_ARCH__
    v = __longlong_as_double((long long)b);
#else
    __builtin_memcpy(&v, &b, 8);
#endif
    return v;
}

#ifdef __CUDACC__

// Exact mutual information (bits) from the fixed-point table: the integer
// numerator m*I*2^F is summed modulo 2^64 (exact, |result| < 2^62), then one
// ldexp and one IEEE division; identical on host and device.
__device__ __forceinline__ double exact_mi(const uint64_t *__restrict__ T, int F, int w, int x,
                                           int y, int z) {
    int m = y + z, xx = w + x;
    if (m == 0) return 0.0;
    uint64_t num = __ldg(T + m) + __ldg(T + w) + __ldg(T + (y - w)) + __ldg(T + x) +
                   __ldg(T + (z - x)) - __ldg(T + xx) - __ldg(T + (m - xx)) - __ldg(T + y) -
                   __ldg(T + z);
    return scalbn((double)(long long)num, -F) / (double)m;
}

// Float-float values hi + lo (|lo| <= ulp(hi) / 2) and the error-free
// transformations they are built from: Dekker's product (1971, with a fused
// multiply-add) and Knuth's sum (TAOCP vol. 2, 4.2.2).  About 46 significant
// bits.  The explicit _rn intrinsics keep the compiler from contracting the
// steps whose rounding errors are being captured.
struct FFloat {
    float hi, lo;
};

__device__ __forceinline__ FFloat ff_fast_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ FFloat ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), v = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}

__device__ __forceinline__ FFloat ff_two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

// a + b for a, b >= 0 (no cancellation to guard against)
__device__ __forceinline__ FFloat ff_add(FFloat a, FFloat b) {
    const FFloat s = ff_two_sum(a.hi, b.hi);
    return ff_fast_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ FFloat ff_mul(FFloat a, FFloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return ff_fast_sum(p, e);
}

// a / b: a first quotient q1, the remainder a - q1 b (a.hi - q1 b.hi is exact
// by Sterbenz's lemma, q1 b.hi being within a few ulps of a.hi), and the
// remainder's quotient as the correction.
__device__ __forceinline__ FFloat ff_div(FFloat a, FFloat b) {
    const float rb = __fdividef(1.f, b.hi);
    const float q1 = __fmul_rn(a.hi, rb);
    const FFloat p = ff_two_prod(q1, b.hi);
    float r = __fsub_rn(a.hi, p.hi);
    r = __fadd_rn(r, __fsub_rn(a.lo, p.lo));
    r = __fmaf_rn(-q1, b.lo, r);
    return ff_fast_sum(q1, __fmul_rn(r, rb));
}

__device__ __forceinline__ FFloat ff_of(double v) {
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}

// The end of a tail walk, once its terms add < 1e-9 of the sum S: continued
// in FP32 until a term adds < 1e-17 of the sum; returns the terms' sum.  The
// hypergeometric is log-concave, so what is left is at most 1e-9 r / (1 - r)
// of S (r the term ratio there, falling further out), and FP32's relative
// error on it -- about 1e-4 even over thousands of terms -- moves the sum by
// far less than the 1e-9 relative the p-values are held to.
template <class Ratio>
__device__ inline float fisher_walk_tail(double S, float t, int x, int dir, int x_end,
                                         Ratio ratio) {
    float St = 0.f;
    const float stop = (float)(1e-17 * S);
    while (x != x_end) {
        const int4 f = ratio(x);
        x += dir;
        t *= __fdividef((float)f.x * (float)f.y, (float)f.z * (float)f.w);
        St += t;
        if (t < stop) break;
    }
    return St;
}

// The sum of a tail walk, t_{j+1} = t_j * (f.x f.y) / (f.z f.w) with
// f = ratio(x), x stepping by `dir` from x0 until x reaches x_end: S0 plus
// every term, stopping once a term adds < 1e-17 of the sum.  While the terms
// add >= 1e-9 of the sum they are walked in float-float: the factors are
// counts below 2^24, exact in FP32, so each ratio's numerator and denominator
// are exact two-products; ratio, term and sum carry ~46 bits (CPU emulation
// against exact rational sums, N up to 10^6: <= 3e-13 relative).  The FP64
// pipe of this GPU issues at 1/64 of the FP32 rate, which makes these ~50
// FP32 operations per term cheaper than the ~12 FP64 ones they replace.
template <class Ratio>
__device__ inline double fisher_walk_ff(double S0, double t0, int x, int dir, int x_end,
                                        Ratio ratio) {
    FFloat S = ff_of(S0), t = ff_of(t0);
    bool low = false;
    while (x != x_end) {
        const int4 f = ratio(x);
        x += dir;
        const FFloat n = ff_two_prod((float)f.x, (float)f.y);
        const FFloat d = ff_two_prod((float)f.z, (float)f.w);
        t = ff_mul(t, ff_div(n, d));
        S = ff_add(S, t);
        if (t.hi < 1e-9f * S.hi) {
            low = true;
            break;
        }
    }
    const double Sd = (double)S.hi + (double)S.lo;
    return low ? Sd + (double)fisher_walk_tail(Sd, t.hi, x, dir, x_end, ratio) : Sd;
}

// The same sum in FP64, for counts of 2^24 and more.  No division per term:
// the terms and their sum are kept over one common denominator (tn / td,
// sn / td), folded back every 16 terms (two divisions); each numerator or
// denominator factor is a product of two counts below 2^31, so 16 of them stay
// below 2^1024.
template <class Ratio>
__device__ inline double fisher_walk_fp64(double S0, double t0, int x, int dir, int x_end,
                                          Ratio ratio) {
    double S = S0, tn = t0, td = 1.0, sn = 0.0;
    bool low = false;
    for (int j = 1; x != x_end; ++j) {
        const int4 f = ratio(x);
        x += dir;
        tn *= (double)f.x * (double)f.y;
        const double d = (double)f.z * (double)f.w;
        td *= d;
        sn = fma(sn, d, tn);
        const double tot = fma(S, td, sn);
        if (tn < 1e-9 * tot) {
            low = true;
            break;
        }
        if ((j & 15) == 0) {
            S += sn / td;
            tn /= td;
            sn = 0.0;
            td = 1.0;
        }
    }
    S += sn / td;
    return low ? S + (double)fisher_walk_tail(S, (float)(tn / td), x, dir, x_end, ratio) : S;
}

// ln P(obs) of the table (n11 n12 / n21 n22) under the hypergeometric with
// its margins, from the log-factorial table; K receives the margins' part,
// ln P(x) = K - lf[x] - lf[r1 - x] - lf[c1 - x] - lf[r2 - c1 + x].
__device__ __forceinline__ double fisher_lpo(const double *__restrict__ lf, int n11, int n12,
                                             int n21, int n22, double &K) {
    const int r1 = n11 + n21, r2 = n12 + n22, c1 = n11 + n12, N = r1 + r2;
    K = __ldg(lf + r1) + __ldg(lf + r2) + __ldg(lf + c1) + __ldg(lf + (N - c1)) - __ldg(lf + N);
    return K - __ldg(lf + n11) - __ldg(lf + n21) - __ldg(lf + n12) - __ldg(lf + n22);
}

// Two-sided Fisher exact test for the table (n11 n12 / n21 n22), natural-log
// p-value, given K and lpo = ln P(obs) from fisher_lpo: the quantity the
// reference's fisher_pval_d (src/kernels/fisher_d.cu:249-311) and host
// fisher_pval (src/misc/fisher_p.c:52-76) compute, here in log space and in
// FP64 throughout.  Terms with P(x) <= P(obs) * (1 + 1e-7) are summed (R's
// rule; the reference compares log d(x) <= log d(obs) strictly, fisher_p.c:72,
// so the two differ only on mathematically tied terms).  The hypergeometric is
// log-concave, so the tail beyond xo (away from the mode) is walked with the
// term ratio, a possible plateau between xo and the mode is walked term by
// term, and the first qualifying term past the mode is found by bisection
// before that tail is walked.  Walks stop once a term adds < 1e-17 of the sum.
//
// FP64 issues at 1/64 of the FP32 rate on this GPU, so the search on the far
// side runs in FP32 first: g32(x), ln P(x) - ln lim from the float table
// lf32, is within E = 2e-6 lf32[N] + 1e-6 of the exact value (each table
// entry within half an ulp of lf[N], five terms, four roundings of sums below
// 4 lf[N]: under 1.5e-6 lf[N] in all).  Where g32 > E a term certainly fails
// the rule and where g32 < -E it certainly passes, so two FP32 bisections
// bracket the first qualifying term, and the FP64 bisection that decides it
// runs only inside the bracket (usually one to three terms wide).  The
// plateau's first step is likewise decided in FP32 when the ratio is clearly
// above 1 + 1e-7.  The terms summed, and the FP64 values deciding them, are
// those of the plain FP64 search.
__device__ inline double fisher_lnp(const double *__restrict__ lf, const float *__restrict__ lf32,
                                    int n11, int n12, int n21, int n22, double K, double lpo,
                                    bool fp64_walks = false) {
    const int r1 = n11 + n21;  // column-1 total
    const int r2 = n12 + n22;  // column-2 total
    const int c1 = n11 + n12;  // row-1 total
    const int N = r1 + r2;
    const int lo = c1 <= r2 ? 0 : c1 - r2;
    const int hi = c1 < r1 ? c1 : r1;
    if (lo >= hi) return 0.0;
    auto lpx = [&](int x) {
        return K - __ldg(lf + x) - __ldg(lf + (r1 - x)) - __ldg(lf + (c1 - x)) -
               __ldg(lf + (r2 - c1 + x));
    };
    // P(x+1)/P(x) and P(x-1)/P(x) as (f.x f.y) / (f.z f.w), f four counts
    auto up4 = [&](int x) { return make_int4(r1 - x, c1 - x, x + 1, r2 - c1 + x + 1); };
    auto down4 = [&](int x) { return make_int4(x, r2 - c1 + x, r1 - x + 1, c1 - x + 1); };
    auto ratio64 = [](int4 f) {
        return ((double)f.x * (double)f.y) / ((double)f.z * (double)f.w);
    };
    // the FP32 ratio is within 4 ulps: above 1 + 1e-6 the FP64 one is above 1 + 1e-7
    auto clearly_rising = [](int4 f) {
        return ((float)f.x * (float)f.y) / ((float)f.z * (float)f.w) > 1.000001f;
    };
    const bool ff = !fp64_walks && N < (1 << 24);
    auto walk = [&](double S0, double t0, int x0, int dir, int x_end, auto ratio) {
        return ff ? fisher_walk_ff(S0, t0, x0, dir, x_end, ratio)
                  : fisher_walk_fp64(S0, t0, x0, dir, x_end, ratio);
    };
    const double tol = 1.0 + 1e-7;
    const int xo = n11;
    const double lim = lpo + 9.99999950000003e-08;  // log1p(1e-7)
    int xm = (int)(((long long)(r1 + 1) * (long long)(c1 + 1)) / (long long)(N + 2));
    if (xm < lo) xm = lo;
    if (xm > hi) xm = hi;
    const float E = 2e-6f * __ldg(lf32 + N) + 1e-6f;
    const float gc = (float)(K - lim);
    auto g32 = [&](int x) {
        return gc - __ldg(lf32 + x) - __ldg(lf32 + (r1 - x)) - __ldg(lf32 + (c1 - x)) -
               __ldg(lf32 + (r2 - c1 + x));
    };
    auto passes = [&](int x) {  // lpx(x) <= lim, in FP32 where the margin decides it
        const float g = g32(x);
        return g < -E ? true : g > E ? false : lpx(x) <= lim;
    };
    double S = 1.0;
    if (xo <= xm) {
        // near tail: x < xo
        S = walk(S, 1.0, xo, -1, lo, down4);
        // plateau between xo and the mode
        if (xo < xm && !clearly_rising(up4(xo))) {
            double t = 1.0;
            for (int x = xo; x < xm;) {
                double t2 = t * ratio64(up4(x));
                if (t2 > tol) break;
                ++x;
                t = t2;
                S += t;
            }
        }
        // falling side x in [xm+1, hi]: first x with lpx(x) <= lim
        const int a = xm + 1, b = hi;
        if (a <= b && passes(b)) {
            int l = a, h = b;  // first x with g32 <= E: no x before it passes
            while (l < h) {
                const int mid = (l + h) >> 1;
                if (g32(mid) <= E) h = mid; else l = mid + 1;
            }
            const int t0 = l;
            h = b;  // first x with g32 < -E (or b): it passes
            while (l < h) {
                const int mid = (l + h) >> 1;
                if (g32(mid) < -E) h = mid; else l = mid + 1;
            }
            l = t0;
            while (l < h) {
                const int mid = (l + h) >> 1;
                if (lpx(mid) <= lim) h = mid; else l = mid + 1;
            }
            const double u = exp(lpx(l) - lpo);
            S = walk(S + u, u, l, +1, hi, up4);
        }
    } else {
        // near tail: x > xo
        S = walk(S, 1.0, xo, +1, hi, up4);
        if (!clearly_rising(down4(xo))) {
            double t = 1.0;
            for (int x = xo; x > xm;) {
                double t2 = t * ratio64(down4(x));
                if (t2 > tol) break;
                --x;
                t = t2;
                S += t;
            }
        }
        // falling side x in [lo, xm-1]: last x with lpx(x) <= lim
        const int a = lo, b = xm - 1;
        if (a <= b && passes(a)) {
            int l = a, h = b;  // last x with g32 <= E: no x after it passes
            while (l < h) {
                const int mid = (l + h + 1) >> 1;
                if (g32(mid) <= E) l = mid; else h = mid - 1;
            }
            const int t0 = h;
            l = a;  // last x with g32 < -E (or a): it passes
            while (l < h) {
                const int mid = (l + h + 1) >> 1;
                if (g32(mid) < -E) l = mid; else h = mid - 1;
            }
            h = t0;
            while (l < h) {
                const int mid = (l + h + 1) >> 1;
                if (lpx(mid) <= lim) l = mid; else h = mid - 1;
            }
            const double u = exp(lpx(l) - lpo);
            S = walk(S + u, u, l, -1, lo, down4);
        }
    }
    double lnp = lpo + log(S);
    return lnp > 0.0 ? 0.0 : lnp;
}

// A lower bound on the p of fisher_lnp, against a threshold: true when the
// observed term and up to 8 terms beyond it on its own side of the mode --
// each at most P(obs), the hypergeometric being unimodal, so each is in the
// sum -- already show ln p > ln_thr.  Such a test cannot reach the ranking,
// and the exact tail sums it would cost are skipped.  lpo = ln P(obs) from
// fisher_lpo.  The terms are walked with the term ratio in FP32 and only
// counted while below 1 - 1e-5 of P(obs); the sum is taken 1e-5 low and its
// log 1e-5 low, and the comparison keeps a margin of 1e-7 + 1e-10 |ln_thr|
// nats, far above the rounding of fisher_lnp, so the tests it drops are tests
// the exact evaluation drops.
__device__ inline bool fisher_above(int n11, int n12, int n21, int n22, double lpo,
                                    double ln_thr) {
    if (!(ln_thr < 0.0)) return false;  // no threshold yet
    const int r1 = n11 + n21, r2 = n12 + n22, c1 = n11 + n12;
    const int lo = c1 <= r2 ? 0 : c1 - r2;
    const int hi = c1 < r1 ? c1 : r1;
    if (lo >= hi) return false;
    const double margin = 1e-7 + 1e-10 * -ln_thr;
    const double d = ln_thr + margin - lpo;  // reject when ln(sum of the terms) > d
    if (d > 2.25) return false;              // 9 terms sum to at most 9 < e^2.25
    auto up = [&](int x) {
        return ((float)(r1 - x) * (float)(c1 - x)) / ((float)(x + 1) * (float)(r2 - c1 + x + 1));
    };
    auto down = [&](int x) {
        return ((float)x * (float)(r2 - c1 + x)) / ((float)(r1 - x + 1) * (float)(c1 - x + 1));
    };
    float S = 1.f, t = 1.f;
    const bool toward_hi = n11 < hi && up(n11) < 1.f;
    int x = n11;
#pragma unroll 1
    for (int j = 0; j < 8; ++j) {
        if (toward_hi ? x >= hi : x <= lo) break;
        t *= toward_hi ? up(x) : down(x);
        if (!(t < 1.f - 1e-5f)) break;  // not below P(obs): the mode's side
        S += t;
        x += toward_hi ? 1 : -1;
    }
    return (double)__logf(S * (1.f - 1e-5f)) - 1e-5 > d;
}

__device__ __forceinline__ void append_candidate(const ScanCtx &ctx, double value, int rA,
                                                 int rB, int fun, int w, int x, int y, int z) {
    unsigned long long key = key_of(value);
    if (key < ctx.st->tau_key) return;
    // One atomic per group of lanes appending together: in a scan's first
    // batch, with no threshold yet, every test of a tile is appended, and one
    // atomic per test on the one counter would serialise them.  The lanes are
    // grouped by their scan state: a batched engine step's pending list mixes
    // requests within a warp.
    const unsigned grp =
        __match_any_sync(__activemask(), (unsigned long long)(uintptr_t)ctx.st);
    unsigned lane;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    const int leader = __ffs(grp) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&ctx.st->count, (uint32_t)__popc(grp));
    base = __shfl_sync(grp, base, leader);
    const uint32_t idx = base + (uint32_t)__popc(grp & ((1u << lane) - 1u));
    if (idx >= ctx.cap) {
        ctx.st->overflow = 1u;
        return;
    }
    Cand c;
    c.key = key;
    c.rA = rA;
    c.rBfun = rB * 8 + fun;
    c.n[0] = w;
    c.n[1] = x;
    c.n[2] = y;
    c.n[3] = z;
    ctx.cand[idx] = c;
}

// Exact evaluation of one test that passed the bounds; appends if it ranks.
// Entropy rejects with one FP64 multiply against tau before the division.
static __device__ __noinline__ void exact_test(const ScanCtx &ctx, int rA, int rB, int fun, int w,
                                        int x, int y, int z) {
    long long d = (long long)w * z - (long long)x * y;
    if (d == 0) return;
    double value;
    if (ctx.objective == 0) {
        const int m = y + z, xx = w + x;
        const uint64_t *T = ctx.T;
        const uint64_t num = __ldg(T + m) + __ldg(T + w) + __ldg(T + (y - w)) + __ldg(T + x) +
                             __ldg(T + (z - x)) - __ldg(T + xx) - __ldg(T + (m - xx)) -
                             __ldg(T + y) - __ldg(T + z);
        const double lhs = (double)(long long)num;
        // num * 2^-F / m >= tau  <=>  num >= tau * m * 2^F (checked with 1e-12 slack)
        if (lhs < ctx.st->tau_val * (double)m * scalbn(1.0, ctx.F) * (1.0 - 1e-12)) return;
        value = scalbn(lhs, -ctx.F) / (double)m;
    } else {
        // print order (w, y-w, x, z-x); value = -log10 p, appended when
        // value >= tau_val, i.e. ln p <= -tau_val ln 10
        double K;
        const double lpo = fisher_lpo(ctx.lf, w, y - w, x, z - x, K);
        if (fisher_above(w, y - w, x, z - x, lpo, -ctx.st->tau_val * 2.302585092994045684))
            return;
        value = -fisher_lnp(ctx.lf, ctx.lf32, w, y - w, x, z - x, K, lpo, ctx.fisher_fp64) *
                0.43429448190325182765;
    }
    append_candidate(ctx, value, rA, rB, fun, w, x, y, z);
}

// n * log2(n) in FP32 (0 for n <= 1).
__device__ __forceinline__ float tlog2f(float n) { return n > 1.f ? n * __log2f(n) : 0.f; }

// Row-pair bounds of an SNP pair: bit 2i+j set when row pair (2s+i, 2t+j) may
// hold a test that passes stage 1.  Every function tested for a row pair is a
// function of the cell (bit of row 2s+i, bit of row 2t+j), so its phi^2 is at
// most the class x cell table's chi^2 / m = sum_k D_k^2 / (c_k y z m), with
// D_k = a_k z - b_k y over the four cells (data processing for the chi^2
// divergence).  Entropy: below theta no test of the row pair passes.  Fisher:
// with C(n, k) >= 2^(n H(k/n)) / sqrt(2n) and C(m, k) <= 2^(m H(k/m))
// (MacWilliams and Sloane), P(obs) >= 2^(-m I) / (2 sqrt(y z)), and I <= ln(1 +
// phi^2) nats, so ln P(obs) >= -m ln(1 + chi^2/m) - ln(4 y z) / 2; above
// lp_thr no test passes.  |D_k| carries a rounding margin (below), the sum a
// 2^-18 margin for the approximate reciprocals, the Fisher bound a margin of
// 1e-4 relative plus 0.01.  A class without valid samples leaves every test
// with w z = x y, which is never ranked.  On the diagonal row 2t+j must be <=
// row 2s+i, which drops (i, j) = (0, 1), bit 1.
__device__ __forceinline__ uint32_t rowpair_bounds(const float *G0, const float *G1, bool diag,
                                                   int objective, float theta, float lp_thr) {
    const float y = G0[8], z = G1[8], yz = y * z, m = y + z, yzm = yz * m;
    if (!(yz > 0.f)) return 0u;
    const float lfix = objective == 0 ? 0.f : 0.5f * logf(4.f * yz);
    // The four row-pair tables share their margins: with R_i = a_i2 z - b_i2 y
    // (row 2s+i carriers) and C_j = a_2j z - b_2j y (row 2t+j carriers), the
    // cells give D_11 = a_ij z - b_ij y, D_10 = R_i - D_11, D_01 = C_j - D_11
    // and D_00 = D_11 - R_i - C_j (the D_k sum to 0).  Every D_k is then within
    // y z 2^-19 of its exact value (each product is at most y z, and at most
    // four rounded terms enter), the margin E added to |D_k|.
    const float E = yz * 1.9073486328125e-06f;  // 2^-19
    const float2 zz = make_float2(z, z), nyy = make_float2(-y, -y), neg1 = make_float2(-1.f, -1.f);
    // (R_0, R_1), (RT_0, RT_1), (C_0, C_1), (CT_0, CT_1) in packed FP32x2
    // instructions (rounded per component as the scalar ones are)
    const float2 aR = make_float2(G0[2], G0[5]), bR = make_float2(G1[2], G1[5]);
    const float2 aC = make_float2(G0[6], G0[7]), bC = make_float2(G1[6], G1[7]);
    const float2 R2 = __ffma2_rn(bR, nyy, __fmul2_rn(aR, zz)), RT2 = __fadd2_rn(aR, bR);
    const float2 Cj = __ffma2_rn(bC, nyy, __fmul2_rn(aC, zz)), CTj = __fadd2_rn(aC, bC);
    const float R[2] = {R2.x, R2.y}, RT[2] = {RT2.x, RT2.y};
    // S = sum_k t_k^2 / c_k is compared in product form, sum_k t_k^2 P_k with
    // P_k the product of the other three c_l (c_l clamped to 1), against
    // theta y z m prod c_l: no reciprocals.  Every quantity is positive; each
    // side carries at most seven float roundings (products below 2^128: t_k^2
    // <= (y z)^2, prod c_l <= (m / 4)^4), so a 1 + 2^-18 factor on the sum keeps
    // the comparison conservative.
    //
    // The row pairs (2s+i, 2t) and (2s+i, 2t+1) are computed side by side in
    // the halves of packed FP32x2 instructions (FFMA2 / FADD2 / FMUL2, rounded
    // per component as the scalar instructions are), in the same operations
    // and order as one row pair alone: half the issue slots for the bulk of
    // the bound, which the scoring warps share with the producers.
    const float th = theta * yzm;
    const float2 nCj = __fmul2_rn(Cj, neg1), nCTj = __fmul2_rn(CTj, neg1);
    const float2 slack = make_float2(1.0000038146972656f, 1.0000038146972656f);  // 1 + 2^-18
    const float2 thh = make_float2(th, th);
    uint32_t ok = 0;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float2 a11 = make_float2(G0[i * 3], G0[i * 3 + 1]);
        const float2 b11 = make_float2(G1[i * 3], G1[i * 3 + 1]);
        const float2 Ri = make_float2(R[i], R[i]), nRi = make_float2(-R[i], -R[i]);
        const float2 RTi = make_float2(RT[i], RT[i]);
        const float mr = m - RT[i];
        const float2 mri = make_float2(mr, mr);
        const float2 D11 = __ffma2_rn(b11, nyy, __fmul2_rn(a11, zz));  // a11 z - b11 y
        const float2 c11 = __fadd2_rn(a11, b11);
        float2 D[4];
        D[0] = D11;
        D[1] = __ffma2_rn(D11, neg1, Ri);                 // R_i - D11
        D[2] = __ffma2_rn(D11, neg1, Cj);                 // C_j - D11
        D[3] = __fadd2_rn(__fadd2_rn(D11, nRi), nCj);     // D11 - R_i - C_j
        const float2 u1 = __ffma2_rn(c11, neg1, RTi);     // RT_i - c11
        const float2 u2 = __ffma2_rn(c11, neg1, CTj);     // CT_j - c11
        const float2 u3 = __fadd2_rn(__fadd2_rn(mri, nCTj), c11);  // m - RT_i - CT_j + c11
        const float2 c0 = make_float2(fmaxf(c11.x, 1.f), fmaxf(c11.y, 1.f));
        const float2 c1 = make_float2(fmaxf(u1.x, 1.f), fmaxf(u1.y, 1.f));
        const float2 c2 = make_float2(fmaxf(u2.x, 1.f), fmaxf(u2.y, 1.f));
        const float2 c3 = make_float2(fmaxf(u3.x, 1.f), fmaxf(u3.y, 1.f));
        const float2 c01 = __fmul2_rn(c0, c1), c23 = __fmul2_rn(c2, c3);
        const float2 P[4] = {__fmul2_rn(c1, c23), __fmul2_rn(c0, c23), __fmul2_rn(c3, c01),
                             __fmul2_rn(c2, c01)};
        float2 S = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 t = make_float2(fabsf(D[k].x) + E, fabsf(D[k].y) + E);
            S = __ffma2_rn(__fmul2_rn(t, t), P[k], S);
        }
        S = __fmul2_rn(S, slack);
        const float2 pc = __fmul2_rn(c01, c23);
        bool pass0, pass1;
        if (objective == 0) {
            const float2 tp = __fmul2_rn(thh, pc);
            pass0 = S.x >= tp.x;
            pass1 = S.y >= tp.y;
        } else {
            // chi^2 itself (one division, its error inside the same factor)
            const float lo0 = -m * log1pf(__fdividef(S.x, pc.x) / yzm) - lfix;
            const float lo1 = -m * log1pf(__fdividef(S.y, pc.y) / yzm) - lfix;
            pass0 = lo0 - (1e-4f * fabsf(lo0) + 1e-2f) <= lp_thr;
            pass1 = lo1 - (1e-4f * fabsf(lo1) + 1e-2f) <= lp_thr;
        }
        ok |= ((uint32_t)pass0 | ((uint32_t)pass1 << 1)) << (2 * i);
    }
    return ok & (diag ? 0xDu : 0xFu);
}

// Scores every test of SNP pair (s >= t) from the Gram counts of both classes
// (G0 class 0, G1 class 1; float holding exact integers).  Row pairs (2s+i,
// 2t+j) with 2t+j <= 2s+i, 5 functions each.
//
// Bound (entropy): I(F;C) <= log2(1 + phi^2), phi^2 = D^2 / Q with
// D = w z - x y and Q = (w+x)(m-w-x) y z, since KL <= log(1 + chi^2).  A test
// is dropped when (|D| + e)^2 < theta * Q, theta = (2^tau - 1)(1 - 2^-10) and e
// bounding the float rounding of D.
// Bound (Fisher): p >= P(obs); dropped when log P(obs) > lp_thr.
// Entropy survivors then meet an FP32 estimate of m*I with an error margin,
// and only tests within that margin of tau reach the exact integer key.
__device__ __forceinline__ void score_tests(const ScanCtx &ctx, const float *G0,
                                            const float *G1, int s, int t, float theta,
                                            float lp_thr, uint32_t *fq, int fq_cap) {
    const float y = G0[8], z = G1[8];
    const float m = y + z;
    const float yz = y * z;
    const bool diag = (s == t);
    // row pairs that may hold a passing test (almost always none)
    const uint32_t rp = rowpair_bounds(G0, G1, diag, ctx.objective, theta, lp_thr);
    if (!rp) return;
    // Pair-level terms of the FP32 entropy estimate (stage 2), made on demand.
    float Tm = -1.f, Ty = 0.f, Tz = 0.f;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (!((rp >> (2 * i + j)) & 1u)) continue;  // includes row 2t+j > row 2s+i
            float on0[5], on1[5];
            {
                float n11 = G0[i * 3 + j], r = G0[i * 3 + 2], c = G0[6 + j];
                float n10 = r - n11, n01 = c - n11, n00 = y - r - c + n11;
                on0[0] = n11; on0[1] = n01; on0[2] = n10; on0[3] = n00; on0[4] = n10 + n01;
            }
            {
                float n11 = G1[i * 3 + j], r = G1[i * 3 + 2], c = G1[6 + j];
                float n10 = r - n11, n01 = c - n11, n00 = z - r - c + n11;
                on1[0] = n11; on1[1] = n01; on1[2] = n10; on1[3] = n00; on1[4] = n10 + n01;
            }
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                const float w = on0[f], x = on1[f];
                bool pass;
                if (ctx.objective == 0) {
                    const float xx = w + x;
                    const float Q = xx * (m - xx) * yz;
                    const float wz = w * z, xy = x * y;
                    const float D = fabsf(wz - xy) + (wz + xy) * 2.384185791015625e-07f;  // 2^-22
                    pass = D * D >= theta * Q;
                } else {
                    // log P(obs) = lf(r1)+lf(r2)+lf(y)+lf(z)-lf(m)-lf(w)-lf(y-w)-lf(x)-lf(z-x)
                    const int iw = (int)w, ix = (int)x, iy = (int)y, iz = (int)z;
                    const float *L = ctx.lf32;
                    float lp = __ldg(L + (iw + ix)) + __ldg(L + (iy + iz - iw - ix)) + __ldg(L + iy) +
                               __ldg(L + iz) - __ldg(L + (iy + iz)) - __ldg(L + iw) -
                               __ldg(L + (iy - iw)) - __ldg(L + ix) - __ldg(L + (iz - ix));
                    pass = lp <= lp_thr;
                }
                if (pass && ctx.objective == 0) {
                    // Stage 2: m*I in FP32 from __log2f (relative error of each
                    // n*log2(n) <= 2.5 ulp, 8 additions) with a rigorous margin;
                    // drop when estimate + margin < tau * m.
                    if (Tm < 0.f) {
                        Tm = tlog2f(m);
                        Ty = tlog2f(y);
                        Tz = tlog2f(z);
                    }
                    const float xx = w + x;
                    const float a = tlog2f(w), b = tlog2f(y - w), c = tlog2f(x), d = tlog2f(z - x);
                    const float e = tlog2f(xx), g = tlog2f(m - xx);
                    const float est = ((Tm + a) + (b + c)) + d - (e + g) - (Ty + Tz);
                    const float tm = ctx.st->tau_f * m;
                    const float mag = Tm + a + b + c + d + e + g + Ty + Tz + fabsf(tm);
                    pass = est + (2e-6f * mag + 1e-3f) >= tm;
                }
                if (!pass) continue;
                if (ctx.pend) {  // Fisher: left for the launch across the GPU after this one
                    PendList &L = *ctx.pend;
                    const uint32_t e = atomicAdd(&L.n, 1u);
                    if (e < L.cap) {
                        L.ent[e] = make_uint4((uint32_t)(2 * s + i),
                                              (uint32_t)(2 * t + j) << 3 | (uint32_t)f,
                                              (uint32_t)w | (uint32_t)x << 16,
                                              (uint32_t)y | (uint32_t)z << 16);
                        if (L.tag) L.tag[e] = ctx.pend_req;
                        continue;
                    }
                } else if (fq) {  // Fisher: queue for the CTA's threads to evaluate together
                    const uint32_t e = atomicAdd(fq, 1u);
                    if (e < (uint32_t)fq_cap) {
                        int4 *qa = reinterpret_cast<int4 *>(fq + 4);
                        reinterpret_cast<int2 *>(qa + fq_cap)[e] = make_int2((int)y, (int)z);
                        qa[e] = make_int4(2 * s + i, (2 * t + j) * 8 + f, (int)w, (int)x);
                        continue;
                    }
                }
                exact_test(ctx, 2 * s + i, 2 * t + j, f, (int)w, (int)x, (int)y, (int)z);
            }
        }
    }
}

// Out-of-line wrapper: G points at 18 floats (class 0 Gram, class 1 Gram);
// fq, when not null, the CTA's Fisher queue of fq_cap entries.
static __device__ __noinline__ void score_pair(const ScanCtx &ctx, const float *G, int s, int t,
                                        float theta, float lp_thr, uint32_t *fq, int fq_cap) {
    float G0[9], G1[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        G0[k] = G[k];
        G1[k] = G[9 + k];
    }
    score_tests(ctx, G0, G1, s, t, theta, lp_thr, fq, fq_cap);
}

#endif  // __CUDACC__

}  // namespace gepi
