/*
 * oracle.c -- TEST INFRASTRUCTURE ONLY: CPU restatement of gEpiCount's gold
 * path, the parity checker for the CUDA scan.  Never linked into the product.
 * See oracle.h for the interface; each function cites the reference code
 * (paths inside the gEpiCount project) whose behaviour it restates.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* Reader: BinPlinkReader.h:101-244 (2-bit decode), PlinkReader.h:408-440.    */
/* ------------------------------------------------------------------------- */
void orc_decode_bed(const uint8_t *bed, int n_lines, int n_samples, uint64_t *bits,
                    uint64_t *valid) {
    const int nw = (n_samples + 63) / 64;
    const size_t bps = ((size_t)n_samples + 3) / 4;
    for (int s = 0; s < n_lines; ++s) {
        const uint8_t *row = bed + 3 + (size_t)s * bps;
        uint64_t *b0 = bits + (size_t)(2 * s) * nw, *b1 = b0 + nw;
        uint64_t *v0 = valid + (size_t)(2 * s) * nw, *v1 = v0 + nw;
        memset(b0, 0, 2 * (size_t)nw * 8);
        memset(v0, 0, 2 * (size_t)nw * 8);
        for (int k = 0; k < n_samples; ++k) {
            int code = (row[k / 4] >> (2 * (k % 4))) & 3;
            uint64_t bit = 1ull << (k % 64);
            /* 0: homozygous col-5 allele, 2: heterozygous, 3: homozygous col-6,
               1: missing (BinPlinkReader.h:174-195). */
            if (code == 0 || code == 2) b0[k / 64] |= bit;
            if (code == 2 || code == 3) b1[k / 64] |= bit;
            if (code != 1) {
                v0[k / 64] |= bit;
                v1[k / 64] |= bit;
            }
        }
    }
}

void orc_class_masks(const int32_t *pheno, int n_samples, uint64_t *mask1, uint64_t *mask2) {
    const int nw = (n_samples + 63) / 64;
    memset(mask1, 0, (size_t)nw * 8);
    memset(mask2, 0, (size_t)nw * 8);
    for (int k = 0; k < n_samples; ++k) {
        uint64_t bit = 1ull << (k % 64);
        if (pheno[k] == 1) mask1[k / 64] |= bit;
        if (pheno[k] == 2) mask2[k / 64] |= bit;
    }
}

/* ------------------------------------------------------------------------- */
/* Counting: proc_gold.h:38-71, masks per proc_gold_1.h:106-112.               */
/* ------------------------------------------------------------------------- */
static inline uint64_t bfun(uint64_t a, uint64_t b, int fun) {
    switch (fun) {
    case 0: return a & b;     /* AND   */
    case 1: return ~a & b;    /* NAND  */
    case 2: return a & ~b;    /* ANDN  */
    case 3: return ~(a | b);  /* NANDN */
    case 4: return a ^ b;     /* XOR   */
    default: return 0;
    }
}

void orc_binfunc(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                 const uint64_t *mask2, int n_words, int rA, int rB, int fun, int32_t out[4]) {
    const uint64_t *a = bits + (size_t)rA * n_words, *b = bits + (size_t)rB * n_words;
    const uint64_t *va = valid + (size_t)rA * n_words, *vb = valid + (size_t)rB * n_words;
    int w = 0, x = 0, y = 0, z = 0;
    for (int j = 0; j < n_words; ++j) {
        uint64_t m0 = mask1[j] & va[j] & vb[j];
        uint64_t m1 = mask2[j] & va[j] & vb[j];
        uint64_t c = bfun(a[j], b[j], fun);
        w += __builtin_popcountll(c & m0);
        x += __builtin_popcountll(c & m1);
        y += __builtin_popcountll(m0);
        z += __builtin_popcountll(m1);
    }
    out[0] = w;
    out[1] = x;
    out[2] = y;
    out[3] = z;
}

void orc_pair_gram(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                   const uint64_t *mask2, int n_words, int s, int t, uint32_t out[18]) {
    const uint64_t *P[3], *Q[3];
    P[0] = bits + (size_t)(2 * s) * n_words;
    P[1] = bits + (size_t)(2 * s + 1) * n_words;
    P[2] = valid + (size_t)(2 * s) * n_words;
    Q[0] = bits + (size_t)(2 * t) * n_words;
    Q[1] = bits + (size_t)(2 * t + 1) * n_words;
    Q[2] = valid + (size_t)(2 * t) * n_words;
    for (int i = 0; i < 18; ++i) out[i] = 0;
    for (int j = 0; j < n_words; ++j)
        for (int p = 0; p < 3; ++p)
            for (int q = 0; q < 3; ++q) {
                uint64_t v = P[p][j] & Q[q][j];
                out[p * 3 + q] += (uint32_t)__builtin_popcountll(v & mask1[j]);
                out[9 + p * 3 + q] += (uint32_t)__builtin_popcountll(v & mask2[j]);
            }
}

/* ------------------------------------------------------------------------- */
/* Entropy: entropyDelta4, entropy_inline.h:30-80 (host branch :70-77).        */
/* ------------------------------------------------------------------------- */
float orc_entropy_ref_f32(int w, int x, int y, int z) {
    float m = (float)(y + z);
    float xx = (float)(w + x);
    float ret = 0.0f;
    if (xx > 0.0f && xx < m)
        ret += (xx / m) * log2f(xx / m) + ((m - xx) / m) * log2f((m - xx) / m);
    if (y > 0 && y > w && w > 0)
        ret -= ((float)w / m) * log2f((float)w / (float)y) +
               ((float)(y - w) / m) * log2f((float)(y - w) / (float)y);
    if (z > 0 && z > x && x > 0)
        ret -= ((float)x / m) * log2f((float)x / (float)z) +
               ((float)(z - x) / m) * log2f((float)(z - x) / (float)z);
    return ret;
}

double orc_entropy_f64(int w, int x, int y, int z) {
    double m = (double)y + (double)z;
    double xx = (double)w + (double)x;
    double ret = 0.0;
    if (xx > 0.0 && xx < m) ret += (xx / m) * log2(xx / m) + ((m - xx) / m) * log2((m - xx) / m);
    if (y > 0 && y > w && w > 0)
        ret -= ((double)w / m) * log2((double)w / y) + ((double)(y - w) / m) * log2((double)(y - w) / y);
    if (z > 0 && z > x && x > 0)
        ret -= ((double)x / m) * log2((double)x / z) + ((double)(z - x) / m) * log2((double)(z - x) / z);
    return ret;
}

/* Fixed-point T(n) = n * round(log2(n) * 2^F).  log2 is evaluated with pure
 * integer arithmetic (64 fraction bits by repeated squaring), so the table is
 * bit-identical on every host.  F is the largest value <= 52 with
 * n_max * (floor(log2 n_max) + 1) * 2^F < 2^62. */
int orc_tfix_bits(int64_t n_max) {
    if (n_max < 2) return 52;
    int e = 63 - __builtin_clzll((unsigned long long)n_max);
    int F = 52;
    while (F > 0) {
        unsigned __int128 lim = (unsigned __int128)n_max * (unsigned __int128)(e + 1);
        lim <<= F;
        if (lim < ((unsigned __int128)1 << 62)) break;
        --F;
    }
    return F;
}

static uint64_t orc_log2_fixed(uint64_t n, int F) {
    if (n <= 1) return 0;
    int e = 63 - __builtin_clzll(n);
    uint64_t x = n << (63 - e); /* Q1.63 in [1, 2) */
    uint64_t frac = 0;
    for (int i = 1; i <= 64; ++i) {
        unsigned __int128 sq = (unsigned __int128)x * x; /* Q2.126 in [1, 4) */
        if ((uint64_t)(sq >> 127)) {
            x = (uint64_t)(sq >> 64);
            frac |= 1ull << (64 - i);
        } else {
            x = (uint64_t)(sq >> 63);
        }
    }
    uint64_t r = (frac >> (64 - F)) + ((frac >> (63 - F)) & 1ull);
    return ((uint64_t)e << F) + r;
}

void orc_tfix_table(int64_t n_max, int F, uint64_t *T) {
    for (int64_t n = 0; n <= n_max; ++n) T[n] = (uint64_t)n * orc_log2_fixed((uint64_t)n, F);
}

double orc_entropy_fixed(const uint64_t *T, int F, int w, int x, int y, int z, int *nonzero) {
    int m = y + z, xx = w + x;
    int64_t d = (int64_t)w * z - (int64_t)x * y;
    if (nonzero) *nonzero = (d != 0);
    if (m == 0) return 0.0;
    uint64_t num = T[m] + T[w] + T[y - w] + T[x] + T[z - x] - T[xx] - T[m - xx] - T[y] - T[z];
    return ldexp((double)(int64_t)num, -F) / (double)m;
}

/* ------------------------------------------------------------------------- */
/* Fisher: fisher_p.c:52-245 (R / C. Loader's saddle-point dbinom_raw).        */
/* ------------------------------------------------------------------------- */
static double orc_stirl_tab[16];
static int orc_stirl_ready = 0;

/* Error of Stirling's formula: log(n!) - log(sqrt(2 pi n) (n/e)^n). */
static double orc_stirlerr(int n) {
    if (!orc_stirl_ready) {
        orc_stirl_tab[0] = 0.0; /* place holder, as the reference */
        for (int i = 1; i < 16; ++i) {
            long double ln = (long double)i;
            orc_stirl_tab[i] = (double)(lgammal(ln + 1.0L) - (ln + 0.5L) * logl(ln) + ln -
                                        0.5L * logl(2.0L * 3.14159265358979323846264338327950288L));
        }
        orc_stirl_ready = 1;
    }
    if (n <= 15) return orc_stirl_tab[n];
    const double S0 = 1.0 / 12.0, S1 = 1.0 / 360.0, S2 = 1.0 / 1260.0, S3 = 1.0 / 1680.0,
                 S4 = 1.0 / 1188.0;
    double nn = (double)n * (double)n;
    if (n > 500) return (S0 - S1 / nn) / n;
    if (n > 80) return (S0 - (S1 - S2 / nn) / nn) / n;
    if (n > 35) return (S0 - (S1 - (S2 - S3 / nn) / nn) / nn) / n;
    return (S0 - (S1 - (S2 - (S3 - S4 / nn) / nn) / nn) / nn) / n;
}

/* Deviance term x log(x/np) + np - x, series for x close to np. */
static double orc_bd0(double x, double np) {
    if (isinf(x) || isinf(np) || np == 0.0) return NAN;
    if (fabs(x - np) < 0.1 * (x + np)) {
        double v = (x - np) / (x + np);
        double s = (x - np) * v;
        double ej = 2 * x * v;
        v = v * v;
        for (int j = 1;; j++) {
            ej *= v;
            double s1 = s + ej / ((j << 1) + 1);
            if (s1 == s) return s1;
            s = s1;
        }
    }
    return x * log(x / np) + np - x;
}

static double orc_dbinom_raw_log(int x, int n, double p, double q) {
    if (p == 0) return x == 0 ? 0.0 : -INFINITY;
    if (q == 0) return x == 0 ? 0.0 : -INFINITY;
    if (x == 0) {
        if (n == 0) return 0.0;
        return (p < 0.1) ? -orc_bd0((double)n, (double)n * q) - (double)n * p : (double)n * log(q);
    }
    if (x == n) return (q < 0.1) ? -orc_bd0((double)n, (double)n * p) - (double)n * q : (double)n * log(p);
    if (x < 0 || x > n) return -INFINITY;
    double lc = orc_stirlerr(n) - orc_stirlerr(x) - orc_stirlerr(n - x) -
                orc_bd0((double)x, (double)n * p) - orc_bd0((double)(n - x), (double)n * q);
    double lf = log(2.0 * 3.14159265358979323846) + log((double)x) + log1p(-(double)x / (double)n);
    return lc - 0.5 * lf;
}

static double orc_dhyper_log(int x, int r, int b, int n) {
    if (n < x || r < x || n - x > b) return -INFINITY;
    if (n == 0) return x == 0 ? 0.0 : -INFINITY;
    double p = (double)n / (double)(r + b);
    double q = (double)(r + b - n) / (double)(r + b);
    return orc_dbinom_raw_log(x, r, p, q) + orc_dbinom_raw_log(n - x, b, p, q) -
           orc_dbinom_raw_log(n, r + b, p, q);
}

double orc_fisher_log10p(int n11, int n12, int n21, int n22, int strict) {
    if (n11 < 0 || n12 < 0 || n21 < 0 || n22 < 0) return NAN;
    int m = n11 + n21, n = n12 + n22, o = n11 + n12;
    int lo = o <= n ? 0 : o - n;
    int hi = o < m ? o : m;
    double dthr = orc_dhyper_log(n11, m, n, o);
    double lim = strict ? dthr : dthr + log1p(1e-7);
    double dsumd = 0.0, dsumn = 0.0;
    for (int j = lo; j <= hi; ++j) {
        double daux = orc_dhyper_log(j, m, n, o);
        double e = exp(daux);
        dsumd += e;
        if (daux <= lim) dsumn += e;
    }
    return log10(dsumn) - log10(dsumd);
}

/* log of the observed table's hypergeometric probability, for pruning. */
static double orc_fisher_lpobs(int n11, int n12, int n21, int n22) {
    return orc_dhyper_log(n11, n11 + n21, n12 + n22, n11 + n12);
}

/* ------------------------------------------------------------------------- */
/* Gold scan with an exact, deterministic top-k (replaces the 2*topmost buffer */
/* and thrust::sort of proc_gold_1.h:114-137,167-172).                         */
/* ------------------------------------------------------------------------- */
typedef struct {
    double key; /* larger = better: I bits, or -log10 p */
    int32_t sA, sB, fun;
    int32_t n[4];
} orc_item;

static inline int orc_better(const orc_item *a, const orc_item *b) {
    if (a->key != b->key) return a->key > b->key;
    if (a->sA != b->sA) return a->sA < b->sA;
    if (a->sB != b->sB) return a->sB < b->sB;
    return a->fun < b->fun;
}

/* Min-heap on "better": root is the worst item kept. */
typedef struct {
    orc_item *v;
    int n, cap;
} orc_heap;

static void orc_heap_push(orc_heap *h, const orc_item *it) {
    if (h->cap <= 0) return;
    if (h->n < h->cap) {
        int i = h->n++;
        h->v[i] = *it;
        while (i > 0) {
            int p = (i - 1) / 2;
            if (orc_better(&h->v[p], &h->v[i])) {
                orc_item t = h->v[p];
                h->v[p] = h->v[i];
                h->v[i] = t;
                i = p;
            } else
                break;
        }
        return;
    }
    if (!orc_better(it, &h->v[0])) return;
    h->v[0] = *it;
    int i = 0;
    for (;;) {
        int l = 2 * i + 1, r = l + 1, w = i;
        if (l < h->n && orc_better(&h->v[w], &h->v[l])) w = l;
        if (r < h->n && orc_better(&h->v[w], &h->v[r])) w = r;
        if (w == i) break;
        orc_item t = h->v[w];
        h->v[w] = h->v[i];
        h->v[i] = t;
        i = w;
    }
}

static int orc_cmp_items(const void *pa, const void *pb) {
    const orc_item *a = (const orc_item *)pa, *b = (const orc_item *)pb;
    if (orc_better(a, b)) return -1;
    if (orc_better(b, a)) return 1;
    return 0;
}

int64_t orc_scan_topk_range(const uint64_t *bits, const uint64_t *valid,
                            const uint64_t *mask1, const uint64_t *mask2, int n_words,
                            int ra0, int ra1, int rb0, int rb1, int objective, int k,
                            orc_result *tops, double *keys, int threads) {
    int64_t nmax = 0;
    for (int j = 0; j < n_words; ++j)
        nmax += __builtin_popcountll(mask1[j]) + __builtin_popcountll(mask2[j]);
    int F = orc_tfix_bits(nmax);
    uint64_t *T = (uint64_t *)malloc((size_t)(nmax + 1) * sizeof(uint64_t));
    orc_tfix_table(nmax, F, T);
    orc_stirlerr(0);

    int nt = 1;
#ifdef _OPENMP
    nt = threads > 0 ? threads : omp_get_max_threads();
#endif
    orc_heap *heaps = (orc_heap *)calloc((size_t)nt, sizeof(orc_heap));
    for (int t = 0; t < nt; ++t) {
        heaps[t].v = (orc_item *)malloc((size_t)(k > 0 ? k : 1) * sizeof(orc_item));
        heaps[t].cap = k;
    }
    int64_t ranked = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt) reduction(+ : ranked)
#endif
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        orc_heap *h = &heaps[tid];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int rA = ra0; rA < ra1; ++rA) {
            int hiB = rA + 1 < rb1 ? rA + 1 : rb1;
            for (int rB = rb0; rB < hiB; ++rB) {
                for (int fun = 0; fun < 5; ++fun) {
                    int32_t c[4];
                    orc_binfunc(bits, valid, mask1, mask2, n_words, rA, rB, fun, c);
                    int w = c[0], x = c[1], y = c[2], z = c[3];
                    int nz = 0;
                    double key;
                    if (objective == 0) {
                        key = orc_entropy_fixed(T, F, w, x, y, z, &nz);
                    } else {
                        nz = ((int64_t)w * z - (int64_t)x * y) != 0;
                        if (!nz) continue;
                        /* p >= P(obs): skip the full sum when the observed
                           table alone already loses to the current k-th. */
                        if (h->n == h->cap && h->cap > 0) {
                            double lp = orc_fisher_lpobs(w, y - w, x, z - x) / log(10.0);
                            if (-lp < h->v[0].key - 1e-6 * (1.0 + fabs(h->v[0].key))) continue;
                        }
                        key = -orc_fisher_log10p(w, y - w, x, z - x, 0);
                    }
                    if (!nz) continue;
                    ++ranked;
                    orc_item it;
                    it.key = key;
                    it.sA = rA;
                    it.sB = rB;
                    it.fun = fun;
                    it.n[0] = w;
                    it.n[1] = x;
                    it.n[2] = y;
                    it.n[3] = z;
                    orc_heap_push(h, &it);
                }
            }
        }
    }
    /* Merge per-thread heaps: concatenate, sort, keep k. */
    size_t tot = 0;
    for (int t = 0; t < nt; ++t) tot += (size_t)heaps[t].n;
    orc_item *all = (orc_item *)malloc((tot > 0 ? tot : 1) * sizeof(orc_item));
    size_t o = 0;
    for (int t = 0; t < nt; ++t) {
        memcpy(all + o, heaps[t].v, (size_t)heaps[t].n * sizeof(orc_item));
        o += (size_t)heaps[t].n;
        free(heaps[t].v);
    }
    free(heaps);
    qsort(all, tot, sizeof(orc_item), orc_cmp_items);
    memset(tops, 0, (size_t)k * sizeof(orc_result));
    for (int i = 0; i < k; ++i) {
        if (keys) keys[i] = 0.0;
        if ((size_t)i >= tot) continue;
        tops[i].sA = all[i].sA;
        tops[i].sB = all[i].sB;
        tops[i].fun = (char)all[i].fun;
        for (int j = 0; j < 4; ++j) tops[i].n[j] = all[i].n[j];
        tops[i].ent = (float)(-all[i].key);
        if (keys) keys[i] = -all[i].key;
    }
    free(all);
    free(T);
    return ranked;
}

int64_t orc_scan_topk(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                      const uint64_t *mask2, int n_rows, int n_words, int objective, int k,
                      orc_result *tops, double *keys, int threads) {
    return orc_scan_topk_range(bits, valid, mask1, mask2, n_words, 0, n_rows, 0, n_rows,
                               objective, k, tops, keys, threads);
}

/* ------------------------------------------------------------------------- */
/* CPU baseline: the reference gold loop (proc_gold_1.h:68-178) with its own   */
/* cost model: masks per row pair, 5 binFunc calls (proc_gold.h:38-71) whose   */
/* popcounts go through the 64K-entry byte table of bitops.h:33-62 (four       */
/* lookups per 64-bit word), float entropyDelta4, and the 2 x topmost result   */
/* buffer: a test better than the current limit is stored, and a full buffer   */
/* is sorted by score and cut back to topmost (proc_gold_1.h:114-137).  With   */
/* threads > 1 every thread keeps its own buffer over its share of the rows.   */
/* ------------------------------------------------------------------------- */
static unsigned char orc_bits_in16[65536];
static int orc_bits_ready = 0;

static void orc_bits_init(void) {
    if (orc_bits_ready) return;
    for (int j = 0; j < 65536; ++j) {
        int c = 0, v = j;
        while (v) {
            ++c;
            v &= v - 1;
        }
        orc_bits_in16[j] = (unsigned char)c;
    }
    orc_bits_ready = 1;
}

static inline int orc_bits_lut(uint64_t a) {
    return orc_bits_in16[a & 0xffff] + orc_bits_in16[(a >> 16) & 0xffff] +
           orc_bits_in16[(a >> 32) & 0xffff] + orc_bits_in16[a >> 48];
}

typedef struct {
    float ent;
    int32_t sA, sB, fun;
    int32_t n[4];
} orc_gold_item;

static int orc_gold_cmp(const void *a, const void *b) {
    const float x = ((const orc_gold_item *)a)->ent, y = ((const orc_gold_item *)b)->ent;
    return x < y ? -1 : (x > y ? 1 : 0);
}

int64_t orc_gold_loop(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                      const uint64_t *mask2, int n_words, int r0, int r1, int topmost,
                      int threads, double *checksum) {
    int nt = 1;
#ifdef _OPENMP
    nt = threads > 0 ? threads : omp_get_max_threads();
#endif
    if (topmost < 1) topmost = 1;
    orc_bits_init();
    int64_t pairs = 0;
    double acc = 0.0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt) reduction(+ : pairs, acc)
#endif
    {
        uint64_t *am0 = (uint64_t *)malloc((size_t)n_words * 8);
        uint64_t *am1 = (uint64_t *)malloc((size_t)n_words * 8);
        orc_gold_item *buf = (orc_gold_item *)calloc((size_t)2 * topmost, sizeof(orc_gold_item));
        float worst = 3.0e38f;
        int widx = -1;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int j = r0; j < r1; ++j) {
            const uint64_t *a = bits + (size_t)j * n_words, *va = valid + (size_t)j * n_words;
            for (int k = 0; k <= j; ++k) {
                const uint64_t *b = bits + (size_t)k * n_words, *vb = valid + (size_t)k * n_words;
                for (int m = 0; m < n_words; ++m) {
                    am0[m] = mask1[m] & va[m] & vb[m];
                    am1[m] = mask2[m] & va[m] & vb[m];
                }
                for (int fun = 0; fun < 5; ++fun) {
                    int w = 0, x = 0, y = 0, z = 0;
                    for (int m = 0; m < n_words; ++m) {
                        uint64_t c = bfun(a[m], b[m], fun);
                        w += orc_bits_lut(c & am0[m]);
                        x += orc_bits_lut(c & am1[m]);
                        y += orc_bits_lut(am0[m]);
                        z += orc_bits_lut(am1[m]);
                    }
                    float ee = orc_entropy_ref_f32(w, x, y, z);
                    if (ee < worst) {
                        if (widx >= 2 * topmost - 1) {
                            qsort(buf, (size_t)2 * topmost, sizeof(orc_gold_item), orc_gold_cmp);
                            widx = topmost - 1;
                            worst = buf[widx].ent;
                            if (!(ee < worst)) continue;
                        }
                        orc_gold_item *it = &buf[++widx];
                        it->ent = ee;
                        it->sA = j;
                        it->sB = k;
                        it->fun = fun;
                        it->n[0] = w;
                        it->n[1] = x;
                        it->n[2] = y;
                        it->n[3] = z;
                    }
                }
                ++pairs;
            }
        }
        for (int i = 0; i <= widx; ++i) acc += buf[i].ent;
        free(buf);
        free(am0);
        free(am1);
    }
    if (checksum) *checksum = acc;
    return pairs;
}
