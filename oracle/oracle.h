/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of gEpiCount's gold path (the parity checker).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the product
 * library never links or calls it.  Every function cites the reference code it
 * follows (paths inside the gEpiCount project).
 *
 * Pinned against the reference: tests/golden/ holds outputs of the unmodified
 * reference gold binary (built by oracle/Makefile.ref) on the 2-SNP test
 * fileset and on seeded synthetic filesets; tests/test_oracle_golden.py checks
 * this restatement against them.
 */
#ifndef GEPI_ORACLE_H_
#define GEPI_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_result {
    int32_t sA, sB;
    int32_t _pad0[2];
    int32_t n[4]; /* w, x, y, z as InteractionResult.n */
    float ent;
    char fun;
    char _pad1[11];
} orc_result;

/* .bed image -> reference row-major bit/valid planes (BinPlinkReader.h:101-244). */
void orc_decode_bed(const uint8_t *bed, int n_lines, int n_samples, uint64_t *bits,
                    uint64_t *valid);
/* Class masks of phenotypes 1 and 2 (PlinkReader.h:408-440). */
void orc_class_masks(const int32_t *pheno, int n_samples, uint64_t *mask1, uint64_t *mask2);

/* binFunc counts (proc_gold.h:38-71) with the gold masks
 * aMask_c = class_c & vA & vB (proc_gold_1.h:106-112): out = {w, x, y, z}. */
void orc_binfunc(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                 const uint64_t *mask2, int n_words, int rA, int rB, int fun, int32_t out[4]);

/* entropyDelta4 host branch (entropy_inline.h:70-77): float, log2 on floats. */
float orc_entropy_ref_f32(int w, int x, int y, int z);
/* The same formula evaluated in double precision. */
double orc_entropy_f64(int w, int x, int y, int z);

/* Fixed-point n*log2(n) table used for exact, reproducible entropy ranking. */
int orc_tfix_bits(int64_t n_max);
void orc_tfix_table(int64_t n_max, int F, uint64_t *T /* n_max+1 */);
/* Mutual information I(F;C) in bits from the fixed-point table (exact integer
 * numerator, one IEEE division).  *nonzero = (w*z != x*y). */
double orc_entropy_fixed(const uint64_t *T, int F, int w, int x, int y, int z, int *nonzero);

/* Two-sided Fisher exact test, log10 p, restating fisher_p.c:52-245 in double.
 * strict=1: terms with log d <= log d_obs (the reference's comparison);
 * strict=0: terms with d <= d_obs * (1 + 1e-7) (R's fisher.test rule). */
double orc_fisher_log10p(int n11, int n12, int n21, int n22, int strict);

/* 18 Gram counts of .bim SNP pair (s, t): index c*9 + p*3 + q, planes
 * {row 2s, row 2s+1, valid}. */
void orc_pair_gram(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                   const uint64_t *mask2, int n_words, int s, int t, uint32_t out[18]);

/* Gold scan (proc_gold_1.h:68-178) over all allele-row pairs rB <= rA (rows
 * [0, n_rows)), ranked by the exact objective: entropy via orc_entropy_fixed,
 * Fisher via orc_fisher_log10p(strict=0) in print order (w, y-w, x, z-x).
 * Only tests with w*z != x*y are ranked; ties broken by (sA, sB, fun)
 * ascending; unused slots zeroed.  ent is the objective as float (-I bits or
 * log10 p).  If keys != NULL it receives the double objective per slot.
 * threads <= 0 uses all OpenMP threads.  Returns the number of tests ranked. */
int64_t orc_scan_topk(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                      const uint64_t *mask2, int n_rows, int n_words, int objective, int k,
                      orc_result *tops, double *keys, int threads);

/* Same scan restricted to row ranges: rA in [ra0, ra1), rB in [rb0, rb1), rB <= rA. */
int64_t orc_scan_topk_range(const uint64_t *bits, const uint64_t *valid,
                            const uint64_t *mask1, const uint64_t *mask2, int n_words,
                            int ra0, int ra1, int rb0, int rb1, int objective, int k,
                            orc_result *tops, double *keys, int threads);

/* The reference's gold loop for a CPU baseline: processes rows [r0, r1)
 * against all rB <= rA as proc_gold_1.h:68-178 does (masks, 5 binFunc calls
 * with the 64K-entry popcount table of bitops.h:33-62, float entropyDelta4,
 * the 2 x topmost result buffer sorted when full) and returns the number of
 * row pairs. */
int64_t orc_gold_loop(const uint64_t *bits, const uint64_t *valid, const uint64_t *mask1,
                      const uint64_t *mask2, int n_words, int r0, int r1, int topmost,
                      int threads, double *checksum);

#ifdef __cplusplus
}
#endif

#endif
