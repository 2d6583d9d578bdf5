/*
 * gepi.h -- C ABI of the GB300-native pairwise Boolean epistasis scan.
 *
 * This is the drop-in boundary for gEpiCount's `proc_gpu` path.  Every entry
 * point takes plain pointers and sizes, returns a gepi_status, and never
 * throws.  Reference interfaces replaced (paths are inside the gEpiCount
 * project):
 *
 *   process_gpu_1(PlinkReader<ui8>*, InteractionResult*, const _paramP1&)
 *       src/proc_gpu.h:134, src/kernels/kernel1.cu:508-511
 *       -> gepi_process_gpu_1()  (same inputs as plain arrays, same output)
 *   InteractionResult                 inc/gEpiCount.h:75-82  -> gepi_result
 *   struct _paramP1                   inc/gEpiCount.h:116-132 -> gepi_params
 *   BinaryFunction / FitnessFunction  inc/gEpiCount.h:58-73
 *   float fisher_pval(int,int,int,int)  inc/gEpiCount.h:137-139,
 *       src/misc/fisher_p.c:52-76     -> gepi_fisher_pval()
 *   BinPlinkReader::checkConsistency/readData
 *       src/reader/BinPlinkReader.h:58-244 -> gepi_plink_open() (host parse)
 *       + gepi_planes_from_bed() (2-bit decode on the device)
 *   allocSendData_device  src/kernels/setup1.h:72-102 -> gepi_planes_from_rows()
 *
 * Threading: a handle (gepi_planes) may be used by one host thread at a time.
 * All calls are synchronous on return unless stated otherwise.
 */
#ifndef GEPI_H_
#define GEPI_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GEPI_ABI_VERSION 2

typedef enum gepi_status {
    GEPI_OK = 0,
    GEPI_ERR_ARG = 1,          /* invalid argument (null pointer, bad size, ...)     */
    GEPI_ERR_IO = 2,           /* file missing / unreadable                          */
    GEPI_ERR_FORMAT = 3,       /* bad .bed magic / size mismatch / unparsable text   */
    GEPI_ERR_CUDA = 4,         /* CUDA runtime error (message via gepi_last_error)   */
    GEPI_ERR_OOM = 5,          /* device memory admission failed                     */
    GEPI_ERR_NOCLASS = 6,      /* phenotype class 1 or 2 has no sample               */
    GEPI_ERR_TIMEOUT = 7,      /* a bounded device wait ran out                      */
    GEPI_ERR_UNSUPPORTED = 8,  /* option not available on this device / build       */
    GEPI_ERR_LIMIT = 9         /* request beyond a documented maximum                */
} gepi_status;

/* Boolean functions, same values as BinaryFunction (inc/gEpiCount.h:58-66). */
enum { GEPI_AND = 0, GEPI_NAND = 1, GEPI_ANDN = 2, GEPI_NANDN = 3, GEPI_XOR = 4 };
/* Objective, same values as FitnessFunction (inc/gEpiCount.h:68-73). */
enum { GEPI_ENTROPY = 0, GEPI_FISHER = 1 };
/* Counting method. */
enum { GEPI_METHOD_AUTO = 0, GEPI_METHOD_POPC = 1, GEPI_METHOD_TENSOR = 2 };
/* Counting variants: a counting kernel with its tile shape and plane words per
 * pipeline stage, ids 1..4 (gepi_count_variant_name / _shape):
 *   1 popc_32x32_w32   popcount, 32 x 32 SNP tiles, 32 words per stage (GEPI_METHOD_POPC)
 *   2 popc_32x32_w16   popcount, 32 x 32 SNP tiles, 16 words per stage
 *   3 popc_64x32_w32   popcount, 64 x 32 SNP tiles, 32 words per stage
 *   4 tensor_80x64_w12 tensor cores, 80 x 64 SNP tiles on a CTA pair, 12 words
 *                      (384 samples) per stage (GEPI_METHOD_TENSOR)
 * Every variant returns the same results bit for bit.  GEPI_VARIANT(v) passed
 * as the `method` of gepi_pair_counts selects variant v. */
#define GEPI_NUM_VARIANTS 4
#define GEPI_VARIANT(v) (16 + (v))

/* One ranked interaction.  Byte layout identical to InteractionResult
 * (inc/gEpiCount.h:75-82, sizeof 48, int4 aligned at offset 16):
 *   sA, sB : allele-row indices (row 2s = .bim column-5 allele carrier,
 *            row 2s+1 = column-6 allele carrier), sB <= sA
 *   n      : {w = on count class 1 (controls), x = on count class 2 (cases),
 *             y = valid count class 1,          z = valid count class 2}
 *   ent    : objective, ascending = best.  Entropy: -I(F;C) in bits.
 *            Fisher: log10 of the two-sided p-value.
 *   fun    : GEPI_AND .. GEPI_XOR */
typedef struct gepi_result {
    int32_t sA;
    int32_t sB;
    int32_t _pad0[2];
    int32_t n[4];
    float ent;
    char fun;
    char _pad1[11];
} gepi_result;

/* Scan parameters: the subset of struct _paramP1 (inc/gEpiCount.h:116-132)
 * that changes results, plus the new knobs. */
typedef struct gepi_params {
    int32_t gpu_num;        /* -G  : CUDA device ordinal                           */
    int32_t topmost;        /* -N  : length of the ranked list                     */
    int32_t objective;      /* -f  : GEPI_ENTROPY / GEPI_FISHER                     */
    int32_t method;         /* GEPI_METHOD_*                                        */
    int32_t verbose;        /* 0 silent, 1 progress lines on stderr                 */
    int32_t variant;        /* 0: by `method`; 1..GEPI_NUM_VARIANTS: that variant   */
    int32_t reserved[6];
} gepi_params;

/* Opaque device-resident genotype bit-planes (one cohort). */
typedef struct gepi_planes gepi_planes;

/* Host-side PLINK fileset, parsed with BinPlinkReader semantics. */
typedef struct gepi_plink gepi_plink;

/* ---- status / version ---------------------------------------------------- */
const char *gepi_status_string(gepi_status s);
/* Last error message of the calling thread ("" if none). */
const char *gepi_last_error(void);
int gepi_abi_version(void);

/* ---- host PLINK reader (replaces BinPlinkReader/PlinkReader host parsing) -- */
/* Parses BASE.fam / BASE.bim and maps BASE.bed (checkConsistency semantics:
 * magic 6c 1b, size == (rows/2)*ceil(samples/4)+3).  Rows = 2 x .bim lines. */
gepi_status gepi_plink_open(const char *base, gepi_plink **out);
void gepi_plink_close(gepi_plink *p);
int gepi_plink_num_rows(const gepi_plink *p);        /* numSNPs(): 2 x .bim lines */
int gepi_plink_num_samples(const gepi_plink *p);     /* numSamples()              */
int gepi_plink_elements_snp(const gepi_plink *p);    /* elementsSNP(): 64-bit words */
const uint8_t *gepi_plink_bed(const gepi_plink *p, size_t *nbytes); /* whole .bed */
const int32_t *gepi_plink_phenotypes(const gepi_plink *p); /* .fam column 6       */
/* .fam info of sample i: name (first field), sex, phenotype. */
gepi_status gepi_plink_sample_info(const gepi_plink *p, int i, const char **name, int *sex,
                                   int *phenotype);
/* .bim info of allele row r: id, allele char, chromosome, position. */
gepi_status gepi_plink_row_info(const gepi_plink *p, int row, const char **id,
                                char *allele, int *chr, int *pos);
/* Host decode to the reference's row-major ui8 bit-planes (BitData/ValidData,
 * BinPlinkReader.h:101-244) and class masks (PlinkReader.h:408-440); for the
 * process_gpu_1 view and for tests.  Arrays are rows x words, words =
 * elementsSNP(); masks have `words` entries. */
gepi_status gepi_plink_decode_rows(const gepi_plink *p, uint64_t *bits, uint64_t *valid,
                                   uint64_t *mask1, uint64_t *mask2);

/* ---- device genotype planes ---------------------------------------------- */
/* Upload a whole .bed file image (header included) and decode it on the device
 * into class-sorted bit-planes.  phenotype[i] is .fam column 6 of sample i;
 * samples with phenotype 1 form class 0 (controls, CLASS0), phenotype 2 class 1
 * (cases, CLASS1); all other samples are left out of every count. */
gepi_status gepi_planes_from_bed(const uint8_t *bed, size_t bed_bytes, int n_bim_snps,
                                 int n_samples, const int32_t *phenotype, int device,
                                 gepi_planes **out);
/* Build planes from the reference reader's host arrays (BitData, ValidData:
 * rows x words ui8, row-major; class masks mask1 (phenotype 1) and mask2
 * (phenotype 2), `words` entries each).  n_rows must be even. */
gepi_status gepi_planes_from_rows(const uint64_t *bits, const uint64_t *valid, int n_rows,
                                  int n_words, const uint64_t *mask1, const uint64_t *mask2,
                                  int device, gepi_planes **out);
/* Frees the plane set.  Its device buffers (planes, operand blocks, candidate
 * buffers, tables) come from a stream-ordered pool per device that keeps up to
 * 8 GiB of freed memory for the next plane set, so building one plane set per
 * cohort, request or step costs no cudaMalloc / cudaFree of the large buffers. */
void gepi_planes_destroy(gepi_planes *pl);
int gepi_planes_num_snps(const gepi_planes *pl);
/* Samples per class (class 0 = phenotype 1, class 1 = phenotype 2). */
gepi_status gepi_planes_class_sizes(const gepi_planes *pl, int *n0, int *n1);

/* ---- the scan ------------------------------------------------------------ */
/* All-pairs scan over allele rows rB <= rA of 5 Boolean functions; writes the
 * `k` best results, ascending by ent with ties broken by (sA, sB, fun)
 * ascending.  Slots beyond the number of tests with a non-zero association
 * are zero-filled (the reference's zeroed tops, gEpiCount.cpp:81-82). */
gepi_status gepi_scan(gepi_planes *pl, const gepi_params *par, gepi_result *tops, int k);

/* Range request: SNP ranges [a0, a0+na) x [b0, b0+nb) (.bim SNP indices).
 * Tests every allele-row pair (rA, rB) with rA in the A range, rB in the B
 * range and rB <= rA, once.  The whole-genome scan is a0=b0=0, na=nb=N. */
gepi_status gepi_scan_range(gepi_planes *pl, const gepi_params *par, int a0, int na,
                            int b0, int nb, gepi_result *tops, int k);

/* Progress of a scan, reported at tile-band ends.  Tiles are walked in bands of
 * about 320 A SNPs (4 A-tile rows of the tensor-core kernel, 10 of the popcount
 * kernel); when a callback fires, every band before the current one is done,
 * so for a whole-genome scan all pairs (s, t), t <= s < snps_done, are tested.
 * Replaces the reference's progress block at diagonal points
 * (src/kernels/kernel1.cu:417-439; gold path src/proc_gold_1.h:140-163). */
typedef struct gepi_progress {
    double elapsed_s;          /* wall time since the scan started                       */
    uint64_t tiles_done;       /* tiles of the scan's list processed                      */
    uint64_t tiles_total;
    int32_t snps_done;         /* A-range SNPs [a0, snps_done) complete                   */
    int32_t ntops;             /* entries in tops: the scan's k when asked for, else 0     */
    const gepi_result *tops;   /* ranked top-k of every test done so far, or NULL;
                                  valid during the callback only                          */
} gepi_progress;
typedef void (*gepi_progress_fn)(void *user, const gepi_progress *p);

/* gepi_scan_range with a progress callback.  points > 0: at most that many
 * callbacks, at the first band end past each 1/points of the tile list;
 * points <= 0: at every band end.  with_tops != 0: each callback also gets the
 * exact ranked top-k of the tests done so far (the batches are cut at the
 * callback's band end for it, and every snapshot reads the candidate buffer
 * back).  Results are identical to gepi_scan_range's. */
gepi_status gepi_scan_progress(gepi_planes *pl, const gepi_params *par, int a0, int na, int b0,
                               int nb, gepi_result *tops, int k, gepi_progress_fn fn, void *user,
                               int32_t points, int32_t with_tops);

/* ---- sharding a scan across GPUs or processes --------------------------------- */
/* Shard `shard` of `n_shards` of the whole-genome triangle of `n_snps` SNPs, as
 * the gepi_scan_range arguments: A rows [r_s, r_{s+1}) against B rows
 * [0, r_{s+1}), r_s = round(n_snps * sqrt(s / n_shards)), so the shards are
 * disjoint, cover every pair once and hold about equal numbers of pairs.  Tile
 * ranges are independent, so a sharded scan needs no exchange but the merge
 * below.  No counterpart in the reference. */
gepi_status gepi_shard_range(int32_t n_snps, int32_t n_shards, int32_t shard, int32_t *a0,
                             int32_t *na, int32_t *b0, int32_t *nb);

/* k-way merge of ranked result lists from disjoint scans of one cohort of
 * `n_samples` samples (e.g. the shards above), on the host: each result is
 * re-keyed from its counts exactly as the scan keys it and the k best are
 * written ranked as one scan ranks them, zero-filling the rest.  For entropy
 * the merged list equals the whole-triangle scan bit for bit; for Fisher it
 * agrees within the objective's 1e-9 relative tolerance. */
gepi_status gepi_merge_results(int32_t n_samples, int32_t objective,
                               const gepi_result *const *lists, const int32_t *lens,
                               int32_t n_lists, gepi_result *out, int32_t k);

/* Per-SNP-pair Gram counts, for verification: for every s in [a0,a0+na),
 * t in [b0,b0+nb) writes 18 uint32 at out[((s-a0)*nb + (t-b0))*18]:
 * class c (0,1) x planes (p,q) in {A-carrier row, a-carrier row, valid}^2,
 * index c*9 + p*3 + q, counting samples of class c with plane p of SNP s and
 * plane q of SNP t both set.  method: GEPI_METHOD_POPC or _TENSOR. */
gepi_status gepi_pair_counts(gepi_planes *pl, int method, int a0, int na, int b0, int nb,
                             uint32_t *out);

/* Timing and work counters of the last gepi_scan / gepi_scan_range on `pl`,
 * measured with CUDA events on the library's stream. */
typedef struct gepi_scan_stats {
    double scan_ms;           /* device time from first to last launch of the scan      */
    double count_ms;          /* summed device time of the counting launches            */
    double max_count_ms;      /* longest counting launch                                */
    int32_t count_launches;   /* counting-kernel launches (one per batch)               */
    int32_t other_launches;   /* select / compaction launches                           */
    int32_t batches;          /* batches completed                                      */
    int32_t overflows;        /* batches retried after a candidate-buffer overflow      */
    uint64_t snp_pairs;       /* SNP pairs s > t tested (pair-tests)                    */
    uint64_t diag_snps;       /* SNPs whose same-SNP allele-row pairs were tested        */
    uint64_t tiles;           /* SNP tile pairs processed                               */
    uint64_t candidates;      /* candidates left for the final host sort                */
    int32_t method;           /* GEPI_METHOD_POPC or GEPI_METHOD_TENSOR actually used   */
    int32_t tile_snps;        /* A SNPs per tile of the variant used                    */
    int32_t variant;          /* counting variant used (1..GEPI_NUM_VARIANTS)           */
    int32_t reserved;
} gepi_scan_stats;
gepi_status gepi_last_scan_stats(const gepi_planes *pl, gepi_scan_stats *out);

/* The FP64 objective each `ent` of the last ranked list on `pl` (gepi_scan,
 * gepi_scan_range, gepi_scan_progress) was rounded from, before the float
 * rounding of the InteractionResult field: entropy -I(F;C) in bits from the
 * exact fixed-point key, Fisher log10 p from the device's log-space tail sums
 * (src/kernels/fisher_d.cu:249-311 computes the same p in FP64 and returns it
 * as float).  out[i] pairs with tops[i]; zero-filled slots give 0.  k may not
 * exceed the last list's length. */
gepi_status gepi_last_scan_values(const gepi_planes *pl, double *out, int32_t k);

/* Counting-method autotuner (replaces the reference's --block-sizes /
 * --max-grid-area tuning, gEpiCount.cpp:135-141 and misc1.cu:35-89, which
 * size its batch grid).  GEPI_METHOD_AUTO requests on `pl` use the method this
 * picks: the first call times both counting kernels on the leading triangle
 * of up to 4,096 SNPs at the plane set's full sample width and keeps the
 * faster; later calls return the cached choice, and later plane sets of the
 * same shape (class widths, tuning triangle, device) in the process reuse it
 * with the first set's timings.  Sets under 256 SNPs use
 * the popcount kernel untimed (times reported as 0).  Outputs may be NULL. */
gepi_status gepi_planes_autotune(gepi_planes *pl, int32_t *method, float *popc_ms,
                                 float *tensor_ms);

/* The autotuner's full report: GEPI_METHOD_AUTO times every counting variant
 * (tile shape, words per stage, popcount or tensor cores) on the tuning
 * triangle and uses the fastest; ms[v-1] is variant v's time (0: not timed --
 * sets under 256 SNPs, or the tensor-core variant above its class-size limit).
 * gepi_planes_autotune reports the fastest variant of each kernel. */
typedef struct gepi_tune_report {
    int32_t variant;     /* the variant AUTO uses on this plane set */
    int32_t n_variants;  /* GEPI_NUM_VARIANTS                        */
    float ms[8];
} gepi_tune_report;
gepi_status gepi_planes_autotune_variants(gepi_planes *pl, gepi_tune_report *out);
/* Name ("" if unknown) and shape of counting variant v. */
const char *gepi_count_variant_name(int32_t variant);
gepi_status gepi_count_variant_shape(int32_t variant, int32_t *method, int32_t *tile_a,
                                     int32_t *tile_b, int32_t *stage_words);

/* Dense kind::mxf4 (packed FP4) tensor-core rate of `device` in TFLOP/s (2 per
 * multiply-accumulate), measured now: one CTA per SM issues back-to-back
 * M=128 x N=256 x K=64 MMAs; best of 3 timed launches.  It is the roofline
 * denominator of the tensor-core counting kernel.  No counterpart in the
 * reference. */
gepi_status gepi_tensor_peak_tflops(int32_t device, double *tflops);

/* The same measurement for each exact FP4 encoding of 0/1 operands (E2M1 A
 * and B, unit block scales): GEPI_PEAK_MXF4 = kind::mxf4 scale_vec::2X UE8M0
 * (the counting kernel's instruction; gepi_tensor_peak_tflops),
 * GEPI_PEAK_MXF4NVF4_2X = kind::mxf4nvf4 scale_vec::2X UE8M0,
 * GEPI_PEAK_MXF4NVF4_4X = kind::mxf4nvf4 scale_vec::4X UE4M3.  No counterpart
 * in the reference. */
enum { GEPI_PEAK_MXF4 = 0, GEPI_PEAK_MXF4NVF4_2X = 1, GEPI_PEAK_MXF4NVF4_4X = 2 };
gepi_status gepi_tensor_peak_probe(int32_t device, int32_t kind, double *tflops);

/* ---- many scans at once: cohort batches and the serving loop ---------------- */
/* One scan request: SNP ranges [a0, a0+na) x [b0, b0+nb) of `planes` (na < 0 or
 * nb < 0: the whole plane set), the `topmost` best results by `objective`
 * (GEPI_ENTROPY / GEPI_FISHER), counting `method` (GEPI_METHOD_*).  Results are
 * those gepi_scan_range gives for the same arguments, bit for bit. */
typedef struct gepi_scan_req {
    gepi_planes *planes;
    int32_t a0, na, b0, nb;
    int32_t topmost;
    int32_t objective;
    int32_t method;
    int32_t variant;  /* 0: by `method`; else a counting variant id */
} gepi_scan_req;

/* Runs `n` requests together on the device of their plane sets (all on one
 * device; plane sets may differ, so a call scans many cohorts): every request
 * walks its tile list in its own adaptive batches, and each engine step -- one
 * CUDA graph replay -- runs the next batch of every unfinished request in ONE
 * persistent counting launch per kernel group (CTAs claim the tiles of all
 * requests from one work list with an atomic counter), then every request's
 * threshold select in one chain of batched launches.
 * Replaces a loop of one reference process per cohort (the batch loop of
 * launch_process_gpu_1, src/kernels/kernel1.cu:387-483, run per cohort).
 * tops[i] receives reqs[i].topmost results; stats (may be NULL) receives one
 * gepi_scan_stats per request.  The first failing request's status is
 * returned.  Calls on one device are serialised internally; a plane set must
 * not be used by another call while it runs.  No counterpart in the reference. */
gepi_status gepi_scan_batch(const gepi_scan_req *reqs, int32_t n, gepi_result *const *tops,
                            gepi_scan_stats *stats);

/* Launch counts of the last gepi_scan_batch call on `device`: engine steps,
 * counting launches (one per kernel group present in a step: the tensor-core
 * kernel per objective, the popcount kernel per variant), select launches
 * (20 per step, batched over every request) and step-graph replays; the
 * device time of the steps (upload to read-back, CUDA events) and the host
 * time spent in them (planning to results consumed), in ms.  No counterpart
 * in the reference. */
typedef struct gepi_batch_stats {
    int64_t steps;
    int64_t count_launches;
    int64_t select_launches;
    int64_t graph_launches;
    double device_ms;
    double wall_ms;
} gepi_batch_stats;
gepi_status gepi_scan_batch_stats(int32_t device, gepi_batch_stats *out);

/* Serving loop: a thread that admits submitted requests first-in first-out
 * while their device footprint (2 candidate buffers each: 256 MiB at topmost
 * <= 512 Ki) fits `hbm_budget_bytes` (0: 16 GiB; the oldest request is always
 * admitted when nothing runs), and runs all admitted requests together as
 * gepi_scan_batch does, admitting new ones between engine steps.  A step is
 * capped at about 4 ms of device time (GEPI_QUANTUM_MS); the requests get
 * their batches -- and the first tiles of the step's work lists -- in policy
 * order, every request at least one tile per step.  GEPI_SERVE_POLICY:
 * "short" (the default): least work left first; "deadline": by submission
 * time + GEPI_SERVE_SLACK (default 1.5) x the request's estimated device time
 * alone; "oldest": first come, first served.
 * Plane sets submitted to a server must not be used by other calls until
 * their requests are waited for.  No counterpart in the reference (it runs
 * one scan per process). */
typedef struct gepi_server gepi_server;
typedef struct gepi_request_info {
    double queue_ms;    /* submit -> admission                          */
    double latency_ms;  /* submit -> results ready                      */
    double device_ms;   /* device time of the request's scan            */
    uint64_t snp_pairs; /* SNP pairs the request tested                 */
    int32_t method;     /* counting method used                          */
    int32_t reserved;
} gepi_request_info;
gepi_status gepi_server_create(int32_t device, size_t hbm_budget_bytes, gepi_server **out);
/* Queues a request; returns at once with its ticket. */
gepi_status gepi_server_submit(gepi_server *srv, const gepi_scan_req *req, uint64_t *ticket);
/* Blocks until the ticket's request is done; copies its topmost results to
 * tops and its timings to info (may be NULL); returns the request's status.
 * Each ticket is waited for once. */
gepi_status gepi_server_wait(gepi_server *srv, uint64_t ticket, gepi_result *tops,
                             gepi_request_info *info);
/* The server's engine counters since it was created (the fields of
 * gepi_batch_stats), as of the last completed step. */
gepi_status gepi_server_stats(gepi_server *srv, gepi_batch_stats *out);
/* Finishes admitted requests, fails queued ones, stops the thread.  No wait
 * may be in progress. */
void gepi_server_destroy(gepi_server *srv);

/* ---- drop-in for the reference's process_gpu_1 ----------------------------- */
/* Same inputs as process_gpu_1 reads from its PlinkReader (BitData, ValidData,
 * numSNPs() = n_rows, elementsSNP() = n_words, classData(1|2)->mask()), same
 * output: tops[par->topmost] filled ascending.  tops must be zeroed by the
 * caller as gEpiCount.cpp:81-82 does. */
gepi_status gepi_process_gpu_1(const uint64_t *bits, const uint64_t *valid, int n_rows,
                               int n_words, const uint64_t *mask1, const uint64_t *mask2,
                               gepi_result *tops, const gepi_params *par);

/* Same inputs, output and results as gepi_process_gpu_1, for callers that
 * cannot allocate device memory (their GPU memory is owned by a pool or a
 * framework that forbids cudaMalloc/cudaFree in libraries it loads).  It
 * allocates nothing: all device scratch comes from one fixed 32 MiB array in
 * device memory (held by every GPU that loads the library until exit).
 * Requests whose rows, planes, tables and tile list do not fit next to the
 * 2 x 65,536-record candidate buffers, or with topmost > 16,384, return
 * GEPI_ERR_LIMIT before any device work.  Each call looks up the array's
 * device address on the device it runs on (cudaGetSymbolAddress, checked).
 * Calls share the array and find the previous call's contents there (each
 * call initialises what it reads): overlapping calls on one GPU race and must
 * be serialised.  The log-factorial tables are the same host std::lgamma
 * values gepi_process_gpu_1 uses, so both entry points return the same bits
 * for either objective.  Only the success path is free of host heap
 * allocation (an error message is a std::string).  Popcount counting only.
 * This entry point has no counterpart in the reference. */
gepi_status gepi_process_gpu_1_noalloc(const uint64_t *bits, const uint64_t *valid, int n_rows,
                                       int n_words, const uint64_t *mask1, const uint64_t *mask2,
                                       gepi_result *tops, const gepi_params *par);

/* ---- host scoring helpers -------------------------------------------------- */
/* Two-sided Fisher exact test, log10(p) as float; replaces fisher_pval()
 * (src/misc/fisher_p.c:52-76), argument order (n11, n12, n21, n22). */
float gepi_fisher_pval(int n11, int n12, int n21, int n22);
/* Same test in double. */
double gepi_fisher_log10p(int n11, int n12, int n21, int n22);

/* ---- seeded synthetic PLINK data -------------------------------------------- */
typedef struct gepi_synth_spec {
    int32_t n_snps;          /* .bim lines                                          */
    int32_t n_cases;         /* phenotype 2                                         */
    int32_t n_controls;      /* phenotype 1                                         */
    double maf_lo, maf_hi;   /* per-SNP minor allele frequency ~ U(maf_lo, maf_hi)  */
    double missing;          /* i.i.d. missing-call probability                     */
    int32_t n_planted;       /* interacting SNP pairs with a case-risk effect        */
    double odds_ratio;       /* planted effect size                                 */
    uint64_t seed;
} gepi_synth_spec;

/* Size in bytes of the .bed image gepi_synth_bed writes. */
size_t gepi_synth_bed_bytes(const gepi_synth_spec *spec);
/* Writes the .bed image (header included), phenotype[n_cases+n_controls]
 * (1 or 2) and, if planted != NULL, planted[2*n_planted] SNP indices. */
gepi_status gepi_synth_bed(const gepi_synth_spec *spec, uint8_t *bed, int32_t *phenotype,
                           int32_t *planted);
/* Writes BASE.bed/.bim/.fam for the same data. */
gepi_status gepi_synth_write(const gepi_synth_spec *spec, const char *base);

#ifdef __cplusplus
}
#endif

#endif /* GEPI_H_ */
