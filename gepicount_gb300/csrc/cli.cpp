// gepi -- command-line drop-in for gEpiCount (src/gEpiCount.cpp:47-187).
//
// Same flags, same stdout lines ("Element Size", "Size of each Data Matrix",
// "Size of array of ... topmost", "Cleaned"), same stderr QC report
// (PlinkReader::checkQuality, src/reader/PlinkReader.h:237-335, emitted in
// single-thread order) and the same ranked table (printInteractions,
// src/misc/print_misc.h:57-78).  The scan runs on the GPU through the C ABI:
// the .bed image is decoded on the device and scanned there.
//
// Flags that only shaped the reference's launch geometry (--block-sizes,
// --max-grid-area, --shared-memory, -t) are accepted and reported as ignored;
// -g (the CPU gold path) runs the same GPU scan, whose ranking is the gold
// ranking under the deterministic tie-break.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gepi.h"

namespace {

const int kDefaultTopmost = 1000000;
const char *kFuncName[6] = {"AND", "NAND", "ANDN", "NANDN", "XOR", "Invalid"};

struct Par {
    int gpuNum = 0;
    int topmost = kDefaultTopmost;
    bool gold = false, shmem = false, alt = false, intermediate = false;
    std::string name;
    int blkSzX = 16, blkSzY = 16, maxGridBlocks = 16;
    int ffun = GEPI_ENTROPY;
    float qaMissSNPs = 0.05f, qaMissSamp = 0.05f;
    int method = GEPI_METHOD_AUTO;
    bool verbose = false;
};

void print_help() {
    std::fprintf(stderr,
                 "gEpiCount -i <input-root> [options]\n\n"
                 "   -i | --input-root      BASE Use BASE as full path and filename for .bed,.bim,.fam\n\n"
                 "   -g | --gold                 Process \"gold\" on CPU  [no]\n"
                 "   -f | --fisher-pvals         Computes Fisher P-value instead of Entropy [no]\n"
                 "   -G | --gpu-num         N    Use GPU number N  [0]\n"
                 "   -t | --alternate-grid       For some block sizes, use different layout during init & entropy  [no]\n"
                 "   -D | --print-diagonal       Print a few results from time to time  [no]\n"
                 "   -N | --topmost         M    Maintain a list of M results  [%d]\n\n"
                 "        --block-sizes     N M  Use block size (N,M)  [16,16]\n"
                 "        --max-grid-area   N    Use max N x 1024 x 1024 results  [16]\n"
                 "        --shared-memory        Use shared memory kernel [no]\n"
                 "        --miss-snps       F    Max missing values fraction for SNPs [0.05]>\n"
                 "        --miss-samples    F    Max missing values fraction for samples  [0.05]\n"
                 "        --method          M    popc | tensor | auto  [auto]\n\n",
                 kDefaultTopmost);
}

bool get_params(int argc, char **argv, Par &par) {
    bool ok = true;
    for (int j = 1; j < argc; ++j) {
        std::string a(argv[j]);
        auto need = [&](int n) {
            if (j + n >= argc) {
                std::fprintf(stderr, "Missing value for option: %s\n", a.c_str());
                ok = false;
                return false;
            }
            return true;
        };
        if (a == "-g" || a == "--gold") par.gold = true;
        else if (a == "-t" || a == "--alternate-grid") par.alt = true;
        else if (a == "-G" || a == "--gpu-num") { if (need(1)) par.gpuNum = std::atoi(argv[++j]); }
        else if (a == "-D" || a == "--print-diagonal") par.intermediate = true;
        else if (a == "-f" || a == "--fisher-pvals") par.ffun = GEPI_FISHER;
        else if (a == "-i" || a == "--input-root") { if (need(1)) par.name = argv[++j]; }
        else if (a == "-N" || a == "--topmost") { if (need(1)) par.topmost = std::atoi(argv[++j]); }
        else if (a == "--block-sizes") {
            if (need(2)) {
                par.blkSzX = std::atoi(argv[++j]);
                par.blkSzY = std::atoi(argv[++j]);
            }
        } else if (a == "--max-grid-area") { if (need(1)) par.maxGridBlocks = std::atoi(argv[++j]); }
        else if (a == "--shared-memory") par.shmem = true;
        else if (a == "--miss-snps") { if (need(1)) par.qaMissSNPs = (float)std::atof(argv[++j]); }
        else if (a == "--miss-samples") { if (need(1)) par.qaMissSamp = (float)std::atof(argv[++j]); }
        else if (a == "--method") {
            if (need(1)) {
                std::string m(argv[++j]);
                par.method = m == "popc" ? GEPI_METHOD_POPC : m == "tensor" ? GEPI_METHOD_TENSOR
                                                                           : GEPI_METHOD_AUTO;
            }
        } else if (a == "-v" || a == "--verbose") par.verbose = true;
        else {
            std::fprintf(stderr, "Unknown option: %s\n", a.c_str());
            ok = false;
        }
    }
    if ((par.blkSzX * par.blkSzY) % 32 != 0) {
        std::fprintf(stderr, "Block size not multiple of war size (32)\n");
        ok = false;
    }
    if (par.name.empty()) {
        std::fprintf(stderr, "Insufficient arguments\n");
        ok = false;
    }
    if (par.topmost <= 0) {
        std::fprintf(stderr, "Topmost must be positive\n");
        ok = false;
    }
    if (!ok) print_help();
    return ok;
}

// checkQuality (PlinkReader.h:237-335): reports samples and SNP rows whose
// missing fraction exceeds the thresholds; nothing is removed.
void check_quality(gepi_plink *p, const std::vector<uint64_t> &valid, float maxMissSNPs,
                   float maxMissSamples) {
    const int nS = gepi_plink_num_samples(p), nR = gepi_plink_num_rows(p);
    const int nw = gepi_plink_elements_snp(p);
    const int32_t *ph = gepi_plink_phenotypes(p);
    std::fprintf(stderr, "Checking data in 1 chunks of %d Samples.\n", nS);
    int ncSamp = 0;
    for (int j = 0; j < nS; ++j) {
        const uint64_t sele = 1ull << (j % 64);
        int v = 0;
        for (int k = 0; k < nR; ++k) v += (valid[(size_t)k * nw + j / 64] & sele) ? 1 : 0;
        float sMiss = (float)(nR - v) / (float)nR;
        if (sMiss > maxMissSamples) {
            const char *nm = "";
            gepi_plink_sample_info(p, j, &nm, nullptr, nullptr);
            std::fprintf(stderr, "Sample %d:\t%s(%d)\tnMiss:%d\t(%4g)\n", j, nm, ph[j], nR - v, sMiss);
            ++ncSamp;
        }
        if (j % 100 == 0) std::fprintf(stderr, "%d %d %g\n", j, nR - v, sMiss);
    }
    std::fprintf(stderr, "\n%d Samples checked, %d with more than %4g missing values\n\n", nS, ncSamp,
                 maxMissSamples);
    std::fprintf(stderr, "Checking data in 1 chunks of %d SNPs.\n", nR);
    int ncSNPs = 0;
    for (int j = 0; j < nR; ++j) {
        int v = 0;
        for (int k = 0; k < nw; ++k) v += __builtin_popcountll(valid[(size_t)j * nw + k]);
        float sMiss = (float)(nS - v) / (float)nS;
        if (sMiss > maxMissSNPs) {
            const char *id = "";
            gepi_plink_row_info(p, j, &id, nullptr, nullptr, nullptr);
            std::fprintf(stderr, "SNP %d:\t%s\tnMiss:%d\t(%4g)\n", j, id, nS - v, sMiss);
            ++ncSNPs;
        }
        if (j % 10000 == 0) std::fprintf(stderr, "%d %d %g\n", j, nS - v, sMiss);
    }
    std::fprintf(stderr, "\n%d SNPs checked, %d with more than %4g missing values\n\n", nR, ncSNPs,
                 maxMissSNPs);
}

void print_interaction(gepi_plink *p, int num, const gepi_result &ir) {
    const char *ia = "", *ib = "";
    char aa = '?', ab = '?';
    int ca = 0, pa = 0, cb = 0, pb = 0;
    gepi_plink_row_info(p, ir.sA, &ia, &aa, &ca, &pa);
    gepi_plink_row_info(p, ir.sB, &ib, &ab, &cb, &pb);
    const int w = ir.n[0], x = ir.n[1], y = ir.n[2], z = ir.n[3];
    float pv = gepi_fisher_pval(w, y - w, x, z - x);
    int f = (ir.fun >= 0 && ir.fun < 5) ? ir.fun : 5;
    std::fprintf(stderr, "%d:\t%d[%s %c %d:%d]\t%s\t%d[%s %c %d:%d]\t%g\t%g\t(%d,%d,%d,%d)\n", num,
                 ir.sA, ia, aa, ca, pa, kFuncName[f], ir.sB, ib, ab, cb, pb, ir.ent, pv, w, y - w, x,
                 z - x);
}

// printInteractions (print_misc.h:57-66): ranks within `context` of every
// multiple of `stride`.
void print_interactions(gepi_plink *p, const gepi_result *tops, int n, int stride = 1,
                        int context = 0) {
    std::fprintf(stderr,
                 "\nRank:\tidxA[id allele chr:pos]\tFunc\tidxB[id allele chr:pos]\tObj\tFPv\t(c00,c01,c10,c11)\n");
    if (stride - 2 * context < 1) context = stride / 2;
    for (int j = 0; j < n; j += stride)
        for (int k = j - context < 0 ? 0 : j - context; k < (j + context + 1 > n ? n : j + context + 1); ++k)
            print_interaction(p, k, tops[k]);
}

constexpr int kPrintStride = 100000, kPrintContext = 5;  // print_misc.h:30-31

// Progress lines at tile-band ends, as the reference prints them at the
// diagonal points of its batch grid (kernel1.cu:417-439, "K1") or every 1,024
// rows of the gold loop (proc_gold_1.h:140-163, "G1"); with -D the ranked
// results so far follow.
struct CliProgress {
    gepi_plink *p = nullptr;
    int rows = 0;  // allele rows (the reference's numSNPs())
    bool gold = false, intermediate = false;
};

void cli_progress(void *user, const gepi_progress *pr) {
    const CliProgress *c = static_cast<const CliProgress *>(user);
    if (pr->snps_done <= 0) return;
    const char *tag = c->gold ? "G1" : "K1";
    const int done_rows = 2 * pr->snps_done;
    float nt = (float)c->rows / (float)done_rows;  // fraction so far is 1/nt
    nt = nt * nt;
    const float tot = (float)pr->elapsed_s;
    float rem = (nt - 1.0f) * tot;
    const float pct = 100.0f / nt;
    const char *uu = "sec";
    if (rem > 3600.0f) {
        rem /= 3600.0f;
        uu = "hr";
    }
    std::fprintf(stderr, "%s: Total time %gsec (%g%%) Remaining: %g%s\n", tag, tot, pct, rem, uu);
    if (c->intermediate && pr->tops && pr->ntops > 0) {
        if (c->gold) std::fprintf(stderr, "G1: Sorting... Limit: %g\n", pr->tops[pr->ntops - 1].ent);
        std::fprintf(stderr, "%s: Last processed: %d,%d\n", tag, done_rows - 1, done_rows - 1);
        print_interactions(c->p, pr->tops, pr->ntops, kPrintStride, kPrintContext);
    }
}

}  // namespace

int main(int argc, char **argv) {
    std::fprintf(stderr, "gEpiCount, version: gepi-gb300 (ABI %d)\n\n", gepi_abi_version());
    Par par;
    if (!get_params(argc, argv, par)) return 3;
    if (par.shmem || par.alt || par.blkSzX != 16 || par.blkSzY != 16 || par.maxGridBlocks != 16)
        std::fprintf(stderr, "Note: launch-geometry options are ignored (tiles are autotuned)\n");
    if (par.gold)
        std::fprintf(stderr, "Note: -g runs the GPU scan; its ranking equals the gold ranking\n");

    gepi_plink *p = nullptr;
    gepi_status st = gepi_plink_open(par.name.c_str(), &p);
    if (st != GEPI_OK) {
        std::fprintf(stderr, "%s\n", gepi_last_error());
        std::printf("Error in %s\n", par.name.c_str());
        return 2;
    }
    const int nR = gepi_plink_num_rows(p), nS = gepi_plink_num_samples(p);
    const int nw = gepi_plink_elements_snp(p);
    std::fprintf(stderr, "%s.fam: %d samples\n%s.bim: %d lines read, %d SNPs\n", par.name.c_str(), nS,
                 par.name.c_str(), nR / 2, nR);
    std::vector<uint64_t> valid((size_t)nR * nw), bits((size_t)nR * nw);
    gepi_plink_decode_rows(p, bits.data(), valid.data(), nullptr, nullptr);
    const long dsz = 8L * nw * nR;
    std::printf("\nElement Size: %d\n", 8);
    std::printf("Size of each Data Matrix: %ld (%ldMB)\n", dsz, (dsz + (1 << 20) - 1) / (1 << 20));
    check_quality(p, valid, par.qaMissSNPs, par.qaMissSamp);
    const long tb = 2L * par.topmost * (long)sizeof(gepi_result);
    std::printf("Size of array of %d topmost interaction results: %ld (%ldMB) (+1x buffer)\n",
                par.topmost, tb, (tb + (1 << 20) - 1) / (1 << 20));
    std::fflush(stdout);

    std::vector<gepi_result> tops((size_t)par.topmost);
    std::memset(tops.data(), 0, tops.size() * sizeof(gepi_result));
    size_t nbytes = 0;
    const uint8_t *bed = gepi_plink_bed(p, &nbytes);
    auto t0 = std::chrono::steady_clock::now();
    gepi_planes *pl = nullptr;
    st = gepi_planes_from_bed(bed, nbytes, nR / 2, nS, gepi_plink_phenotypes(p), par.gpuNum, &pl);
    if (st == GEPI_OK) {
        gepi_params gp{};
        gp.gpu_num = par.gpuNum;
        gp.topmost = par.topmost;
        gp.objective = par.ffun;
        gp.method = par.method;
        gp.verbose = par.verbose;
        if (!par.gold)
            std::fprintf(stderr, "K1: Objective function is %s\n",
                         par.ffun == GEPI_FISHER ? "FISHER PV" : "ENTROPY");
        CliProgress cp;
        cp.p = p;
        cp.rows = nR;
        cp.gold = par.gold;
        cp.intermediate = par.intermediate;
        // every band end for the progress lines; with -D at most 32 snapshots
        st = gepi_scan_progress(pl, &gp, 0, nR / 2, 0, nR / 2, tops.data(), par.topmost, cli_progress,
                                &cp, par.intermediate ? 32 : 0, par.intermediate ? 1 : 0);
        gepi_planes_destroy(pl);
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st != GEPI_OK) {
        std::fprintf(stderr, "E[%d]: %s: %s\n", par.gpuNum, gepi_status_string(st), gepi_last_error());
        gepi_plink_close(p);
        return 1;
    }
    if (par.gold) std::fprintf(stderr, "G1: Sorting... Limit: %g\n", tops[par.topmost - 1].ent);
    std::fprintf(stderr, par.gold ? "process_gold_1: %g \n" : "process_gpu_1: %g \n", secs);
    print_interactions(p, tops.data(), (int)tops.size());
    gepi_plink_close(p);
    std::printf("Cleaned\n");
    return 0;
}
