// Seeded synthetic PLINK genotype generator.
//
// Produces byte-identical .bed/.bim/.fam on every host: one splitmix64 stream
// per SNP (and one for the cohort simulation), per-sample decisions taken by
// integer compares against thresholds fixed once per SNP.  Build with
// -ffp-contract=off so the few double operations round the same way on x86
// and Arm.
//
// Model (HWE, minor allele = .bim column 5 = PLINK code 00):
//   P(00) = p^2, P(10) = 2p(1-p), P(11) = (1-p)^2, p ~ U(maf_lo, maf_hi) per SNP;
//   each call independently missing (code 01) with probability `missing`.
// Planted pairs (s, t): dominant coding D = (minor allele count >= 1); pair j
// contributes log(odds_ratio) * rule_j(D_s, D_t) to the case log-odds, rule_j =
// XOR for even j, AND for odd j.  Individuals are simulated one at a time and
// accepted into the case or control set until both hold their exact counts.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.h"

namespace gepi {

static inline uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t stream_seed(uint64_t seed, uint64_t stream) {
    uint64_t s = seed ^ (0xD1B54A32D192ED03ull * (stream + 1));
    return splitmix64(s);
}

static inline double unit53(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

static inline uint32_t prob_to_u32(double p) {
    if (p <= 0.0) return 0u;
    if (p >= 1.0) return 0xFFFFFFFFu;
    return (uint32_t)(p * 4294967296.0);
}

struct SnpModel {
    uint32_t t00, t10;  // genotype draw g < t00 -> code 0; g < t10 -> code 2; else 3
};

static SnpModel snp_model(const gepi_synth_spec &sp, uint64_t &st) {
    double u = unit53(splitmix64(st));
    double p = sp.maf_lo + (sp.maf_hi - sp.maf_lo) * u;
    double p2 = p * p;
    double het = 2.0 * p * (1.0 - p);
    SnpModel m;
    m.t00 = prob_to_u32(p2);
    double c = p2 + het;
    m.t10 = prob_to_u32(c);
    if (m.t10 < m.t00) m.t10 = m.t00;
    return m;
}

static inline int draw_code(const SnpModel &m, uint32_t miss_thr, uint64_t r) {
    uint32_t lo = (uint32_t)r, hi = (uint32_t)(r >> 32);
    if (lo < miss_thr) return 1;
    if (hi < m.t00) return 0;
    if (hi < m.t10) return 2;
    return 3;
}

static bool spec_ok(const gepi_synth_spec *sp) {
    if (!sp) return false;
    if (sp->n_snps <= 0 || sp->n_cases < 0 || sp->n_controls < 0) return false;
    if (sp->n_cases + sp->n_controls <= 0) return false;
    if (!(sp->maf_lo >= 0.0 && sp->maf_hi <= 0.5 && sp->maf_lo <= sp->maf_hi)) return false;
    if (!(sp->missing >= 0.0 && sp->missing < 1.0)) return false;
    if (sp->n_planted < 0 || 2 * (int64_t)sp->n_planted > sp->n_snps) return false;
    if (sp->n_planted > 0 && !(sp->odds_ratio > 0.0)) return false;
    return true;
}

static void planted_snps(const gepi_synth_spec &sp, std::vector<int32_t> &out) {
    // Distinct SNP indices drawn without replacement from the cohort stream.
    out.clear();
    uint64_t st = stream_seed(sp.seed, 0xFFFFFFF0ull);
    std::vector<char> used(sp.n_snps, 0);
    while ((int)out.size() < 2 * sp.n_planted) {
        int32_t s = (int32_t)(splitmix64(st) % (uint64_t)sp.n_snps);
        if (used[s]) continue;
        used[s] = 1;
        out.push_back(s);
    }
}

}  // namespace gepi

using namespace gepi;

extern "C" size_t gepi_synth_bed_bytes(const gepi_synth_spec *sp) {
    if (!spec_ok(sp)) return 0;
    size_t ns = (size_t)sp->n_cases + (size_t)sp->n_controls;
    return 3 + (size_t)sp->n_snps * ((ns + 3) / 4);
}

extern "C" gepi_status gepi_synth_bed(const gepi_synth_spec *sp, uint8_t *bed,
                                      int32_t *phenotype, int32_t *planted_out) {
    if (!spec_ok(sp) || !bed || !phenotype) return set_error(GEPI_ERR_ARG, "gepi_synth_bed: bad spec");
    const int ns = sp->n_cases + sp->n_controls;
    const size_t bps = ((size_t)ns + 3) / 4;
    const uint32_t miss_thr = prob_to_u32(sp->missing);
    bed[0] = 0x6c;
    bed[1] = 0x1b;
    bed[2] = 0x01;

    std::vector<int32_t> planted;
    planted_snps(*sp, planted);
    if (planted_out)
        for (size_t i = 0; i < planted.size(); ++i) planted_out[i] = planted[i];

    // Cohort simulation: genotypes of planted SNPs per accepted individual.
    const int np = 2 * sp->n_planted;
    std::vector<uint8_t> pcode((size_t)np * ns, 1);
    {
        uint64_t cst = stream_seed(sp->seed, 0xFFFFFFF1ull);
        std::vector<SnpModel> pm(np);
        for (int j = 0; j < np; ++j) {
            uint64_t st = stream_seed(sp->seed, (uint64_t)planted[j]);
            pm[j] = snp_model(*sp, st);
        }
        // Case odds = OR^r / sqrt(OR) for r active rules (baseline centred so
        // both classes fill).  Only IEEE-exact operations (*, /, sqrt) are used,
        // so the acceptance thresholds are identical on every host.
        std::vector<uint64_t> thr(sp->n_planted + 1);
        {
            double base = sp->n_planted > 0 ? std::sqrt(sp->odds_ratio) : 1.0;
            double pw = 1.0;
            for (int r = 0; r <= sp->n_planted; ++r) {
                double odds = pw / base;
                double pc = odds / (1.0 + odds);
                thr[r] = (uint64_t)(pc * 9007199254740992.0);
                pw *= sp->odds_ratio;
            }
        }
        int cases = 0, controls = 0, got = 0;
        std::vector<int> code(np);
        // Exact counts: label order is decided by acceptance; with no planted
        // pairs this is a seeded shuffle of n_cases 2s and n_controls 1s.
        while (got < ns) {
            int active = 0;
            for (int j = 0; j < np; ++j) code[j] = draw_code(pm[j], 0u, splitmix64(cst));
            for (int q = 0; q < sp->n_planted; ++q) {
                int ds = code[2 * q] != 3, dt = code[2 * q + 1] != 3;  // carries minor allele
                active += (q % 2 == 0) ? (ds ^ dt) : (ds & dt);
            }
            bool is_case = (splitmix64(cst) >> 11) < thr[active];
            if (is_case ? cases >= sp->n_cases : controls >= sp->n_controls) continue;
            if (is_case) ++cases; else ++controls;
            phenotype[got] = is_case ? 2 : 1;
            for (int j = 0; j < np; ++j) {
                uint64_t r = splitmix64(cst);
                int c = code[j];
                if ((uint32_t)r < miss_thr) c = 1;
                pcode[(size_t)j * ns + got] = (uint8_t)c;
            }
            ++got;
        }
    }
    std::vector<int32_t> pidx(sp->n_snps, -1);
    for (int j = 0; j < np; ++j) pidx[planted[j]] = j;

#pragma omp parallel for schedule(dynamic, 64)
    for (int s = 0; s < sp->n_snps; ++s) {
        uint8_t *row = bed + 3 + (size_t)s * bps;
        std::memset(row, 0, bps);
        if (pidx[s] >= 0) {
            const uint8_t *pc = &pcode[(size_t)pidx[s] * ns];
            for (int k = 0; k < ns; ++k) row[k >> 2] |= (uint8_t)(pc[k] << (2 * (k & 3)));
            continue;
        }
        uint64_t st = stream_seed(sp->seed, (uint64_t)s);
        SnpModel m = snp_model(*sp, st);
        for (int k = 0; k < ns; ++k) {
            int c = draw_code(m, miss_thr, splitmix64(st));
            row[k >> 2] |= (uint8_t)(c << (2 * (k & 3)));
        }
    }
    return GEPI_OK;
}

extern "C" gepi_status gepi_synth_write(const gepi_synth_spec *sp, const char *base) {
    if (!spec_ok(sp) || !base) return set_error(GEPI_ERR_ARG, "gepi_synth_write: bad spec");
    const int ns = sp->n_cases + sp->n_controls;
    size_t nb = gepi_synth_bed_bytes(sp);
    std::vector<uint8_t> bed(nb);
    std::vector<int32_t> ph(ns);
    gepi_status st = gepi_synth_bed(sp, bed.data(), ph.data(), nullptr);
    if (st != GEPI_OK) return st;
    std::string b(base);
    FILE *f = std::fopen((b + ".bed").c_str(), "wb");
    if (!f) return set_error(GEPI_ERR_IO, "cannot write " + b + ".bed");
    size_t w = std::fwrite(bed.data(), 1, nb, f);
    std::fclose(f);
    if (w != nb) return set_error(GEPI_ERR_IO, "short write " + b + ".bed");
    f = std::fopen((b + ".fam").c_str(), "w");
    if (!f) return set_error(GEPI_ERR_IO, "cannot write " + b + ".fam");
    for (int i = 0; i < ns; ++i)
        std::fprintf(f, "F%d I%d 0 0 %d %d\n", i + 1, i + 1, 1 + (i & 1), ph[i]);
    std::fclose(f);
    f = std::fopen((b + ".bim").c_str(), "w");
    if (!f) return set_error(GEPI_ERR_IO, "cannot write " + b + ".bim");
    static const char a1[4] = {'A', 'C', 'A', 'C'}, a2[4] = {'G', 'T', 'T', 'G'};
    for (int s = 0; s < sp->n_snps; ++s) {
        int chr = 1 + (int)(((int64_t)s * 22) / sp->n_snps);
        std::fprintf(f, "%d\trs%d\t0\t%d\t%c\t%c\n", chr, s + 1, 1000 + 100 * s, a1[s & 3],
                     a2[s & 3]);
    }
    std::fclose(f);
    return GEPI_OK;
}
