// Host PLINK fileset reader with the semantics of gEpiCount's PlinkReader /
// BinPlinkReader (src/reader/PlinkReader.h:345-440, BinPlinkReader.h:58-244):
//   .fam  : lines shorter than 5 chars skipped; sample name = first token;
//           sex and phenotype = 5th and 6th fields parsed as integers.
//   .bim  : lines shorter than 9 chars skipped; "chr id cM pos a1 a2" with chr,
//           cM, pos integers and alleles the first character of their token;
//           each line yields TWO allele rows (a1 row, then a2 row).
//   .bed  : magic 6c 1b, size = (rows/2) * ceil(samples/4) + 3; the order byte
//           is reported but the data is always read SNP-major.
// Decoding 2-bit calls (low bits = first sample): 00 -> a1 row, 10 -> both rows,
// 11 -> a2 row, 01 -> missing; valid = not missing; sample j at bit j%64 of
// word j/64.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "common.h"

struct gepi_plink {
    std::string base;
    std::vector<std::string> sample_name;
    std::vector<int32_t> sex, pheno;
    std::vector<std::string> snp_id;  // per .bim line
    std::vector<char> allele;         // per allele row (2 per line)
    std::vector<int32_t> chr, pos;    // per .bim line
    std::vector<uint8_t> bed;         // whole file image
    bool snp_major = true;
};

namespace gepi {

static gepi_status read_fam(gepi_plink &p) {
    std::ifstream is(p.base + ".fam");
    if (!is.is_open()) return set_error(GEPI_ERR_IO, "cannot open " + p.base + ".fam");
    std::string line;
    while (std::getline(is, line)) {
        if (line.size() < 5) continue;
        size_t n = line.find_first_of(" \t", 0);
        int d = 0, e = -9;
        if (std::sscanf(line.c_str(), "%*s %*s %*d %*d %d %d", &d, &e) < 2) e = -9;
        p.sample_name.push_back(line.substr(0, n));
        p.sex.push_back(d);
        p.pheno.push_back(e);
    }
    return GEPI_OK;
}

static gepi_status read_bim(gepi_plink &p) {
    std::ifstream is(p.base + ".bim");
    if (!is.is_open()) return set_error(GEPI_ERR_IO, "cannot open " + p.base + ".bim");
    std::string line;
    while (std::getline(is, line)) {
        if (line.size() < 9) continue;
        std::istringstream sis(line);
        int a = 0, b = 0, c = 0;
        std::string sn;
        char d = '0', e = '0';
        sis >> a >> sn >> b >> c >> d >> e;
        if (sis.fail())
            return set_error(GEPI_ERR_FORMAT, "unparsable .bim line: " + line);
        p.snp_id.push_back(sn);
        p.chr.push_back(a);
        p.pos.push_back(c);
        p.allele.push_back(d);
        p.allele.push_back(e);
    }
    return GEPI_OK;
}

static gepi_status read_bed(gepi_plink &p) {
    std::string fname = p.base + ".bed";
    FILE *f = std::fopen(fname.c_str(), "rb");
    if (!f) return set_error(GEPI_ERR_IO, "cannot open " + fname);
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 3) {
        std::fclose(f);
        return set_error(GEPI_ERR_FORMAT, fname + ": too short");
    }
    p.bed.resize((size_t)sz);
    size_t got = std::fread(p.bed.data(), 1, (size_t)sz, f);
    std::fclose(f);
    if (got != (size_t)sz) return set_error(GEPI_ERR_IO, fname + ": short read");
    if (p.bed[0] != 0x6c || p.bed[1] != 0x1b)
        return set_error(GEPI_ERR_FORMAT, fname + ": Incorrect Magic");
    size_t expect = p.snp_id.size() * ((p.pheno.size() + 3) / 4) + 3;
    if (expect != (size_t)sz)
        return set_error(GEPI_ERR_FORMAT, fname + ": Size (" + std::to_string(sz) +
                                              ") different than expected (" +
                                              std::to_string(expect) + ")");
    p.snp_major = (p.bed[2] == 0x1);
    return GEPI_OK;
}

}  // namespace gepi

using namespace gepi;

extern "C" gepi_status gepi_plink_open(const char *base, gepi_plink **out) {
    if (!base || !out) return set_error(GEPI_ERR_ARG, "gepi_plink_open: null argument");
    *out = nullptr;
    gepi_plink *p = new gepi_plink();
    p->base = base;
    gepi_status s = read_fam(*p);
    if (s == GEPI_OK) s = read_bim(*p);
    if (s == GEPI_OK) s = read_bed(*p);
    if (s != GEPI_OK) {
        delete p;
        return s;
    }
    *out = p;
    return GEPI_OK;
}

extern "C" void gepi_plink_close(gepi_plink *p) { delete p; }

extern "C" int gepi_plink_num_rows(const gepi_plink *p) { return p ? (int)p->allele.size() : 0; }

extern "C" int gepi_plink_num_samples(const gepi_plink *p) { return p ? (int)p->pheno.size() : 0; }

extern "C" int gepi_plink_elements_snp(const gepi_plink *p) {
    return p ? (int)((p->pheno.size() + 63) / 64) : 0;
}

extern "C" const uint8_t *gepi_plink_bed(const gepi_plink *p, size_t *nbytes) {
    if (!p) return nullptr;
    if (nbytes) *nbytes = p->bed.size();
    return p->bed.data();
}

extern "C" const int32_t *gepi_plink_phenotypes(const gepi_plink *p) {
    return p ? p->pheno.data() : nullptr;
}

extern "C" gepi_status gepi_plink_sample_info(const gepi_plink *p, int i, const char **name,
                                              int *sex, int *phenotype) {
    if (!p || i < 0 || i >= (int)p->pheno.size())
        return set_error(GEPI_ERR_ARG, "gepi_plink_sample_info: bad sample");
    if (name) *name = p->sample_name[i].c_str();
    if (sex) *sex = p->sex[i];
    if (phenotype) *phenotype = p->pheno[i];
    return GEPI_OK;
}

extern "C" gepi_status gepi_plink_row_info(const gepi_plink *p, int row, const char **id,
                                           char *allele, int *chr, int *pos) {
    if (!p || row < 0 || row >= (int)p->allele.size())
        return set_error(GEPI_ERR_ARG, "gepi_plink_row_info: bad row");
    int s = row / 2;
    if (id) *id = p->snp_id[s].c_str();
    if (allele) *allele = p->allele[row];
    if (chr) *chr = p->chr[s];
    if (pos) *pos = p->pos[s];
    return GEPI_OK;
}

extern "C" gepi_status gepi_plink_decode_rows(const gepi_plink *p, uint64_t *bits,
                                              uint64_t *valid, uint64_t *mask1,
                                              uint64_t *mask2) {
    if (!p) return set_error(GEPI_ERR_ARG, "gepi_plink_decode_rows: null reader");
    const int ns = (int)p->pheno.size();
    const int nw = (ns + 63) / 64;
    const int nl = (int)p->snp_id.size();
    const size_t bps = ((size_t)ns + 3) / 4;
    if (bits && valid) {
        for (int s = 0; s < nl; ++s) {
            const uint8_t *row = p->bed.data() + 3 + (size_t)s * bps;
            uint64_t *bA = bits + (size_t)(2 * s) * nw, *ba = bits + (size_t)(2 * s + 1) * nw;
            uint64_t *vA = valid + (size_t)(2 * s) * nw, *va = valid + (size_t)(2 * s + 1) * nw;
            std::memset(bA, 0, nw * 8);
            std::memset(ba, 0, nw * 8);
            std::memset(vA, 0, nw * 8);
            for (int k = 0; k < ns; ++k) {
                int code = (row[k >> 2] >> (2 * (k & 3))) & 3;
                uint64_t bit = 1ull << (k & 63);
                int w = k >> 6;
                if (code != 1) vA[w] |= bit;
                if (code == 0 || code == 2) bA[w] |= bit;
                if (code == 2 || code == 3) ba[w] |= bit;
            }
            std::memcpy(va, vA, nw * 8);
        }
    }
    if (mask1) std::memset(mask1, 0, nw * 8);
    if (mask2) std::memset(mask2, 0, nw * 8);
    for (int k = 0; k < ns; ++k) {
        uint64_t bit = 1ull << (k & 63);
        if (mask1 && p->pheno[k] == 1) mask1[k >> 6] |= bit;
        if (mask2 && p->pheno[k] == 2) mask2[k >> 6] |= bit;
    }
    return GEPI_OK;
}
