// gepi-synth: writes a seeded synthetic PLINK fileset (BASE.bed/.bim/.fam)
// with the package's generator (synth.cpp) and nothing else -- no CUDA, no
// scan code -- so a process that must not load the scan library (the CPU
// baseline leg of the benchmark) can still make the benchmark's inputs.
//
//   gepi-synth BASE n_snps n_cases n_controls maf_lo maf_hi missing n_planted odds_ratio seed
#include <cstdio>
#include <cstdlib>
#include <string>

#include "common.h"

namespace gepi {

// synth.cpp reports errors through the library's error slot; this tool
// prints them instead.
static std::string g_msg;
gepi_status set_error(gepi_status s, const std::string &msg) {
    g_msg = msg;
    return s;
}
void clear_error() { g_msg.clear(); }

}  // namespace gepi

int main(int argc, char **argv) {
    if (argc != 11) {
        std::fprintf(stderr,
                     "usage: %s BASE n_snps n_cases n_controls maf_lo maf_hi missing n_planted "
                     "odds_ratio seed\n",
                     argv[0]);
        return 2;
    }
    gepi_synth_spec sp{};
    sp.n_snps = std::atoi(argv[2]);
    sp.n_cases = std::atoi(argv[3]);
    sp.n_controls = std::atoi(argv[4]);
    sp.maf_lo = std::atof(argv[5]);
    sp.maf_hi = std::atof(argv[6]);
    sp.missing = std::atof(argv[7]);
    sp.n_planted = std::atoi(argv[8]);
    sp.odds_ratio = std::atof(argv[9]);
    sp.seed = std::strtoull(argv[10], nullptr, 10);
    const gepi_status s = gepi_synth_write(&sp, argv[1]);
    if (s != GEPI_OK) {
        std::fprintf(stderr, "gepi-synth: %s\n", gepi::g_msg.c_str());
        return 1;
    }
    return 0;
}
