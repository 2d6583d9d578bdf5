// Host-built scoring tables and the host Fisher test.
//
// Entropy ranking uses T(n) = n * round(log2(n) * 2^F), an integer table whose
// log2 is computed with integer arithmetic only (64 fraction bits by repeated
// squaring), so every host builds the same bits.  With it the numerator
// m * I(F;C) * 2^F of any 2x2 table is an exact integer sum: mathematically
// equal tables tie exactly and the ranking is reproducible on CPU and GPU.
//
// Fisher uses log(n!) (lgamma) tables; gepi_fisher_pval replaces the reference's
// host fisher_pval (src/misc/fisher_p.c:52-76) used when printing.
#include <cmath>
#include <cstdint>
#include <vector>

#include "common.h"
#include "tables.h"

namespace gepi {

int tfix_bits(int64_t n_max) {
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

// round(log2(n) * 2^F) with log2 from 64 fraction bits (repeated squaring of
// the mantissa in Q1.63, truncating each square).
static uint64_t log2_fixed(uint64_t n, int F) {
    if (n <= 1) return 0;
    int e = 63 - __builtin_clzll(n);
    uint64_t x = n << (63 - e);
    uint64_t frac = 0;
    for (int i = 1; i <= 64; ++i) {
        unsigned __int128 sq = (unsigned __int128)x * x;
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

void build_tfix(int64_t n_max, int F, std::vector<uint64_t> &T) {
    T.resize((size_t)n_max + 1);
    for (int64_t n = 0; n <= n_max; ++n) T[(size_t)n] = (uint64_t)n * log2_fixed((uint64_t)n, F);
}

void build_lfact(int64_t n_max, std::vector<double> &lf, std::vector<float> &lf32) {
    lf.resize((size_t)n_max + 1);
    lf32.resize((size_t)n_max + 1);
    for (int64_t n = 0; n <= n_max; ++n) {
        double v = std::lgamma((double)n + 1.0);
        lf[(size_t)n] = v;
        lf32[(size_t)n] = (float)v;
    }
}

// Host two-sided Fisher test, natural-log p.  Same summation rule as the
// device (terms with P(x) <= P(obs)(1 + 1e-7)), evaluated over the whole
// support in log space: the tail sum is taken relative to P(obs) and the
// normaliser relative to the largest term, so p far below 1e-308 stays finite
// (the reference's linear-space sum prints -inf there).
double fisher_lnp_host(int n11, int n12, int n21, int n22) {
    if (n11 < 0 || n12 < 0 || n21 < 0 || n22 < 0) return NAN;
    const int r1 = n11 + n21, r2 = n12 + n22, c1 = n11 + n12, N = r1 + r2;
    const int lo = c1 <= r2 ? 0 : c1 - r2;
    const int hi = c1 < r1 ? c1 : r1;
    if (lo >= hi) return 0.0;
    auto lfa = [](int n) { return std::lgamma((double)n + 1.0); };
    const double K = lfa(r1) + lfa(r2) + lfa(c1) + lfa(N - c1) - lfa(N);
    auto lpx = [&](int x) { return K - lfa(x) - lfa(r1 - x) - lfa(c1 - x) - lfa(r2 - c1 + x); };
    const double lpo = lpx(n11);
    const double lim = lpo + std::log1p(1e-7);
    std::vector<double> l((size_t)(hi - lo + 1));
    double lmax = lpo;
    for (int x = lo; x <= hi; ++x) {
        l[(size_t)(x - lo)] = lpx(x);
        if (l[(size_t)(x - lo)] > lmax) lmax = l[(size_t)(x - lo)];
    }
    double num = 0.0, den = 0.0;
    bool all = true;
    for (int x = lo; x <= hi; ++x) {
        const double v = l[(size_t)(x - lo)];
        den += std::exp(v - lmax);
        if (v <= lim) num += std::exp(v - lpo);
        else all = false;
    }
    // every term of the support qualifies: p = 1 exactly (the reference's
    // linear-space ratio of two equal sums prints 0 there)
    if (all) return 0.0;
    double r = lpo + std::log(num) - (lmax + std::log(den));
    return r > 0.0 ? 0.0 : r;
}

}  // namespace gepi

extern "C" double gepi_fisher_log10p(int n11, int n12, int n21, int n22) {
    return gepi::fisher_lnp_host(n11, n12, n21, n22) / std::log(10.0);
}

extern "C" float gepi_fisher_pval(int n11, int n12, int n21, int n22) {
    return (float)gepi_fisher_log10p(n11, n12, n21, n22);
}
