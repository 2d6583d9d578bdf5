// Host-built scoring tables (see tables.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace gepi {

// Fraction bits F of the fixed-point n*log2(n) table for counts up to n_max.
int tfix_bits(int64_t n_max);
// T[n] = n * round(log2(n) * 2^F), n in [0, n_max].
void build_tfix(int64_t n_max, int F, std::vector<uint64_t> &T);
// lf[n] = log(n!) in double and float.
void build_lfact(int64_t n_max, std::vector<double> &lf, std::vector<float> &lf32);
// Natural-log two-sided Fisher p-value of (n11 n12 / n21 n22).
double fisher_lnp_host(int n11, int n12, int n21, int n22);

}  // namespace gepi
