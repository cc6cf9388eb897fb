// Separable starting weights for the optimal-transport solver (declarations).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gbv {

// Length of the padded sort (the power of two >= n) and number of prefix-sum
// chunks for n seeds: the scratch separable_start needs is key[len] (double),
// val[len] (uint32) and chunk[chunks] (double).
size_t start_sort_len(uint32_t n);
size_t start_chunks(uint32_t n);

// w[i] = |p_i|^2 - 2 sum_a Phi_a(p_ia) for the n seeds xyz[3n] in the box
// [lo, hi]; Phi_a' is the piecewise-linear empirical CDF of axis a mapped
// onto [lo_a, hi_a].  Deterministic; not centred.
void separable_start(const double* xyz, uint32_t n, const double lo[3], const double hi[3],
                     double* key, uint32_t* val, double* chunk, double* w, cudaStream_t st);

}  // namespace gbv
