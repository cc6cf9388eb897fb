// Separable starting weights for the optimal-transport solver.
//
// w_i = |p_i|^2 - 2 sum_a Phi_a(p_ia), where Phi_a' = F_a interpolates axis
// a's empirical CDF linearly (the seed of rank k maps to
// lo_a + (k + 1/2) / n (hi_a - lo_a)).  For product measures grad phi,
// phi = sum_a Phi_a, is the Brenier map onto the uniform box.  phi is convex
// and grad phi(p_i) lies strictly inside the box, so no cell of distinct
// seeds is empty: seed i's cell is where x.p_i - phi(p_i) is largest over
// the seeds (the power distance |x - p|^2 - w rearranged), and at
// x = grad phi(p_i) convexity makes every other seed strictly smaller.
// The reference has no counterpart: its solver starts from zero weights.
//
// Per axis the coordinates are sorted with their indices (a bitonic network,
// ties broken by index, padded to a power of two with +inf); with s_k the
// sorted coordinates and P_k their exclusive prefix sum, summation by parts
// gives
//   Phi_k = sum_{m<k} (s_{m+1} - s_m) (F_m + F_{m+1}) / 2
//         = lo (s_k - s_0) + (hi - lo) (k s_k - P_k) / n,
// and w[index_k] -= 2 Phi_k.  The prefix sum runs over fixed chunks in a
// fixed order, so the weights are the same from run to run.
#include "gbv_start.cuh"

#include <cmath>

#include "gbv_common.cuh"

namespace gbv {

namespace {

constexpr uint32_t kStartChunk = 256;
constexpr unsigned kStartThreads = 256;

unsigned grid_for(size_t n) { return (unsigned)((n + kStartThreads - 1) / kStartThreads); }

__global__ void norm2_kernel(const double* __restrict__ xyz, uint32_t n, double* __restrict__ w) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  w[i] = x * x + y * y + z * z;
}

// Coordinate a of every seed with its index; +inf past n.
__global__ void load_axis_kernel(const double* __restrict__ xyz, uint32_t n, size_t m, int a,
                                 double* __restrict__ key, uint32_t* __restrict__ val) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  key[i] = i < n ? xyz[3 * i + a] : INFINITY;
  val[i] = i < n ? (uint32_t)i : 0xffffffffu;
}

// One compare-exchange stage of the bitonic network: distance j inside
// sequences of length k, ascending where (i & k) == 0.  m is a power of two,
// so the partner i ^ j of i < m is below m.
__global__ void bitonic_kernel(double* __restrict__ key, uint32_t* __restrict__ val, size_t m,
                               size_t j, size_t k) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const size_t l = i ^ j;
  if (l <= i) return;
  const double a = key[i], b = key[l];
  const uint32_t va = val[i], vb = val[l];
  const bool greater = a > b || (a == b && va > vb);
  if (greater == ((i & k) == 0)) {
    key[i] = b;
    key[l] = a;
    val[i] = vb;
    val[l] = va;
  }
}

// Sum of each chunk of the sorted coordinates, in order.
__global__ void chunk_sum_kernel(const double* __restrict__ s, uint32_t n, uint32_t nchunks,
                                 double* __restrict__ chunk) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nchunks) return;
  const size_t b = (size_t)t * kStartChunk, e = min((size_t)n, b + kStartChunk);
  double acc = 0.0;
  for (size_t k = b; k < e; ++k) acc += s[k];
  chunk[t] = acc;
}

// Exclusive prefix sum of the chunk sums, in place, in order (one thread).
__global__ void chunk_scan_kernel(double* __restrict__ chunk, uint32_t nchunks) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double acc = 0.0;
  for (uint32_t t = 0; t < nchunks; ++t) {
    const double v = chunk[t];
    chunk[t] = acc;
    acc += v;
  }
}

// w[index_k] -= 2 Phi_k along each chunk.
__global__ void phi_kernel(const double* __restrict__ s, const uint32_t* __restrict__ idx,
                           uint32_t n, uint32_t nchunks, const double* __restrict__ chunk,
                           double lo, double span, double* __restrict__ w) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nchunks) return;
  const size_t b = (size_t)t * kStartChunk, e = min((size_t)n, b + kStartChunk);
  const double s0 = s[0], inv_n = 1.0 / (double)n;
  double P = chunk[t];
  for (size_t k = b; k < e; ++k) {
    const double sk = s[k];
    const double phi = lo * (sk - s0) + span * (((double)k * sk - P) * inv_n);
    const uint32_t i = idx[k];
    if (i < n) w[i] -= 2.0 * phi;  // always true for finite coordinates
    P += sk;
  }
}

}  // namespace

size_t start_sort_len(uint32_t n) {
  size_t m = 1;
  while (m < n) m <<= 1;
  return m;
}

size_t start_chunks(uint32_t n) { return ((size_t)n + kStartChunk - 1) / kStartChunk; }

void separable_start(const double* xyz, uint32_t n, const double lo[3], const double hi[3],
                     double* key, uint32_t* val, double* chunk, double* w, cudaStream_t st) {
  const size_t m = start_sort_len(n);
  const uint32_t nch = (uint32_t)start_chunks(n);
  norm2_kernel<<<grid_for(n), kStartThreads, 0, st>>>(xyz, n, w); count_launch();
  for (int a = 0; a < 3; ++a) {
    load_axis_kernel<<<grid_for(m), kStartThreads, 0, st>>>(xyz, n, m, a, key, val); count_launch();
    for (size_t k = 2; k <= m; k <<= 1)
      for (size_t j = k >> 1; j > 0; j >>= 1) {
        bitonic_kernel<<<grid_for(m), kStartThreads, 0, st>>>(key, val, m, j, k); count_launch();
      }
    chunk_sum_kernel<<<grid_for(nch), kStartThreads, 0, st>>>(key, n, nch, chunk); count_launch();
    chunk_scan_kernel<<<1, 1, 0, st>>>(chunk, nch); count_launch();
    phi_kernel<<<grid_for(nch), kStartThreads, 0, st>>>(key, val, n, nch, chunk, lo[a],
                                                       hi[a] - lo[a], w); count_launch();
  }
}

}  // namespace gbv
