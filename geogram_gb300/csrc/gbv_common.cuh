// Shared device helpers for the GB300 Laguerre cell engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbv.h"

namespace gbv {

// ---------------------------------------------------------------------
// Per-cell status codes (written to the caller's cell_status array).
// The first four mirror the outcomes of the reference's security-radius
// loop (generic_RVD.h:2278-2352) composed with delaunay_nn.cpp:104-145.
// ---------------------------------------------------------------------
enum CellStatus : int32_t {
  CELL_CERTIFIED = GBV_CELL_CERTIFIED,      // stopped by d2 > 4.1 R2
  CELL_ALL_NEIGHBOURS = GBV_CELL_ALL_NEIGHBOURS,  // every other seed clipped
  CELL_DUPLICATE = GBV_CELL_DUPLICATE,      // a lower-index duplicate exists
  CELL_STALLED = GBV_CELL_STALLED,          // list growth stalled (copies)
  CELL_NEED_MORE_K = GBV_CELL_NEED_MORE_K,  // list exhausted (internal, retried)
  CELL_OVERFLOW = GBV_CELL_OVERFLOW,        // capacity exceeded (internal, retried)
  CELL_RECHECK = GBV_CELL_RECHECK,          // FP32 could not certify (internal)
  CELL_ERROR = GBV_CELL_ERROR,              // inconsistent polytope (reported)
};

constexpr uint32_t kNone = 0xFFFFFFFFu;

// Neighbour-list counts carry, besides the length (bits 0-23), the number of
// higher-index copies of the seed (bits 24-30) and a lower-index copy flag
// (bit 31).
constexpr uint32_t kCntMask = 0x00FFFFFFu;
__host__ __device__ __forceinline__ uint32_t pack_cnt(uint32_t cnt, uint32_t copies, bool lower) {
  return lower ? 0x80000000u : ((cnt & kCntMask) | ((copies > 127u ? 127u : copies) << 24));
}

// Longest list the reference's security-radius loop will ever clip for a
// seed with m > 0 higher-index copies.  Delaunay_NearestNeighbors asks for
// k + 1 points and drops the seed and its copies (delaunay_nn.cpp:104-145),
// so every list is m shorter than asked; clip_by_cell_SR grows k by k/8
// (k > 8) or 1 (generic_RVD.h:2332-2345) and stops when a list did not grow
// (:2297-2299).  Returns the list length at which that happens.
__host__ __device__ inline uint32_t reference_list_cap(uint32_t k0, uint32_t n, uint32_t m,
                                                       bool check_sr) {
  const uint32_t nm1 = n - 1;
  auto listlen = [&](uint32_t asked) -> uint32_t {
    const uint32_t got = (asked + 1 < n ? asked + 1 : n) - 1;  // minus the seed
    return got > m ? got - m : 0u;
  };
  uint32_t a = listlen(k0 < nm1 ? k0 : nm1);
  if (!check_sr) return a;
  for (int it = 0; it < 64; ++it) {
    uint32_t g = a > 8 ? a + a / 8 : a + 1;
    if (g > nm1) g = nm1;
    const uint32_t a2 = listlen(g);
    if (a2 <= a) return a;
    a = a2;
  }
  return a;
}

// Host-side count of this library's kernel launches (gbv_kernel_launches).
void count_launch();
// Sets the calling thread's gbv_last_error() message.
void set_last_error(const char* msg);

// Exact FP64 squared distance with the reference's evaluation order
// (geometry_nd.h:65-73): ((((0 + dx^2) + dy^2) + dz^2) + dh^2), no fusion.
__device__ __forceinline__ double dist2_exact(double4 a, double4 b) {
  double dx = __dsub_rn(b.x, a.x), dy = __dsub_rn(b.y, a.y);
  double dz = __dsub_rn(b.z, a.z), dh = __dsub_rn(b.w, a.w);
  double r = __dmul_rn(dx, dx);
  r = __dadd_rn(r, __dmul_rn(dy, dy));
  r = __dadd_rn(r, __dmul_rn(dz, dz));
  r = __dadd_rn(r, __dmul_rn(dh, dh));
  return r;
}

// 3-bit interleave helpers for 30-bit Morton codes (x in bit 0).
__host__ __device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__host__ __device__ __forceinline__ uint32_t compact3(uint32_t v) {
  v &= 0x09249249u;
  v = (v | (v >> 2)) & 0x030C30C3u;
  v = (v | (v >> 4)) & 0x0300F00Fu;
  v = (v | (v >> 8)) & 0x030000FFu;
  v = (v | (v >> 16)) & 0x3FFu;
  return v;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

// Grid over the seeds' bounding box: G = 2^L fine cells per axis, fine
// cells numbered in Morton order so that every octree node at level l is a
// contiguous range of fine cells, hence of sorted seeds.
struct GridDesc {
  double lo[3];
  double h;        // fine cell edge
  double inv_h;
  float lo_f[3];
  float h_f;
  int L;           // levels
  int G;           // 1 << L
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}

}  // namespace gbv
