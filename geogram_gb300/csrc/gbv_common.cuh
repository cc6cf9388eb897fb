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
  CELL_NEED_MORE_K = GBV_CELL_NEED_MORE_K,  // list exhausted (internal, retried)
  CELL_OVERFLOW = GBV_CELL_OVERFLOW,        // capacity exceeded (internal, retried)
  CELL_RECHECK = GBV_CELL_RECHECK,          // FP32 could not certify (internal)
  CELL_ERROR = GBV_CELL_ERROR,              // inconsistent polytope (reported)
};

constexpr uint32_t kNone = 0xFFFFFFFFu;

// Host-side count of this library's kernel launches (gbv_kernel_launches).
void count_launch();

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
