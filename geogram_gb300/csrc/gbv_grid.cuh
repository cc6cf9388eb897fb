// Grid build and kNN search (declarations shared by the .cu files).
#pragma once

#include "gbv_common.cuh"

namespace gbv {

// Seeds re-ordered by fine grid cell (Morton order), one record per slot.
struct SortedSeeds {
  double4* xd = nullptr;  // (x, y, z, h): h = sqrt(W - w), 0 for Voronoi
  double* q = nullptr;    // w - |p|^2 with the reference's arithmetic
  float4* xf = nullptr;   // (x, y, z, h) rounded to FP32
  float4* xl = nullptr;   // FP32 remainders: x = xf + xl to about 2^-48 |x|
  float2* wf = nullptr;   // weight as FP32 (value, remainder); nullptr: Voronoi
  double* ws = nullptr;   // weights by slot (nullptr for Voronoi)
  uint32_t* perm = nullptr;   // slot -> original index
  uint32_t* slot_of = nullptr;  // original index -> slot
  uint32_t* cell_start = nullptr;  // G^3 + 1 entries
  GridDesc* gd = nullptr;   // device: grid descriptor
  double* aux = nullptr;    // device: [0] W = max w, [1] max |coordinate|, [2] largest
                            // squared lift difference, [3] unused
  uint32_t n = 0;
  int L = 0;
};

// Scratch owned by the caller (the context's arena).
struct GridScratch {
  uint32_t* cid = nullptr;     // n
  uint32_t* rank = nullptr;    // n
  uint32_t* scan_tmp = nullptr;
  size_t scan_tmp_elems = 0;
  double* red = nullptr;       // reduction partials
};

// Exclusive scan of n uint32 values in place; tmp must hold
// scan_tmp_elems(n) entries (1024 values per block, partial sums scanned
// recursively).
constexpr size_t kScanBlockElems = 1024;
constexpr size_t scan_tmp_elems(size_t n) {
  size_t tot = 0;
  while (n > kScanBlockElems) {
    n = (n + kScanBlockElems - 1) / kScanBlockElems;
    tot += n + 1;
  }
  return tot + 1;
}
// Blocks of the bounding-box reduction of build_grid; GridScratch::red holds
// 8 doubles per block.
constexpr int kBboxParts = 120;
void exclusive_scan_u32(uint32_t* data, size_t n, uint32_t* tmp, cudaStream_t st);

// Chooses L from n (about one seed per fine cell, 1 <= L <= 9).
int choose_levels(uint32_t n);

// Builds the sorted seed arrays.  xyz: n points of `stride` doubles,
// w: n weights or nullptr.  Fills S (whose buffers are preallocated,
// cell_start with 8^L + 1 entries) and S.gd / S.aux on the device.
// dim = 4: the 4th coordinate of each point is its lift h (no weights).
void build_grid(const double* xyz, uint32_t stride, uint32_t dim, const double* w,
                uint32_t n, int L, SortedSeeds& S, GridScratch& scr, cudaStream_t st);

// Max weight of the seeds in every node of the implicit octree, all levels:
// level l occupies [node_offset(l), node_offset(l) + 8^l), empty nodes hold
// -inf (weights are 0 for Voronoi diagrams).
__host__ __device__ inline size_t node_offset(int l) {
  return (((size_t)1 << (3 * l)) - 1) / 7;
}
inline size_t node_count(int L) { return node_offset(L + 1); }
void build_node_wmax(const SortedSeeds& S, double* wmax, cudaStream_t st);

// Linear upper bound of the weights per octree node: for every seed j of
// node B (centre m), w_j <= a + g . (p_j - m) + e, with (a, g) the
// least-squares fit of the node's weights and e the largest excess.  For
// any point c it bounds the power of the node's seeds from below:
//   |c - p_j|^2 - w_j >= dist(c + g/2, box)^2 - (c - m) . g - |g|^2 / 4 - a - e.
// lin[node] = (a, gx, gy, gz), ex[node] = e; moments: 14 doubles per node of
// scratch.  Deterministic (fixed combination order; the maxima are
// order-independent).
void build_node_linear(const SortedSeeds& S, double4* lin, double* ex, double* moments,
                       cudaStream_t st);

// True when no seed of the node (box [b, b + side]^3, padded by pad) can
// have power below `best` at corner c by the linear bound (FP32, with a
// margin that only keeps more nodes).
__device__ __forceinline__ bool linear_bound_clears(float cx, float cy, float cz, float best,
                                                    float bx, float by, float bz, float side,
                                                    float pad, const float4& fl, float ge) {
  const float ga = fl.x, gx = fl.y, gy = fl.z, gz = fl.w;
  const float px = cx + 0.5f * gx, py = cy + 0.5f * gy, pz = cz + 0.5f * gz;
  const float dx = fmaxf(fmaxf(bx - pad - px, px - (bx + side + pad)), 0.f);
  const float dy = fmaxf(fmaxf(by - pad - py, py - (by + side + pad)), 0.f);
  const float dz = fmaxf(fmaxf(bz - pad - pz, pz - (bz + side + pad)), 0.f);
  const float d2 = dx * dx + dy * dy + dz * dz;
  const float h = 0.5f * side;
  const float lin = (cx - (bx + h)) * gx + (cy - (by + h)) * gy + (cz - (bz + h)) * gz;
  const float g2 = 0.25f * (gx * gx + gy * gy + gz * gz);
  const float lb = d2 - lin - g2 - ga - ge;
  // rounding of the FP32 copies of a, g, e (g times |p - m| <= side) and of
  // this evaluation
  const float margin = 1e-5f * (fabsf(best) + fabsf(ga) + fabsf(ge) + fabsf(lin) + g2 + d2 +
                                (fabsf(gx) + fabsf(gy) + fabsf(gz)) * side) +
                       1e-7f;
  return lb >= best + margin;
}

enum KnnMode : int {
  KNN_CELLS = 0,  // exclude self and zero-distance seeds (delaunay_nn rule)
  KNN_ALL = 1,    // all stored points, self included (get_nearest_neighbors)
  KNN_QUERY = 2,  // separate query points
};

struct KnnArgs {
  const SortedSeeds* S;
  uint32_t nq;          // number of queries
  const uint32_t* qlist;   // optional list of query slots (KNN_CELLS / ALL)
  const double4* qpts;  // KNN_QUERY: query points (x,y,z,h)
  uint32_t k;
  int mode;
  // optional lower bound per query: only neighbours after (lo_d2, lo_idx)
  // in (d2, original index) order are returned (the next batch of a list)
  const double* lo_d2;
  const uint32_t* lo_idx;
  // outputs, [k][out_stride] slot-major (sorted slots of neighbours)
  uint32_t* nbr;        // may be null if only idx/d2 wanted
  uint32_t out_stride;
  uint32_t* cnt;        // [nq] list lengths (bit 31: lower-index duplicate)
  // optional: (d2, original index) of each query's last returned neighbour
  double* last_d2;
  uint32_t* last_idx;
  // optional exported results in caller order: idx (original indices) and
  // d2, row-major [row][k]; row = perm[slot] (ALL) or query index (QUERY)
  uint32_t* exp_idx;
  double* exp_d2;
  // scratch: global lists for k > kKnnSmemK ([k][nq] each), and the queries
  // the FP32 screening could not settle (count + list, nq entries)
  double* gl_d2;
  uint32_t* gl_slot;
  uint32_t* flag_count;
  uint32_t* flag_list;
  // every stored point as a query, in slot order (qlist null, nq = n): the
  // tiled search may take them, with tile_scratch of
  // knn_tile_scratch_elems(n, L) entries
  bool coherent;
  uint32_t* tile_scratch;
};

// Launches the kNN search.  Every stored point in slot order, k <=
// kKnnMaxK: the tiled FP32 screening with an exact FP64 re-rank, then the
// exact search for the queries it could not settle (needs flag_count /
// flag_list).  Other queries, k <= kKnnSmemK: the same per thread.  Larger
// k: the exact search with global lists gl_d2 / gl_slot (k > kKnnMaxK).
constexpr uint32_t kKnnSmemK = 64;
constexpr uint32_t kKnnMaxK = 128;
size_t knn_tile_scratch_elems(uint32_t n, int L);
void launch_knn(const KnnArgs& a, cudaStream_t st);

}  // namespace gbv
