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
  double* aux = nullptr;    // device: [0] W = max w, [1] max |coordinate|
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
// scan_tmp_elems(n) entries.
size_t scan_tmp_elems(size_t n);
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
};

// Launches the kNN search.  For k <= kKnnSmemK: FP32 screening with an
// exact FP64 re-rank, then the exact search for the queries it could not
// settle (needs flag_count / flag_list).  Larger k: the exact search with
// global lists gl_d2 / gl_slot.
constexpr uint32_t kKnnSmemK = 64;
void launch_knn(const KnnArgs& a, cudaStream_t st);

}  // namespace gbv
