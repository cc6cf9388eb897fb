// Laguerre cell clipping and geometry kernels (declarations).
#pragma once

#include "gbv_grid.cuh"

namespace gbv {

// Capacities of the two clipping shapes.  The small one runs every cell;
// the large one runs the few cells whose polytope overflows the small one.
constexpr int kSmallT = 64, kSmallP = 32;
constexpr int kLargeT = 128, kLargeP = 64;
constexpr int kTMax = kLargeT, kPMax = kLargeP;
constexpr int kMaxFacets = kLargeP;   // facet slots per cell in the outputs
constexpr uint32_t kBoxBase = 0xFFFFFF00u;  // plane owner of box face b: kBoxBase + b

// Combinatorics of the clipped cells, one record per sorted slot, written
// by the clipping kernels and read by the geometry kernel.
struct CombBuf {
  uint32_t* tv;     // [n][kTMax] plane slots of each triangle, i | j<<8 | k<<16
  uint32_t* ta;     // [n][kTMax] adjacent triangles across edges opposite i, j, k
  int16_t* key;     // [n][kTMax] stored list-order key (effective = parity * key)
  uint32_t* pown;   // [n][kPMax] plane owner: seed slot or kBoxBase + face
  uint16_t* prank;  // [n][kPMax] position of the plane's seed in the neighbour list
  ulonglong2* tmask;  // [n] used triangle slots (bits 0-63, 64-127)
  uint64_t* pmask;    // [n] used plane slots
  uint32_t* flags;    // [n] bit 0: parity is -1; bit 1: bits 8-31 hold the
                      // number of list positions the polytope has clipped
};

struct ClipArgs {
  SortedSeeds S;
  // neighbour lists: list position r of list row `row` at nbr[r * nbr_stride + row]
  const uint32_t* nbr;
  uint32_t nbr_stride;
  const uint32_t* nbr_cnt;    // per row; bit 31 = lower-index duplicate
  uint32_t list_k;            // capacity of the lists
  uint32_t n_total;           // number of seeds
  uint32_t k0;                // first list length asked (reference_list_cap)
  const uint32_t* qlist;      // sorted slots to process (nullptr: all)
  const uint32_t* qrow;       // list row of each query (nullptr: row = qi)
  uint32_t nq;
  double box[6];              // xmin ymin zmin xmax ymax zmax
  int check_sr;
  int fast_pred;              // 1: the reference's inexact predicates (gbv_predicates)
  int32_t* status;            // by sorted slot
  uint32_t* nclip;            // by sorted slot: neighbours visited
  CombBuf comb;
  unsigned long long* counters;  // [0] exact predicate calls, [1] max clips,
                                 // [2] conflict tests, [3] corners created
  // set (nonzero) by the first cell clipped away entirely; the cells not
  // started yet are then skipped (null: off).  An empty cell in this pass
  // is empty for good: a caller that rejects any empty cell stops here.
  unsigned int* abort_on_empty;
  // nonzero: a cell whose record in `comb` holds the polytope of the first
  // d <= (its list length) positions of its list continues from there (the
  // caller keeps the records of earlier passes over the same seeds and
  // lists that only grew at their end, and clears the flags otherwise)
  int resume;
};

enum ClipShape : int { CLIP_SMALL = 0, CLIP_LARGE = 1 };

// Error of the last launch of this module (launch configuration errors are
// not sticky, so the orchestration checks this after every launch).
extern cudaError_t last_launch_error;

// FP64 clipping (exact conflict signs).
void launch_clip_fp64(const ClipArgs& a, int shape, cudaStream_t st);
// FP32 clipping with certified signs.  A sign the FP32 bound cannot decide
// is taken exactly from the FP64 planes when exact_fallback is set (always
// for the large shape), else the cell gets status GBV_CELL_RECHECK; so do
// cells whose security-radius stop FP32 cannot certify.
void launch_clip_fp32(const ClipArgs& a, int shape, bool exact_fallback, cudaStream_t st);

struct GeomArgs {
  SortedSeeds S;
  const uint32_t* nbr;        // the lists the cells were clipped with
  uint32_t nbr_stride;
  const uint32_t* qlist;      // sorted slots (nullptr: all)
  const uint32_t* qrow;
  uint32_t nq;
  double box[6];
  int verify_sr;              // FP32 clipping: check its stops in FP64
  int shape;                  // ClipShape of the clipping pass
  int g32;                    // FP32 corners, tetrahedra and facet triangles
                              // (security-radius cells only)
  CombBuf comb;
  int32_t* status;
  const uint32_t* nclip;
  // outputs by sorted slot
  double* vol;
  double* mg;                 // [3][n]
  uint32_t* nf;
  uint32_t* f_nbr;            // [kMaxFacets][n] original index
  double* f_area;             // [kMaxFacets][n]
  uint32_t out_stride;
  // Cell-centred certification (off when node_wmax is null): every seed
  // that could still cut the cell and is not in its candidate list is
  // written to extra[k * nbr_stride + row], k < max_extra (row: the cell's
  // list row), and counted in extra_cnt[row] (bit 31: more were found than
  // fit).
  const double* node_wmax;
  const double4* node_lin;    // per-node linear weight bound (a, g) and its excess
  const double* node_ex;      //   (build_node_linear); may be null
  // the same rounded to FP32 once per call (the walk compares in FP32)
  const float* node_wmax_f;
  const float4* node_lin_f;
  const float* node_ex_f;
  const uint32_t* cand_cnt;   // candidate list lengths, per list row
  uint32_t* extra;
  uint32_t* extra_cnt;
  uint32_t max_extra;
  // optional certification counters: [0] nodes, [1] seeds scanned, [2] max
  // nodes of one cell, [3] max seeds of one cell, [4] cells
  unsigned long long* cert_stats;
};

// FP64 geometry of the final cells, one warp per cell, with the reference's
// formulas and summation order.
void launch_geometry(const GeomArgs& a, cudaStream_t st);

// Cells beyond the large shape: one single-thread block per cell, polytope in global
// memory (kHugeT corners, kHugeV planes), clipping and geometry in one
// kernel.  Their facets go to a separate area: nf[slot] carries
// kHugeFacets and hp_nbr[slot] / hp_area[slot] point at the cell's
// neighbours and areas.
constexpr uint32_t kHugeT = 4096, kHugeV = 2048;
constexpr uint32_t kHugeFacets = 0x80000000u;

struct HugeArgs {
  SortedSeeds S;
  const uint32_t* nbr;
  uint32_t nbr_stride;
  const uint32_t* nbr_cnt;
  uint32_t list_k;
  uint32_t n_total;
  uint32_t k0;
  const uint32_t* qlist;      // sorted slots (required)
  const uint32_t* qrow;       // list rows (nullptr: row = qi)
  uint32_t nq;
  double box[6];
  int check_sr;
  int fast_pred;
  int32_t* status;
  uint32_t* nclip;
  unsigned long long* counters;
  // scratch, per query: [nq][kHugeT] and [nq][kHugeV]
  ushort4* scr_t;
  ushort4* scr_adj;
  double4* scr_cor;
  float* scr_eps;
  double4* scr_pl;
  uint32_t* scr_vg;
  uint16_t* scr_v2t;
  uint8_t* scr_v2e;
  // outputs by sorted slot (as GeomArgs) and the facet area [nq][kHugeV]
  double* vol;
  double* mg;
  uint32_t* nf;
  uint32_t out_stride;
  uint32_t* fac_nbr;
  double* fac_area;
  uint32_t** hp_nbr;
  double** hp_area;
  // certification (as GeomArgs; off when node_wmax is null)
  const double* node_wmax;
  const double4* node_lin;
  const double* node_ex;
  uint32_t* extra;
  uint32_t* extra_cnt;
  uint32_t max_extra;
  // optional per-query counters (kHugeStats each): cycles of the clipping,
  // geometry and certification phases, clips, conflict tests, triangles,
  // planes, octree nodes and seeds visited by the certification
  unsigned long long* stats;
};
constexpr int kHugeStats = 9;

void launch_huge(const HugeArgs& a, cudaStream_t st);

}  // namespace gbv
