// Laguerre cell clipping kernels (declarations).
#pragma once

#include "gbv_grid.cuh"

namespace gbv {

// Capacities of the two kernel shapes.  The small one runs every cell; the
// large one runs the few cells whose polytope overflows the small one.
constexpr int kSmallT = 64, kSmallP = 32;
constexpr int kLargeT = 128, kLargeP = 64;
constexpr int kMaxFacets = kLargeP;  // facet slots per cell in the outputs

struct ClipArgs {
  SortedSeeds S;
  // neighbour lists: list r of query qi at nbr[r * nbr_stride + qi]
  const uint32_t* nbr;
  uint32_t nbr_stride;
  const uint32_t* nbr_cnt;    // [nq]; bit 31 = lower-index duplicate
  uint32_t list_k;            // capacity of the lists
  uint32_t n_total;           // number of seeds
  const uint32_t* qlist;      // sorted slots to process (nullptr: all)
  const uint32_t* qrow;       // list row of each query (nullptr: row = qi)
  uint32_t nq;
  double box[6];              // xmin ymin zmin xmax ymax zmax
  int check_sr;
  // outputs indexed by sorted slot
  int32_t* status;
  double* vol;
  double* mg;                 // [3][n] (component-major)
  uint32_t* nf;               // facets between seeds
  uint32_t* nclip;            // neighbours visited
  uint32_t* f_nbr;            // [kMaxFacets][n] original index
  double* f_area;             // [kMaxFacets][n]
  uint32_t out_stride;        // n
  // per-call counters: [0] exact predicate calls, [1] max clips
  unsigned long long* counters;
};

enum ClipShape : int { CLIP_SMALL = 0, CLIP_LARGE = 1 };

// Error of the last clipping launch (launch configuration errors are not
// sticky, so the orchestration checks this after every launch).
extern cudaError_t last_launch_error;

// FP64 clipping (exact conflict signs).
void launch_clip_fp64(const ClipArgs& a, int shape, cudaStream_t st);
// FP32 clipping with certified signs and FP64 geometry; cells that FP32
// cannot certify get status GBV_CELL_RECHECK.
void launch_clip_fp32(const ClipArgs& a, cudaStream_t st);

}  // namespace gbv
