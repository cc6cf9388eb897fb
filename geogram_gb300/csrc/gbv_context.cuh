// The context behind the C ABI's gbv_context handle (device buffers, the
// stream, the last cell results) and the error types the entry points turn
// into status codes.  Shared by the .cu files that implement entry points.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <string>

#include "gbv_clip.cuh"

namespace gbv {

struct CudaError {
  cudaError_t e;
  std::string where;
};

#define GBV_CUDA(call)                                                     \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) throw ::gbv::CudaError{e_, #call};              \
  } while (0)

struct StatusError {
  gbv_status st;
  std::string msg;
};

}  // namespace gbv

struct gbv_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  std::map<std::string, std::pair<void*, size_t>> bufs;

  gbv::SortedSeeds S;
  gbv::GridScratch scr;
  unsigned long long* counters = nullptr;  // [0] exact calls [1] max clips
                                           // [2] conflict tests [3] corners created
  uint32_t* list_counts = nullptr;         // [4] classification counters
  uint32_t* h_counts = nullptr;            // pinned mirror
  unsigned long long* h_clipc = nullptr;   // pinned: first clipping pass's tests, corners

  // last cell results, caller order; their combinatorics stay in the
  // arena's cb_* buffers (by sorted slot) until the seeds are re-sorted
  uint32_t n = 0;
  uint64_t nnz = 0;
  bool has_cells = false;
  double* vol = nullptr;
  double* mg = nullptr;
  uint32_t* rowptr = nullptr;
  uint32_t* nbr = nullptr;
  double* area = nullptr;
  int32_t* status = nullptr;
  double box[6] = {0.0, 0.0, 0.0, 1.0, 1.0, 1.0};  // the clipping box of the last cells
  // last periodic cells: the first per_n cells above are the original
  // seeds; their facets' seeds and image translations
  bool has_periodic = false;
  uint32_t per_n = 0, per_nnz = 0;
  uint32_t* per_nbr = nullptr;
  uint8_t* per_shift = nullptr;

  // nearest-neighbour search state
  bool nn_ready = false;
  uint32_t nn_n = 0, nn_dim = 3;

  template <class T>
  T* buf(const std::string& name, size_t count) {
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    auto it = bufs.find(name);
    if (it != bufs.end() && it->second.second >= bytes) return (T*)it->second.first;
    if (it != bufs.end()) {
      GBV_CUDA(cudaFree(it->second.first));
      bufs.erase(it);
    }
    void* p = nullptr;
    GBV_CUDA(cudaMalloc(&p, bytes));
    bufs[name] = {p, bytes};
    size_t total = 0;
    for (const auto& kv : bufs) total += kv.second.second;
    peak_bytes = std::max(peak_bytes, total);
    return (T*)p;
  }
  size_t peak_bytes = 0;  // most device memory the arena held at once
};

namespace gbv {
// Cells restricted to a tetrahedral mesh (gbv_restrict.cu), after a cell
// computation on the mesh's bounding box; device arrays.
void restricted_cells(gbv_context* c, const double* d_xyz, const double* d_w, uint32_t n,
                      const double* d_mv, uint32_t nv, const uint32_t* d_tets, uint32_t nt,
                      cudaStream_t st, double* d_m, double* d_mg, double* d_F, double* d_g);
}  // namespace gbv

namespace gbv {
// Periodic cells (gbv_periodic.cu): the seeds and their ghost images in
// the layer of width delta (returns the augmented count), the original
// cells whose security ball leaves the ghost box, and the originals'
// facets as (seed, translation code).
uint32_t periodic_ghosts(gbv_context* c, const double* d_xyz, const double* d_w, uint32_t n,
                         double P, double delta, cudaStream_t st, double** aug_xyz,
                         double** aug_w);
uint32_t periodic_reach_failures(gbv_context* c, uint32_t n, const double* aug_xyz,
                                 const double* aug_w, double W, double P, double delta,
                                 cudaStream_t st);
void periodic_remap(gbv_context* c, uint32_t n, cudaStream_t st, uint32_t** out_nbr,
                    uint8_t** out_shift, uint32_t* nnz);
}  // namespace gbv
