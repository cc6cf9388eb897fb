// C ABI of the cell engine: context, device buffers and the passes that
// take every seed to a certified cell.
//
// A compute call runs, on the context's stream:
//   1. build_grid: bounding box, counting sort of the seeds by Morton cell;
//   2. kNN with a list of 64 (or k0 without the security radius);
//   3. the clipping kernel over all cells (FP64, or FP32 + FP64 geometry);
//   4. the cells FP32 could not certify: FP64 clipping with the same lists;
//   5. cells that overflowed the small capacity: the large FP64 kernel;
//   6. cells whose list ran out before certification: a longer list (x4,
//      up to n - 1) for those cells only, then 4-5 again on them;
//   7. unsort into the caller's order and compact the facets into CSR.
// Steps 4-6 are the security-radius growth of generic_RVD.h:2278-2352:
// since a certified cell does not depend on how long the list was, growing
// the list of the few uncertified cells gives the reference's result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gbv_context.cuh"
#include "gbv_ot.cuh"
#include "gbv_lbfgs.h"
#include "gbv_mlp.cuh"
#include "gbv_start.cuh"

namespace {

thread_local std::string g_last_error;

gbv_status fail(gbv_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

}  // namespace


namespace gbv {

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void set_last_error(const char* msg) { g_last_error = msg; }

// ---------------------------------------------------------------------
// Small kernels of the orchestration
// ---------------------------------------------------------------------

// Collects the queries of a pass whose cell ended with one of the retry
// statuses, with the list row each used.
__global__ void classify_kernel(const uint32_t* __restrict__ qlist,
                                const uint32_t* __restrict__ qrow, uint32_t nq,
                                const int32_t* __restrict__ status, uint32_t* __restrict__ counts,
                                uint32_t* __restrict__ recheck_s, uint32_t* __restrict__ recheck_r,
                                uint32_t* __restrict__ over_s, uint32_t* __restrict__ over_r,
                                uint32_t* __restrict__ morek_s, uint32_t* __restrict__ morek_r) {
  const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= nq) return;
  const uint32_t s = qlist ? qlist[qi] : qi;
  const uint32_t r = qrow ? qrow[qi] : qi;
  const int32_t st = status[s];
  if (st == CELL_RECHECK) {
    uint32_t k = atomicAdd(&counts[0], 1u);
    recheck_s[k] = s;
    recheck_r[k] = r;
  } else if (st == CELL_OVERFLOW) {
    uint32_t k = atomicAdd(&counts[1], 1u);
    over_s[k] = s;
    over_r[k] = r;
  } else if (st == CELL_NEED_MORE_K) {
    uint32_t k = atomicAdd(&counts[2], 1u);
    morek_s[k] = s;
    morek_r[k] = r;
  } else if (st == CELL_ERROR) {
    atomicAdd(&counts[3], 1u);
  }
}

// Starts the extended lists of cells that ran out of neighbours: copies the
// first k entries of each cell's current list and its lower bound.
__global__ void extend_lists_kernel(const uint32_t* __restrict__ rows, uint32_t m,
                                    const uint32_t* __restrict__ old_lists, uint32_t old_stride,
                                    uint32_t k, const double* __restrict__ old_last_d2,
                                    const uint32_t* __restrict__ old_last_idx,
                                    uint32_t* __restrict__ new_lists, double* __restrict__ lo_d2,
                                    uint32_t* __restrict__ lo_idx) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint32_t r = rows[i];
  for (uint32_t j = 0; j < k; ++j) new_lists[(size_t)j * m + i] = old_lists[(size_t)j * old_stride + r];
  lo_d2[i] = old_last_d2[r];
  lo_idx[i] = old_last_idx[r];
}

// Length of an extended list: the k entries copied plus the new batch; the
// copies count of the first list is kept.
__global__ void add_count_kernel(uint32_t* __restrict__ cnt, uint32_t m, uint32_t k,
                                 const uint32_t* __restrict__ rows,
                                 const uint32_t* __restrict__ old_cnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) cnt[i] = pack_cnt(k + (cnt[i] & kCntMask), (old_cnt[rows[i]] >> 24) & 0x7Fu, false);
}

__global__ void facet_count_kernel(const uint32_t* __restrict__ slot_of,
                                   const uint32_t* __restrict__ nf, uint32_t n,
                                   uint32_t* __restrict__ rowptr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) rowptr[i] = nf[slot_of[i]] & ~kHugeFacets;
  if (i == n) rowptr[n] = 0;
}

// Sum of the n per-cell facet counts in 64 bits (the CSR offsets are 32-bit);
// *total must be zero on entry.
__global__ void facet_total_kernel(const uint32_t* __restrict__ counts, uint32_t n,
                                   unsigned long long* __restrict__ total) {
  unsigned long long s = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    s += counts[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0) atomicAdd(total, s);
}

// Unsorts the per-cell results into the caller's order and writes the CSR.
__global__ void unsort_kernel(const uint32_t* __restrict__ slot_of, uint32_t n,
                              const double* __restrict__ vol_s, const double* __restrict__ mg_s,
                              const int32_t* __restrict__ st_s, const uint32_t* __restrict__ nf,
                              const uint32_t* __restrict__ f_nbr,
                              const double* __restrict__ f_area,
                              uint32_t* const* __restrict__ hp_nbr,
                              double* const* __restrict__ hp_area,
                              const uint32_t* __restrict__ rowptr, double* __restrict__ vol,
                              double* __restrict__ mg, int32_t* __restrict__ status,
                              uint32_t* __restrict__ nbr, double* __restrict__ area) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = slot_of[i];
  vol[i] = vol_s[s];
  mg[3 * (size_t)i] = mg_s[s];
  mg[3 * (size_t)i + 1] = mg_s[(size_t)n + s];
  mg[3 * (size_t)i + 2] = mg_s[2 * (size_t)n + s];
  status[i] = st_s[s];
  const uint32_t b = rowptr[i], c = nf[s];
  if (c & kHugeFacets) {
    const uint32_t* hn = hp_nbr[s];
    const double* ha = hp_area[s];
    for (uint32_t f = 0; f < (c & ~kHugeFacets); ++f) {
      nbr[b + f] = hn[f];
      area[b + f] = ha[f];
    }
    return;
  }
  for (uint32_t f = 0; f < c; ++f) {
    nbr[b + f] = f_nbr[(size_t)f * n + s];
    area[b + f] = f_area[(size_t)f * n + s];
  }
}

// Compensated (Neumaier) FP64 sum, deterministic: fixed partition into
// blocks, fixed order inside each block, then one block over the partials.
constexpr int kSumThreads = 256;

__device__ __forceinline__ void neumaier_add(double& s, double& c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x)) c += (s - t) + x;
  else c += (x - t) + s;
  s = t;
}

__global__ void sum_partial_kernel(const double* __restrict__ x, size_t n,
                                   double* __restrict__ part) {
  __shared__ double ss[kSumThreads], sc[kSumThreads];
  double s = 0.0, c = 0.0;
  const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const size_t b = blockIdx.x * chunk, e = min(n, b + chunk);
  for (size_t i = b + threadIdx.x; i < e; i += kSumThreads) neumaier_add(s, c, x[i]);
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0, C = 0.0;
    for (int t = 0; t < kSumThreads; ++t) {
      neumaier_add(S, C, ss[t]);
      C += sc[t];
    }
    part[2 * blockIdx.x] = S;
    part[2 * blockIdx.x + 1] = C;
  }
}

__global__ void sum_final_kernel(const double* __restrict__ part, int np, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double S = 0.0, C = 0.0;
  for (int b = 0; b < np; ++b) {
    neumaier_add(S, C, part[2 * b]);
    C += part[2 * b + 1];
  }
  out[0] = S + C;
}

__global__ void sum_u32_kernel(const uint32_t* __restrict__ x, size_t n,
                               unsigned long long* __restrict__ out) {
  unsigned long long s = 0;
  for (size_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s += x[i];
  s = __reduce_add_sync(0xFFFFFFFFu, (unsigned)min(s, 0xFFFFFFFFull)) ;
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// Lloyd update (CVT.cpp:150-160): x_i <- mg_i / m_i when m_i > 1e-30.
__global__ void lloyd_update_kernel(double* __restrict__ xyz, const double* __restrict__ vol,
                                    const double* __restrict__ mg, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double m = vol[i];
  if (m > 1e-30) {
    xyz[3 * (size_t)i] = mg[3 * (size_t)i] / m;
    xyz[3 * (size_t)i + 1] = mg[3 * (size_t)i + 1] / m;
    xyz[3 * (size_t)i + 2] = mg[3 * (size_t)i + 2] / m;
  }
}

__global__ void to_query4_kernel(const double* __restrict__ q, uint32_t nq, uint32_t dim,
                                 double4* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  out[i] = make_double4(q[(size_t)i * dim], q[(size_t)i * dim + 1], q[(size_t)i * dim + 2],
                        dim == 4 ? q[(size_t)i * dim + 3] : 0.0);
}

// ---------------------------------------------------------------------
// Host helpers
// ---------------------------------------------------------------------

static void setup_seeds(gbv_context* c, uint32_t n, bool weighted) {
  const int L = choose_levels(n);
  SortedSeeds& S = c->S;
  S.xd = c->buf<double4>("xd", n);
  S.q = c->buf<double>("q", n);
  S.xf = c->buf<float4>("xf", n);
  S.xl = c->buf<float4>("xl", n);
  S.wf = weighted ? c->buf<float2>("wf", n) : nullptr;
  S.ws = weighted ? c->buf<double>("ws", n) : nullptr;
  S.perm = c->buf<uint32_t>("perm", n);
  S.slot_of = c->buf<uint32_t>("slot_of", n);
  S.cell_start = c->buf<uint32_t>("cell_start", ((size_t)1 << (3 * L)) + 1);
  S.gd = c->buf<GridDesc>("gd", 1);
  S.aux = c->buf<double>("aux", 4);
  S.L = L;
  c->scr.cid = c->buf<uint32_t>("cid", n);
  c->scr.rank = c->buf<uint32_t>("rank", n);
  c->scr.scan_tmp_elems = scan_tmp_elems(((size_t)1 << (3 * L)) + 1);
  c->scr.scan_tmp = c->buf<uint32_t>("scan_tmp", c->scr.scan_tmp_elems);
  c->scr.red = c->buf<double>("red", 8 * (size_t)kBboxParts);
}

static inline unsigned nblocks(size_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

struct CellsTiming {
  float grid = 0, knn = 0, clip = 0, total = 0;
};

// One list buffer: lists[r * stride + row], counts and the exact (d2, index)
// of each row's last entry (the lower bound of the next batch).
struct ListSet {
  const uint32_t* lists = nullptr;
  uint32_t stride = 0;
  const uint32_t* cnt = nullptr;
  uint32_t k = 0;
  const double* last_d2 = nullptr;
  const uint32_t* last_idx = nullptr;
};

// Order of candidates in Laguerre mode: twice the distance from the seed
// to the power bisector, (|d|^2 + w_i - w_j) / |d|, ties by original index.
// Clipping the nearest planes first keeps the intermediate polytopes small.
__device__ __forceinline__ float plane_key(const double4& pi, double wi, const double4& pj,
                                           double wj) {
  const float dx = (float)(pj.x - pi.x), dy = (float)(pj.y - pi.y), dz = (float)(pj.z - pi.z);
  const float d2 = dx * dx + dy * dy + dz * dz;
  return (d2 + (float)(wi - wj)) * rsqrtf(fmaxf(d2, 1e-30f));
}

__device__ __forceinline__ bool key_less(float ka, uint32_t oa, float kb, uint32_t ob) {
  return ka < kb || (ka == kb && oa < ob);
}

// Cells with extra candidates from the certification: their slots, list
// rows and counts.
// FP32 copies of the per-node weight bounds (the certification compares in FP32).
__global__ void node_bounds_f32_kernel(const double* __restrict__ wmax,
                                       const double4* __restrict__ lin,
                                       const double* __restrict__ ex, uint32_t m,
                                       float* __restrict__ wf, float4* __restrict__ lf,
                                       float* __restrict__ ef) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  wf[i] = (float)wmax[i];
  if (lin) {
    const double4 l = lin[i];
    lf[i] = make_float4((float)l.x, (float)l.y, (float)l.z, (float)l.w);
    ef[i] = (float)ex[i];
  }
}

__global__ void collect_extra_kernel(const uint32_t* __restrict__ qlist, uint32_t nq,
                                     const uint32_t* __restrict__ extra_cnt,
                                     const int32_t* __restrict__ status,
                                     uint32_t* __restrict__ count, uint32_t* __restrict__ out_s,
                                     uint32_t* __restrict__ out_r) {
  const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qi >= nq) return;
  const uint32_t s = qlist ? qlist[qi] : qi;
  if (status[s] >= CELL_NEED_MORE_K) return;
  if (extra_cnt[qi] == 0) return;
  const uint32_t k = atomicAdd(count, 1u);
  out_s[k] = s;
  out_r[k] = qi;
}

// New lists = old list of the row, then the certification's extras in
// plane order.  The range query meets the extras in slot order, and slots
// within a grid cell depend on the order of the counting sort's atomics;
// sorting makes the clipping order, hence the results, deterministic.
__global__ void append_extra_kernel(const uint32_t* __restrict__ sl, const uint32_t* __restrict__ rows,
                                    uint32_t m, const uint32_t* __restrict__ old_lists,
                                    uint32_t old_stride, const uint32_t* __restrict__ old_cnt,
                                    const uint32_t* __restrict__ extra,
                                    const uint32_t* __restrict__ extra_cnt, uint32_t ex_stride,
                                    uint32_t max_extra, const double4* __restrict__ xd,
                                    const double* __restrict__ ws,
                                    const uint32_t* __restrict__ perm,
                                    uint32_t* __restrict__ new_lists,
                                    uint32_t* __restrict__ new_cnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint32_t r = rows[i], s = sl[i];
  const uint32_t c0 = old_cnt[r] & kCntMask;
  for (uint32_t j = 0; j < c0; ++j) new_lists[(size_t)j * m + i] = old_lists[(size_t)j * old_stride + r];
  const uint32_t ce = min(extra_cnt[r] & 0x7FFFFFFFu, max_extra);
  const double4 pi = xd[s];
  const double wi = ws ? ws[s] : 0.0;
  // insertion sort into place (few extras per cell; a handful of cells
  // next to dense clusters have hundreds)
  for (uint32_t j = 0; j < ce; ++j) {
    const uint32_t v = extra[(size_t)j * ex_stride + r];
    const float kv = plane_key(pi, wi, xd[v], ws ? ws[v] : 0.0);
    const uint32_t ov = perm[v];
    uint32_t k = j;
    while (k > 0) {
      const uint32_t u = new_lists[(size_t)(c0 + k - 1) * m + i];
      if (key_less(plane_key(pi, wi, xd[u], ws ? ws[u] : 0.0), perm[u], kv, ov)) break;
      new_lists[(size_t)(c0 + k) * m + i] = u;
      --k;
    }
    new_lists[(size_t)(c0 + k) * m + i] = v;
  }
  new_cnt[i] = c0 + ce;
}

// Candidate lists from a CSR adjacency in the caller's order (at most k
// per row, k <= kMaxCsrCandidates), in plane order.
constexpr uint32_t kMaxCsrCandidates = 96;

__global__ void csr_to_lists_kernel(const uint32_t* __restrict__ rowptr,
                                    const uint32_t* __restrict__ idx,
                                    const uint32_t* __restrict__ slot_of, uint32_t n, uint32_t k,
                                    const double4* __restrict__ xd,
                                    const double* __restrict__ ws,
                                    uint32_t* __restrict__ lists, uint32_t* __restrict__ cnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = slot_of[i];
  const uint32_t b = rowptr[i];
  const uint32_t c = min(min(rowptr[i + 1] - b, k), kMaxCsrCandidates);
  const double4 pi = xd[s];
  const double wi = ws ? ws[s] : 0.0;
  float key[kMaxCsrCandidates];
  uint32_t ord[kMaxCsrCandidates];
  // insertion sort by (plane key, original index); the previous cells'
  // facets come in their clipping order, so rows are nearly sorted
  for (uint32_t j = 0; j < c; ++j) {
    const uint32_t o = idx[b + j];
    const float kv = plane_key(pi, wi, xd[slot_of[o]], ws ? ws[slot_of[o]] : 0.0);
    uint32_t q = j;
    while (q > 0 && key_less(kv, o, key[q - 1], ord[q - 1])) {
      key[q] = key[q - 1];
      ord[q] = ord[q - 1];
      --q;
    }
    key[q] = kv;
    ord[q] = o;
  }
  for (uint32_t j = 0; j < c; ++j) lists[(size_t)j * n + s] = slot_of[ord[j]];
  cnt[s] = c;
}

__global__ void max_degree_kernel(const uint32_t* __restrict__ rowptr, uint32_t n,
                                  uint32_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t d = (i < n) ? rowptr[i + 1] - rowptr[i] : 0u;
  d = __reduce_max_sync(0xFFFFFFFFu, d);
  if ((threadIdx.x & 31) == 0) atomicMax(out, d);
}

// The passes that take every seed to a final cell: clipping, geometry,
// the FP64 fixes, and the caller-order outputs.
struct Pipeline {
  gbv_context* c;
  cudaStream_t st;
  uint32_t n;
  bool fp32;
  bool check_sr;
  SortedSeeds S;
  ClipArgs cbase{};
  GeomArgs gbase{};
  int32_t* status_s;
  double* vol_s;
  double* mg_s;
  uint32_t* nf;
  uint32_t* nclip;
  uint32_t* f_nbr;
  double* f_area;
  uint32_t *rs, *rr, *os, *orw, *ms, *mr, *mk_s, *mk_r;
  uint32_t n_recheck = 0, n_over = 0, n_morek = 0;
  // certification (Laguerre mode)
  const double* node_wmax = nullptr;
  const double4* node_lin = nullptr;
  const double* node_ex = nullptr;
  uint32_t* extra = nullptr;
  uint32_t* extra_cnt = nullptr;
  uint32_t max_extra = 32;
  // cells beyond the large shape
  uint32_t n_huge = 0;
  uint32_t** hp_nbr = nullptr;
  double** hp_area = nullptr;
  int huge_chunks = 0;

  Pipeline(gbv_context* ctx, uint32_t n_, const double* box_min, const double* box_max,
           bool fp32_, bool check_sr_, uint32_t k0, cudaStream_t st_, bool fast_pred = false)
      : c(ctx), st(st_), n(n_), fp32(fp32_), check_sr(check_sr_) {
    S = c->S;
    for (int k = 0; k < 3; ++k) {
      c->box[k] = box_min[k];
      c->box[3 + k] = box_max[k];
    }
    c->h_counts[4] = 0;  // first-pass kNN exact fallbacks (cells_device sets it)
    status_s = c->buf<int32_t>("status_s", n);
    vol_s = c->buf<double>("vol_s", n);
    mg_s = c->buf<double>("mg_s", 3 * (size_t)n);
    nf = c->buf<uint32_t>("nf", n);
    nclip = c->buf<uint32_t>("nclip", n);
    f_nbr = c->buf<uint32_t>("f_nbr", (size_t)kMaxFacets * n);
    f_area = c->buf<double>("f_area", (size_t)kMaxFacets * n);
    CombBuf cb;
    cb.tv = c->buf<uint32_t>("cb_tv", (size_t)kTMax * n);
    cb.ta = c->buf<uint32_t>("cb_ta", (size_t)kTMax * n);
    cb.key = c->buf<int16_t>("cb_key", (size_t)kTMax * n);
    cb.pown = c->buf<uint32_t>("cb_pown", (size_t)kPMax * n);
    cb.prank = c->buf<uint16_t>("cb_prank", (size_t)kPMax * n);
    cb.tmask = c->buf<ulonglong2>("cb_tmask", n);
    cb.pmask = c->buf<uint64_t>("cb_pmask", n);
    cb.flags = c->buf<uint32_t>("cb_flags", n);
    cbase.S = S;
    cbase.n_total = n;
    cbase.k0 = k0;
    gbase.S = S;
    for (int k = 0; k < 3; ++k) {
      cbase.box[k] = gbase.box[k] = box_min[k];
      cbase.box[3 + k] = gbase.box[3 + k] = box_max[k];
    }
    cbase.check_sr = check_sr ? 1 : 0;
    cbase.fast_pred = fast_pred ? 1 : 0;
    cbase.status = gbase.status = status_s;
    cbase.nclip = nclip;
    gbase.nclip = nclip;
    cbase.comb = gbase.comb = cb;
    cbase.counters = c->counters;
    gbase.vol = vol_s;
    gbase.mg = mg_s;
    gbase.nf = nf;
    gbase.f_nbr = f_nbr;
    gbase.f_area = f_area;
    gbase.out_stride = n;
    rs = c->buf<uint32_t>("cls_rs", n);
    rr = c->buf<uint32_t>("cls_rr", n);
    os = c->buf<uint32_t>("cls_os", n);
    orw = c->buf<uint32_t>("cls_or", n);
    ms = c->buf<uint32_t>("cls_ms", n);
    mr = c->buf<uint32_t>("cls_mr", n);
    mk_s = c->buf<uint32_t>("mk_s", n);
    mk_r = c->buf<uint32_t>("mk_r", n);
    GBV_CUDA(cudaMemsetAsync(c->counters, 0, 4 * sizeof(unsigned long long), st));
  }

  bool timed_first = false;  // the first clipping pass has been timed
  unsigned int* abort_on_empty = nullptr;  // first pass stops at an empty cell
  bool aborted = false;
  bool geom32 = false;       // FP32 geometry after FP32 clipping passes
  bool resume = false;       // clipping continues from the stored polytopes

  // certification counters (GBV_CERT_STATS in the environment)
  unsigned long long* cert_stats = nullptr;

  const float* node_wmax_f = nullptr;
  const float4* node_lin_f = nullptr;
  const float* node_ex_f = nullptr;

  void enable_certification(const double* wmax, const double4* lin, const double* ex,
                            uint32_t nodes) {
    node_wmax = wmax;
    node_lin = lin;
    node_ex = ex;
    float* wf = c->buf<float>("node_wmax_f", nodes);
    float4* lf = lin ? c->buf<float4>("node_lin_f", nodes) : nullptr;
    float* ef = lin ? c->buf<float>("node_ex_f", nodes) : nullptr;
    node_bounds_f32_kernel<<<nblocks(nodes, 256), 256, 0, st>>>(wmax, lin, ex, nodes, wf, lf, ef); count_launch();
    node_wmax_f = wf;
    node_lin_f = lf;
    node_ex_f = ef;
    if (std::getenv("GBV_CERT_STATS")) {
      cert_stats = c->buf<unsigned long long>("cert_stats", 5);
      GBV_CUDA(cudaMemsetAsync(cert_stats, 0, 5 * sizeof(unsigned long long), st));
    }
  }

  void print_cert_stats() {
    if (!cert_stats) return;
    unsigned long long h[5];
    GBV_CUDA(cudaMemcpyAsync(h, cert_stats, sizeof(h), cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    std::fprintf(stderr,
                 "[cert] %llu cells: nodes %.1f/cell (max %llu), seeds scanned %.1f/cell (max "
                 "%llu)\n",
                 h[4], (double)h[0] / std::max(1ull, h[4]), h[2],
                 (double)h[1] / std::max(1ull, h[4]), h[3]);
  }

  // Room for up to `per_row` extra candidates of each of `rows` list rows.
  void size_extras(uint32_t per_row, uint32_t rows) {
    max_extra = per_row;
    extra = c->buf<uint32_t>("cert_extra", (size_t)per_row * rows);
    extra_cnt = c->buf<uint32_t>("cert_extra_cnt", rows);
    GBV_CUDA(cudaMemsetAsync(extra_cnt, 0, sizeof(uint32_t) * rows, st));
  }

  void classify(const uint32_t* ql, const uint32_t* qr, uint32_t nq, uint32_t out[4]) {
    GBV_CUDA(cudaMemsetAsync(c->list_counts, 0, 4 * sizeof(uint32_t), st));
    classify_kernel<<<nblocks(nq, 256), 256, 0, st>>>(ql, qr, nq, status_s, c->list_counts, rs,
                                                      rr, os, orw, ms, mr); count_launch();
    GBV_CUDA(cudaMemcpyAsync(c->h_counts, c->list_counts, 4 * sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 4; ++k) out[k] = c->h_counts[k];
    if (out[3]) {
      throw StatusError{GBV_ERR_STATE, "inconsistent polytope in " + std::to_string(out[3]) +
                                           " cell(s) (conflict zone not a disk)"};
    }
  }

  // clip + geometry of a set of cells with the given lists
  // (kind 0: the pipeline's precision, 1: FP64 small, 2: FP64 large,
  // 3: FP32 large, 4: FP32 small with exact signs where FP32 cannot decide)
  void run(const ListSet& L, const uint32_t* ql, const uint32_t* qr, uint32_t nq, int kind) {
    ClipArgs a = cbase;
    a.nbr = L.lists;
    a.nbr_stride = L.stride;
    a.nbr_cnt = L.cnt;
    a.list_k = L.k;
    a.qlist = ql;
    a.qrow = qr;
    a.nq = nq;
    a.resume = resume ? 1 : 0;
    const bool f32 = (kind == 0 && fp32) || kind == 3 || kind == 4;
    const int shape = (kind == 2 || kind == 3) ? CLIP_LARGE : CLIP_SMALL;
    // the first pass over every cell: its kernel time and counters alone
    const bool first = kind == 0 && !timed_first;
    if (first) GBV_CUDA(cudaEventRecord(c->ev[6], st));
    if (abort_on_empty && kind == 0) {
      GBV_CUDA(cudaMemsetAsync(abort_on_empty, 0, sizeof(unsigned int), st));
      a.abort_on_empty = abort_on_empty;
    }
    if (f32) launch_clip_fp32(a, shape, kind != 0, st);
    else launch_clip_fp64(a, shape, st);
    if (abort_on_empty && kind == 0) {
      unsigned int h = 0;
      GBV_CUDA(cudaMemcpyAsync(&h, abort_on_empty, sizeof h, cudaMemcpyDeviceToHost, st));
      GBV_CUDA(cudaStreamSynchronize(st));
      if (h) {
        aborted = true;
        return;
      }
    }
    if (first) {
      timed_first = true;
      GBV_CUDA(cudaEventRecord(c->ev[7], st));
      GBV_CUDA(cudaMemcpyAsync(c->h_clipc, c->counters + 2, 2 * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, st));
    }
    GBV_CUDA(last_launch_error);
    GeomArgs g = gbase;
    g.nbr = L.lists;
    g.nbr_stride = L.stride;
    g.qlist = ql;
    g.qrow = qr;
    g.nq = nq;
    g.verify_sr = (f32 && check_sr) ? 1 : 0;
    g.shape = shape;
    g.g32 = (f32 && geom32 && !node_wmax) ? 1 : 0;
    if (node_wmax) {
      g.node_wmax = node_wmax;
      g.node_lin = node_lin;
      g.node_ex = node_ex;
      g.node_wmax_f = node_wmax_f;
      g.node_lin_f = node_lin_f;
      g.node_ex_f = node_ex_f;
      g.cand_cnt = L.cnt;
      g.extra = extra;
      g.extra_cnt = extra_cnt;
      g.max_extra = max_extra;
      g.cert_stats = cert_stats;
    }
    launch_geometry(g, st);
    GBV_CUDA(last_launch_error);
  }

  // Cells beyond the large shape (slots hs, rows hr of L), in chunks.
  void run_huge(const ListSet& L, const uint32_t* hs, const uint32_t* hr, uint32_t m) {
    if (!hp_nbr) {
      hp_nbr = c->buf<uint32_t*>("huge_hp_nbr", n);
      hp_area = c->buf<double*>("huge_hp_area", n);
    }
    constexpr uint32_t kChunk = 1024;
    const size_t cap = std::min<uint32_t>(m, kChunk);
    for (uint32_t off = 0; off < m; off += kChunk) {
      const uint32_t cm = std::min<uint32_t>(kChunk, m - off);
      HugeArgs h{};
      h.S = S;
      h.nbr = L.lists;
      h.nbr_stride = L.stride;
      h.nbr_cnt = L.cnt;
      h.list_k = L.k;
      h.n_total = n;
      h.k0 = cbase.k0;
      h.qlist = hs + off;
      h.qrow = hr ? hr + off : nullptr;
      h.nq = cm;
      for (int k = 0; k < 6; ++k) h.box[k] = cbase.box[k];
      h.check_sr = cbase.check_sr;
      h.fast_pred = cbase.fast_pred;
      h.status = status_s;
      h.nclip = nclip;
      h.counters = c->counters;
      h.scr_t = c->buf<ushort4>("huge_t", cap * kHugeT);
      h.scr_adj = c->buf<ushort4>("huge_adj", cap * kHugeT);
      h.scr_cor = c->buf<double4>("huge_cor", cap * kHugeT);
      h.scr_eps = c->buf<float>("huge_eps", cap * kHugeT);
      h.scr_pl = c->buf<double4>("huge_pl", cap * kHugeV);
      h.scr_vg = c->buf<uint32_t>("huge_vg", cap * kHugeV);
      h.scr_v2t = c->buf<uint16_t>("huge_v2t", cap * kHugeV);
      h.scr_v2e = c->buf<uint8_t>("huge_v2e", cap * kHugeV);
      h.vol = vol_s;
      h.mg = mg_s;
      h.nf = nf;
      h.out_stride = n;
      const std::string tag = std::to_string(huge_chunks++);
      h.fac_nbr = c->buf<uint32_t>("huge_fn" + tag, (size_t)cm * kHugeV);
      h.fac_area = c->buf<double>("huge_fa" + tag, (size_t)cm * kHugeV);
      h.hp_nbr = hp_nbr;
      h.hp_area = hp_area;
      if (node_wmax) {
        h.node_wmax = node_wmax;
        h.node_lin = node_lin;
        h.node_ex = node_ex;
        h.extra = extra;
        h.extra_cnt = extra_cnt;
        h.max_extra = max_extra;
      }
      const bool stats = std::getenv("GBV_HUGE_STATS") != nullptr;
      if (stats) {
        h.stats = c->buf<unsigned long long>("huge_stats", (size_t)cm * kHugeStats);
        GBV_CUDA(cudaMemsetAsync(h.stats, 0, sizeof(unsigned long long) * cm * kHugeStats, st));
      }
      launch_huge(h, st);
      GBV_CUDA(last_launch_error);
      if (stats) {
        // per-phase cycles and work of the cells of this launch, on stderr
        std::vector<unsigned long long> v((size_t)cm * kHugeStats);
        GBV_CUDA(cudaMemcpyAsync(v.data(), h.stats, v.size() * 8, cudaMemcpyDeviceToHost, st));
        GBV_CUDA(cudaStreamSynchronize(st));
        unsigned long long mx[kHugeStats] = {}, sum[kHugeStats] = {};
        for (uint32_t q = 0; q < cm; ++q)
          for (int k = 0; k < kHugeStats; ++k) {
            mx[k] = std::max(mx[k], v[(size_t)q * kHugeStats + k]);
            sum[k] += v[(size_t)q * kHugeStats + k];
          }
        std::fprintf(stderr,
                     "[huge] %u cells  max/mean: clip Mcyc %.1f/%.1f geom %.1f/%.1f certify "
                     "%.1f/%.1f clips %llu/%.0f tests %llu/%.0f tri %llu/%.0f planes %llu/%.0f "
                     "nodes %llu/%.0f seeds %llu/%.0f\n",
                     cm, mx[0] * 1e-6, sum[0] * 1e-6 / cm, mx[1] * 1e-6, sum[1] * 1e-6 / cm,
                     mx[2] * 1e-6, sum[2] * 1e-6 / cm, mx[3], (double)sum[3] / cm, mx[4],
                     (double)sum[4] / cm, mx[5], (double)sum[5] / cm, mx[6], (double)sum[6] / cm,
                     mx[7], (double)sum[7] / cm, mx[8], (double)sum[8] / cm);
      }
    }
  }

  // A pass and its FP64 fixes; returns the cells that still need a longer
  // list (slots in mk_s, rows of L in mk_r).
  uint32_t process(const ListSet& L, const uint32_t* ql, const uint32_t* qr, uint32_t nq) {
    uint32_t* rc_s = c->buf<uint32_t>("rc_s", n);
    uint32_t* rc_r = c->buf<uint32_t>("rc_r", n);
    uint32_t* ov_s = c->buf<uint32_t>("ov_s", n);
    uint32_t* ov_r = c->buf<uint32_t>("ov_r", n);
    auto append = [&](uint32_t* dst, uint32_t at, const uint32_t* src, uint32_t cnt) {
      if (cnt) GBV_CUDA(cudaMemcpyAsync(dst + at, src, cnt * sizeof(uint32_t),
                                        cudaMemcpyDeviceToDevice, st));
    };
    run(L, ql, qr, nq, 0);
    if (aborted) return 0;
    uint32_t c1[4];
    classify(ql, qr, nq, c1);
    uint32_t nrc = c1[0], nov = c1[1], nmk = c1[2];
    append(rc_s, 0, rs, nrc);
    append(rc_r, 0, rr, nrc);
    append(ov_s, 0, os, nov);
    append(ov_r, 0, orw, nov);
    append(mk_s, 0, ms, nmk);
    append(mk_r, 0, mr, nmk);
    if (nrc && fp32) {
      // FP32 again, undecided signs taken exactly; what is left (stops of
      // the security radius FP32 could not certify) goes to FP64 below
      n_recheck += nrc;
      run(L, rc_s, rc_r, nrc, 4);
      uint32_t c6[4];
      classify(rc_s, rc_r, nrc, c6);
      append(ov_s, nov, os, c6[1]);
      append(ov_r, nov, orw, c6[1]);
      nov += c6[1];
      append(mk_s, nmk, ms, c6[2]);
      append(mk_r, nmk, mr, c6[2]);
      nmk += c6[2];
      append(rc_s, 0, rs, c6[0]);
      append(rc_r, 0, rr, c6[0]);
      nrc = c6[0];
    }
    if (nrc) {
      if (!fp32) n_recheck += nrc;
      run(L, rc_s, rc_r, nrc, 1);
      uint32_t c2[4];
      classify(rc_s, rc_r, nrc, c2);
      append(ov_s, nov, os, c2[1]);
      append(ov_r, nov, orw, c2[1]);
      nov += c2[1];
      append(mk_s, nmk, ms, c2[2]);
      append(mk_r, nmk, mr, c2[2]);
      nmk += c2[2];
    }
    if (nov && fp32) {
      // the large shape in FP32 first; its rechecks go to FP64 below
      n_over += nov;
      run(L, ov_s, ov_r, nov, 3);
      uint32_t c5[4];
      classify(ov_s, ov_r, nov, c5);
      uint32_t* lr_s = c->buf<uint32_t>("lr_s", n);
      uint32_t* lr_r = c->buf<uint32_t>("lr_r", n);
      append(lr_s, 0, rs, c5[0]);
      append(lr_r, 0, rr, c5[0]);
      append(mk_s, nmk, ms, c5[2]);
      append(mk_r, nmk, mr, c5[2]);
      nmk += c5[2];
      // beyond the large shape, and the large cells FP32 could not certify:
      // the FP64 large pass
      append(ov_s, 0, os, c5[1]);
      append(ov_r, 0, orw, c5[1]);
      append(ov_s, c5[1], lr_s, c5[0]);
      append(ov_r, c5[1], lr_r, c5[0]);
      nov = c5[1] + c5[0];
      n_recheck += c5[0];
    }
    if (nov) {
      if (!fp32) n_over += nov;
      run(L, ov_s, ov_r, nov, 2);
      uint32_t c3[4];
      classify(ov_s, ov_r, nov, c3);
      if (c3[0]) throw StatusError{GBV_ERR_STATE, "FP64 clipping asked for a recheck"};
      append(mk_s, nmk, ms, c3[2]);
      append(mk_r, nmk, mr, c3[2]);
      nmk += c3[2];
      if (c3[1]) {
        const uint32_t nh = c3[1];
        uint32_t* hg_s = c->buf<uint32_t>("hg_s", n);
        uint32_t* hg_r = c->buf<uint32_t>("hg_r", n);
        append(hg_s, 0, os, nh);
        append(hg_r, 0, orw, nh);
        n_huge += nh;
        run_huge(L, hg_s, hg_r, nh);
        uint32_t c4[4];
        classify(hg_s, hg_r, nh, c4);
        if (c4[0] || c4[1]) {
          throw StatusError{GBV_ERR_CAPACITY, std::to_string(c4[1]) + " cell(s) exceed " +
                                                  std::to_string(kHugeT) + " corners or " +
                                                  std::to_string(kHugeV) + " planes"};
        }
        append(mk_s, nmk, ms, c4[2]);
        append(mk_r, nmk, mr, c4[2]);
        nmk += c4[2];
      }
    }
    return nmk;
  }

  // Caller-order results and CSR into the context.
  void finish() {
    c->vol = c->buf<double>("vol", n);
    c->mg = c->buf<double>("mg", 3 * (size_t)n);
    c->status = c->buf<int32_t>("status", n);
    c->rowptr = c->buf<uint32_t>("rowptr", (size_t)n + 1);
    facet_count_kernel<<<nblocks((size_t)n + 1, 256), 256, 0, st>>>(S.slot_of, nf, n, c->rowptr); count_launch();
    // A cell has at most kHugeV facets, so below 2^32 / kHugeV cells the
    // 32-bit offsets cannot wrap; above, the total is checked exactly.
    if ((uint64_t)n * kHugeV > 0xffffffffull) {
      unsigned long long* tot = c->buf<unsigned long long>("facet_total", 1);
      GBV_CUDA(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), st));
      facet_total_kernel<<<4 * 152, 256, 0, st>>>(c->rowptr, n, tot); count_launch();
      unsigned long long h_tot = 0;
      GBV_CUDA(cudaMemcpyAsync(&h_tot, tot, sizeof h_tot, cudaMemcpyDeviceToHost, st));
      GBV_CUDA(cudaStreamSynchronize(st));
      if (h_tot > 0xffffffffull)
        throw StatusError{GBV_ERR_CAPACITY, std::to_string(h_tot) +
                                                " facets exceed the 32-bit CSR offsets"};
    }
    uint32_t* stmp = c->buf<uint32_t>("csr_scan_tmp", scan_tmp_elems((size_t)n + 1));
    exclusive_scan_u32(c->rowptr, (size_t)n + 1, stmp, st);
    GBV_CUDA(cudaMemcpyAsync(&c->h_counts[0], c->rowptr + n, 4, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    const uint32_t nnz32 = c->h_counts[0];
    c->nnz = nnz32;
    c->nbr = c->buf<uint32_t>("nbr", std::max<uint32_t>(nnz32, 1));
    c->area = c->buf<double>("area", std::max<uint32_t>(nnz32, 1));
    unsort_kernel<<<nblocks(n, 256), 256, 0, st>>>(S.slot_of, n, vol_s, mg_s, status_s, nf,
                                                   f_nbr, f_area, hp_nbr, hp_area, c->rowptr,
                                                   c->vol, c->mg,
                                                   c->status, c->nbr, c->area); count_launch();
    c->n = n;
    c->has_cells = true;
  }

  void report(gbv_cell_report* rep, uint32_t K, float t_grid, float t_knn, float t_clip,
              float t_retry, float t_total) {
    double* part = c->buf<double>("sum_part", 2 * 256);
    double* out = c->buf<double>("sum_out", 1);
    sum_partial_kernel<<<256, kSumThreads, 0, st>>>(c->vol, n, part); count_launch();
    sum_final_kernel<<<1, 32, 0, st>>>(part, 256, out); count_launch();
    unsigned long long* clips = c->buf<unsigned long long>("clip_sum", 1);
    GBV_CUDA(cudaMemsetAsync(clips, 0, 8, st));
    sum_u32_kernel<<<256, 256, 0, st>>>(nclip, n, clips); count_launch();
    double vs = 0;
    unsigned long long cs = 0, hc[4] = {0, 0, 0, 0};
    GBV_CUDA(cudaMemcpyAsync(&vs, out, 8, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaMemcpyAsync(&cs, clips, 8, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaMemcpyAsync(hc, c->counters, 32, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    rep->nnz = c->nnz;
    rep->n_cells = n;
    rep->n_recheck_fp64 = n_recheck;
    rep->n_more_k = n_morek;
    rep->n_overflow = n_over;
    rep->max_clips = (uint32_t)hc[1];
    rep->knn_k = K;
    rep->mean_clips = (double)cs / n;
    rep->volume_sum = vs;
    rep->n_exact = hc[0];
    rep->ms_grid = t_grid;
    rep->ms_knn = t_knn;
    rep->ms_clip = t_clip;
    rep->ms_retry = t_retry;
    rep->ms_total = t_total;
    rep->n_huge = n_huge;
    rep->n_knn_exact = c->h_counts[4];
    rep->n_conflict_tests = timed_first ? c->h_clipc[0] : 0;
    rep->n_corners_created = timed_first ? c->h_clipc[1] : 0;
    float ms = 0.f;
    if (timed_first) GBV_CUDA(cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]));
    rep->ms_clip_kernel = ms;
  }
};

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float t = 0.f;
  GBV_CUDA(cudaEventElapsedTime(&t, a, b));
  return t;
}

// The whole cell computation on device inputs (the reference's
// security-radius semantics).
static void cells_device(gbv_context* c, const double* d_xyz, const double* d_w, uint32_t n,
                         const gbv_cell_options& o, cudaStream_t st, gbv_cell_report* rep) {
  if (n == 0) throw StatusError{GBV_ERR_INVALID_ARGUMENT, "n must be > 0"};
  setup_seeds(c, n, d_w != nullptr);
  c->nn_ready = false;
  c->has_periodic = false;
  SortedSeeds& S = c->S;
  GBV_CUDA(cudaEventRecord(c->ev[0], st));
  build_grid(d_xyz, 3, 3, d_w, n, S.L, S, c->scr, st);
  GBV_CUDA(cudaEventRecord(c->ev[1], st));
  Pipeline P(c, n, o.box_min, o.box_max, o.precision != GBV_PRECISION_FP64,
             o.check_sr != 0, o.k0, st, o.predicates == GBV_PREDICATES_FAST);
  P.geom32 = o.precision == GBV_PRECISION_FP32_GEOMETRY;
  uint32_t* flag_count = c->buf<uint32_t>("knn_flag_count", 1);
  uint32_t* flag_list = c->buf<uint32_t>("knn_flag_list", n);

  // first lists: the security-radius loop's cells need about 40-70
  // neighbours (Voronoi / weights on the squared-spacing scale), a few up to
  // twice that.  96 covers about 90% of the cells of a 1M-seed power diagram
  // with weights up to the squared spacing; the others take a second pass
  // with longer lists.  Longer first lists cost more in the search (its
  // heaps grow) than the second pass saves (measured: 80.7 ms per 1M-seed
  // diagram at 96, 83.6 at 112, 87.8 at 128, 88.6 at 80).  The cells come
  // out the same whatever the list length.
  const uint32_t nm1 = n > 1 ? n - 1 : 0;
  const uint32_t auto_k = 96u;
  const uint32_t K = o.check_sr ? std::min<uint32_t>(o.first_k ? o.first_k : auto_k, nm1)
                                : std::min<uint32_t>(o.k0, nm1);
  uint32_t* knn = c->buf<uint32_t>("knn", (size_t)std::max<uint32_t>(K, 1) * n);
  uint32_t* kcnt = c->buf<uint32_t>("kcnt", n);
  double* klast_d = c->buf<double>("klast_d", n);
  uint32_t* klast_i = c->buf<uint32_t>("klast_i", n);
  {
    KnnArgs ka{};
    ka.S = &S;
    ka.nq = n;
    ka.k = K;
    ka.mode = KNN_CELLS;
    ka.nbr = knn;
    ka.out_stride = n;
    ka.cnt = kcnt;
    ka.last_d2 = klast_d;
    ka.last_idx = klast_i;
    ka.flag_count = flag_count;
    ka.flag_list = flag_list;
    ka.coherent = true;  // every slot, in sorted order
    ka.tile_scratch = c->buf<uint32_t>("knn_tiles", knn_tile_scratch_elems(n, S.L));
    if (K > kKnnMaxK) {  // only without the security radius
      ka.gl_d2 = c->buf<double>("knn_gd2", (size_t)K * n);
      ka.gl_slot = c->buf<uint32_t>("knn_gslot", (size_t)K * n);
    }
    c->h_counts[4] = 0;
    if (K > 0) {
      launch_knn(ka, st);
      // read with the report (the pipeline synchronises before it)
      GBV_CUDA(cudaMemcpyAsync(&c->h_counts[4], flag_count, sizeof(uint32_t),
                               cudaMemcpyDeviceToHost, st));
    } else {
      GBV_CUDA(cudaMemsetAsync(kcnt, 0, sizeof(uint32_t) * n, st));
    }
    GBV_CUDA(cudaGetLastError());
  }
  GBV_CUDA(cudaEventRecord(c->ev[2], st));

  ListSet L0;
  L0.lists = knn;
  L0.stride = n;
  L0.cnt = kcnt;
  L0.k = K;
  L0.last_d2 = klast_d;
  L0.last_idx = klast_i;
  uint32_t morek = P.process(L0, nullptr, nullptr, n);
  GBV_CUDA(cudaEventRecord(c->ev[5], st));
  ListSet cur = L0;
  int round = 0;
  while (morek > 0) {
    P.n_morek += morek;
    if (cur.k >= nm1) throw StatusError{GBV_ERR_STATE, "list growth did not terminate"};
    // Up to 256 neighbours the lists grow by 64 (the FP32-screened search,
    // a cell needing fewer than 256 takes at most two extra rounds); beyond,
    // every round doubles them, so a cell that needs k neighbours (outer
    // seeds of clustered inputs need thousands) takes O(log k) rounds and
    // O(k) clips in all
    const uint32_t want = cur.k < 4 * kKnnSmemK ? kKnnSmemK : cur.k;
    const uint32_t batch = std::min<uint32_t>(want, nm1 - cur.k);
    const uint32_t newk = cur.k + batch;
    const std::string tag = std::to_string(round & 1);
    uint32_t* q_s = c->buf<uint32_t>("ext_s" + tag, morek);
    uint32_t* q_r = c->buf<uint32_t>("ext_r" + tag, morek);
    GBV_CUDA(cudaMemcpyAsync(q_s, P.mk_s, morek * 4, cudaMemcpyDeviceToDevice, st));
    GBV_CUDA(cudaMemcpyAsync(q_r, P.mk_r, morek * 4, cudaMemcpyDeviceToDevice, st));
    uint32_t* lists = c->buf<uint32_t>("ext_lists" + tag, (size_t)newk * morek);
    uint32_t* cnt = c->buf<uint32_t>("ext_cnt" + tag, morek);
    double* lo_d = c->buf<double>("ext_lo_d" + tag, morek);
    uint32_t* lo_i = c->buf<uint32_t>("ext_lo_i" + tag, morek);
    double* last_d = c->buf<double>("ext_last_d" + tag, morek);
    uint32_t* last_i = c->buf<uint32_t>("ext_last_i" + tag, morek);
    extend_lists_kernel<<<nblocks(morek, 128), 128, 0, st>>>(q_r, morek, cur.lists, cur.stride,
                                                             cur.k, cur.last_d2, cur.last_idx,
                                                             lists, lo_d, lo_i); count_launch();
    KnnArgs ka{};
    ka.S = &S;
    ka.nq = morek;
    ka.qlist = q_s;
    ka.k = batch;
    ka.mode = KNN_CELLS;
    ka.lo_d2 = lo_d;
    ka.lo_idx = lo_i;
    ka.nbr = lists + (size_t)cur.k * morek;
    ka.out_stride = morek;
    ka.cnt = cnt;
    ka.last_d2 = last_d;
    ka.last_idx = last_i;
    ka.flag_count = flag_count;
    ka.flag_list = flag_list;
    if (batch > kKnnMaxK) {  // lists beyond the shared-memory lists
      ka.gl_d2 = c->buf<double>("ext_gd2", (size_t)batch * morek);
      ka.gl_slot = c->buf<uint32_t>("ext_gslot", (size_t)batch * morek);
    }
    launch_knn(ka, st);
    add_count_kernel<<<nblocks(morek, 128), 128, 0, st>>>(cnt, morek, cur.k, q_r, cur.cnt); count_launch();
    GBV_CUDA(cudaGetLastError());
    ListSet nx;
    nx.lists = lists;
    nx.stride = morek;
    nx.cnt = cnt;
    nx.k = newk;
    nx.last_d2 = last_d;
    nx.last_idx = last_i;
    morek = P.process(nx, q_s, nullptr, morek);
    cur = nx;
    ++round;
  }
  GBV_CUDA(cudaEventRecord(c->ev[3], st));
  P.finish();
  GBV_CUDA(cudaEventRecord(c->ev[4], st));
  if (rep) {
    GBV_CUDA(cudaEventSynchronize(c->ev[4]));
    P.report(rep, K, elapsed(c->ev[0], c->ev[1]), elapsed(c->ev[1], c->ev[2]),
             elapsed(c->ev[2], c->ev[5]), elapsed(c->ev[5], c->ev[3]),
             elapsed(c->ev[0], c->ev[4]));
  } else {
    GBV_CUDA(cudaStreamSynchronize(st));
  }
  GBV_CUDA(cudaGetLastError());
}

// Laguerre cells certified by the cell-centred power range query (no
// security radius): the path of the optimal-transport solver, whose weights
// vary too much for the 4-d lift's radius to stop.  Candidates come from a
// CSR adjacency in the caller's order (e.g. the previous Newton iterate's
// cells) or, when none is given, from the kNN (lifted when weighted).
//
// abort_below > 0: after the first pass every cell's volume bounds its final
// volume from above (clipping by more seeds only removes volume), so when
// one is below abort_below the call stops there and returns false -- the
// line search of the optimal-transport solver rejects such steps, and
// their cells are the costliest to certify.  Returns true when the cells
// are complete.
__global__ void min_partial_kernel(const double* __restrict__ v, uint32_t n,
                                   double* __restrict__ part) {
  __shared__ double sm[256];
  double m = DBL_MAX;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = fmin(m, v[i]);
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] = fmin(sm[threadIdx.x], sm[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

static bool laguerre_device(gbv_context* c, const double* d_xyz, const double* d_w, uint32_t n,
                            const double* box_min, const double* box_max, bool fp32,
                            const uint32_t* cand_rowptr, const uint32_t* cand_idx,
                            cudaStream_t st, gbv_cell_report* rep, double abort_below = 0.0) {
  if (n < 2) throw StatusError{GBV_ERR_INVALID_ARGUMENT, "n must be >= 2"};
  setup_seeds(c, n, d_w != nullptr);
  c->nn_ready = false;
  SortedSeeds& S = c->S;
  GBV_CUDA(cudaEventRecord(c->ev[0], st));
  build_grid(d_xyz, 3, 3, d_w, n, S.L, S, c->scr, st);
  double* wmax = c->buf<double>("node_wmax", node_count(S.L));
  build_node_wmax(S, wmax, st);
  // linear weight bounds per node (they prune where the weights have a
  // large smooth gradient, as optimal-transport weights do)
  double4* nlin = nullptr;
  double* nex = nullptr;
  if (d_w) {
    nlin = c->buf<double4>("node_lin", node_count(S.L));
    nex = c->buf<double>("node_ex", node_count(S.L));
    build_node_linear(S, nlin, nex, c->buf<double>("node_mom", 14 * node_count(S.L)), st);
  }
  GBV_CUDA(cudaEventRecord(c->ev[1], st));
  // no list cap for seeds with copies (the security-radius loop is not used)
  Pipeline P(c, n, box_min, box_max, fp32, false, n, st);
  P.enable_certification(wmax, nlin, nex, node_count(S.L));
  // a certification round extends lists at their end: its cells continue
  // from the polytopes of the round before (GBV_CERT_RESUME=0: from the box)
  const char* rs_env = std::getenv("GBV_CERT_RESUME");
  P.resume = !(rs_env && rs_env[0] == '0');
  if (P.resume) GBV_CUDA(cudaMemsetAsync(P.cbase.comb.flags, 0, sizeof(uint32_t) * n, st));
  uint32_t K;
  uint32_t* lists;
  uint32_t* cnt = c->buf<uint32_t>("lag_cnt", n);
  if (cand_rowptr) {
    uint32_t* dmax = c->buf<uint32_t>("lag_maxdeg", 1);
    GBV_CUDA(cudaMemsetAsync(dmax, 0, 4, st));
    max_degree_kernel<<<nblocks(n, 256), 256, 0, st>>>(cand_rowptr, n, dmax); count_launch();
    GBV_CUDA(cudaMemcpyAsync(&c->h_counts[0], dmax, 4, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    K = std::max<uint32_t>(1, std::min<uint32_t>(c->h_counts[0], kMaxCsrCandidates));
    lists = c->buf<uint32_t>("lag_lists", (size_t)K * n);
    csr_to_lists_kernel<<<nblocks(n, 128), 128, 0, st>>>(cand_rowptr, cand_idx, S.slot_of, n, K,
                                                         S.xd, S.ws, lists, cnt); count_launch();
  } else {
    K = std::min<uint32_t>(32, n - 1);
    lists = c->buf<uint32_t>("lag_lists", (size_t)K * n);
    KnnArgs ka{};
    ka.S = &S;
    ka.nq = n;
    ka.k = K;
    ka.mode = KNN_CELLS;
    ka.nbr = lists;
    ka.out_stride = n;
    ka.cnt = cnt;
    ka.flag_count = c->buf<uint32_t>("knn_flag_count", 1);
    ka.flag_list = c->buf<uint32_t>("knn_flag_list", n);
    ka.coherent = true;
    ka.tile_scratch = c->buf<uint32_t>("knn_tiles", knn_tile_scratch_elems(n, S.L));
    launch_knn(ka, st);
  }
  GBV_CUDA(cudaGetLastError());
  GBV_CUDA(cudaEventRecord(c->ev[2], st));
  ListSet cur;
  cur.lists = lists;
  cur.stride = n;
  cur.cnt = cnt;
  cur.k = K;
  const uint32_t* ql = nullptr;
  uint32_t nq = n;
  uint32_t* ex_s = c->buf<uint32_t>("lag_ex_s", n);
  uint32_t* ex_r = c->buf<uint32_t>("lag_ex_r", n);
  uint32_t* ex_count = c->buf<uint32_t>("lag_ex_count", 1);
  // A call that may stop (abort_below > 0): the first clipping pass stops
  // at the first cell it empties, and after the first round (clipping,
  // geometry and certification) the volumes bound the final ones from
  // above (later rounds only add planes), so a volume below abort_below
  // already decides.
  if (abort_below > 0.0) P.abort_on_empty = c->buf<unsigned int>("lag_abort", 1);
  for (int round = 0;; ++round) {
    // cells far from their final shape (e.g. next to dense clusters) may
    // need hundreds of extra candidates, a few next to the densest clusters
    // of 10M seeds tens of thousands: the room per cell doubles each round,
    // up to 65536 and to 2^28 entries over the round's cells (at least 2048)
    const uint64_t room_cap = std::max<uint64_t>(kHugeV, (1ull << 28) / std::max<uint32_t>(nq, 1));
    P.size_extras((uint32_t)std::min<uint64_t>(32ull << std::min(round, 11), room_cap),
                  cur.stride);
    if (P.process(cur, ql, nullptr, nq) != 0)
      throw StatusError{GBV_ERR_STATE, "unexpected list exhaustion in Laguerre mode"};
    if (round == 0 && abort_below > 0.0) {
      P.abort_on_empty = nullptr;
      if (P.aborted) {
        c->has_cells = false;
        if (std::getenv("GBV_OT_LOG"))
          std::fprintf(stderr, "[ot]   first clipping pass emptied a cell: stopped\n");
        return false;
      }
      double* part = c->buf<double>("lag_min_part", 256);
      min_partial_kernel<<<256, 256, 0, st>>>(P.vol_s, n, part); count_launch();
      double hp[256];
      GBV_CUDA(cudaMemcpyAsync(hp, part, sizeof(hp), cudaMemcpyDeviceToHost, st));
      GBV_CUDA(cudaStreamSynchronize(st));
      double mn = DBL_MAX;
      for (double v : hp) mn = std::min(mn, v);
      if (mn < abort_below) {
        c->has_cells = false;
        if (std::getenv("GBV_OT_LOG"))
          std::fprintf(stderr, "[ot]   first-round min volume %.3e < %.3e: stopped\n", mn,
                       abort_below);
        return false;
      }
    }
    if (round == 0) GBV_CUDA(cudaEventRecord(c->ev[5], st));
    GBV_CUDA(cudaMemsetAsync(ex_count, 0, 4, st));
    collect_extra_kernel<<<nblocks(nq, 256), 256, 0, st>>>(ql, nq, P.extra_cnt, P.status_s,
                                                           ex_count, ex_s, ex_r); count_launch();
    GBV_CUDA(cudaMemcpyAsync(&c->h_counts[0], ex_count, 4, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    const uint32_t m = c->h_counts[0];
    if (m == 0) break;
    P.n_morek += m;
    if (std::getenv("GBV_OT_LOG"))
      std::fprintf(stderr, "[ot]   round %d: %u cells with extra candidates (room %u)\n", round, m,
                   P.max_extra);
    if (round >= 48)
      throw StatusError{GBV_ERR_NOT_CONVERGED,
                        "certification did not settle: " + std::to_string(m) +
                            " cell(s) still found candidates after 48 rounds"};
    const std::string tag = std::to_string(round & 1);
    const uint32_t newk = cur.k + P.max_extra;
    uint32_t* q_s = c->buf<uint32_t>("lag_q" + tag, m);
    uint32_t* nl = c->buf<uint32_t>("lag_nl" + tag, (size_t)newk * m);
    uint32_t* nc = c->buf<uint32_t>("lag_nc" + tag, m);
    GBV_CUDA(cudaMemcpyAsync(q_s, ex_s, m * 4, cudaMemcpyDeviceToDevice, st));
    append_extra_kernel<<<nblocks(m, 128), 128, 0, st>>>(ex_s, ex_r, m, cur.lists, cur.stride,
                                                         cur.cnt, P.extra, P.extra_cnt,
                                                         cur.stride, P.max_extra, S.xd, S.ws,
                                                         S.perm, nl, nc); count_launch();
    cur.lists = nl;
    cur.stride = m;
    cur.cnt = nc;
    cur.k = newk;
    ql = q_s;
    nq = m;
  }
  GBV_CUDA(cudaEventRecord(c->ev[3], st));
  P.finish();
  GBV_CUDA(cudaEventRecord(c->ev[4], st));
  if (rep) {
    GBV_CUDA(cudaEventSynchronize(c->ev[4]));
    P.report(rep, K, elapsed(c->ev[0], c->ev[1]), elapsed(c->ev[1], c->ev[2]),
             elapsed(c->ev[2], c->ev[5]), elapsed(c->ev[5], c->ev[3]),
             elapsed(c->ev[0], c->ev[4]));
  } else {
    GBV_CUDA(cudaStreamSynchronize(st));
  }
  P.print_cert_stats();
  GBV_CUDA(cudaGetLastError());
  return true;
}

// ---------------------------------------------------------------------
// Learned warm start: buffers and features
// ---------------------------------------------------------------------
static MlpBuffers mlp_buffers(gbv_context* c, uint32_t rows) {
  const size_t r = (size_t)(rows + 31) / 32 * 32;
  const size_t e = r * kMlpHid;
  MlpBuffers B;
  B.xn = c->buf<bf16>("mlp_xn", r * kMlpInPad);
  B.h1 = c->buf<bf16>("mlp_h1", e);
  B.h2 = c->buf<bf16>("mlp_h2", e);
  B.h3 = c->buf<bf16>("mlp_h3", e);
  B.z1 = c->buf<float>("mlp_z1", e);
  B.z2 = c->buf<float>("mlp_z2", e);
  B.z3 = c->buf<float>("mlp_z3", e);
  B.acc = c->buf<float>("mlp_acc", e);
  B.y = c->buf<float>("mlp_y", r);
  B.dy = c->buf<float>("mlp_dy", r);
  B.dz = c->buf<float>("mlp_dz", e);
  B.dzb = c->buf<bf16>("mlp_dzb", e);
  B.dzt = c->buf<bf16>("mlp_dzt", e);
  B.ht = c->buf<bf16>("mlp_ht", e);
  B.part = c->buf<float>("mlp_part", mlp_part_floats());
  B.w1b = c->buf<bf16>("mlp_w1b", kMlpHid * kMlpInPad);
  B.w2b = c->buf<bf16>("mlp_w2b", kMlpHid * kMlpHid);
  B.w3b = c->buf<bf16>("mlp_w3b", kMlpHid * kMlpHid);
  B.w1t = c->buf<bf16>("mlp_w1t", kMlpHid * kMlpInPad);
  B.w2t = c->buf<bf16>("mlp_w2t", kMlpHid * kMlpHid);
  B.w3t = c->buf<bf16>("mlp_w3t", kMlpHid * kMlpHid);
  B.lpart = c->buf<double>("mlp_lpart", kMlpLossParts);
  return B;
}

// Raw features of n seeds (device, caller order); uses the context's grid.
static void mlp_features_device(gbv_context* c, const double* d_xyz, uint32_t n, float* d_raw,
                                cudaStream_t st) {
  if (n < 17) throw StatusError{GBV_ERR_INVALID_ARGUMENT, "the features need n >= 17"};
  setup_seeds(c, n, false);
  c->nn_ready = false;
  c->has_cells = false;
  SortedSeeds& S = c->S;
  build_grid(d_xyz, 3, 3, nullptr, n, S.L, S, c->scr, st);
  uint32_t* oi = c->buf<uint32_t>("mlp_knn_i", (size_t)n * 17);
  double* od = c->buf<double>("mlp_knn_d", (size_t)n * 17);
  KnnArgs ka{};
  ka.S = &S;
  ka.nq = n;
  ka.k = 17;
  ka.mode = KNN_ALL;
  ka.exp_idx = oi;
  ka.exp_d2 = od;
  ka.flag_count = c->buf<uint32_t>("knn_flag_count", 1);
  ka.flag_list = c->buf<uint32_t>("nn_flag_list", n);
  ka.coherent = true;
  ka.tile_scratch = c->buf<uint32_t>("knn_tiles", knn_tile_scratch_elems(n, S.L));
  launch_knn(ka, st);
  mlp_features(d_xyz, od, n, d_raw, st);
  GBV_CUDA(cudaGetLastError());
}

static void mlp_forward_all(gbv_context* c, const float* params, const float* norm,
                            const float* raw, uint32_t n, float* y, cudaStream_t st) {
  const uint32_t cap = std::min<uint32_t>(n, kMlpChunk);
  MlpBuffers B = mlp_buffers(c, cap);
  for (uint32_t off = 0; off < n; off += kMlpChunk) {
    const uint32_t rows = std::min<uint32_t>(kMlpChunk, n - off);
    mlp_forward(params, norm, raw + (size_t)off * kMlpIn, rows, B, false, st);
    GBV_CUDA(cudaMemcpyAsync(y + off, B.y, sizeof(float) * rows, cudaMemcpyDeviceToDevice, st));
  }
  GBV_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------
// Semi-discrete optimal transport: damped Newton with FP64 PCG
// ---------------------------------------------------------------------
struct OtWork {
  gbv_context* c;
  cudaStream_t st;
  uint32_t n;
  double* part;      // device partials
  std::vector<double> hpart;
  explicit OtWork(gbv_context* ctx, uint32_t n_, cudaStream_t s) : c(ctx), st(s), n(n_) {
    part = c->buf<double>("ot_part", 4 * kOtParts);
    hpart.resize(4 * kOtParts);
  }
  // Neumaier sum of the (s, c) pairs of the first 2*kOtParts partials
  double fetch_sum() {
    GBV_CUDA(cudaMemcpyAsync(hpart.data(), part, sizeof(double) * 2 * kOtParts,
                             cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    double S = 0.0, C = 0.0;
    for (int b = 0; b < kOtParts; ++b) {
      const double x = hpart[2 * b], t = S + x;
      if (std::fabs(S) >= std::fabs(x)) C += (S - t) + x;
      else C += (x - t) + S;
      S = t;
      C += hpart[2 * b + 1];
    }
    return S + C;
  }
  double dot(const double* a, const double* b) {
    dot_parts(a, b, n, part, st);
    return fetch_sum();
  }
  // residual r = vol - nu; returns ||r||^2, max |r_i|/nu_i, min vol
  void residual_stats(const double* vol, const double* nu, double* r, double& r2, double& rel_inf,
                      double& vmin) {
    residual(vol, nu, n, r, part, st);
    GBV_CUDA(cudaMemcpyAsync(hpart.data(), part, sizeof(double) * 4 * kOtParts,
                             cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    double S = 0.0, C = 0.0;
    rel_inf = 0.0;
    vmin = DBL_MAX;
    for (int b = 0; b < kOtParts; ++b) {
      const double x = hpart[2 * b], t = S + x;
      if (std::fabs(S) >= std::fabs(x)) C += (S - t) + x;
      else C += (x - t) + S;
      S = t;
      C += hpart[2 * b + 1];
      rel_inf = std::max(rel_inf, hpart[2 * kOtParts + b]);
      vmin = std::min(vmin, hpart[3 * kOtParts + b]);
    }
    r2 = S + C;
  }
};

__global__ void mul_kernel(double* __restrict__ y, const double* __restrict__ x, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] *= x[i];
}

__global__ void fill_kernel(double* __restrict__ y, double v, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = v;
}

// Laguerre cells at weights w with the given candidates (CSR in caller
// order, may be null); results in the context.
// Progress lines on stderr when the environment sets GBV_OT_LOG (the
// solver's counterpart of the reference's Logger output).
static bool ot_log_enabled() {
  static const bool on = std::getenv("GBV_OT_LOG") != nullptr;
  return on;
}

static bool ot_cells(gbv_context* c, const double* xyz, const double* w, uint32_t n,
                     const gbv_ot_options& o, const uint32_t* cand_rp, const uint32_t* cand_ix,
                     cudaStream_t st, double abort_below = 0.0) {
  gbv_cell_report rep{};
  const bool log = ot_log_enabled();
  const bool done =
      laguerre_device(c, xyz, w, n, o.box_min, o.box_max, o.precision == GBV_PRECISION_FP32_RECHECK,
                      cand_rp, cand_ix, st, log ? &rep : nullptr, abort_below);
  if (!done) return false;
  if (log)
    std::fprintf(stderr,
                 "[ot] cells: %.1f ms (knn %.1f, first pass %.1f, rounds %.1f) extra %u huge %u "
                 "overflow %u recheck %u max_clips %u mean_clips %.1f candidates %u exact %llu\n",
                 rep.ms_total, rep.ms_knn, rep.ms_clip, rep.ms_retry, rep.n_more_k, rep.n_huge,
                 rep.n_overflow, rep.n_recheck_fp64, rep.max_clips, rep.mean_clips, rep.knn_k,
                 (unsigned long long)rep.n_exact);
  return true;
}

// Saves the current cells' adjacency as the next call's candidates.
static void save_adjacency(gbv_context* c, uint32_t n, cudaStream_t st, uint32_t** rp,
                           uint32_t** ix) {
  *rp = c->buf<uint32_t>("ot_adj_rp", (size_t)n + 1);
  *ix = c->buf<uint32_t>("ot_adj_ix", std::max<uint64_t>(c->nnz, 1));
  GBV_CUDA(cudaMemcpyAsync(*rp, c->rowptr, sizeof(uint32_t) * ((size_t)n + 1),
                           cudaMemcpyDeviceToDevice, st));
  if (c->nnz)
    GBV_CUDA(cudaMemcpyAsync(*ix, c->nbr, sizeof(uint32_t) * c->nnz, cudaMemcpyDeviceToDevice, st));
}

// Hessian of the current cells, in buffers of the context; with `sell`,
// also its sliced-ELL copy for the CG product.
static Hessian current_hessian(gbv_context* c, const double* xyz, uint32_t n, cudaStream_t st,
                               bool sell = true) {
  Hessian H;
  uint32_t* rp = c->buf<uint32_t>("ot_h_rp", (size_t)n + 1);
  uint32_t* col = c->buf<uint32_t>("ot_h_col", std::max<uint64_t>(c->nnz, 1));
  GBV_CUDA(cudaMemcpyAsync(rp, c->rowptr, sizeof(uint32_t) * ((size_t)n + 1),
                           cudaMemcpyDeviceToDevice, st));
  if (c->nnz)
    GBV_CUDA(cudaMemcpyAsync(col, c->nbr, sizeof(uint32_t) * c->nnz, cudaMemcpyDeviceToDevice, st));
  H.val = c->buf<double>("ot_h_val", std::max<uint64_t>(c->nnz, 1));
  H.diag = c->buf<double>("ot_h_diag", n);
  H.invd = c->buf<double>("ot_h_invd", n);
  assemble_hessian(xyz, rp, col, c->area, n, H, st);
  if (!sell) return H;
  const uint32_t nsl = sell_slices(n);
  uint32_t* sl_off = c->buf<uint32_t>("ot_sl_off", (size_t)nsl + 1);
  GBV_CUDA(cudaMemsetAsync(sl_off, 0, sizeof(uint32_t) * ((size_t)nsl + 1), st));
  sell_widths(H, sl_off, st);
  if (32ull * c->nnz > 0xffffffffull) {  // the slices may not fit 32-bit offsets
    unsigned long long* tot = c->buf<unsigned long long>("ot_sl_total", 1);
    GBV_CUDA(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), st));
    sum_u32_kernel<<<256, 256, 0, st>>>(sl_off, nsl, tot); count_launch();
    unsigned long long h_tot = 0;
    GBV_CUDA(cudaMemcpyAsync(&h_tot, tot, sizeof h_tot, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    if (h_tot > 0xffffffffull)
      throw StatusError{GBV_ERR_CAPACITY, std::to_string(h_tot) +
                                              " padded Hessian entries exceed 32-bit offsets"};
  }
  uint32_t* stmp = c->buf<uint32_t>("ot_sl_scan_tmp", scan_tmp_elems((size_t)nsl + 1));
  exclusive_scan_u32(sl_off, (size_t)nsl + 1, stmp, st);
  uint32_t total = 0;
  GBV_CUDA(cudaMemcpyAsync(&total, sl_off + nsl, 4, cudaMemcpyDeviceToHost, st));
  GBV_CUDA(cudaStreamSynchronize(st));
  uint32_t* s_col = c->buf<uint32_t>("ot_sl_col", std::max<uint32_t>(total, 1));
  double* s_val = c->buf<double>("ot_sl_val", std::max<uint32_t>(total, 1));
  sell_pack(H, sl_off, s_col, s_val, st);
  return H;
}

// Learned start (params non-null): the network predicts t_i = (H0 w*)_i /
// vol_i(0), the Hessian at zero weights applied to the optimal weights over
// the zero-weight cell volume -- the cell-averaged Laplacian of the
// potential, by the Monge-Ampere relation a function of the local density,
// which its inputs see -- and the start solves H0 w = t vol(0).  An exact t
// would give w* itself; errors in t come out smoothed by the inverse
// Laplacian instead of as seed-to-seed noise, which would empty cells.
static void ot_solve(gbv_context* c, const double* xyz, const double* nu_in, uint32_t n,
                     const gbv_ot_options& o, double* w, cudaStream_t st, gbv_ot_report* rep,
                     const float* params = nullptr, const float* norm = nullptr) {
  if (n < 2) throw StatusError{GBV_ERR_INVALID_ARGUMENT, "n must be >= 2"};
  const auto t0 = std::chrono::steady_clock::now();
  double ms_cells = 0.0, ms_lin = 0.0;
  auto now_ms = [&](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  OtWork W(c, n, st);
  const double boxvol = (o.box_max[0] - o.box_min[0]) * (o.box_max[1] - o.box_min[1]) *
                        (o.box_max[2] - o.box_min[2]);
  double* nu = c->buf<double>("ot_nu", n);
  if (nu_in) {
    GBV_CUDA(cudaMemcpyAsync(nu, nu_in, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  } else {
    fill_kernel<<<nblocks(n, 256), 256, 0, st>>>(nu, boxvol / n, n); count_launch();
  }
  double* r = c->buf<double>("ot_r", n);
  double* x = c->buf<double>("ot_x", n);
  double* rr = c->buf<double>("ot_cg_r", n);
  double* p = c->buf<double>("ot_cg_p", n);
  double* Ap = c->buf<double>("ot_cg_ap", n);
  double* z = c->buf<double>("ot_cg_z", n);
  double* ones = c->buf<double>("ot_ones", n);
  double* wt = c->buf<double>("ot_wt", n);
  fill_kernel<<<nblocks(n, 256), 256, 0, st>>>(ones, 1.0, n); count_launch();
  CgScalars* cg_sc = c->buf<CgScalars>("ot_cg_scalars", 1);
  double* cg_part = c->buf<double>("ot_cg_part", 2 * kPcgParts);
  const double nu_norm = std::sqrt(W.dot(nu, nu));
  // x = H^+ b by Jacobi-preconditioned CG; b (overwritten: the residual) is
  // first projected on mean zero (H has the constants as kernel), and so
  // is x at the end.  Returns the iterations.
  auto pcg = [&](const Hessian& H, double* b, double tol) -> uint32_t {
    const double mean = W.dot(b, ones) / n;
    add_scalar(b, -mean, n, st);
    const double bnorm = std::sqrt(W.dot(b, b));
    GBV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
    cg_precond(b, H.invd, z, n, st);
    GBV_CUDA(cudaMemcpyAsync(p, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    const double rz = W.dot(b, z);
    // the iterations run on the device; the host looks at the iteration
    // count and the convergence flag every kCgChunk iterations
    constexpr uint32_t kCgChunk = 16;
    CgScalars h{};
    h.rz = rz;
    h.b2 = bnorm * bnorm;
    h.tol2 = tol * tol;
    h.done = (bnorm > 0.0) ? 0u : 1u;
    GBV_CUDA(cudaMemcpyAsync(cg_sc, &h, sizeof h, cudaMemcpyHostToDevice, st));
    uint32_t k = 0;
    while (!h.done && k < o.max_cg) {
      const uint32_t m = std::min<uint32_t>(kCgChunk, o.max_cg - k);
      pcg_iterations(H, x, b, p, Ap, z, cg_part, cg_sc, m, st);
      GBV_CUDA(cudaMemcpyAsync(&h, cg_sc, sizeof h, cudaMemcpyDeviceToHost, st));
      GBV_CUDA(cudaStreamSynchronize(st));
      k = h.k;
      if (k % kCgChunk != 0) break;  // stopped inside the chunk
    }
    const double xmean = W.dot(x, ones) / n;
    add_scalar(x, -xmean, n, st);
    return k;
  };

  uint32_t *adj_rp = nullptr, *adj_ix = nullptr;
  uint32_t cell_calls = 0, cg_total = 0, halvings = 0, it = 0;
  auto cells = [&](const double* ww, bool with_adj, double abort_below = 0.0) {
    const auto tc = std::chrono::steady_clock::now();
    const bool done = ot_cells(c, xyz, ww, n, o, with_adj ? adj_rp : nullptr,
                               with_adj ? adj_ix : nullptr, st, abort_below);
    ++cell_calls;
    ms_cells += now_ms(tc);
    return done;
  };
  double nu_min = DBL_MAX;
  {
    // min nu through the residual of ones * nu: reuse the min-vol slot
    double a, b2, m;
    W.residual_stats(nu, ones, Ap, a, b2, m);
    nu_min = m;
  }
  double ms_start = 0.0;
  uint32_t start_cg = 0;
  if (params) {
    const auto ts = std::chrono::steady_clock::now();
    GBV_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
    cells(w, false);
    Hessian H0 = current_hessian(c, xyz, n, st);
    float* raw = c->buf<float>("ws_raw", (size_t)n * kMlpIn);
    float* y = c->buf<float>("ws_y", n);
    // b_i = t_i vol_i(0): the network predicts the cell-averaged Laplacian
    double* vol0 = c->buf<double>("ws_vol0", n);
    GBV_CUDA(cudaMemcpyAsync(vol0, c->vol, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    mlp_features_device(c, xyz, n, raw, st);
    mlp_forward_all(c, params, norm, raw, n, y, st);
    mlp_denorm(y, norm, n, rr, st);
    mul_kernel<<<nblocks(n, 256), 256, 0, st>>>(rr, vol0, n); count_launch();
    start_cg = pcg(H0, rr, 1e-6);
    GBV_CUDA(cudaMemcpyAsync(w, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    ms_start = now_ms(ts);
    if (ot_log_enabled())
      std::fprintf(stderr, "[ot] learned start: %.1f ms, %u CG iterations\n", ms_start, start_cg);
  }
  // The damped Newton method needs a start whose cells all have volume
  // (its floor eps0 comes from the start's smallest cell).  A given start
  // (a warm start) with a cell below start_min is scaled toward zero,
  // halving, and replaced by zeros after 10 halvings.
  const double start_min = 1e-8 * nu_min;
  const bool nonzero_start = std::sqrt(W.dot(w, w)) > 0.0;
  double start_scale = 1.0;
  double r2, rel_inf, vmin;
  if (nonzero_start) {
    for (int k = 0;; ++k) {
      if (cells(w, false, start_min)) {
        W.residual_stats(c->vol, nu, r, r2, rel_inf, vmin);
        if (vmin >= start_min) break;
      }
      if (k == 10) {
        GBV_CUDA(cudaMemsetAsync(w, 0, sizeof(double) * n, st));
        start_scale = 0.0;
        break;
      }
      scale_copy(w, w, 0.5, n, st);
      start_scale *= 0.5;
    }
    if (ot_log_enabled())
      std::fprintf(stderr, "[ot] start scaled by %g (min volume %.3e, min nu %.3e)\n",
                   start_scale, vmin, nu_min);
  }
  if (!nonzero_start || start_scale == 0.0) {
    cells(w, false);
    W.residual_stats(c->vol, nu, r, r2, rel_inf, vmin);
  }
  // a start with an empty cell (duplicated seeds) still gets a positive floor
  const double eps0 = vmin > 0.0 ? 0.5 * std::min(nu_min, vmin) : 1e-6 * nu_min;
  bool converged = rel_inf < o.tol;
  double alpha_prev = 1.0;
  for (it = 0; it < o.max_newton && !converged; ++it) {
    save_adjacency(c, n, st, &adj_rp, &adj_ix);
    const auto tl = std::chrono::steady_clock::now();
    Hessian H = current_hessian(c, xyz, n, st);
    // b = -(vol - nu)
    scale_copy(rr, r, -1.0, n, st);
    cg_total += pcg(H, rr, o.cg_rtol > 0.0 ? o.cg_rtol : 1e-4);
    ms_lin += now_ms(tl);
    // damped step (Kitagawa-Merigot-Thibert): halve until every cell keeps
    // at least eps0 and the residual drops by (1 - alpha / 2); the first
    // trial is min(1, step_growth * the previous step), which skips the
    // full steps that early iterations always reject (and whose cells are
    // the costliest to compute)
    double alpha = o.step_growth > 0.0 ? std::min(1.0, o.step_growth * alpha_prev) : 1.0;
    bool accepted = false;
    for (int h = 0; h < 30; ++h) {
      GBV_CUDA(cudaMemcpyAsync(wt, w, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      axpy(wt, x, alpha, n, st);
      // a cell already below eps0 after the first pass rejects the step
      if (!cells(wt, true, eps0)) {
        if (ot_log_enabled())
          std::fprintf(stderr, "[ot] newton %u alpha %g rejected: a cell below eps0\n", it, alpha);
        alpha *= 0.5;
        ++halvings;
        continue;
      }
      double r2t, relt, vmint;
      W.residual_stats(c->vol, nu, r, r2t, relt, vmint);
      if (ot_log_enabled())
        std::fprintf(stderr, "[ot] newton %u alpha %g |r| %.3e -> %.3e max rel %.3e min vol %.3e (eps0 %.3e)\n",
                     it, alpha, std::sqrt(r2), std::sqrt(r2t), relt, vmint, eps0);
      if (vmint >= eps0 && std::sqrt(r2t) <= (1.0 - 0.5 * alpha) * std::sqrt(r2)) {
        GBV_CUDA(cudaMemcpyAsync(w, wt, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        r2 = r2t;
        rel_inf = relt;
        vmin = vmint;
        accepted = true;
        alpha_prev = alpha;
        break;
      }
      alpha *= 0.5;
      ++halvings;
    }
    if (!accepted) {
      // restore the cells of the current weights and stop
      cells(w, true);
      W.residual_stats(c->vol, nu, r, r2, rel_inf, vmin);
      break;
    }
    converged = rel_inf < o.tol;
  }
  GBV_CUDA(cudaStreamSynchronize(st));
  if (rep) {
    rep->converged = converged ? 1 : 0;
    rep->newton_iters = it;
    rep->cg_iters = cg_total;
    rep->halvings = halvings;
    rep->cell_calls = cell_calls;
    rep->mass_error_inf = rel_inf;
    rep->mass_error_l2 = std::sqrt(r2) / nu_norm;
    rep->min_volume = vmin;
    rep->ms_total = now_ms(t0);
    rep->ms_cells = ms_cells;
    rep->ms_linear = ms_lin;
    rep->start_scale = start_scale;
    rep->ms_start = ms_start;
    rep->start_cg_iters = start_cg;
    rep->levels = 1;
  }
}

// ---------------------------------------------------------------------
// Multilevel optimal transport (optimize_levels of the reference's compute_OTM,
// compute_OTM/main.cpp:292-294): solve on nested random subsets of the
// seeds, coarse to fine, each level starting from the coarser one's weights
// interpolated at its seeds.
// ---------------------------------------------------------------------
// Integer hash (the "lowbias32" finaliser published by C. Wellons): the
// level of seed i is set by where hash(i) falls, so levels are nested.
__device__ __forceinline__ uint32_t level_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__global__ void level_flag_kernel(uint32_t n, uint32_t thr, uint32_t* __restrict__ flag) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n) flag[i] = (i < n && level_hash(i) < thr) ? 1u : 0u;
}

__global__ void level_gather_kernel(const double* __restrict__ xyz, const double* __restrict__ nu,
                                    const uint32_t* __restrict__ flag,
                                    const uint32_t* __restrict__ pos, uint32_t n,
                                    double* __restrict__ xo, double* __restrict__ nuo) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flag[i]) return;
  const uint32_t k = pos[i];
  xo[3 * (size_t)k] = xyz[3 * (size_t)i];
  xo[3 * (size_t)k + 1] = xyz[3 * (size_t)i + 1];
  xo[3 * (size_t)k + 2] = xyz[3 * (size_t)i + 2];
  if (nu) nuo[k] = nu[i];
}

// Weighted local linear fit of the coarse weights around each fine seed:
// minimise sum_m g_m (w_m - a - b . (q_m - p))^2 over the kk nearest coarse
// seeds, g_m = exp(-d_m^2 / h^2) with h the distance to the 8th nearest;
// w(p) = a.  Smooth across seeds (no seed-to-seed noise) and exact for
// linear potentials.
__global__ void mls_kernel(const double* __restrict__ xf, const double* __restrict__ xc,
                           const double* __restrict__ wc, const uint32_t* __restrict__ nidx,
                           const double* __restrict__ nd2, uint32_t nf, uint32_t kk,
                           double* __restrict__ wf) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  const double px = xf[3 * (size_t)i], py = xf[3 * (size_t)i + 1], pz = xf[3 * (size_t)i + 2];
  const double h2 = fmax(nd2[(size_t)i * kk + min(kk - 1, 7u)], 1e-300);
  double A[4][4] = {}, r[4] = {};
  double gsum = 0.0, gw = 0.0;
  for (uint32_t m = 0; m < kk; ++m) {
    const uint32_t j = nidx[(size_t)i * kk + m];
    const double g = exp(-nd2[(size_t)i * kk + m] / h2);
    const double v[4] = {1.0, xc[3 * (size_t)j] - px, xc[3 * (size_t)j + 1] - py,
                         xc[3 * (size_t)j + 2] - pz};
    for (int a = 0; a < 4; ++a) {
      r[a] += g * wc[j] * v[a];
      for (int b = 0; b < 4; ++b) A[a][b] += g * v[a] * v[b];
    }
    gsum += g;
    gw += g * wc[j];
  }
  // a little ridge on the slope terms keeps flat neighbourhoods solvable
  for (int a = 1; a < 4; ++a) A[a][a] += 1e-6 * h2 * gsum;
  // Gaussian elimination with partial pivoting (4 x 4)
  bool ok = true;
  for (int c = 0; c < 4 && ok; ++c) {
    int piv = c;
    for (int q = c + 1; q < 4; ++q)
      if (fabs(A[q][c]) > fabs(A[piv][c])) piv = q;
    if (!(fabs(A[piv][c]) > 1e-300)) {
      ok = false;
      break;
    }
    if (piv != c) {
      for (int b = 0; b < 4; ++b) {
        const double t = A[c][b];
        A[c][b] = A[piv][b];
        A[piv][b] = t;
      }
      const double t = r[c];
      r[c] = r[piv];
      r[piv] = t;
    }
    for (int q = c + 1; q < 4; ++q) {
      const double f = A[q][c] / A[c][c];
      for (int b = c; b < 4; ++b) A[q][b] -= f * A[c][b];
      r[q] -= f * r[c];
    }
  }
  double x[4] = {};
  if (ok) {
    for (int c = 3; c >= 0; --c) {
      double t = r[c];
      for (int b = c + 1; b < 4; ++b) t -= A[c][b] * x[b];
      x[c] = t / A[c][c];
    }
  }
  wf[i] = (ok && isfinite(x[0])) ? x[0] : gw / gsum;
}

// Weights at the fine seeds xf (device, nf x 3) from the coarse seeds xc
// and their weights wc.
static void interpolate_weights(gbv_context* c, const double* xc, const double* wc, uint32_t nc,
                                const double* xf, uint32_t nf, double* wf, cudaStream_t st) {
  const uint32_t kk = std::min<uint32_t>(16, nc);
  setup_seeds(c, nc, false);
  c->nn_ready = false;
  c->has_cells = false;
  SortedSeeds& S = c->S;
  build_grid(xc, 3, 3, nullptr, nc, S.L, S, c->scr, st);
  double4* q4 = c->buf<double4>("lvl_q4", nf);
  to_query4_kernel<<<nblocks(nf, 256), 256, 0, st>>>(xf, nf, 3, q4); count_launch();
  uint32_t* oi = c->buf<uint32_t>("lvl_oi", (size_t)nf * kk);
  double* od = c->buf<double>("lvl_od", (size_t)nf * kk);
  KnnArgs ka{};
  ka.S = &S;
  ka.nq = nf;
  ka.qpts = q4;
  ka.k = kk;
  ka.mode = KNN_QUERY;
  ka.exp_idx = oi;
  ka.exp_d2 = od;
  ka.flag_count = c->buf<uint32_t>("knn_flag_count", 1);
  ka.flag_list = c->buf<uint32_t>("lvl_flag_list", nf);
  launch_knn(ka, st);
  mls_kernel<<<nblocks(nf, 128), 128, 0, st>>>(xf, xc, wc, oi, od, nf, kk, wf); count_launch();
  GBV_CUDA(cudaGetLastError());
}

static void ot_solve_levels(gbv_context* c, const double* xyz, const double* nu, uint32_t n,
                            const gbv_ot_options& o, uint32_t ratio, uint32_t min_level,
                            double* w, cudaStream_t st, gbv_ot_report* rep) {
  if (ratio < 2) throw StatusError{GBV_ERR_INVALID_ARGUMENT, "ratio must be >= 2"};
  min_level = std::max<uint32_t>(min_level, 64);
  // level sizes, finest first: n, n / ratio, ... down to >= min_level
  std::vector<uint32_t> target{n};
  while (target.back() / ratio >= min_level) target.push_back(target.back() / ratio);
  std::reverse(target.begin(), target.end());
  const int nl = (int)target.size();
  const auto t0 = std::chrono::steady_clock::now();
  gbv_ot_report total{};
  uint32_t* flag = c->buf<uint32_t>("lvl_flag", (size_t)n + 1);
  uint32_t* pos = c->buf<uint32_t>("lvl_pos", (size_t)n + 1);
  uint32_t* stmp = c->buf<uint32_t>("lvl_scan_tmp", scan_tmp_elems((size_t)n + 1));
  const double* xprev = nullptr;
  double* wprev = nullptr;
  uint32_t mprev = 0;
  for (int l = 0; l < nl; ++l) {
    const bool finest = l == nl - 1;
    const double* xl = xyz;
    const double* nul = nu;
    uint32_t m = n;
    const std::string tag = std::to_string(l & 1);
    if (!finest) {
      // hash threshold for about target[l] seeds
      const uint32_t thr = (uint32_t)std::min<double>(4294967295.0,
                                                      4294967296.0 * target[l] / (double)n);
      level_flag_kernel<<<nblocks((size_t)n + 1, 256), 256, 0, st>>>(n, thr, flag); count_launch();
      GBV_CUDA(cudaMemcpyAsync(pos, flag, sizeof(uint32_t) * ((size_t)n + 1),
                               cudaMemcpyDeviceToDevice, st));
      exclusive_scan_u32(pos, (size_t)n + 1, stmp, st);
      GBV_CUDA(cudaMemcpyAsync(&c->h_counts[0], pos + n, 4, cudaMemcpyDeviceToHost, st));
      GBV_CUDA(cudaStreamSynchronize(st));
      m = c->h_counts[0];
      if (m < 2) continue;
      double* xo = c->buf<double>("lvl_x" + tag, 3 * (size_t)m);
      double* nuo = nu ? c->buf<double>("lvl_nu" + tag, m) : nullptr;
      level_gather_kernel<<<nblocks(n, 256), 256, 0, st>>>(xyz, nu, flag, pos, n, xo, nuo);
      count_launch();
      if (nuo) {
        // the level's masses sum to the box volume
        double* part = c->buf<double>("sum_part", 2 * 256);
        double* outs = c->buf<double>("sum_out", 1);
        sum_partial_kernel<<<256, kSumThreads, 0, st>>>(nuo, m, part); count_launch();
        sum_final_kernel<<<1, 32, 0, st>>>(part, 256, outs); count_launch();
        double sum = 0.0;
        GBV_CUDA(cudaMemcpyAsync(&sum, outs, 8, cudaMemcpyDeviceToHost, st));
        GBV_CUDA(cudaStreamSynchronize(st));
        const double bv = (o.box_max[0] - o.box_min[0]) * (o.box_max[1] - o.box_min[1]) *
                          (o.box_max[2] - o.box_min[2]);
        scale_copy(nuo, nuo, bv / sum, m, st);
      }
      xl = xo;
      nul = nuo;
    }
    double* wl = finest ? w : c->buf<double>("lvl_w" + tag, m);
    if (wprev) interpolate_weights(c, xprev, wprev, mprev, xl, m, wl, st);
    else GBV_CUDA(cudaMemsetAsync(wl, 0, sizeof(double) * m, st));
    gbv_ot_options ol = o;
    if (!finest) ol.tol = std::max(o.tol, 1e-3);
    gbv_ot_report r{};
    ot_solve(c, xl, nul, m, ol, wl, st, &r);
    if (ot_log_enabled())
      std::fprintf(stderr, "[ot] level %d/%d: %u seeds, %u Newton, %u cell passes, %.0f ms, "
                   "start scale %g, mass error %.2e\n", l + 1, nl, m, r.newton_iters,
                   r.cell_calls, r.ms_total, r.start_scale, r.mass_error_inf);
    total.cg_iters += r.cg_iters;
    total.halvings += r.halvings;
    total.cell_calls += r.cell_calls;
    total.ms_cells += r.ms_cells;
    total.ms_linear += r.ms_linear;
    if (finest) {
      total.converged = r.converged;
      total.newton_iters = r.newton_iters;
      total.mass_error_inf = r.mass_error_inf;
      total.mass_error_l2 = r.mass_error_l2;
      total.min_volume = r.min_volume;
      total.start_scale = r.start_scale;
    }
    xprev = xl;
    wprev = wl;
    mprev = m;
  }
  if (rep) {
    *rep = total;
    rep->levels = (uint32_t)nl;
    rep->ms_total =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
}

// Device arguments must be memory of the context's device (or managed
// memory): the kernels run on c->device, and another GPU's memory read
// without peer access is an illegal address.  Checked before any launch.
static void require_device(const gbv_context* c, const void* p, const char* name) {
  if (!p) return;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    throw StatusError{GBV_ERR_INVALID_ARGUMENT, std::string(name) + " is not device memory"};
  }
  if (at.type == cudaMemoryTypeManaged) return;
  if (at.type != cudaMemoryTypeDevice || at.device != c->device)
    throw StatusError{GBV_ERR_INVALID_ARGUMENT,
                      std::string(name) + " must be device memory of the context's device " +
                          std::to_string(c->device)};
}

template <class F>
static gbv_status guarded(F&& f) {
  try {
    f();
    return GBV_OK;
  } catch (const CudaError& e) {
    return fail(GBV_ERR_CUDA, e.where + ": " + cudaGetErrorString(e.e));
  } catch (const StatusError& e) {
    return fail(e.st, e.msg);
  } catch (const std::exception& e) {
    return fail(GBV_ERR_STATE, e.what());
  }
}

static gbv_status check_opts(const gbv_cell_options* o, bool geometry32_ok = true) {
  if (!o) return fail(GBV_ERR_INVALID_ARGUMENT, "options is NULL");
  if (o->precision != GBV_PRECISION_FP64 && o->precision != GBV_PRECISION_FP32_RECHECK &&
      o->precision != GBV_PRECISION_FP32_GEOMETRY)
    return fail(GBV_ERR_INVALID_ARGUMENT, "unknown precision");
  if (o->precision == GBV_PRECISION_FP32_GEOMETRY && !geometry32_ok)
    return fail(GBV_ERR_INVALID_ARGUMENT,
                "GBV_PRECISION_FP32_GEOMETRY is for gbv_cells_* and the Lloyd steps");
  for (int k = 0; k < 3; ++k)
    if (!(o->box_max[k] > o->box_min[k])) return fail(GBV_ERR_INVALID_ARGUMENT, "empty box");
  if (o->k0 == 0) return fail(GBV_ERR_INVALID_ARGUMENT, "k0 must be > 0");
  if (o->certification != GBV_CERTIFY_SECURITY_RADIUS &&
      o->certification != GBV_CERTIFY_POWER_RANGE)
    return fail(GBV_ERR_INVALID_ARGUMENT, "unknown certification");
  if (o->predicates != GBV_PREDICATES_EXACT && o->predicates != GBV_PREDICATES_FAST)
    return fail(GBV_ERR_INVALID_ARGUMENT, "unknown predicates");
  if (o->first_k > kKnnMaxK)
    return fail(GBV_ERR_INVALID_ARGUMENT,
                "first_k must be at most " + std::to_string(kKnnMaxK) + " (0: automatic)");
  return GBV_OK;
}

static gbv_status check_ot_opts(const gbv_ot_options* o) {
  if (!o) return fail(GBV_ERR_INVALID_ARGUMENT, "options is NULL");
  if (o->precision != GBV_PRECISION_FP64 && o->precision != GBV_PRECISION_FP32_RECHECK)
    return fail(GBV_ERR_INVALID_ARGUMENT, "unknown precision");
  for (int k = 0; k < 3; ++k)
    if (!(o->box_max[k] > o->box_min[k])) return fail(GBV_ERR_INVALID_ARGUMENT, "empty box");
  if (!(o->tol > 0.0)) return fail(GBV_ERR_INVALID_ARGUMENT, "tol must be > 0");
  return GBV_OK;
}

}  // namespace gbv

using namespace gbv;

extern "C" {

const char* gbv_last_error(void) { return g_last_error.c_str(); }

uint64_t gbv_kernel_launches(void) { return g_launches.load(); }

uint64_t gbv_device_bytes(const gbv_context* c, uint64_t* peak) {
  if (!c) return 0;
  uint64_t total = 0;
  for (const auto& kv : c->bufs) total += kv.second.second;
  if (peak) *peak = c->peak_bytes;
  return total;
}

void gbv_cell_options_default(gbv_cell_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  for (int k = 0; k < 3; ++k) {
    o->box_min[k] = 0.0;
    o->box_max[k] = 1.0;
  }
  o->k0 = 20;
  o->check_sr = 1;
  o->precision = GBV_PRECISION_FP64;
}

gbv_status gbv_create(int device, gbv_context** out) {
  if (!out) return fail(GBV_ERR_INVALID_ARGUMENT, "out is NULL");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(GBV_ERR_NO_DEVICE, "no CUDA device");
  }
  if (device < 0 || device >= ndev) return fail(GBV_ERR_INVALID_ARGUMENT, "bad device index");
  gbv_context* c = new gbv_context();
  c->device = device;
  gbv_status st = guarded([&] {
    GBV_CUDA(cudaSetDevice(device));
    GBV_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    for (auto& e : c->ev) GBV_CUDA(cudaEventCreate(&e));
    c->counters = c->buf<unsigned long long>("counters", 4);
    c->list_counts = c->buf<uint32_t>("list_counts", 4);
    GBV_CUDA(cudaMallocHost(&c->h_counts, 8 * sizeof(uint32_t)));
    GBV_CUDA(cudaMallocHost(&c->h_clipc, 2 * sizeof(unsigned long long)));
  });
  if (st != GBV_OK) {
    gbv_destroy(c);  // releases whatever was created before the failure
    return st;
  }
  *out = c;
  return GBV_OK;
}

gbv_status gbv_destroy(gbv_context* c) {
  if (!c) return GBV_OK;
  cudaSetDevice(c->device);
  for (auto& kv : c->bufs) cudaFree(kv.second.first);
  if (c->h_counts) cudaFreeHost(c->h_counts);
  if (c->h_clipc) cudaFreeHost(c->h_clipc);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return GBV_OK;
}

gbv_status gbv_cells_compute_device(gbv_context* c, const double* d_xyz, const double* d_w,
                                    uint32_t n, const gbv_cell_options* opt, void* stream,
                                    gbv_cell_report* report) {
  if (!c || !d_xyz) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_w, "d_w");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    if (opt->certification == GBV_CERTIFY_POWER_RANGE)
      laguerre_device(c, d_xyz, d_w, n, opt->box_min, opt->box_max,
                      opt->precision != GBV_PRECISION_FP64, nullptr, nullptr, st, report);
    else
      cells_device(c, d_xyz, d_w, n, *opt, st, report);
  });
}

gbv_status gbv_cells_compute(gbv_context* c, const double* xyz, const double* w, uint32_t n,
                             const gbv_cell_options* opt, gbv_cell_report* report) {
  if (!c || !xyz) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    double* dx = c->buf<double>("in_xyz", 3 * (size_t)n);
    double* dw = w ? c->buf<double>("in_w", n) : nullptr;
    GBV_CUDA(cudaMemcpyAsync(dx, xyz, 3 * sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    if (w) GBV_CUDA(cudaMemcpyAsync(dw, w, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    if (opt->certification == GBV_CERTIFY_POWER_RANGE)
      laguerre_device(c, dx, dw, n, opt->box_min, opt->box_max,
                      opt->precision != GBV_PRECISION_FP64, nullptr, nullptr, c->stream,
                      report);
    else
      cells_device(c, dx, dw, n, *opt, c->stream, report);
  });
}

gbv_status gbv_periodic_cells(gbv_context* c, const double* xyz, const double* w, uint32_t n,
                              double period, const gbv_cell_options* opt,
                              gbv_cell_report* report) {
  if (!c || !xyz) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n < 2) return fail(GBV_ERR_INVALID_ARGUMENT, "n must be >= 2");
  if (!(period > 0.0)) return fail(GBV_ERR_INVALID_ARGUMENT, "period must be > 0");
  gbv_status s = check_opts(opt, false);
  if (s != GBV_OK) return s;
  if (opt->certification != GBV_CERTIFY_SECURITY_RADIUS || !opt->check_sr)
    return fail(GBV_ERR_INVALID_ARGUMENT, "periodic cells use the security-radius loop");
  for (uint32_t i = 0; i < 3 * n; ++i)
    if (!(xyz[i] >= 0.0 && xyz[i] < period))
      return fail(GBV_ERR_INVALID_ARGUMENT, "seeds must lie in [0, period)^3");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    c->has_periodic = false;
    double W = 0.0, wmin = 0.0;
    if (w) {
      W = wmin = w[0];
      for (uint32_t i = 1; i < n; ++i) {
        W = std::max(W, w[i]);
        wmin = std::min(wmin, w[i]);
      }
    }
    double* dx = c->buf<double>("per_in_xyz", 3 * (size_t)n);
    double* dw = w ? c->buf<double>("per_in_w", n) : nullptr;
    GBV_CUDA(cudaMemcpyAsync(dx, xyz, 24 * (size_t)n, cudaMemcpyHostToDevice, st));
    if (w) GBV_CUDA(cudaMemcpyAsync(dw, w, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    // a first layer of about four seed spacings plus the lift range; widened
    // (doubling) while some cell's security ball leaves the ghost box
    double delta = std::min(period, 4.0 * period * std::cbrt(1.0 / n) + 2.0 * std::sqrt(W - wmin));
    for (int round = 0;; ++round) {
      double *ax = nullptr, *aw = nullptr;
      const uint32_t na = periodic_ghosts(c, dx, dw, n, period, delta, st, &ax, &aw);
      gbv_cell_options o = *opt;
      for (int k = 0; k < 3; ++k) {
        o.box_min[k] = -delta;
        o.box_max[k] = period + delta;
      }
      cells_device(c, ax, aw, na, o, st, report);
      const uint32_t fails = periodic_reach_failures(c, n, ax, aw, W, period, delta, st);
      if (fails == 0) break;
      if (delta >= period || round >= 8)
        throw StatusError{GBV_ERR_NOT_CONVERGED,
                          std::to_string(fails) + " periodic cell(s) reach beyond one period"};
      delta = std::min(period, 2.0 * delta);
    }
    uint32_t nnz = 0;
    periodic_remap(c, n, st, &c->per_nbr, &c->per_shift, &nnz);
    GBV_CUDA(cudaStreamSynchronize(st));
    c->per_n = n;
    c->per_nnz = nnz;
    c->has_periodic = true;
    if (report) {
      report->n_cells = n;
      report->nnz = nnz;
    }
  });
}

gbv_status gbv_periodic_fetch(gbv_context* c, double* vol, double* mg, uint32_t* rowptr,
                              uint32_t* nbr, uint8_t* shift, double* area) {
  if (!c) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL context");
  if (!c->has_periodic || !c->has_cells) return fail(GBV_ERR_STATE, "no periodic cells computed");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const size_t n = c->per_n, nnz = c->per_nnz;
    if (vol) GBV_CUDA(cudaMemcpyAsync(vol, c->vol, 8 * n, cudaMemcpyDeviceToHost, st));
    if (mg) GBV_CUDA(cudaMemcpyAsync(mg, c->mg, 24 * n, cudaMemcpyDeviceToHost, st));
    if (rowptr) GBV_CUDA(cudaMemcpyAsync(rowptr, c->rowptr, 4 * (n + 1), cudaMemcpyDeviceToHost, st));
    if (nbr && nnz) GBV_CUDA(cudaMemcpyAsync(nbr, c->per_nbr, 4 * nnz, cudaMemcpyDeviceToHost, st));
    if (shift && nnz) GBV_CUDA(cudaMemcpyAsync(shift, c->per_shift, nnz, cudaMemcpyDeviceToHost, st));
    if (area && nnz) GBV_CUDA(cudaMemcpyAsync(area, c->area, 8 * nnz, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

// Restricted cells of the seeds xyz (host) on the mesh already on the device
// (dmv, dt): per-cell m, mg, the CVT energy and its gradient; the box is
// the bounding box of the mesh and the seeds.
static void restricted_eval(gbv_context* c, const double* mesh_xyz, uint32_t nv, const double* dmv,
                            const uint32_t* dt, uint32_t nt, const double* xyz, const double* w,
                            uint32_t n, const gbv_cell_options& opt, double* m, double* mg,
                            double* f, double* g, gbv_cell_report* report) {
  cudaStream_t st = c->stream;
  gbv_cell_options o = opt;
  for (int k = 0; k < 3; ++k) {
    o.box_min[k] = DBL_MAX;
    o.box_max[k] = -DBL_MAX;
  }
  auto grow = [&](const double* p) {
    for (int k = 0; k < 3; ++k) {
      o.box_min[k] = std::min(o.box_min[k], p[k]);
      o.box_max[k] = std::max(o.box_max[k], p[k]);
    }
  };
  for (uint32_t v = 0; v < nv; ++v) grow(mesh_xyz + 3 * (size_t)v);
  for (uint32_t i = 0; i < n; ++i) grow(xyz + 3 * (size_t)i);
  for (int k = 0; k < 3; ++k)
    if (!(o.box_max[k] > o.box_min[k])) throw StatusError{GBV_ERR_INVALID_ARGUMENT, "flat mesh"};
  double* dx = c->buf<double>("in_xyz", 3 * (size_t)n);
  double* dw = w ? c->buf<double>("in_w", n) : nullptr;
  GBV_CUDA(cudaMemcpyAsync(dx, xyz, 24 * (size_t)n, cudaMemcpyHostToDevice, st));
  if (w) GBV_CUDA(cudaMemcpyAsync(dw, w, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
  cells_device(c, dx, dw, n, o, st, report);
  double* dm = c->buf<double>("rv_m", n);
  double* dmg = c->buf<double>("rv_mg", 3 * (size_t)n);
  double* dF = c->buf<double>("rv_F", n);
  double* dg = c->buf<double>("rv_g", 3 * (size_t)n);
  restricted_cells(c, dx, dw, n, dmv, nv, dt, nt, st, dm, dmg, dF, dg);
  if (m) GBV_CUDA(cudaMemcpyAsync(m, dm, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
  if (mg) GBV_CUDA(cudaMemcpyAsync(mg, dmg, 24 * (size_t)n, cudaMemcpyDeviceToHost, st));
  if (g) GBV_CUDA(cudaMemcpyAsync(g, dg, 24 * (size_t)n, cudaMemcpyDeviceToHost, st));
  if (f) {
    // deterministic FP64 sum of the per-cell energies
    double* part = c->buf<double>("rv_part", 2 * kOtParts);
    double* ones = c->buf<double>("rv_ones", n);
    fill_kernel<<<nblocks(n, 256), 256, 0, st>>>(ones, 1.0, n); count_launch();
    dot_parts(dF, ones, n, part, st);
    std::vector<double> hp(2 * kOtParts);
    GBV_CUDA(cudaMemcpyAsync(hp.data(), part, 16 * kOtParts, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    double S = 0.0, C = 0.0;
    for (int b = 0; b < kOtParts; ++b) {
      const double x = hp[2 * b], t = S + x;
      if (std::fabs(S) >= std::fabs(x)) C += (S - t) + x;
      else C += (x - t) + S;
      S = t;
      C += hp[2 * b + 1];
    }
    *f = S + C;
  }
  GBV_CUDA(cudaStreamSynchronize(st));
}

gbv_status gbv_restricted_cells(gbv_context* c, const double* mesh_xyz, uint32_t nv,
                                const uint32_t* tets, uint32_t nt, const double* xyz,
                                const double* w, uint32_t n, const gbv_cell_options* opt,
                                double* m, double* mg, double* f, double* g,
                                gbv_cell_report* report) {
  if (!c || !mesh_xyz || !tets || !xyz) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (nv == 0 || nt == 0 || n == 0) return fail(GBV_ERR_INVALID_ARGUMENT, "empty mesh or seeds");
  gbv_status s = check_opts(opt, false);
  if (s != GBV_OK) return s;
  if (opt->certification != GBV_CERTIFY_SECURITY_RADIUS)
    return fail(GBV_ERR_INVALID_ARGUMENT, "restricted cells use the security-radius loop");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    double* dmv = c->buf<double>("rv_mesh_xyz", 3 * (size_t)nv);
    uint32_t* dt = c->buf<uint32_t>("rv_tets_in", 4 * (size_t)nt);
    GBV_CUDA(cudaMemcpyAsync(dmv, mesh_xyz, 24 * (size_t)nv, cudaMemcpyHostToDevice, c->stream));
    GBV_CUDA(cudaMemcpyAsync(dt, tets, 16 * (size_t)nt, cudaMemcpyHostToDevice, c->stream));
    restricted_eval(c, mesh_xyz, nv, dmv, dt, nt, xyz, w, n, *opt, m, mg, f, g, report);
  });
}

gbv_status gbv_cvt_newton(gbv_context* c, const double* mesh_xyz, uint32_t nv,
                          const uint32_t* tets, uint32_t nt, double* xyz, uint32_t n,
                          const gbv_cell_options* opt, uint32_t nb_iter, uint32_t m,
                          double* energy, uint32_t* iterations) {
  if (!c || !mesh_xyz || !tets || !xyz) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (nv == 0 || nt == 0 || n == 0) return fail(GBV_ERR_INVALID_ARGUMENT, "empty mesh or seeds");
  if (m == 0) return fail(GBV_ERR_INVALID_ARGUMENT, "m must be > 0");
  gbv_status s = check_opts(opt, false);
  if (s != GBV_OK) return s;
  if (opt->certification != GBV_CERTIFY_SECURITY_RADIUS)
    return fail(GBV_ERR_INVALID_ARGUMENT, "restricted cells use the security-radius loop");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    double* dmv = c->buf<double>("rv_mesh_xyz", 3 * (size_t)nv);
    uint32_t* dt = c->buf<uint32_t>("rv_tets_in", 4 * (size_t)nt);
    GBV_CUDA(cudaMemcpyAsync(dmv, mesh_xyz, 24 * (size_t)nv, cudaMemcpyHostToDevice, c->stream));
    GBV_CUDA(cudaMemcpyAsync(dt, tets, 16 * (size_t)nt, cudaMemcpyHostToDevice, c->stream));
    std::vector<double> x(xyz, xyz + 3 * (size_t)n);
    // HLBFGS stops once its iteration count exceeds max_iter
    // (third_party/HLBFGS/HLBFGS.cpp:580), so the reference's
    // Newton_iterations(nb_iter) takes nb_iter + 1 steps: so does this
    LbfgsParams prm;
    prm.m = (int)m;
    prm.max_iter = (int)nb_iter + 1;
    auto fg = [&](const std::vector<double>& p, std::vector<double>& g) -> double {
      double f = 0.0;
      restricted_eval(c, mesh_xyz, nv, dmv, dt, nt, p.data(), nullptr, n, *opt, nullptr, nullptr,
                      &f, g.data(), nullptr);
      return f;
    };
    if (energy) energy[0] = 0.0;
    bool first = true;
    auto newiter = [&](int it, const std::vector<double>&, double f, const std::vector<double>&) {
      if (energy && (uint32_t)it <= nb_iter + 1) energy[it] = f;
    };
    const LbfgsResult r = lbfgs_minimize(
        x, prm,
        [&](const std::vector<double>& p, std::vector<double>& g) {
          const double f = fg(p, g);
          if (first && energy) energy[0] = f;
          first = false;
          return f;
        },
        newiter);
    std::copy(x.begin(), x.end(), xyz);
    if (iterations) *iterations = (uint32_t)r.iterations;
  });
}

gbv_status gbv_cells_fetch(gbv_context* c, double* vol, double* mg, uint32_t* rowptr,
                           uint32_t* nbr, double* area, int32_t* status) {
  if (!c) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL context");
  if (!c->has_cells) return fail(GBV_ERR_STATE, "no cells computed");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const size_t n = c->n;
    if (vol) GBV_CUDA(cudaMemcpyAsync(vol, c->vol, 8 * n, cudaMemcpyDeviceToHost, st));
    if (mg) GBV_CUDA(cudaMemcpyAsync(mg, c->mg, 24 * n, cudaMemcpyDeviceToHost, st));
    if (rowptr) GBV_CUDA(cudaMemcpyAsync(rowptr, c->rowptr, 4 * (n + 1), cudaMemcpyDeviceToHost, st));
    if (nbr && c->nnz) GBV_CUDA(cudaMemcpyAsync(nbr, c->nbr, 4 * c->nnz, cudaMemcpyDeviceToHost, st));
    if (area && c->nnz) GBV_CUDA(cudaMemcpyAsync(area, c->area, 8 * c->nnz, cudaMemcpyDeviceToHost, st));
    if (status) GBV_CUDA(cudaMemcpyAsync(status, c->status, 4 * n, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

gbv_status gbv_cells_device_results(gbv_context* c, const double** vol, const double** mg,
                                    const uint32_t** rowptr, const uint32_t** nbr,
                                    const double** area, const int32_t** status) {
  if (!c) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL context");
  if (!c->has_cells) return fail(GBV_ERR_STATE, "no cells computed");
  if (vol) *vol = c->vol;
  if (mg) *mg = c->mg;
  if (rowptr) *rowptr = c->rowptr;
  if (nbr) *nbr = c->nbr;
  if (area) *area = c->area;
  if (status) *status = c->status;
  return GBV_OK;
}

gbv_status gbv_lloyd_device(gbv_context* c, double* d_xyz, const double* d_w, uint32_t n,
                            uint32_t iters, const gbv_cell_options* opt, void* stream,
                            gbv_cell_report* report) {
  if (!c || !d_xyz) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_w, "d_w");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    for (uint32_t it = 0; it < iters; ++it) {
      cells_device(c, d_xyz, d_w, n, *opt, st, report);
      lloyd_update_kernel<<<nblocks(n, 256), 256, 0, st>>>(d_xyz, c->vol, c->mg, n); count_launch();
    }
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

gbv_status gbv_lloyd_step(gbv_context* c, double* xyz, const double* w, uint32_t n,
                          const gbv_cell_options* opt, gbv_cell_report* report) {
  if (!c || !xyz) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    double* dx = c->buf<double>("lloyd_xyz", 3 * (size_t)n);
    double* dw = w ? c->buf<double>("in_w", n) : nullptr;
    GBV_CUDA(cudaMemcpyAsync(dx, xyz, 24 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    if (w) GBV_CUDA(cudaMemcpyAsync(dw, w, 8 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    cells_device(c, dx, dw, n, *opt, c->stream, report);
    lloyd_update_kernel<<<nblocks(n, 256), 256, 0, c->stream>>>(dx, c->vol, c->mg, n); count_launch();
    GBV_CUDA(cudaMemcpyAsync(xyz, dx, 24 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    GBV_CUDA(cudaStreamSynchronize(c->stream));
  });
}

gbv_status gbv_nn_set_points(gbv_context* c, uint32_t n, const double* pts, uint32_t dim,
                             uint32_t stride) {
  if (!c || !pts) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n == 0) return fail(GBV_ERR_INVALID_ARGUMENT, "n must be > 0");
  if (dim != 3 && dim != 4) return fail(GBV_ERR_INVALID_ARGUMENT, "dim must be 3 or 4");
  if (stride < dim) return fail(GBV_ERR_INVALID_ARGUMENT, "stride < dim");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    double* dp = c->buf<double>("nn_pts", (size_t)n * stride);
    GBV_CUDA(cudaMemcpyAsync(dp, pts, sizeof(double) * (size_t)n * stride,
                             cudaMemcpyHostToDevice, c->stream));
    setup_seeds(c, n, false);
    build_grid(dp, stride, dim, nullptr, n, c->S.L, c->S, c->scr, c->stream);
    GBV_CUDA(cudaStreamSynchronize(c->stream));
    c->nn_ready = true;
    c->nn_n = n;
    c->nn_dim = dim;
    c->has_cells = false;
  });
}

gbv_status gbv_nn_get_nearest_neighbors(gbv_context* c, uint32_t nq, const double* q, uint32_t k,
                                        uint32_t* idx, double* d2) {
  if (!c || !q || !idx) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!c->nn_ready) return fail(GBV_ERR_STATE, "set_points was not called");
  if (k == 0 || k > c->nn_n) return fail(GBV_ERR_INVALID_ARGUMENT, "need 0 < k <= n");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    double* dq = c->buf<double>("nn_q", (size_t)nq * c->nn_dim);
    double4* q4 = c->buf<double4>("nn_q4", nq);
    uint32_t* oi = c->buf<uint32_t>("nn_oi", (size_t)nq * k);
    double* od = c->buf<double>("nn_od", (size_t)nq * k);
    GBV_CUDA(cudaMemcpyAsync(dq, q, sizeof(double) * (size_t)nq * c->nn_dim,
                             cudaMemcpyHostToDevice, st));
    to_query4_kernel<<<nblocks(nq, 256), 256, 0, st>>>(dq, nq, c->nn_dim, q4); count_launch();
    KnnArgs ka{};
    ka.S = &c->S;
    ka.nq = nq;
    ka.qpts = q4;
    ka.k = k;
    ka.mode = KNN_QUERY;
    ka.exp_idx = oi;
    ka.exp_d2 = od;
    ka.flag_count = c->buf<uint32_t>("knn_flag_count", 1);
    ka.flag_list = c->buf<uint32_t>("nn_flag_list", nq);
    if (k > kKnnMaxK) {
      ka.gl_d2 = c->buf<double>("nn_gd2", (size_t)k * nq);
      ka.gl_slot = c->buf<uint32_t>("nn_gslot", (size_t)k * nq);
    }
    launch_knn(ka, st);
    GBV_CUDA(cudaMemcpyAsync(idx, oi, 4 * (size_t)nq * k, cudaMemcpyDeviceToHost, st));
    if (d2) GBV_CUDA(cudaMemcpyAsync(d2, od, 8 * (size_t)nq * k, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    GBV_CUDA(cudaGetLastError());
  });
}

gbv_status gbv_nn_get_nearest_neighbors_all(gbv_context* c, uint32_t k, uint32_t* idx,
                                            double* d2) {
  if (!c || !idx) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!c->nn_ready) return fail(GBV_ERR_STATE, "set_points was not called");
  if (k == 0 || k > c->nn_n) return fail(GBV_ERR_INVALID_ARGUMENT, "need 0 < k <= n");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const uint32_t n = c->nn_n;
    uint32_t* oi = c->buf<uint32_t>("nn_oi", (size_t)n * k);
    double* od = c->buf<double>("nn_od", (size_t)n * k);
    KnnArgs ka{};
    ka.S = &c->S;
    ka.nq = n;
    ka.k = k;
    ka.mode = KNN_ALL;
    ka.exp_idx = oi;
    ka.exp_d2 = od;
    ka.flag_count = c->buf<uint32_t>("knn_flag_count", 1);
    ka.flag_list = c->buf<uint32_t>("nn_flag_list", n);
    ka.coherent = true;
    ka.tile_scratch = c->buf<uint32_t>("knn_tiles", knn_tile_scratch_elems(n, c->S.L));
    if (k > kKnnMaxK) {
      ka.gl_d2 = c->buf<double>("nn_gd2", (size_t)k * n);
      ka.gl_slot = c->buf<uint32_t>("nn_gslot", (size_t)k * n);
    }
    launch_knn(ka, st);
    GBV_CUDA(cudaMemcpyAsync(idx, oi, 4 * (size_t)n * k, cudaMemcpyDeviceToHost, st));
    if (d2) GBV_CUDA(cudaMemcpyAsync(d2, od, 8 * (size_t)n * k, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    GBV_CUDA(cudaGetLastError());
  });
}

gbv_status gbv_mlp_features(gbv_context* c, const double* d_xyz, uint32_t n, float* d_raw,
                            void* stream) {
  if (!c || !d_xyz || !d_raw) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_raw, "d_raw");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    mlp_features_device(c, d_xyz, n, d_raw, st);
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

gbv_status gbv_mlp_forward(gbv_context* c, const float* d_params, const float* d_norm,
                           const float* d_raw, uint32_t n, float* d_y, void* stream) {
  if (!c || !d_params || !d_norm || !d_raw || !d_y)
    return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n == 0) return fail(GBV_ERR_INVALID_ARGUMENT, "n must be > 0");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_params, "d_params"); require_device(c, d_norm, "d_norm");
    require_device(c, d_raw, "d_raw"); require_device(c, d_y, "d_y");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    mlp_forward_all(c, d_params, d_norm, d_raw, n, d_y, st);
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

gbv_status gbv_mlp_loss_grad(gbv_context* c, const float* d_params, const float* d_norm,
                             const float* d_raw, const float* d_target, uint32_t n,
                             float* d_grad, double* loss, void* stream) {
  if (!c || !d_params || !d_norm || !d_raw || !d_target || !d_grad)
    return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n == 0 || n > kMlpChunk)
    return fail(GBV_ERR_INVALID_ARGUMENT, "batch must hold 1 to GBV_MLP_MAX_BATCH rows");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_params, "d_params"); require_device(c, d_norm, "d_norm");
    require_device(c, d_raw, "d_raw"); require_device(c, d_target, "d_target");
    require_device(c, d_grad, "d_grad");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    MlpBuffers B = mlp_buffers(c, n);
    mlp_loss_grad(d_params, d_norm, d_raw, d_target, n, d_grad, B, st);
    double hp[kMlpLossParts];
    GBV_CUDA(cudaMemcpyAsync(hp, B.lpart, sizeof(hp), cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
    double s = 0.0;
    for (double v : hp) s += v;
    if (loss) *loss = s;
    GBV_CUDA(cudaGetLastError());
  });
}

gbv_status gbv_mlp_adam(gbv_context* c, float* d_params, float* d_m, float* d_v,
                        const float* d_grad, uint32_t step, float lr, float beta1, float beta2,
                        float eps, void* stream) {
  if (!c || !d_params || !d_m || !d_v || !d_grad)
    return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (step == 0) return fail(GBV_ERR_INVALID_ARGUMENT, "step counts from 1");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_params, "d_params"); require_device(c, d_m, "d_m");
    require_device(c, d_v, "d_v"); require_device(c, d_grad, "d_grad");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    mlp_adam(d_params, d_m, d_v, d_grad, step, lr, beta1, beta2, eps, st);
    GBV_CUDA(cudaGetLastError());
  });
}

gbv_status gbv_ot_warm_start(gbv_context* c, const double* d_xyz, uint32_t n,
                             const gbv_ot_options* opt, const float* d_params,
                             const float* d_norm, double* d_w, void* stream) {
  if (!c || !d_xyz || !d_params || !d_norm || !d_w)
    return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_params, "d_params");
    require_device(c, d_norm, "d_norm"); require_device(c, d_w, "d_w");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    gbv_ot_options o = *opt;
    o.max_newton = 0;
    ot_solve(c, d_xyz, nullptr, n, o, d_w, st, nullptr, d_params, d_norm);
  });
}

gbv_status gbv_ot_separable_start(gbv_context* c, const double* d_xyz, uint32_t n,
                                  const gbv_ot_options* opt, double* d_w, void* stream) {
  if (!c || !d_xyz || !d_w) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n == 0 || n > 0x80000000u) return fail(GBV_ERR_INVALID_ARGUMENT, "n must be in [1, 2^31]");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_w, "d_w");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    const size_t m = start_sort_len(n);
    double* key = c->buf<double>("start_key", m);
    uint32_t* val = c->buf<uint32_t>("start_val", m);
    double* chunk = c->buf<double>("start_chunk", start_chunks(n));
    separable_start(d_xyz, n, opt->box_min, opt->box_max, key, val, chunk, d_w, st);
    GBV_CUDA(cudaGetLastError());
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

gbv_status gbv_ot_solve_levels_device(gbv_context* c, const double* d_xyz, const double* d_nu,
                                      uint32_t n, const gbv_ot_options* opt, uint32_t ratio,
                                      uint32_t min_level, double* d_w, void* stream,
                                      gbv_ot_report* report) {
  if (!c || !d_xyz || !d_w) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_nu, "d_nu");
    require_device(c, d_w, "d_w");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    ot_solve_levels(c, d_xyz, d_nu, n, *opt, ratio, min_level, d_w, st, report);
  });
}

gbv_status gbv_ot_solve_levels(gbv_context* c, const double* xyz, const double* nu, uint32_t n,
                               const gbv_ot_options* opt, uint32_t ratio, uint32_t min_level,
                               double* w, gbv_ot_report* report) {
  if (!c || !xyz || !w) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    double* dx = c->buf<double>("ot_in_xyz", 3 * (size_t)n);
    double* dw = c->buf<double>("ot_in_w", n);
    double* dnu = nu ? c->buf<double>("ot_in_nu", n) : nullptr;
    GBV_CUDA(cudaMemcpyAsync(dx, xyz, 24 * (size_t)n, cudaMemcpyHostToDevice, st));
    if (nu) GBV_CUDA(cudaMemcpyAsync(dnu, nu, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    ot_solve_levels(c, dx, dnu, n, *opt, ratio, min_level, dw, st, report);
    GBV_CUDA(cudaMemcpyAsync(w, dw, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

gbv_status gbv_ot_solve_learned_device(gbv_context* c, const double* d_xyz, const double* d_nu,
                                       uint32_t n, const gbv_ot_options* opt,
                                       const float* d_params, const float* d_norm, double* d_w,
                                       void* stream, gbv_ot_report* report) {
  if (!c || !d_xyz || !d_params || !d_norm || !d_w)
    return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_nu, "d_nu");
    require_device(c, d_params, "d_params"); require_device(c, d_norm, "d_norm");
    require_device(c, d_w, "d_w");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    ot_solve(c, d_xyz, d_nu, n, *opt, d_w, st, report, d_params, d_norm);
  });
}

gbv_status gbv_mlp_gemm_nt(gbv_context* c, const void* d_a, int lda, const void* d_bt, int ldb,
                           float* d_c, int ldc, int M, int N, int K, void* stream) {
  if (!c || !d_a || !d_bt || !d_c) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (M <= 0 || N <= 0 || K <= 0 || K % 32 || lda % 8 || ldb % 8 || lda < K || ldb < K ||
      ldc < N)
    return fail(GBV_ERR_INVALID_ARGUMENT, "bad GEMM shape");
  if (((uintptr_t)d_a | (uintptr_t)d_bt) & 15)
    return fail(GBV_ERR_INVALID_ARGUMENT, "operands must be 16-byte aligned");
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_a, "d_a"); require_device(c, d_bt, "d_bt"); require_device(c, d_c, "d_c");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    gemm_nt((const bf16*)d_a, lda, (const bf16*)d_bt, ldb, d_c, ldc, M, N, K, 1, 0, st);
    GBV_CUDA(cudaStreamSynchronize(st));
    GBV_CUDA(cudaGetLastError());
  });
}

void gbv_ot_options_default(gbv_ot_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  for (int k = 0; k < 3; ++k) {
    o->box_min[k] = 0.0;
    o->box_max[k] = 1.0;
  }
  o->tol = 1e-6;
  o->max_newton = 100;
  o->max_cg = 4000;
  o->precision = GBV_PRECISION_FP32_RECHECK;
  o->cg_rtol = 1e-4;
  o->step_growth = 4.0;
}

gbv_status gbv_ot_solve_device(gbv_context* c, const double* d_xyz, const double* d_nu, uint32_t n,
                               const gbv_ot_options* opt, double* d_w, void* stream,
                               gbv_ot_report* report) {
  if (!c || !d_xyz || !d_w) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    require_device(c, d_xyz, "d_xyz"); require_device(c, d_nu, "d_nu");
    require_device(c, d_w, "d_w");
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    ot_solve(c, d_xyz, d_nu, n, *opt, d_w, st, report);
  });
}

gbv_status gbv_ot_solve(gbv_context* c, const double* xyz, const double* nu, uint32_t n,
                        const gbv_ot_options* opt, double* w, gbv_ot_report* report) {
  if (!c || !xyz || !w) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    double* dx = c->buf<double>("ot_in_xyz", 3 * (size_t)n);
    double* dw = c->buf<double>("ot_in_w", n);
    double* dnu = nu ? c->buf<double>("ot_in_nu", n) : nullptr;
    GBV_CUDA(cudaMemcpyAsync(dx, xyz, 24 * (size_t)n, cudaMemcpyHostToDevice, st));
    GBV_CUDA(cudaMemcpyAsync(dw, w, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    if (nu) GBV_CUDA(cudaMemcpyAsync(dnu, nu, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    ot_solve(c, dx, dnu, n, *opt, dw, st, report);
    GBV_CUDA(cudaMemcpyAsync(w, dw, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

gbv_status gbv_ot_gradient_hessian(gbv_context* c, const double* xyz, const double* w,
                                   const double* nu, uint32_t n, const gbv_ot_options* opt,
                                   double* g, uint32_t* h_rowptr, uint32_t* h_col, double* h_val,
                                   double* h_diag, uint64_t h_capacity, uint64_t* nnz) {
  if (!c || !xyz || !w) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  gbv_status s = check_ot_opts(opt);
  if (s != GBV_OK) return s;
  return guarded([&] {
    GBV_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    double* dx = c->buf<double>("ot_in_xyz", 3 * (size_t)n);
    double* dw = c->buf<double>("ot_in_w", n);
    double* dnu = c->buf<double>("ot_in_nu", n);
    GBV_CUDA(cudaMemcpyAsync(dx, xyz, 24 * (size_t)n, cudaMemcpyHostToDevice, st));
    GBV_CUDA(cudaMemcpyAsync(dw, w, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    const double boxvol = (opt->box_max[0] - opt->box_min[0]) * (opt->box_max[1] - opt->box_min[1]) *
                          (opt->box_max[2] - opt->box_min[2]);
    if (nu) GBV_CUDA(cudaMemcpyAsync(dnu, nu, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    else { fill_kernel<<<nblocks(n, 256), 256, 0, st>>>(dnu, boxvol / n, n); count_launch(); }
    ot_cells(c, dx, dw, n, *opt, nullptr, nullptr, st);
    if (nnz) *nnz = c->nnz;
    if (g) {
      double* dg = c->buf<double>("ot_grad", n);
      residual(c->vol, dnu, n, dg, c->buf<double>("ot_part", 4 * kOtParts), st);
      scale_copy(dg, dg, -1.0, n, st);  // g = nu - vol
      GBV_CUDA(cudaMemcpyAsync(g, dg, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
    }
    if (h_capacity > 0) {
      if (h_capacity < c->nnz) throw StatusError{GBV_ERR_CAPACITY, "Hessian capacity too small"};
      Hessian H = current_hessian(c, dx, n, st, false);
      if (h_rowptr) GBV_CUDA(cudaMemcpyAsync(h_rowptr, H.rowptr, 4 * ((size_t)n + 1), cudaMemcpyDeviceToHost, st));
      if (h_col) GBV_CUDA(cudaMemcpyAsync(h_col, H.col, 4 * c->nnz, cudaMemcpyDeviceToHost, st));
      if (h_val) GBV_CUDA(cudaMemcpyAsync(h_val, H.val, 8 * c->nnz, cudaMemcpyDeviceToHost, st));
      if (h_diag) GBV_CUDA(cudaMemcpyAsync(h_diag, H.diag, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
    }
    GBV_CUDA(cudaStreamSynchronize(st));
  });
}

}  // extern "C"
