// gbv_knn_noalloc: the k nearest neighbours of every point, with all the
// search's scratch memory in one fixed array compiled into the library, so
// that the call itself allocates nothing.
//
// Who needs this: code that must not allocate GPU memory while it runs --
// work enqueued from inside a region where the application forbids device
// allocations (allocation can synchronise the device or fail under a hard
// memory budget), callers that own all device memory through their own pool
// and account for every byte, and real-time or latency-bound loops where a
// cudaMalloc/cudaFree pair would add unpredictable stalls.  They pass their
// own device input and output arrays; everything else lives in
// g_knn_scratch below.
//
// The scratch array is a file-scope __device__ array of fixed size: every
// GPU that loads the library holds it (about 3.2 MB) until the process
// exits.  All calls share it and it keeps the last call's contents, so the
// call clears what must start at zero (the grid counts and the flag count)
// and two calls whose work overlaps on the GPU -- on different streams, or
// from different host threads -- race on it and corrupt each other's
// results.  Order them on one stream, or synchronise between them.
//
// Host code must not use the array's name as a device address: in host code
// it names a host-side stand-in.  Every call looks up the array's address in
// the current device's context with cudaGetSymbolAddress, so the address
// stays right after cudaDeviceReset or in another context.  The first call
// in a context loads the library's device code there, array included (that
// load allocates the 3.2 MB and can synchronise): make the first call on
// each device outside any region that must not allocate, and before any
// stream capture begins.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "gbv_grid.cuh"

namespace gbv {

constexpr uint32_t kNoAllocMaxPoints = GBV_NOALLOC_MAX_POINTS;
constexpr int kNoAllocLevels = 5;  // choose_levels(32768): 8^5 fine cells
constexpr size_t kNoAllocCells = ((size_t)1 << (3 * kNoAllocLevels)) + 1;

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// The carve-up must hold what its users write: the scan of the grid counts
// (8^kNoAllocLevels + 1 entries) and the bounding-box partials of build_grid
// (checked below).
constexpr size_t kNoAllocScanTmp = 64;
constexpr size_t kNoAllocRed = 8 * 128;

// Carve-up of the scratch array (byte offsets).
struct NoAllocLayout {
  static constexpr size_t xd = 0;
  static constexpr size_t q = xd + align256(sizeof(double4) * kNoAllocMaxPoints);
  static constexpr size_t xf = q + align256(sizeof(double) * kNoAllocMaxPoints);
  static constexpr size_t xl = xf + align256(sizeof(float4) * kNoAllocMaxPoints);
  static constexpr size_t perm = xl + align256(sizeof(float4) * kNoAllocMaxPoints);
  static constexpr size_t slot_of = perm + align256(sizeof(uint32_t) * kNoAllocMaxPoints);
  static constexpr size_t cell_start = slot_of + align256(sizeof(uint32_t) * kNoAllocMaxPoints);
  static constexpr size_t gd = cell_start + align256(sizeof(uint32_t) * kNoAllocCells);
  static constexpr size_t aux = gd + align256(sizeof(GridDesc));
  static constexpr size_t cid = aux + align256(sizeof(double) * 4);
  static constexpr size_t rank = cid + align256(sizeof(uint32_t) * kNoAllocMaxPoints);
  static constexpr size_t scan_tmp = rank + align256(sizeof(uint32_t) * kNoAllocMaxPoints);
  static constexpr size_t red = scan_tmp + align256(sizeof(uint32_t) * kNoAllocScanTmp);
  static constexpr size_t flag_count = red + align256(sizeof(double) * kNoAllocRed);
  static constexpr size_t flag_list = flag_count + 256;
  static constexpr size_t total = flag_list + align256(sizeof(uint32_t) * kNoAllocMaxPoints);
};

static_assert(scan_tmp_elems(kNoAllocCells) <= kNoAllocScanTmp,
              "scan scratch of the allocation-free kNN is too small");
static_assert(8 * (size_t)kBboxParts <= kNoAllocRed,
              "bounding-box partials of the allocation-free kNN are too small");

static __device__ __align__(256) unsigned char g_knn_scratch[NoAllocLayout::total];

namespace {
// Device address of g_knn_scratch in the current context.
cudaError_t scratch_address(unsigned char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_knn_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<unsigned char*>(p);
  return cudaSuccess;
}

// True when p is device memory of device dev (or managed memory).
bool on_device(const void* p, int dev) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}
}  // namespace

}  // namespace gbv

using namespace gbv;

extern "C" gbv_status gbv_knn_noalloc(const double* d_pts, uint32_t n, uint32_t dim,
                                      uint32_t stride, uint32_t k, uint32_t* d_idx,
                                      double* d_d2, void* stream) {
  auto fail = [](gbv_status st, const std::string& msg) {
    set_last_error(msg.c_str());  // reported by gbv_last_error()
    return st;
  };
  if (!d_pts || !d_idx) return fail(GBV_ERR_INVALID_ARGUMENT, "NULL argument");
  if (dim != 3 && dim != 4) return fail(GBV_ERR_INVALID_ARGUMENT, "dim must be 3 or 4");
  if (stride < dim) return fail(GBV_ERR_INVALID_ARGUMENT, "stride < dim");
  if (n == 0 || n > kNoAllocMaxPoints)
    return fail(GBV_ERR_CAPACITY, "gbv_knn_noalloc takes 1 to " +
                                      std::to_string(kNoAllocMaxPoints) + " points, got " +
                                      std::to_string(n));
  if (k == 0 || k > n || k > kKnnSmemK)
    return fail(GBV_ERR_INVALID_ARGUMENT,
                "gbv_knn_noalloc needs 0 < k <= min(n, " + std::to_string(kKnnSmemK) + ")");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return fail(GBV_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (!on_device(d_pts, dev) || !on_device(d_idx, dev) || (d_d2 && !on_device(d_d2, dev)))
    return fail(GBV_ERR_INVALID_ARGUMENT,
                "gbv_knn_noalloc: arrays must be device memory of the current device " +
                    std::to_string(dev));
  unsigned char* base = nullptr;
  e = scratch_address(&base);
  if (e != cudaSuccess)
    return fail(GBV_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  using Lay = NoAllocLayout;
  SortedSeeds S;
  S.xd = reinterpret_cast<double4*>(base + Lay::xd);
  S.q = reinterpret_cast<double*>(base + Lay::q);
  S.xf = reinterpret_cast<float4*>(base + Lay::xf);
  S.xl = reinterpret_cast<float4*>(base + Lay::xl);
  S.wf = nullptr;
  S.ws = nullptr;
  S.perm = reinterpret_cast<uint32_t*>(base + Lay::perm);
  S.slot_of = reinterpret_cast<uint32_t*>(base + Lay::slot_of);
  S.cell_start = reinterpret_cast<uint32_t*>(base + Lay::cell_start);
  S.gd = reinterpret_cast<GridDesc*>(base + Lay::gd);
  S.aux = reinterpret_cast<double*>(base + Lay::aux);
  GridScratch scr;
  scr.cid = reinterpret_cast<uint32_t*>(base + Lay::cid);
  scr.rank = reinterpret_cast<uint32_t*>(base + Lay::rank);
  scr.scan_tmp = reinterpret_cast<uint32_t*>(base + Lay::scan_tmp);
  scr.scan_tmp_elems = kNoAllocScanTmp;
  scr.red = reinterpret_cast<double*>(base + Lay::red);
  const int L = choose_levels(n);  // <= kNoAllocLevels for n <= kNoAllocMaxPoints
  // build_grid clears the grid counts (cell_start) before counting
  build_grid(d_pts, stride, dim, nullptr, n, L, S, scr, st);
  KnnArgs ka{};
  ka.S = &S;
  ka.nq = n;
  ka.k = k;
  ka.mode = KNN_ALL;
  ka.exp_idx = d_idx;
  ka.exp_d2 = d_d2;
  // launch_knn clears the flag count before the search
  ka.flag_count = reinterpret_cast<uint32_t*>(base + Lay::flag_count);
  ka.flag_list = reinterpret_cast<uint32_t*>(base + Lay::flag_list);
  launch_knn(ka, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GBV_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return GBV_OK;
}
