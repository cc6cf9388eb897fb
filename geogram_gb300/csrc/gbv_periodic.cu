// Laguerre cells in a periodic cube [0, P)^3: what the reference computes with
// PeriodicDelaunay3d and copy_Laguerre_cell_from_Delaunay
// (delaunay/periodic_delaunay_3d.cpp:3634-3734), here without a Delaunay
// triangulation.  The seeds' images under the 26 translations by +-P that
// fall in a layer of width delta around the cube are added as ghost seeds,
// and the cells of the original seeds are certified by the security-radius
// loop in the box [-delta, P + delta]^3.  A ghost layer is wide enough for a
// cell when the cell's security ball (radius^2 = 4.1 (R^2 + h^2), the radius
// at which the loop stopped) stays inside the box: every image the layer
// leaves out is then farther than any neighbour the loop could still need,
// and the box does not cut the cell.  The caller widens the layer until
// every cell passes.  Facet neighbours are reported as the original seed
// and the translation of its image.
#include <cfloat>

#include "gbv_context.cuh"
#include "gbv_refgeom.cuh"

namespace gbv {
namespace {

// translation code t = (tx + 1) * 9 + (ty + 1) * 3 + (tz + 1); 13: none
__device__ __forceinline__ void shift_of(int t, double P, double& sx, double& sy, double& sz) {
  sx = (double)(t / 9 - 1) * P;
  sy = (double)((t / 3) % 3 - 1) * P;
  sz = (double)(t % 3 - 1) * P;
}

__device__ __forceinline__ bool in_layer(double x, double y, double z, double P, double d) {
  return x >= -d && x <= P + d && y >= -d && y <= P + d && z >= -d && z <= P + d;
}

__global__ void ghost_count_kernel(const double* __restrict__ xyz, uint32_t n, double P,
                                   double delta, uint32_t* __restrict__ cnt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  if (i == n) {
    cnt[n] = 0;
    return;
  }
  const double x = xyz[3 * (size_t)i], y = xyz[3 * (size_t)i + 1], z = xyz[3 * (size_t)i + 2];
  uint32_t k = 0;
  for (int t = 0; t < 27; ++t) {
    if (t == 13) continue;
    double sx, sy, sz;
    shift_of(t, P, sx, sy, sz);
    k += in_layer(x + sx, y + sy, z + sz, P, delta) ? 1u : 0u;
  }
  cnt[i] = k;
}

// Originals at 0..n-1, seed i's ghosts from n + off[i] in translation order.
__global__ void ghost_fill_kernel(const double* __restrict__ xyz, const double* __restrict__ w,
                                  uint32_t n, double P, double delta,
                                  const uint32_t* __restrict__ off, double* __restrict__ ax,
                                  double* __restrict__ aw, uint32_t* __restrict__ src,
                                  uint8_t* __restrict__ shift) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = xyz[3 * (size_t)i], y = xyz[3 * (size_t)i + 1], z = xyz[3 * (size_t)i + 2];
  ax[3 * (size_t)i] = x;
  ax[3 * (size_t)i + 1] = y;
  ax[3 * (size_t)i + 2] = z;
  if (w) aw[i] = w[i];
  src[i] = i;
  shift[i] = 13;
  size_t g = (size_t)n + off[i];
  for (int t = 0; t < 27; ++t) {
    if (t == 13) continue;
    double sx, sy, sz;
    shift_of(t, P, sx, sy, sz);
    const double gx = x + sx, gy = y + sy, gz = z + sz;
    if (!in_layer(gx, gy, gz, P, delta)) continue;
    ax[3 * g] = gx;
    ax[3 * g + 1] = gy;
    ax[3 * g + 2] = gz;
    if (w) aw[g] = w[i];
    src[g] = i;
    shift[g] = (uint8_t)t;
    ++g;
  }
}

struct ReachArgs {
  uint32_t n;              // original seeds (the first n of the augmented set)
  const double* xyz;       // augmented seeds, caller order
  const double* w;
  double W;                // largest weight (lift h_i^2 = W - w_i)
  double P, delta;
  const uint32_t* slot_of;
  const uint32_t* nf;
  CombBuf cb;
  const double4* xd;
  const double* q;
  double box[6];
  uint32_t* fails;
};

__device__ __forceinline__ double4 reach_plane(const ReachArgs& a, uint32_t own, const double4& pi,
                                               double qi) {
  if (own >= kBoxBase) {
    switch (own - kBoxBase) {
      case 0: return make_double4(1.0, 0.0, 0.0, -a.box[0]);
      case 1: return make_double4(-1.0, 0.0, 0.0, a.box[3]);
      case 2: return make_double4(0.0, 1.0, 0.0, -a.box[1]);
      case 3: return make_double4(0.0, -1.0, 0.0, a.box[4]);
      case 4: return make_double4(0.0, 0.0, 1.0, -a.box[2]);
      default: return make_double4(0.0, 0.0, -1.0, a.box[5]);
    }
  }
  const double4 pj = a.xd[own];
  return make_double4(2.0 * __dsub_rn(pi.x, pj.x), 2.0 * __dsub_rn(pi.y, pj.y),
                      2.0 * __dsub_rn(pi.z, pj.z), __dsub_rn(qi, a.q[own]));
}

// Counts the original cells whose security ball leaves the ghost box.
__global__ void reach_kernel(ReachArgs a) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const uint32_t s = a.slot_of[i];
  if (a.nf[s] & kHugeFacets) {  // no stored polytope: take it as failing
    atomicAdd(a.fails, 1u);
    return;
  }
  const double px = a.xyz[3 * (size_t)i], py = a.xyz[3 * (size_t)i + 1],
               pz = a.xyz[3 * (size_t)i + 2];
  const ulonglong2 tm = a.cb.tmask[s];
  const size_t tb = (size_t)s * kTMax, pb = (size_t)s * kPMax;
  const double4 pis = a.xd[s];
  const double qis = a.q[s];
  double R2 = 0.0;
  for (int h = 0; h < 2; ++h) {
    uint64_t bits = h ? tm.y : tm.x;
    while (bits) {
      const int t = 64 * h + __ffsll((long long)bits) - 1;
      bits &= bits - 1;
      const uint32_t v = a.cb.tv[tb + t];
      const double3 c = r_corner(reach_plane(a, a.cb.pown[pb + (v & 0xFF)], pis, qis),
                                 reach_plane(a, a.cb.pown[pb + (v >> 8 & 0xFF)], pis, qis),
                                 reach_plane(a, a.cb.pown[pb + (v >> 16 & 0xFF)], pis, qis));
      const double dx = c.x - px, dy = c.y - py, dz = c.z - pz;
      R2 = fmax(R2, dx * dx + dy * dy + dz * dz);
    }
  }
  const double h2 = a.w ? a.W - a.w[i] : 0.0;
  double m = DBL_MAX;
  m = fmin(m, fmin(px + a.delta, a.P + a.delta - px));
  m = fmin(m, fmin(py + a.delta, a.P + a.delta - py));
  m = fmin(m, fmin(pz + a.delta, a.P + a.delta - pz));
  if (!(m * m > 4.1 * (R2 + h2) * (1.0 + 1e-9))) atomicAdd(a.fails, 1u);
}

// Facets of the original cells: the seed across each one and its translation.
__global__ void periodic_remap_kernel(const uint32_t* __restrict__ nbr, uint32_t nnz,
                                      const uint32_t* __restrict__ src,
                                      const uint8_t* __restrict__ shift,
                                      uint32_t* __restrict__ out_nbr,
                                      uint8_t* __restrict__ out_shift) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const uint32_t j = nbr[k];
  out_nbr[k] = src[j];
  out_shift[k] = shift[j];
}

}  // namespace

uint32_t periodic_ghosts(gbv_context* c, const double* d_xyz, const double* d_w, uint32_t n,
                         double P, double delta, cudaStream_t st, double** aug_xyz,
                         double** aug_w) {
  uint32_t* off = c->buf<uint32_t>("per_off", (size_t)n + 1);
  ghost_count_kernel<<<(n + 256) / 256, 256, 0, st>>>(d_xyz, n, P, delta, off); count_launch();
  uint32_t* tmp = c->buf<uint32_t>("per_scan", scan_tmp_elems((size_t)n + 1));
  exclusive_scan_u32(off, (size_t)n + 1, tmp, st);
  uint32_t ng = 0;
  GBV_CUDA(cudaMemcpyAsync(&ng, off + n, sizeof ng, cudaMemcpyDeviceToHost, st));
  GBV_CUDA(cudaStreamSynchronize(st));
  const size_t na = (size_t)n + ng;
  if (na > 0xFFFFFFF0ull) throw StatusError{GBV_ERR_CAPACITY, "too many ghost seeds"};
  *aug_xyz = c->buf<double>("per_xyz", 3 * na);
  *aug_w = d_w ? c->buf<double>("per_w", na) : nullptr;
  uint32_t* src = c->buf<uint32_t>("per_src", na);
  uint8_t* shift = c->buf<uint8_t>("per_shift_of", na);
  ghost_fill_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_xyz, d_w, n, P, delta, off, *aug_xyz,
                                                     *aug_w, src, shift); count_launch();
  return (uint32_t)na;
}

uint32_t periodic_reach_failures(gbv_context* c, uint32_t n, const double* aug_xyz,
                                 const double* aug_w, double W, double P, double delta,
                                 cudaStream_t st) {
  const uint32_t na = c->n;
  ReachArgs a{};
  a.n = n;
  a.xyz = aug_xyz;
  a.w = aug_w;
  a.W = W;
  a.P = P;
  a.delta = delta;
  a.slot_of = c->S.slot_of;
  a.nf = c->buf<uint32_t>("nf", na);
  a.cb.tv = c->buf<uint32_t>("cb_tv", (size_t)kTMax * na);
  a.cb.ta = c->buf<uint32_t>("cb_ta", (size_t)kTMax * na);
  a.cb.key = c->buf<int16_t>("cb_key", (size_t)kTMax * na);
  a.cb.pown = c->buf<uint32_t>("cb_pown", (size_t)kPMax * na);
  a.cb.prank = c->buf<uint16_t>("cb_prank", (size_t)kPMax * na);
  a.cb.tmask = c->buf<ulonglong2>("cb_tmask", na);
  a.cb.pmask = c->buf<uint64_t>("cb_pmask", na);
  a.cb.flags = c->buf<uint32_t>("cb_flags", na);
  a.xd = c->S.xd;
  a.q = c->S.q;
  for (int k = 0; k < 6; ++k) a.box[k] = c->box[k];
  a.fails = c->buf<uint32_t>("per_fails", 1);
  GBV_CUDA(cudaMemsetAsync(a.fails, 0, sizeof(uint32_t), st));
  reach_kernel<<<(n + 127) / 128, 128, 0, st>>>(a); count_launch();
  uint32_t h = 0;
  GBV_CUDA(cudaMemcpyAsync(&h, a.fails, sizeof h, cudaMemcpyDeviceToHost, st));
  GBV_CUDA(cudaStreamSynchronize(st));
  GBV_CUDA(cudaGetLastError());
  return h;
}

void periodic_remap(gbv_context* c, uint32_t n, cudaStream_t st, uint32_t** out_nbr,
                    uint8_t** out_shift, uint32_t* nnz) {
  uint32_t h = 0;
  GBV_CUDA(cudaMemcpyAsync(&h, c->rowptr + n, sizeof h, cudaMemcpyDeviceToHost, st));
  GBV_CUDA(cudaStreamSynchronize(st));
  *out_nbr = c->buf<uint32_t>("per_nbr", std::max<uint32_t>(h, 1));
  *out_shift = c->buf<uint8_t>("per_shift", std::max<uint32_t>(h, 1));
  const uint32_t* src = c->buf<uint32_t>("per_src", c->n);
  const uint8_t* shift = c->buf<uint8_t>("per_shift_of", c->n);
  if (h) {
    periodic_remap_kernel<<<(h + 255) / 256, 256, 0, st>>>(c->nbr, h, src, shift, *out_nbr,
                                                           *out_shift); count_launch();
  }
  *nnz = h;
}

}  // namespace gbv
