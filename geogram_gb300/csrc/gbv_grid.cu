// Grid build (counting sort of Morton-ordered seeds) and kNN search.
//
// Replaces the reference's BalancedKdTree (points/kd_tree.cpp:121-542):
// instead of a median-split tree, seeds are counting-sorted into a uniform
// grid whose fine cells are numbered in Morton order.  Every node of the
// implicit octree over that grid is then a contiguous range of fine cells,
// hence of sorted seeds, found with two loads from cell_start; the kNN
// query is a depth-first traversal of that octree with box-distance
// pruning (the same pruning rule as kd_tree.cpp:300,330).  Distances are
// screened in FP32 against a conservative bound and ranked in exact FP64
// with the reference's arithmetic, ties broken by point index.
#include <cfloat>
#include <cmath>

#include "gbv_grid.cuh"

namespace gbv {

// ---------------------------------------------------------------------
// Exclusive scan (uint32, in place), 1024 elements per block.
// ---------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanPer = 4;
constexpr int kScanBlock = kScanThreads * kScanPer;

__global__ void scan_block_kernel(uint32_t* __restrict__ data, size_t n,
                                  uint32_t* __restrict__ sums) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanPer;
  uint32_t v[kScanPer];
  uint32_t run = 0;
#pragma unroll
  for (int i = 0; i < kScanPer; ++i) {
    v[i] = (base + i < n) ? data[base + i] : 0u;
    uint32_t t = v[i];
    v[i] = run;
    run += t;
  }
  // inclusive warp scan of per-thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = (lane < kScanThreads / 32) ? warp_tot[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  uint32_t off = (x - run) + (warp > 0 ? warp_tot[warp - 1] : 0u);
#pragma unroll
  for (int i = 0; i < kScanPer; ++i)
    if (base + i < n) data[base + i] = v[i] + off;
  if (threadIdx.x == kScanThreads - 1 && sums) sums[blockIdx.x] = off + run;
}

__global__ void scan_add_kernel(uint32_t* __restrict__ data, size_t n,
                                const uint32_t* __restrict__ sums) {
  const uint32_t add = sums[blockIdx.x];
  const size_t base = (size_t)blockIdx.x * kScanBlock;
  for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x) {
    size_t j = base + i;
    if (j < n) data[j] += add;
  }
}

static_assert(kScanBlock == kScanBlockElems, "scan block size and scan_tmp_elems disagree");

void exclusive_scan_u32(uint32_t* data, size_t n, uint32_t* tmp, cudaStream_t st) {
  if (n == 0) return;
  size_t nb = (n + kScanBlock - 1) / kScanBlock;
  if (nb == 1) {
    scan_block_kernel<<<1, kScanThreads, 0, st>>>(data, n, nullptr); count_launch();
    return;
  }
  uint32_t* sums = tmp;
  scan_block_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(data, n, sums); count_launch();
  exclusive_scan_u32(sums, nb, tmp + nb + 1, st);
  scan_add_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(data, n, sums); count_launch();
}

// ---------------------------------------------------------------------
// Bounding box, max weight
// ---------------------------------------------------------------------
constexpr int kRedThreads = 256;

// Per-block min x,y,z / max x,y,z / max w, written to part[8*block].
// v[6] = max w (or max |h| when dim = 4), v[7] = -min w.
__global__ void bbox_partial_kernel(const double* __restrict__ xyz, uint32_t stride,
                                    uint32_t dim, const double* __restrict__ w, uint32_t n,
                                    double* __restrict__ part) {
  double v[8] = {DBL_MAX, DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      double x = xyz[(size_t)i * stride + c];
      v[c] = fmin(v[c], x);
      v[3 + c] = fmax(v[3 + c], x);
    }
    if (w) {
      v[6] = fmax(v[6], w[i]);
      v[7] = fmax(v[7], -w[i]);
    } else if (dim == 4) {
      v[6] = fmax(v[6], fabs(xyz[(size_t)i * stride + 3]));
    }
  }
  __shared__ double sh[8][kRedThreads];
  for (int c = 0; c < 8; ++c) sh[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      for (int c = 0; c < 3; ++c)
        sh[c][threadIdx.x] = fmin(sh[c][threadIdx.x], sh[c][threadIdx.x + s]);
      for (int c = 3; c < 8; ++c)
        sh[c][threadIdx.x] = fmax(sh[c][threadIdx.x], sh[c][threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 8; ++c) part[8 * blockIdx.x + c] = sh[c][0];
}

// Reduces the partials and fills the grid descriptor.
__global__ void bbox_final_kernel(const double* __restrict__ part, int nparts, int L,
                                  int has_w, int dim, GridDesc* __restrict__ gd,
                                  double* __restrict__ wmax_out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double v[8] = {DBL_MAX, DBL_MAX, DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int b = 0; b < nparts; ++b) {
    for (int c = 0; c < 3; ++c) v[c] = fmin(v[c], part[8 * b + c]);
    for (int c = 3; c < 8; ++c) v[c] = fmax(v[c], part[8 * b + c]);
  }
  GridDesc g;
  double ext = fmax(v[3] - v[0], fmax(v[4] - v[1], v[5] - v[2]));
  if (!(ext > 0.0)) ext = 1.0;
  g.L = L;
  g.G = 1 << L;
  g.h = ext / g.G * (1.0 + 1e-9);
  g.inv_h = 1.0 / g.h;
  for (int c = 0; c < 3; ++c) {
    g.lo[c] = v[c];
    g.lo_f[c] = (float)v[c];
  }
  g.h_f = (float)g.h;
  *gd = g;
  *wmax_out = has_w ? v[6] : 0.0;
  // max |coordinate| (lift included) for the FP32 screening bound
  double m = 0.0;
  for (int c = 0; c < 3; ++c) m = fmax(m, fmax(fabs(v[c]), fabs(v[3 + c])));
  if (has_w) m = fmax(m, sqrt(fmax(v[6] + v[7], 0.0)));
  else if (dim == 4) m = fmax(m, v[6]);
  wmax_out[1] = m;
  // the largest squared difference of two lifts: h_i^2 <= W - min w with
  // weights, h^2 <= max |h|^2 for 4-d points, 0 in 3-d
  wmax_out[2] = has_w ? fmax(v[6] + v[7], 0.0) : (dim == 4 ? v[6] * v[6] : 0.0);
}

__global__ void cell_id_kernel(const double* __restrict__ xyz, uint32_t stride, uint32_t n,
                               const GridDesc* __restrict__ gd, uint32_t* __restrict__ cid,
                               uint32_t* __restrict__ rank, uint32_t* __restrict__ count) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const GridDesc g = *gd;
  uint32_t c3[3];
  for (int c = 0; c < 3; ++c) {
    double u = (xyz[(size_t)i * stride + c] - g.lo[c]) * g.inv_h;
    int iu = (int)floor(u);
    c3[c] = (uint32_t)clampi(iu, 0, g.G - 1);
  }
  uint32_t code = morton3(c3[0], c3[1], c3[2]);
  cid[i] = code;
  rank[i] = atomicAdd(&count[code], 1u);
}

__global__ void scatter_kernel(const double* __restrict__ xyz, uint32_t stride,
                               uint32_t dim, const double* __restrict__ w, uint32_t n,
                               const uint32_t* __restrict__ cid,
                               const uint32_t* __restrict__ rank,
                               const uint32_t* __restrict__ start,
                               const double* __restrict__ wmax, SortedSeeds S) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t s = start[cid[i]] + rank[i];
  double x = xyz[(size_t)i * stride], y = xyz[(size_t)i * stride + 1],
         z = xyz[(size_t)i * stride + 2];
  double wi = w ? w[i] : 0.0;
  // h_i = sqrt(W - w_i): the 4-d lift of compute_OTM/main.cpp:280-283
  double h = w ? sqrt(__dsub_rn(*wmax, wi)) : (dim == 4 ? xyz[(size_t)i * stride + 3] : 0.0);
  // q = w - |p|^2 evaluated as periodic_delaunay_3d.cpp:3712-3726 does:
  // (x*x + y*y) + z*z, then w - len2, no fused multiply-add.
  double len2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
  S.xd[s] = make_double4(x, y, z, h);
  S.q[s] = __dsub_rn(wi, len2);
  const float4 hi = make_float4((float)x, (float)y, (float)z, (float)h);
  S.xf[s] = hi;
  S.xl[s] = make_float4((float)(x - (double)hi.x), (float)(y - (double)hi.y),
                        (float)(z - (double)hi.z), (float)(h - (double)hi.w));
  if (S.wf) {
    const float whi = (float)wi;
    S.wf[s] = make_float2(whi, (float)(wi - (double)whi));
  }
  if (S.ws) S.ws[s] = wi;
  S.perm[s] = i;
  S.slot_of[i] = s;
}

// ---------------------------------------------------------------------
// Max weight per octree node
// ---------------------------------------------------------------------
__global__ void wmax_fine_kernel(const uint32_t* __restrict__ cell_start,
                                 const double* __restrict__ ws, size_t ncells,
                                 double* __restrict__ out) {
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const uint32_t b = cell_start[c], e = cell_start[c + 1];
  double m = -INFINITY;
  for (uint32_t s = b; s < e; ++s) m = fmax(m, ws ? ws[s] : 0.0);
  out[c] = m;
}

__global__ void wmax_up_kernel(const double* __restrict__ child, size_t nparent,
                               double* __restrict__ parent) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nparent) return;
  double m = child[8 * p];
#pragma unroll
  for (int k = 1; k < 8; ++k) m = fmax(m, child[8 * p + k]);
  parent[p] = m;
}

// ---------------------------------------------------------------------
// Linear weight bound per octree node
// ---------------------------------------------------------------------
constexpr int kMom = 14;  // S0, S1 (3), S2 (xx xy xz yy yz zz), Sw, Swd (3)

__device__ __forceinline__ double3 node_centre(const GridDesc& gd, int lev, uint32_t code) {
  const double side = gd.h * (double)(1u << (gd.L - lev));
  return make_double3(gd.lo[0] + ((double)compact3(code) + 0.5) * side,
                      gd.lo[1] + ((double)compact3(code >> 1) + 0.5) * side,
                      gd.lo[2] + ((double)compact3(code >> 2) + 0.5) * side);
}

__global__ void leaf_moments_kernel(SortedSeeds S, size_t ncells, double* __restrict__ mom) {
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const GridDesc& gd = *S.gd;
  const double3 m = node_centre(gd, gd.L, (uint32_t)c);
  double v[kMom] = {};
  for (uint32_t s = S.cell_start[c]; s < S.cell_start[c + 1]; ++s) {
    const double4 p = S.xd[s];
    const double w = S.ws ? S.ws[s] : 0.0;
    const double dx = p.x - m.x, dy = p.y - m.y, dz = p.z - m.z;
    v[0] += 1.0;
    v[1] += dx; v[2] += dy; v[3] += dz;
    v[4] += dx * dx; v[5] += dx * dy; v[6] += dx * dz;
    v[7] += dy * dy; v[8] += dy * dz; v[9] += dz * dz;
    v[10] += w;
    v[11] += w * dx; v[12] += w * dy; v[13] += w * dz;
  }
  double* o = mom + (node_offset(gd.L) + c) * kMom;
  for (int k = 0; k < kMom; ++k) o[k] = v[k];
}

// parent moments from the 8 children's, shifted to the parent's centre
__global__ void combine_moments_kernel(const GridDesc* __restrict__ gdp, int lev, size_t nparent,
                                       double* __restrict__ mom) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nparent) return;
  const GridDesc& gd = *gdp;
  const double3 mp = node_centre(gd, lev, (uint32_t)p);
  double v[kMom] = {};
  for (int k = 0; k < 8; ++k) {
    const uint32_t cc = ((uint32_t)p << 3) | (uint32_t)k;
    const double* c = mom + (node_offset(lev + 1) + cc) * kMom;
    if (c[0] == 0.0) continue;
    const double3 mc = node_centre(gd, lev + 1, cc);
    const double ex = mc.x - mp.x, ey = mc.y - mp.y, ez = mc.z - mp.z;
    const double n0 = c[0];
    v[0] += n0;
    v[1] += c[1] + n0 * ex; v[2] += c[2] + n0 * ey; v[3] += c[3] + n0 * ez;
    v[4] += c[4] + 2.0 * c[1] * ex + n0 * ex * ex;
    v[5] += c[5] + c[1] * ey + c[2] * ex + n0 * ex * ey;
    v[6] += c[6] + c[1] * ez + c[3] * ex + n0 * ex * ez;
    v[7] += c[7] + 2.0 * c[2] * ey + n0 * ey * ey;
    v[8] += c[8] + c[2] * ez + c[3] * ey + n0 * ey * ez;
    v[9] += c[9] + 2.0 * c[3] * ez + n0 * ez * ez;
    v[10] += c[10];
    v[11] += c[11] + c[10] * ex; v[12] += c[12] + c[10] * ey; v[13] += c[13] + c[10] * ez;
  }
  double* o = mom + (node_offset(lev) + p) * kMom;
  for (int k = 0; k < kMom; ++k) o[k] = v[k];
}

// least-squares (a, g) per node; empty nodes get zeros
__global__ void fit_nodes_kernel(const double* __restrict__ mom, size_t nn,
                                 double4* __restrict__ lin, unsigned long long* __restrict__ ex) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double* v = mom + i * kMom;
  ex[i] = 0ull;  // the ordered key of -inf (below every double key)
  double4 r = make_double4(0.0, 0.0, 0.0, 0.0);
  if (v[0] > 0.0) {
    r.x = v[10] / v[0];
    if (v[0] >= 4.0) {
      double A[4][4] = {{v[0], v[1], v[2], v[3]},
                        {v[1], v[4], v[5], v[6]},
                        {v[2], v[5], v[7], v[8]},
                        {v[3], v[6], v[8], v[9]}};
      double b[4] = {v[10], v[11], v[12], v[13]};
      const double ridge = 1e-9 * (v[4] + v[7] + v[9]) + 1e-300;
      for (int k = 1; k < 4; ++k) A[k][k] += ridge;
      bool ok = true;
      for (int c = 0; c < 4 && ok; ++c) {
        int piv = c;
        for (int q = c + 1; q < 4; ++q)
          if (fabs(A[q][c]) > fabs(A[piv][c])) piv = q;
        if (!(fabs(A[piv][c]) > 0.0)) { ok = false; break; }
        if (piv != c) {
          for (int k = 0; k < 4; ++k) { const double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
          const double t = b[c]; b[c] = b[piv]; b[piv] = t;
        }
        for (int q = c + 1; q < 4; ++q) {
          const double f = A[q][c] / A[c][c];
          for (int k = c; k < 4; ++k) A[q][k] -= f * A[c][k];
          b[q] -= f * b[c];
        }
      }
      if (ok) {
        double x[4];
        for (int c = 3; c >= 0; --c) {
          double t = b[c];
          for (int k = c + 1; k < 4; ++k) t -= A[c][k] * x[k];
          x[c] = t / A[c][c];
        }
        if (isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(x[3]))
          r = make_double4(x[0], x[1], x[2], x[3]);
      }
    }
  }
  lin[i] = r;
}

// monotone map of doubles to unsigned keys (atomicMax on doubles)
__device__ __forceinline__ unsigned long long dkey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dval(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double((long long)b);
}

// e[node] = max over the node's seeds of w - a - g . (p - m), at level lev
__global__ void node_excess_kernel(SortedSeeds S, int lev, const double4* __restrict__ lin,
                                   unsigned long long* __restrict__ ex) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned FULL = 0xFFFFFFFFu;
  const GridDesc& gd = *S.gd;
  bool live = s < S.n;
  uint32_t node = 0;
  double r = -INFINITY;
  if (live) {
    const double4 p = S.xd[s];
    // the fine cell holding slot s: cell_start[c] <= s < cell_start[c + 1]
    uint32_t lo = 0, hi = 1u << (3 * gd.L);
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (S.cell_start[mid] <= s) lo = mid;
      else hi = mid;
    }
    node = lo >> (3 * (gd.L - lev));
    const double3 m = node_centre(gd, lev, node);
    const double4 f = lin[node_offset(lev) + node];
    const double w = S.ws ? S.ws[s] : 0.0;
    r = w - f.x - (f.y * (p.x - m.x) + f.z * (p.y - m.y) + f.w * (p.z - m.z));
  }
  // one atomic per warp when the whole warp is in one node
  const uint32_t n0 = __shfl_sync(FULL, node, 0);
  const bool same = __all_sync(FULL, !live || node == n0);
  if (same) {
    double mx = r;
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > -INFINITY)
      atomicMax(&ex[node_offset(lev) + n0], dkey(mx));
  } else if (live) {
    atomicMax(&ex[node_offset(lev) + node], dkey(r));
  }
}

// in place: ex holds keys, each thread turns its own entry into a double
__global__ void excess_decode_kernel(double* __restrict__ ex, size_t nn) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const unsigned long long k = reinterpret_cast<unsigned long long*>(ex)[i];
  ex[i] = k ? dval(k) : 0.0;
}

void build_node_linear(const SortedSeeds& S, double4* lin, double* ex, double* moments,
                       cudaStream_t st) {
  const int L = S.L;
  const size_t nf = (size_t)1 << (3 * L);
  const size_t nn = node_count(L);
  leaf_moments_kernel<<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(S, nf, moments);
  count_launch();
  for (int l = L - 1; l >= 0; --l) {
    const size_t np = (size_t)1 << (3 * l);
    combine_moments_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(S.gd, l, np, moments);
    count_launch();
  }
  // the excess maxima are kept as ordered keys in ex itself, decoded at the end
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(ex);
  fit_nodes_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(moments, nn, lin, keys);
  count_launch();
  for (int l = 0; l <= L; ++l) {
    node_excess_kernel<<<(S.n + 255) / 256, 256, 0, st>>>(S, l, lin, keys);
    count_launch();
  }
  excess_decode_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(ex, nn);
  count_launch();
}

void build_node_wmax(const SortedSeeds& S, double* wmax, cudaStream_t st) {
  const int L = S.L;
  const size_t nf = (size_t)1 << (3 * L);
  wmax_fine_kernel<<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(S.cell_start, S.ws, nf,
                                                                  wmax + node_offset(L)); count_launch();
  for (int l = L - 1; l >= 0; --l) {
    const size_t np = (size_t)1 << (3 * l);
    wmax_up_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(wmax + node_offset(l + 1), np,
                                                                  wmax + node_offset(l)); count_launch();
  }
}

int choose_levels(uint32_t n) {
  int L = 1;
  while (L < 9 && (double)(1u << (3 * L)) < (double)n) ++L;
  return L;
}

void build_grid(const double* xyz, uint32_t stride, uint32_t dim, const double* w,
                uint32_t n, int L, SortedSeeds& S, GridScratch& scr, cudaStream_t st) {
  const int nparts = kBboxParts;
  bbox_partial_kernel<<<nparts, kRedThreads, 0, st>>>(xyz, stride, dim, w, n, scr.red); count_launch();
  bbox_final_kernel<<<1, 32, 0, st>>>(scr.red, nparts, L, w != nullptr, (int)dim, S.gd,
                                      S.aux); count_launch();
  const size_t ncells = (size_t)1 << (3 * L);
  cudaMemsetAsync(S.cell_start, 0, sizeof(uint32_t) * (ncells + 1), st);
  const unsigned nb = (n + 255) / 256;
  cell_id_kernel<<<nb, 256, 0, st>>>(xyz, stride, n, S.gd, scr.cid, scr.rank,
                                     S.cell_start); count_launch();
  exclusive_scan_u32(S.cell_start, ncells + 1, scr.scan_tmp, st);
  scatter_kernel<<<nb, 256, 0, st>>>(xyz, stride, dim, w, n, scr.cid, scr.rank,
                                     S.cell_start, S.aux, S); count_launch();
  S.n = n;
  S.L = L;
}

// ---------------------------------------------------------------------
// kNN: depth-first traversal of the implicit Morton octree
// ---------------------------------------------------------------------
constexpr int kKnnThreads = 64;
constexpr uint32_t kLeaf = 24;
constexpr int kKnnExtra = 8;                 // FP32 list slack beyond k
constexpr int kKnnCap = kKnnSmemK + kKnnExtra;

// Squared distance from point u (fine-cell units) to the box of an octree
// node [i*side, (i+1)*side)^3, in fine-cell units, shrunk by a small slack
// so that it never exceeds the true distance to any seed assigned to it.
__device__ __forceinline__ float node_box_d2(float ux, float uy, float uz, uint32_t ix,
                                             uint32_t iy, uint32_t iz, float side) {
  float bx = ix * side, by = iy * side, bz = iz * side;
  float dx = fmaxf(fmaxf(bx - ux, ux - (bx + side)), 0.f);
  float dy = fmaxf(fmaxf(by - uy, uy - (by + side)), 0.f);
  float dz = fmaxf(fmaxf(bz - uz, uz - (bz + side)), 0.f);
  dx = fmaxf(dx - 1e-3f, 0.f);
  dy = fmaxf(dy - 1e-3f, 0.f);
  dz = fmaxf(dz - 1e-3f, 0.f);
  return dx * dx + dy * dy + dz * dz;
}

// Depth-first traversal, nearest child first.  thr() is the current
// squared pruning distance (FP32); leaf(b, e) scans sorted slots [b, e).
template <class Thr, class Leaf>
__device__ __forceinline__ void traverse(const SortedSeeds& S, const GridDesc& g, float ux,
                                         float uy, float uz, Thr thr, Leaf leaf) {
  const float h2f = g.h_f * g.h_f;
  uint32_t stack[8 * 10 + 8];
  int sp = 0;
  stack[sp++] = 0u;  // (code << 4) | level
  while (sp > 0) {
    const uint32_t e = stack[--sp];
    const int lev = (int)(e & 15u);
    const uint32_t code = e >> 4;
    const int shift = g.L - lev;
    const float side = (float)(1u << shift);
    const float t0 = thr();
    if (t0 < FLT_MAX) {
      const float bd = node_box_d2(ux, uy, uz, compact3(code), compact3(code >> 1),
                                   compact3(code >> 2), side) * h2f;
      if (bd > t0) continue;
    }
    const uint32_t c_lo = code << (3 * shift);
    const uint32_t c_hi = (code + 1u) << (3 * shift);
    const uint32_t b = S.cell_start[c_lo], en = S.cell_start[c_hi];
    if (b == en) continue;
    if (en - b <= kLeaf || lev == g.L) {
      leaf(b, en);
      continue;
    }
    const float cside = side * 0.5f;
    float cd[8];
    uint32_t cc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t ch = (code << 3) | (uint32_t)c;
      cd[c] = node_box_d2(ux, uy, uz, compact3(ch), compact3(ch >> 1), compact3(ch >> 2),
                          cside) * h2f;
      cc[c] = ch;
    }
#pragma unroll
    for (int i = 1; i < 8; ++i) {
#pragma unroll
      for (int j = i; j > 0; --j) {
        if (cd[j] > cd[j - 1]) {
          const float td = cd[j];
          cd[j] = cd[j - 1];
          cd[j - 1] = td;
          const uint32_t tc = cc[j];
          cc[j] = cc[j - 1];
          cc[j - 1] = tc;
        }
      }
    }
    const float t1 = thr();
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (cd[c] <= t1) stack[sp++] = (cc[c] << 4) | (uint32_t)(lev + 1);
  }
}

struct QueryCtx {
  uint32_t qslot;  // kNone for external queries
  uint32_t qperm;
  double4 q;
  float4 qf;
  float ux, uy, uz;
  bool has_lo;
  double lo_d;
  uint32_t lo_i;
};

__device__ __forceinline__ QueryCtx make_query(const KnnArgs& a, const SortedSeeds& S,
                                               const GridDesc& g, uint32_t qi) {
  QueryCtx c;
  c.qslot = kNone;
  if (a.mode == KNN_QUERY) {
    c.q = a.qpts[qi];
  } else {
    c.qslot = a.qlist ? a.qlist[qi] : qi;
    c.q = S.xd[c.qslot];
  }
  c.qperm = (c.qslot != kNone) ? S.perm[c.qslot] : 0u;
  c.qf = make_float4((float)c.q.x, (float)c.q.y, (float)c.q.z, (float)c.q.w);
  c.ux = (float)((c.q.x - g.lo[0]) * g.inv_h);
  c.uy = (float)((c.q.y - g.lo[1]) * g.inv_h);
  c.uz = (float)((c.q.z - g.lo[2]) * g.inv_h);
  c.has_lo = a.lo_d2 != nullptr;
  c.lo_d = c.has_lo ? a.lo_d2[qi] : 0.0;
  c.lo_i = c.has_lo ? a.lo_idx[qi] : 0u;
  return c;
}

// (d, i) after the query's lower bound in (d2, original index) order?
__device__ __forceinline__ bool after_lo(const QueryCtx& c, double d, uint32_t i) {
  return !c.has_lo || d > c.lo_d || (d == c.lo_d && i > c.lo_i);
}

__device__ __forceinline__ void write_outputs(const KnnArgs& a, const SortedSeeds& S,
                                              const QueryCtx& c, uint32_t qi, uint32_t cnt,
                                              uint32_t copies, bool dup_lower, const double* ld,
                                              const uint32_t* ls, uint32_t stride) {
  if (a.cnt) a.cnt[qi] = (a.mode == KNN_CELLS) ? pack_cnt(cnt, copies, dup_lower) : cnt;
  if (a.mode == KNN_CELLS && dup_lower) cnt = 0;
  if (a.nbr)
    for (uint32_t r = 0; r < cnt; ++r) a.nbr[(size_t)r * a.out_stride + qi] = ls[(size_t)r * stride];
  if (a.last_d2) {
    a.last_d2[qi] = cnt ? ld[(size_t)(cnt - 1) * stride] : (c.has_lo ? c.lo_d : 0.0);
    a.last_idx[qi] = cnt ? S.perm[ls[(size_t)(cnt - 1) * stride]] : (c.has_lo ? c.lo_i : 0u);
  }
  if (a.exp_idx) {
    const size_t row = (a.mode == KNN_QUERY) ? qi : c.qperm;
    const uint32_t K = a.k;
    for (uint32_t r = 0; r < K; ++r) {
      a.exp_idx[row * K + r] = (r < cnt) ? S.perm[ls[(size_t)r * stride]] : kNone;
      if (a.exp_d2) a.exp_d2[row * K + r] = (r < cnt) ? ld[(size_t)r * stride] : INFINITY;
    }
  }
}

// (da, pa) > (db, pb) in the list order: distance, then original index
__device__ __forceinline__ bool pair_greater(double da, uint32_t pa, double db, uint32_t pb) {
  return da > db || (da == db && pa > pb);
}

// Puts (d, slot) (original index p) at position pos of the max-heap of size
// `size` held in ld/ls (with stride) and sifts it down.
__device__ __forceinline__ void heap_sift_down(double* ld, uint32_t* ls, uint32_t stride,
                                               const uint32_t* __restrict__ perm, uint32_t pos,
                                               uint32_t size, double d, uint32_t slot,
                                               uint32_t p) {
  for (;;) {
    const uint32_t l = 2 * pos + 1;
    if (l >= size) break;
    uint32_t ch = l;
    double dc = ld[(size_t)l * stride];
    uint32_t sc = ls[(size_t)l * stride];
    uint32_t pc = perm[sc];
    if (l + 1 < size) {
      const double dr = ld[(size_t)(l + 1) * stride];
      const uint32_t sr = ls[(size_t)(l + 1) * stride];
      const uint32_t pr = perm[sr];
      if (pair_greater(dr, pr, dc, pc)) {
        ch = l + 1;
        dc = dr;
        sc = sr;
        pc = pr;
      }
    }
    if (!pair_greater(dc, pc, d, p)) break;
    ld[(size_t)pos * stride] = dc;
    ls[(size_t)pos * stride] = sc;
    pos = ch;
  }
  ld[(size_t)pos * stride] = d;
  ls[(size_t)pos * stride] = slot;
}

// ---- exact search: FP64 distances of every candidate, FP64 list ---------
// qsel: when non-null, the kernel runs only the queries qsel[0..*qcount).
// SMEM: the list in dynamic shared memory, [k][blockDim] doubles then
// [k][blockDim] slots (k <= kKnnMaxK); otherwise global lists gl_d2/gl_slot.
template <bool SMEM>
__global__ void __launch_bounds__(kKnnThreads)
knn_exact_kernel(KnnArgs a, SortedSeeds S, const GridDesc* __restrict__ gdp,
                 const double* __restrict__ aux, const uint32_t* __restrict__ qsel,
                 const uint32_t* __restrict__ qcount) {
  extern __shared__ __align__(16) unsigned char exact_smem[];
  uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
  if (qsel) {
    if (qi >= *qcount) return;
    qi = qsel[qi];
  } else if (qi >= a.nq) {
    return;
  }
  const GridDesc g = *gdp;
  double* ld;
  uint32_t* ls;
  uint32_t stride;
  if (SMEM) {
    double* sd = reinterpret_cast<double*>(exact_smem);
    ld = sd + threadIdx.x;
    ls = reinterpret_cast<uint32_t*>(sd + (size_t)a.k * blockDim.x) + threadIdx.x;
    stride = blockDim.x;
  } else {
    ld = a.gl_d2 + qi;
    ls = a.gl_slot + qi;
    stride = a.nq;
  }
  const QueryCtx c = make_query(a, S, g, qi);
  const float delta = 8.0f * (float)aux[1] * 5.9604645e-8f + 1e-30f;
  const uint32_t K = a.k;
  uint32_t cnt = 0, copies = 0;
  double worst = DBL_MAX;
  float thr = FLT_MAX;
  bool dup_lower = false;
  auto L = [&](uint32_t r) -> double& { return ld[(size_t)r * stride]; };
  auto LS = [&](uint32_t r) -> uint32_t& { return ls[(size_t)r * stride]; };
  traverse(S, g, c.ux, c.uy, c.uz, [&]() { return thr; }, [&](uint32_t b, uint32_t en) {
    for (uint32_t s2 = b; s2 < en; ++s2) {
      const float4 p = S.xf[s2];
      const float dx = p.x - c.qf.x, dy = p.y - c.qf.y, dz = p.z - c.qf.z, dh = p.w - c.qf.w;
      const float d32 = dx * dx + dy * dy + dz * dz + dh * dh;
      if (d32 > thr) continue;
      if (a.mode == KNN_CELLS && s2 == c.qslot) continue;
      const double d = dist2_exact(c.q, S.xd[s2]);
      const uint32_t pj = S.perm[s2];
      if (a.mode == KNN_CELLS && d == 0.0) {
        if (pj < c.qperm) dup_lower = true;
        else ++copies;
        continue;
      }
      if (!after_lo(c, d, pj)) continue;
      if constexpr (SMEM) {
        // short lists (k <= 64): insertion into the sorted list
        if (cnt == K) {
          if (d > worst) continue;
          if (d == worst && pj > S.perm[LS(K - 1)]) continue;
        }
        uint32_t pos = (cnt < K) ? cnt : K - 1;
        while (pos > 0) {
          const double dp = L(pos - 1);
          if (dp < d) break;
          if (dp == d && S.perm[LS(pos - 1)] < pj) break;
          L(pos) = dp;
          LS(pos) = LS(pos - 1);
          --pos;
        }
        L(pos) = d;
        LS(pos) = s2;
        if (cnt < K) ++cnt;
        if (cnt == K) worst = L(K - 1);
      } else {
        // long lists (up to every seed): a bounded max-heap on (d, index),
        // O(log k) per candidate, sorted once at the end
        if (cnt < K) {
          uint32_t pos = cnt++;
          while (pos > 0) {
            const uint32_t par = (pos - 1) >> 1;
            const double dp = L(par);
            const uint32_t sp = LS(par);
            if (!pair_greater(d, pj, dp, S.perm[sp])) break;
            L(pos) = dp;
            LS(pos) = sp;
            pos = par;
          }
          L(pos) = d;
          LS(pos) = s2;
        } else {
          if (!pair_greater(L(0), S.perm[LS(0)], d, pj)) continue;
          heap_sift_down(ld, ls, stride, S.perm, 0, K, d, s2, pj);
        }
        if (cnt == K) worst = L(0);
      }
      if (cnt == K) {
        const float r = sqrtf(__double2float_ru(worst)) * 1.0000076f + delta;
        thr = r * r * 1.0000076f;
      }
    }
  });
  if constexpr (!SMEM) {
    // heapsort: the max-heap becomes the ascending list
    for (uint32_t end = cnt; end > 1; --end) {
      const double dl = L(end - 1);
      const uint32_t sl = LS(end - 1);
      L(end - 1) = L(0);
      LS(end - 1) = LS(0);
      heap_sift_down(ld, ls, stride, S.perm, 0, end - 1, dl, sl, S.perm[sl]);
    }
  }
  write_outputs(a, S, c, qi, cnt, copies, dup_lower, ld, ls, stride);
}

// ---- fast search: FP32 selection of k + kKnnExtra, exact FP64 re-rank ------
// The k + kKnnExtra nearest by FP32 distance are kept in a bounded max-heap
// (its root is the pruning threshold).  Every seed of the true k nearest
// (exact (d2, index) order) lies within FP32 distance sqrt(d32_k) + 2 delta
// of the query, where d32_k is the k-th FP32 distance and delta bounds
// |FP32 - FP64| distance; if the heap's root is not beyond that, a seed of
// the true k nearest may have been dropped and the query is flagged for the
// exact search.  The kept seeds are heap-sorted, then re-ranked in FP64.
__global__ void __launch_bounds__(kKnnThreads)
knn_fast_kernel(KnnArgs a, SortedSeeds S, const GridDesc* __restrict__ gdp,
                const double* __restrict__ aux) {
  extern __shared__ __align__(16) unsigned char knn_smem[];
  double(*s_d)[kKnnThreads] = reinterpret_cast<double(*)[kKnnThreads]>(knn_smem);
  uint32_t(*s_s)[kKnnThreads] =
      reinterpret_cast<uint32_t(*)[kKnnThreads]>(knn_smem + sizeof(double) * kKnnCap * kKnnThreads);
  const uint32_t qi = blockIdx.x * kKnnThreads + threadIdx.x;
  if (qi >= a.nq) return;
  const int tid = threadIdx.x;
  const GridDesc g = *gdp;
  const QueryCtx c = make_query(a, S, g, qi);
  const float delta = 8.0f * (float)aux[1] * 5.9604645e-8f + 1e-30f;
  const uint32_t K = a.k;
  const uint32_t cap = K + kKnnExtra;
  // the FP32 distance lives in the low word of the list's double slot
  auto D32 = [&](uint32_t r) -> float& { return *reinterpret_cast<float*>(&s_d[r][tid]); };
  uint32_t cnt = 0, copies = 0;
  float thr = FLT_MAX;
  bool dup_lower = false;
  // lower bound: candidates surely before it are skipped, those near it are
  // compared exactly
  float lo_skip = -1.f, lo_check = -1.f;
  if (c.has_lo) {
    const float r = sqrtf(__double2float_rd(c.lo_d));
    const float r1 = fmaxf(r * 0.9999924f - delta, 0.f);
    const float r2 = r * 1.0000076f + delta;
    lo_skip = r1 * r1 * 0.9999924f;
    lo_check = r2 * r2 * 1.0000076f;
  }
  auto sift_down = [&](uint32_t i, uint32_t n) {
    const float d = D32(i);
    const uint32_t sl = s_s[i][tid];
    for (;;) {
      uint32_t c1 = 2 * i + 1;
      if (c1 >= n) break;
      float dc = D32(c1);
      if (c1 + 1 < n) {
        const float d2 = D32(c1 + 1);
        if (d2 > dc) {
          dc = d2;
          ++c1;
        }
      }
      if (dc <= d) break;
      D32(i) = dc;
      s_s[i][tid] = s_s[c1][tid];
      i = c1;
    }
    D32(i) = d;
    s_s[i][tid] = sl;
  };
  traverse(S, g, c.ux, c.uy, c.uz, [&]() { return thr; }, [&](uint32_t b, uint32_t en) {
    for (uint32_t s2 = b; s2 < en; ++s2) {
      const float4 p = S.xf[s2];
      const float dx = p.x - c.qf.x, dy = p.y - c.qf.y, dz = p.z - c.qf.z, dh = p.w - c.qf.w;
      const float d32 = dx * dx + dy * dy + dz * dz + dh * dh;
      if (d32 >= thr) continue;
      if (a.mode == KNN_CELLS && s2 == c.qslot) continue;
      if (c.has_lo) {
        if (d32 < lo_skip) continue;
        if (d32 <= lo_check && !after_lo(c, dist2_exact(c.q, S.xd[s2]), S.perm[s2])) continue;
      }
      if (a.mode == KNN_CELLS && d32 <= 0.f) {
        if (dist2_exact(c.q, S.xd[s2]) == 0.0) {
          if (S.perm[s2] < c.qperm) dup_lower = true;
          else ++copies;
          continue;
        }
      }
      if (cnt < cap) {
        // push and sift up
        uint32_t i = cnt++;
        while (i > 0) {
          const uint32_t par = (i - 1) >> 1;
          const float dp = D32(par);
          if (dp >= d32) break;
          D32(i) = dp;
          s_s[i][tid] = s_s[par][tid];
          i = par;
        }
        D32(i) = d32;
        s_s[i][tid] = s2;
        if (cnt == cap) thr = D32(0);
      } else {
        // replace the root (the farthest kept) and sift down
        D32(0) = d32;
        s_s[0][tid] = s2;
        sift_down(0, cap);
        thr = D32(0);
      }
    }
  });
  // heap sort: ascending FP32 distance
  for (uint32_t n = cnt; n > 1; --n) {
    const float dr = D32(0);
    const uint32_t sr = s_s[0][tid];
    D32(0) = D32(n - 1);
    s_s[0][tid] = s_s[n - 1][tid];
    D32(n - 1) = dr;
    s_s[n - 1][tid] = sr;
    sift_down(0, n - 1);
  }
  if (cnt == cap) {
    const float r = sqrtf(D32(K - 1)) * 1.0000076f + 2.f * delta;
    if (!(D32(cap - 1) > r * r * 1.0000076f)) {
      // a seed that may belong to the k nearest could have been dropped
      const uint32_t k = atomicAdd(a.flag_count, 1u);
      a.flag_list[k] = qi;
      if (a.cnt) a.cnt[qi] = 0;
      return;
    }
  }
  // exact distances, then insertion sort by (d2, original index)
  for (uint32_t r = 0; r < cnt; ++r) s_d[r][tid] = dist2_exact(c.q, S.xd[s_s[r][tid]]);
  for (uint32_t r = 1; r < cnt; ++r) {
    const double d = s_d[r][tid];
    const uint32_t sl = s_s[r][tid];
    const uint32_t pj = S.perm[sl];
    uint32_t pos = r;
    while (pos > 0) {
      const double dp = s_d[pos - 1][tid];
      if (dp < d || (dp == d && S.perm[s_s[pos - 1][tid]] < pj)) break;
      s_d[pos][tid] = dp;
      s_s[pos][tid] = s_s[pos - 1][tid];
      --pos;
    }
    s_d[pos][tid] = d;
    s_s[pos][tid] = sl;
  }
  write_outputs(a, S, c, qi, cnt < K ? cnt : K, copies, dup_lower, &s_d[0][tid], &s_s[0][tid],
                kKnnThreads);
}

// The exact search of all queries (qsel null) or of the queries qsel[0 ..
// *qcount) (a device count: every query gets a thread, those past the count
// return at once).
static void launch_knn_exact(const KnnArgs& a, const uint32_t* qsel, const uint32_t* qcount,
                             cudaStream_t st) {
  if (a.k <= kKnnMaxK) {
    const int bs = a.k <= kKnnSmemK ? kKnnThreads : 32;
    const size_t sh = (sizeof(double) + sizeof(uint32_t)) * a.k * bs;
    cudaFuncSetAttribute(knn_exact_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sh);
    knn_exact_kernel<true><<<(a.nq + bs - 1) / bs, bs, sh, st>>>(a, *a.S, a.S->gd, a.S->aux,
                                                                qsel, qcount); count_launch();
  } else {
    knn_exact_kernel<false><<<(a.nq + kKnnThreads - 1) / kKnnThreads, kKnnThreads, 0, st>>>(
        a, *a.S, a.S->gd, a.S->aux, qsel, qcount); count_launch();
  }
}

// ---- tiled search: lists up to kKnnMaxK in shared memory --------------------
// The queries are cut into tiles: the largest octree nodes with at most
// kTileMax seeds (a fine cell with more is cut into pieces of 32
// consecutive slots), 32 queries at most per tile, one warp per tile.  A
// warp reads the seeds of the 27 nodes of the tile's level around the tile,
// then those of the surrounding nodes that its pruning distance still
// reaches, gathered 32 at a time across node boundaries (a warp scan of the
// node counts) and staged in shared memory; every lane tests every staged
// seed against its own query.  A seed nearer than the lane's pruning
// distance goes to the lane's buffer; after each chunk of 32 the lanes empty
// their buffers into their own max-heaps of the k + kKnnExtra nearest by
// FP32 distance together (column `lane` of [k][32] arrays: conflict-free).
// The first pruning distance comes from the tile's seed density; a lane
// that finds fewer seeds than the heap holds within it takes the exact
// search instead.  The kept seeds are sorted by FP32 distance; neighbours in
// that order farther apart than their error bound are in exact order
// already, and runs of closer ones are re-ranked in FP64 by (d2, original
// index), so the lists equal the exact search's.
constexpr uint32_t kTileMax = 64;

// Squared distance (fine-cell units) between the box of node (ix, iy, iz)
// of side `side` and the box [lo, hi], shrunk by a small slack as
// node_box_d2.
__device__ __forceinline__ float box_box_d2(uint32_t ix, uint32_t iy, uint32_t iz, float side,
                                            const float* lo, const float* hi) {
  const float bx = ix * side, by = iy * side, bz = iz * side;
  float dx = fmaxf(fmaxf(bx - hi[0], lo[0] - (bx + side)), 0.f);
  float dy = fmaxf(fmaxf(by - hi[1], lo[1] - (by + side)), 0.f);
  float dz = fmaxf(fmaxf(bz - hi[2], lo[2] - (bz + side)), 0.f);
  dx = fmaxf(dx - 1e-3f, 0.f);
  dy = fmaxf(dy - 1e-3f, 0.f);
  dz = fmaxf(dz - 1e-3f, 0.f);
  return dx * dx + dy * dy + dz * dz;
}

// Candidates a lane buffers before emptying them into its heap: a whole
// staged chunk (measured: half-chunk buffers, which leave room for a 7th
// warp per SM, made the search 17% slower by doubling the divergent heap
// updates).
constexpr uint32_t kTileBuf = 32;

size_t knn_tile_smem(uint32_t k) {
  // staged seeds (float4 + slot), the lane buffers, the heaps
  return 32 * (sizeof(float4) + sizeof(uint32_t)) + kTileBuf * 32 * sizeof(uint2) +
         (size_t)(k + kKnnExtra) * 32 * (sizeof(float) + sizeof(uint32_t));
}

size_t knn_tile_scratch_elems(uint32_t n, int L) {
  const size_t nf = ((size_t)1 << (3 * L)) + 1;
  return nf + scan_tmp_elems(nf) + 2 * ((size_t)n + nf) + 2;
}

// Level of the tile holding fine cell f (the highest ancestor with at most
// kTileMax seeds, or L); its seed range in b/e.
__device__ __forceinline__ int tile_level(const uint32_t* __restrict__ cs, uint32_t f, int L,
                                          uint32_t& b, uint32_t& e) {
  int lev = L;
  b = cs[f];
  e = cs[f + 1];
  for (int l = L - 1; l >= 0; --l) {
    const int sh = 3 * (L - l);
    const uint32_t node = f >> sh;
    const uint32_t bb = cs[node << sh], ee = cs[(node + 1u) << sh];
    if (ee - bb > kTileMax) break;
    lev = l;
    b = bb;
    e = ee;
  }
  return lev;
}

// Tiles per fine cell: the cell that starts its tile emits ceil(count / 32).
__global__ void tile_count_kernel(const uint32_t* __restrict__ cs, int L, uint32_t nf,
                                  uint32_t* __restrict__ cnt) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f > nf) return;
  if (f == nf) {
    cnt[nf] = 0;
    return;
  }
  uint32_t b, e;
  const int lev = tile_level(cs, f, L, b, e);
  const int sh = 3 * (L - lev);
  const bool first = ((f >> sh) << sh) == f;
  cnt[f] = first ? (e - b + 31u) / 32u : 0u;
}

// items[t] = (first slot, count | level << 8)
__global__ void tile_fill_kernel(const uint32_t* __restrict__ cs, int L, uint32_t nf,
                                 const uint32_t* __restrict__ off, uint2* __restrict__ items) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const uint32_t m = off[f + 1] - off[f];
  if (m == 0) return;
  uint32_t b, e;
  const int lev = tile_level(cs, f, L, b, e);
  for (uint32_t k = 0; k < m; ++k) {
    const uint32_t s0 = b + 32u * k;
    items[off[f] + k] = make_uint2(s0, min(32u, e - s0) | ((uint32_t)lev << 8));
  }
}

__global__ void __launch_bounds__(32)
knn_tile_kernel(KnnArgs a, SortedSeeds S, const GridDesc* __restrict__ gdp,
                const double* __restrict__ aux, const uint32_t* __restrict__ ntiles,
                const uint2* __restrict__ items) {
  extern __shared__ __align__(16) unsigned char knn_smem[];
  const int lane = threadIdx.x;
  const unsigned FULL = 0xFFFFFFFFu;
  const uint32_t K = a.k;
  const uint32_t cap = K + kKnnExtra;
  float4* s_pt = reinterpret_cast<float4*>(knn_smem);
  uint32_t* s_sl = reinterpret_cast<uint32_t*>(s_pt + 32);
  uint2* s_buf = reinterpret_cast<uint2*>(s_sl + 32);  // [kTileBuf][32] (d32 bits, slot)
  float* hd = reinterpret_cast<float*>(s_buf + kTileBuf * 32);
  uint32_t* hs = reinterpret_cast<uint32_t*>(hd + (size_t)cap * 32);
  if (blockIdx.x >= *ntiles) return;
  const uint2 item = items[blockIdx.x];
  const uint32_t nq_tile = item.y & 0xFFu;
  const int tlev = (int)(item.y >> 8);
  const bool active = (uint32_t)lane < nq_tile;
  const uint32_t qi = item.x + (active ? lane : 0);
  const GridDesc g = *gdp;
  const QueryCtx c = make_query(a, S, g, qi);
  const float delta = 8.0f * (float)aux[1] * 5.9604645e-8f + 1e-30f;
  auto D = [&](uint32_t r) -> float& { return hd[(size_t)r * 32 + lane]; };
  auto SL = [&](uint32_t r) -> uint32_t& { return hs[(size_t)r * 32 + lane]; };

  // the tile's node, its box and seed count; the box of its queries
  const int tsh = g.L - tlev;                    // node side = 2^tsh fine cells
  const float tside = (float)(1u << tsh);
  const int NG = 1 << tlev;                      // nodes per axis at that level
  const int G = g.G;
  const uint32_t fx = (uint32_t)clampi((int)c.ux, 0, G - 1);
  const uint32_t fy = (uint32_t)clampi((int)c.uy, 0, G - 1);
  const uint32_t fz = (uint32_t)clampi((int)c.uz, 0, G - 1);
  const int nx = (int)__shfl_sync(FULL, fx >> tsh, 0);
  const int ny = (int)__shfl_sync(FULL, fy >> tsh, 0);
  const int nz = (int)__shfl_sync(FULL, fz >> tsh, 0);
  float lo[3] = {c.ux, c.uy, c.uz}, hi[3] = {c.ux, c.uy, c.uz};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(FULL, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(FULL, hi[d], o));
    }
  }

  uint32_t cnt = 0, copies = 0;
  bool dup_lower = false;
  auto sift_down = [&](uint32_t i, uint32_t n) {
    const float d = D(i);
    const uint32_t sl = SL(i);
    for (;;) {
      uint32_t c1 = 2 * i + 1;
      if (c1 >= n) break;
      float dc = D(c1);
      if (c1 + 1 < n) {
        const float d2 = D(c1 + 1);
        if (d2 > dc) {
          dc = d2;
          ++c1;
        }
      }
      if (dc <= d) break;
      D(i) = dc;
      SL(i) = SL(c1);
      i = c1;
    }
    D(i) = d;
    SL(i) = sl;
  };
  float thr;
  auto offer = [&](uint32_t s2, float d32) {
    if (a.mode == KNN_CELLS && s2 == c.qslot) return;
    if (a.mode == KNN_CELLS && d32 <= 0.f) {
      if (dist2_exact(c.q, S.xd[s2]) == 0.0) {
        if (S.perm[s2] < c.qperm) dup_lower = true;
        else ++copies;
        return;
      }
    }
    if (cnt < cap) {
      uint32_t i = cnt++;
      while (i > 0) {
        const uint32_t par = (i - 1) >> 1;
        const float dp = D(par);
        if (dp >= d32) break;
        D(i) = dp;
        SL(i) = SL(par);
        i = par;
      }
      D(i) = d32;
      SL(i) = s2;
      if (cnt == cap) thr = fminf(thr, D(0));
    } else {
      D(0) = d32;
      SL(0) = s2;
      sift_down(0, cap);
      thr = D(0);
    }
  };

  // ---- first pruning distance: a ball of 1.35x the radius that holds cap
  // seeds at the tile's density (plus the largest lift difference, 4-d)
  float t0 = FLT_MAX;
  if (a.nq > 4 * cap) {
    const uint32_t tcode = morton3((uint32_t)nx, (uint32_t)ny, (uint32_t)nz);
    const uint32_t tb = S.cell_start[tcode << (3 * tsh)];
    const uint32_t te = S.cell_start[(tcode + 1u) << (3 * tsh)];
    const float rho = (float)max(te - tb, 8u) / (tside * tside * tside);
    const float r = 1.35f * cbrtf(3.f * (float)cap / (4.f * 3.14159265f * rho));
    t0 = (r * g.h_f) * (r * g.h_f) + (float)aux[2] * 1.0001f;
  }
  thr = t0;
  float wthr = t0;
  const float h2f = g.h_f * g.h_f;
  uint2* mybuf = s_buf + lane;  // entry j at mybuf[32 * j]
  uint32_t bn = 0;
  bool searching = active;  // the lane still takes offers in this sweep

  // Offers the seeds of up to 32 nodes (one per lane: first slot b, count
  // n) to every query, 32 at a time.
  auto gather = [&](uint32_t b, uint32_t n) {
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    const uint32_t excl = incl - n;
    for (uint32_t base = 0; base < total; base += 32) {
      const uint32_t i = base + lane;
      // the last lane whose range starts at or before i owns it
      int own = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const uint32_t e = __shfl_sync(FULL, excl, own + step);
        if (e <= i) own += step;
      }
      const uint32_t ob = __shfl_sync(FULL, b, own);
      const uint32_t oe = __shfl_sync(FULL, excl, own);
      __syncwarp();
      if (i < total) {
        const uint32_t s2 = ob + (i - oe);
        s_pt[lane] = S.xf[s2];
        s_sl[lane] = s2;
      }
      __syncwarp();
      const uint32_t m = min(32u, total - base);
      for (uint32_t t0s = 0; t0s < m; t0s += kTileBuf) {
        const uint32_t t1 = min(m, t0s + kTileBuf);
        for (uint32_t t = t0s; t < t1; ++t) {
          const float4 p = s_pt[t];
          const float dx = p.x - c.qf.x, dy = p.y - c.qf.y, dz = p.z - c.qf.z,
                      dh = p.w - c.qf.w;
          const float d32 = dx * dx + dy * dy + dz * dz + dh * dh;
          if (searching && d32 < thr) {
            mybuf[32 * bn] = make_uint2(__float_as_uint(d32), s_sl[t]);
            ++bn;
          }
        }
        // every lane empties its buffer into its heap
        for (uint32_t j = 0; j < bn; ++j) {
          const uint2 v = mybuf[32 * j];
          const float d32 = __uint_as_float(v.x);
          if (d32 < thr) offer(v.y, d32);
        }
        bn = 0;
      }
    }
    wthr = searching ? thr : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wthr = fmaxf(wthr, __shfl_xor_sync(FULL, wthr, o));
  };

  // squared distance (world units) from the query box to node (x, y, z)
  auto node_d2 = [&](int x, int y, int z) {
    return box_box_d2((uint32_t)x, (uint32_t)y, (uint32_t)z, tside, lo, hi) * h2f;
  };
  auto node_range = [&](int x, int y, int z, uint32_t& b, uint32_t& n) {
    const uint32_t code = morton3((uint32_t)x, (uint32_t)y, (uint32_t)z);
    b = S.cell_start[code << (3 * tsh)];
    n = S.cell_start[(code + 1u) << (3 * tsh)] - b;
  };

  // A lane that finds fewer than cap seeds within its first pruning
  // distance (a query near the domain's boundary, where the ball of the
  // density estimate is cut) starts over with a ball of twice the radius,
  // up to twice; the other lanes keep their heaps.
  float t_lane = t0;
  for (int sweep = 0; sweep < 3; ++sweep) {
  // ---- the 27 nodes around the tile, nearest first (the node, its 6
  // faces, 12 edges, 8 corners): the heaps fill with near seeds early, so
  // that their bounds prune more of the farther ones
  {
    uint32_t b = 0, n = 0;
    if (lane < 27) {
      // offsets + 1 per axis, as x + 3 y + 9 z, sorted by |dx| + |dy| + |dz|
      constexpr uint8_t kNear[27] = {13, 4, 10, 12, 14, 16, 22, 1, 3, 5, 7, 9, 11,
                                     15, 17, 19, 21, 23, 25, 0, 2, 6, 8, 18, 20, 24, 26};
      const int o = kNear[lane];
      const int x = nx + o % 3 - 1, y = ny + (o / 3) % 3 - 1, z = nz + o / 9 - 1;
      if (x >= 0 && y >= 0 && z >= 0 && x < NG && y < NG && z < NG) node_range(x, y, z, b, n);
    }
    gather(b, n);
  }
  // ---- the nodes beyond them that the pruning distance still reaches
  {
    // reach in fine cells, with a margin for the FP32 arithmetic
    const float rr = (wthr < FLT_MAX) ? sqrtf(wthr) / g.h_f * 1.001f + 0.01f : 2.f * (float)G;
    const int x0 = max(0, (int)floorf((lo[0] - rr) / tside)), x1 = min(NG - 1, (int)floorf((hi[0] + rr) / tside));
    const int y0 = max(0, (int)floorf((lo[1] - rr) / tside)), y1 = min(NG - 1, (int)floorf((hi[1] + rr) / tside));
    const int z0 = max(0, (int)floorf((lo[2] - rr) / tside)), z1 = min(NG - 1, (int)floorf((hi[2] + rr) / tside));
    const int sx = x1 - x0 + 1, sy = y1 - y0 + 1, sz = z1 - z0 + 1;
    const int total = (x1 >= x0 && y1 >= y0 && z1 >= z0) ? sx * sy * sz : 0;
    for (int base = 0; base < total; base += 32) {
      uint32_t b = 0, n = 0;
      const int idx = base + lane;
      if (idx < total) {
        const int x = x0 + idx % sx, y = y0 + (idx / sx) % sy, z = z0 + idx / (sx * sy);
        const bool inner = abs(x - nx) <= 1 && abs(y - ny) <= 1 && abs(z - nz) <= 1;
        if (!inner && !(wthr < FLT_MAX && node_d2(x, y, z) > wthr)) node_range(x, y, z, b, n);
      }
      gather(b, n);
    }
  }
    searching = active && cnt < cap && t_lane < FLT_MAX;
    if (!__any_sync(FULL, searching)) break;
    if (searching) {
      t_lane = 4.f * t_lane;
      thr = t_lane;
      cnt = 0;
      copies = 0;
      dup_lower = false;
    }
    wthr = searching ? thr : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wthr = fmaxf(wthr, __shfl_xor_sync(FULL, wthr, o));
  }
  if (!active) return;

  // ---- per lane: heap sort, ascending FP32 distance
  for (uint32_t n = cnt; n > 1; --n) {
    const float dr = D(0);
    const uint32_t sr = SL(0);
    D(0) = D(n - 1);
    SL(0) = SL(n - 1);
    D(n - 1) = dr;
    SL(n - 1) = sr;
    sift_down(0, n - 1);
  }
  bool unsure = cnt < cap && t_lane < FLT_MAX;  // fewer than cap within the last distance
  if (cnt == cap) {
    // a seed that may belong to the k nearest could have been dropped
    const float r = sqrtf(D(K - 1)) * 1.0000076f + 2.f * delta;
    unsure = !(D(cap - 1) > r * r * 1.0000076f);
  }
  if (unsure) {
    const uint32_t k = atomicAdd(a.flag_count, 1u);
    a.flag_list[k] = qi;
    if (a.cnt) a.cnt[qi] = 0;
    return;
  }
  // ---- exact order: runs of neighbours whose FP32 distances are within
  // their error bound of each other are sorted by exact (d2, index)
  auto exact_run = [&](uint32_t r0, uint32_t r1) {
    for (uint32_t r = r0 + 1; r < r1; ++r) {
      const uint32_t sl = SL(r);
      const double d = dist2_exact(c.q, S.xd[sl]);
      const uint32_t p = S.perm[sl];
      uint32_t pos = r;
      while (pos > r0) {
        const uint32_t s1 = SL(pos - 1);
        if (!pair_greater(dist2_exact(c.q, S.xd[s1]), S.perm[s1], d, p)) break;
        SL(pos) = s1;
        --pos;
      }
      SL(pos) = sl;
    }
  };
  {
    uint32_t run0 = 0;
    for (uint32_t r = 1; r <= cnt; ++r) {
      bool split = r == cnt;
      if (!split) {
        const float rr = sqrtf(D(r - 1)) * 1.0000076f + 2.f * delta;
        split = D(r) > rr * rr * 1.0000076f;
      }
      if (split) {
        if (r - run0 > 1) exact_run(run0, r);
        run0 = r;
      }
    }
  }
  uint32_t out = cnt < K ? cnt : K;
  if (a.cnt) a.cnt[qi] = (a.mode == KNN_CELLS) ? pack_cnt(out, copies, dup_lower) : out;
  if (a.mode == KNN_CELLS && dup_lower) out = 0;
  if (a.nbr)
    for (uint32_t r = 0; r < out; ++r) a.nbr[(size_t)r * a.out_stride + qi] = SL(r);
  if (a.last_d2) {
    if (out) {
      const uint32_t sl = SL(out - 1);
      a.last_d2[qi] = dist2_exact(c.q, S.xd[sl]);
      a.last_idx[qi] = S.perm[sl];
    } else {
      a.last_d2[qi] = c.has_lo ? c.lo_d : 0.0;
      a.last_idx[qi] = c.has_lo ? c.lo_i : 0u;
    }
  }
  if (a.exp_idx) {
    const size_t row = (a.mode == KNN_QUERY) ? qi : c.qperm;
    for (uint32_t r = 0; r < K; ++r) {
      const bool h = r < out;
      a.exp_idx[row * K + r] = h ? S.perm[SL(r)] : kNone;
      if (a.exp_d2) a.exp_d2[row * K + r] = h ? dist2_exact(c.q, S.xd[SL(r)]) : INFINITY;
    }
  }
}

void launch_knn(const KnnArgs& a, cudaStream_t st) {
  if (a.nq == 0) return;
  if (a.k <= kKnnMaxK && a.flag_count && a.coherent && a.tile_scratch && !a.qlist &&
      a.nq == a.S->n) {
    // tiles of the octree, the tiled search, then the exact search of the
    // queries whose FP32 screening could not settle the list
    const int L = a.S->L;
    const uint32_t nf = 1u << (3 * L);
    uint32_t* off = a.tile_scratch;                       // nf + 1
    uint32_t* tmp = off + nf + 1;                         // scan scratch
    size_t items_at = (size_t)nf + 1 + scan_tmp_elems((size_t)nf + 1);
    items_at += items_at & 1;  // 8-byte aligned
    uint2* items = reinterpret_cast<uint2*>(a.tile_scratch + items_at);
    tile_count_kernel<<<(nf + 256) / 256, 256, 0, st>>>(a.S->cell_start, L, nf, off); count_launch();
    exclusive_scan_u32(off, (size_t)nf + 1, tmp, st);
    tile_fill_kernel<<<(nf + 255) / 256, 256, 0, st>>>(a.S->cell_start, L, nf, off, items); count_launch();
    const size_t sh = knn_tile_smem(a.k);
    cudaFuncSetAttribute(knn_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    cudaMemsetAsync(a.flag_count, 0, sizeof(uint32_t), st);
    // tiles <= fine cells + queries / 32
    const unsigned grid = nf + (a.nq + 31) / 32;
    knn_tile_kernel<<<grid, 32, sh, st>>>(a, *a.S, a.S->gd, a.S->aux, off + nf, items); count_launch();
    launch_knn_exact(a, a.flag_list, a.flag_count, st);
    return;
  }
  if (a.k <= kKnnSmemK && a.flag_count) {
    const size_t sh = (sizeof(double) + sizeof(uint32_t)) * kKnnCap * kKnnThreads;
    cudaFuncSetAttribute(knn_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    cudaMemsetAsync(a.flag_count, 0, sizeof(uint32_t), st);
    const unsigned nb = (a.nq + kKnnThreads - 1) / kKnnThreads;
    knn_fast_kernel<<<nb, kKnnThreads, sh, st>>>(a, *a.S, a.S->gd, a.S->aux); count_launch();
    launch_knn_exact(a, a.flag_list, a.flag_count, st);
  } else {
    launch_knn_exact(a, nullptr, nullptr, st);
  }
}

}  // namespace gbv
