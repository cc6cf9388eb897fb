// Semi-discrete optimal transport on the GPU: the Hessian of the
// Kantorovich dual in CSR, the sparse product and the vector steps of a
// Jacobi-preconditioned conjugate gradient, all in FP64.
//
// The reference's solver (exploragram's OptimalTransportMap3d) is not in
// the checkout; this follows the published method it implements (B. Levy,
// "A numerical algorithm for L2 semi-discrete optimal transport in 3D",
// ESAIM M2AN 49(6), 2015; damped Newton of Kitagawa, Merigot and Thibert,
// JEMS 2019): for weights w, the gradient of the dual is nu_i - |Lag_i(w)|
// and its Hessian is the graph Laplacian with coefficients
// A_ij / (2 |p_i - p_j|) over the Laguerre facets.
//
// Reductions are deterministic: every block sums a fixed part of the
// vector in a fixed order and a fixed tree, and the partial sums are added
// in a fixed order.  FP64 instructions are the scarce resource on this part
// (their pipe, not memory, bounds the CG kernels), so the kernels keep them
// few: plain sums instead of compensated ones, one row per thread in the
// product, the Jacobi preconditioner as a product by the inverse diagonal.
#include <cfloat>

#include "gbv_common.cuh"
#include "gbv_ot.cuh"

namespace gbv {

constexpr int kOtThreads = 256;
constexpr int kOtWarps = kOtThreads / 32;

// Sum of v over the block, in a fixed tree; the result in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[kOtWarps];
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
  __syncthreads();  // ws may still be read by a previous call
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (warp == 0) {
    t = lane < kOtWarps ? ws[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(FULL, t, o);
  }
  return t;
}

// Same for max / min (results in thread 0).
template <bool kMax>
__device__ __forceinline__ double block_ext(double v) {
  __shared__ double ws[kOtWarps];
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_down_sync(FULL, v, o);
    v = kMax ? fmax(v, u) : fmin(v, u);
  }
  __syncthreads();
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  double t = v;
  if (warp == 0) {
    t = ws[lane < kOtWarps ? lane : 0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double u = __shfl_down_sync(FULL, t, o);
      t = kMax ? fmax(t, u) : fmin(t, u);
    }
  }
  return t;
}

// ---------------------------------------------------------------------
// Hessian assembly
// ---------------------------------------------------------------------
__global__ void hessian_kernel(const double* __restrict__ xyz, const uint32_t* __restrict__ rowptr,
                               const uint32_t* __restrict__ col, const double* __restrict__ area,
                               uint32_t n, double* __restrict__ val, double* __restrict__ diag,
                               double* __restrict__ invd) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xi = xyz[3 * (size_t)i], yi = xyz[3 * (size_t)i + 1], zi = xyz[3 * (size_t)i + 2];
  double d = 0.0;
  for (uint32_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
    const uint32_t j = col[k];
    // the facet seen from cell j
    double aji = -1.0;
    for (uint32_t l = rowptr[j]; l < rowptr[j + 1]; ++l)
      if (col[l] == i) {
        aji = area[l];
        break;
      }
    double c = 0.0;
    if (aji >= 0.0) {
      const double dx = xyz[3 * (size_t)j] - xi, dy = xyz[3 * (size_t)j + 1] - yi,
                   dz = xyz[3 * (size_t)j + 2] - zi;
      const double dist = sqrt(dx * dx + dy * dy + dz * dz);
      // (A_ij + A_ji) with the lower index's area first: identical on both sides
      const double asum = (i < j) ? area[k] + aji : aji + area[k];
      c = asum / (4.0 * dist);
    }
    val[k] = -c;
    d += c;
  }
  diag[i] = d;
  invd[i] = d > 0.0 ? 1.0 / d : 1.0;
}

// Slice widths of the sliced-ELL copy: 32 times the longest row of each
// slice of 32 rows (one warp per slice).
__global__ void sell_width_kernel(const uint32_t* __restrict__ rowptr, uint32_t n, uint32_t nsl,
                                  uint32_t* __restrict__ sl_off) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t deg = i < n ? rowptr[i + 1] - rowptr[i] : 0u;
  const uint32_t w = __reduce_max_sync(0xFFFFFFFFu, deg);
  if ((threadIdx.x & 31) == 0 && (i >> 5) < nsl) sl_off[i >> 5] = 32u * w;
}

// Row i of the CSR into its slice: entry k at sl_off[s] + 32 k + lane; rows
// shorter than the slice are padded with zeros on their own column.
__global__ void sell_pack_kernel(const uint32_t* __restrict__ rowptr,
                                 const uint32_t* __restrict__ col, const double* __restrict__ val,
                                 const uint32_t* __restrict__ sl_off, uint32_t n,
                                 uint32_t* __restrict__ s_col, double* __restrict__ s_val) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = i >> 5, lane = i & 31;
  const uint32_t base = sl_off[s], w = (sl_off[s + 1] - base) >> 5;
  const uint32_t b = rowptr[i], deg = rowptr[i + 1] - b;
  for (uint32_t k = 0; k < w; ++k) {
    const size_t pos = (size_t)base + 32u * k + lane;
    s_col[pos] = k < deg ? col[b + k] : i;
    s_val[pos] = k < deg ? val[b + k] : 0.0;
  }
}

void assemble_hessian(const double* xyz, const uint32_t* rowptr, const uint32_t* col,
                      const double* area, uint32_t n, Hessian& H, cudaStream_t st) {
  H.rowptr = rowptr;
  H.col = col;
  H.n = n;
  hessian_kernel<<<(n + kOtThreads - 1) / kOtThreads, kOtThreads, 0, st>>>(
      xyz, rowptr, col, area, n, H.val, H.diag, H.invd); count_launch();
}

uint32_t sell_slices(uint32_t n) { return (n + 31) / 32; }

void sell_widths(const Hessian& H, uint32_t* sl_off, cudaStream_t st) {
  const uint32_t nsl = sell_slices(H.n), threads = nsl * 32u;
  sell_width_kernel<<<(threads + kOtThreads - 1) / kOtThreads, kOtThreads, 0, st>>>(
      H.rowptr, H.n, nsl, sl_off); count_launch();
}

void sell_pack(Hessian& H, const uint32_t* sl_off, uint32_t* s_col, double* s_val,
               cudaStream_t st) {
  H.sl_off = sl_off;
  H.s_col = s_col;
  H.s_val = s_val;
  sell_pack_kernel<<<(H.n + kOtThreads - 1) / kOtThreads, kOtThreads, 0, st>>>(
      H.rowptr, H.col, H.val, sl_off, H.n, s_col, s_val); count_launch();
}

// ---------------------------------------------------------------------
// Reductions and vector steps
// ---------------------------------------------------------------------
__global__ void dot_kernel(const double* __restrict__ a, const double* __restrict__ b, uint32_t n,
                           double* __restrict__ part) {
  double s = 0.0;
  const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s = fma(a[i], b[i], s);
  s = block_sum(s);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s;
    part[2 * blockIdx.x + 1] = 0.0;
  }
}

void dot_parts(const double* a, const double* b, uint32_t n, double* part, cudaStream_t st) {
  dot_kernel<<<kOtParts, kOtThreads, 0, st>>>(a, b, n, part); count_launch();
}

// part layout: [2*kOtParts] sum of r^2 ((s, 0) pairs), then per block
// max |r_i|/nu_i at [2*kOtParts + b] and min vol at [3*kOtParts + b].
__global__ void residual_kernel(const double* __restrict__ vol, const double* __restrict__ nu,
                                uint32_t n, double* __restrict__ r, double* __restrict__ part) {
  double s = 0.0, mx = 0.0, mn = DBL_MAX;
  const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double ri = vol[i] - nu[i];
    r[i] = ri;
    s = fma(ri, ri, s);
    mx = fmax(mx, fabs(ri) / nu[i]);
    mn = fmin(mn, vol[i]);
  }
  s = block_sum(s);
  mx = block_ext<true>(mx);
  mn = block_ext<false>(mn);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s;
    part[2 * blockIdx.x + 1] = 0.0;
    part[2 * kOtParts + blockIdx.x] = mx;
    part[3 * kOtParts + blockIdx.x] = mn;
  }
}

void residual(const double* vol, const double* nu, uint32_t n, double* r, double* part,
              cudaStream_t st) {
  residual_kernel<<<kOtParts, kOtThreads, 0, st>>>(vol, nu, n, r, part); count_launch();
}

__global__ void precond_kernel(const double* __restrict__ r, const double* __restrict__ invd,
                               double* __restrict__ z, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = r[i] * invd[i];
}

__global__ void axpy_kernel(double* __restrict__ y, const double* __restrict__ x, double alpha,
                            uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = fma(alpha, x[i], y[i]);
}

__global__ void add_scalar_kernel(double* __restrict__ y, double c, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += c;
}

__global__ void scale_copy_kernel(double* __restrict__ y, const double* __restrict__ x, double alpha,
                                  uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = alpha * x[i];
}

static inline unsigned nb(uint32_t n) { return (n + kOtThreads - 1) / kOtThreads; }

void cg_precond(const double* r, const double* invd, double* z, uint32_t n, cudaStream_t st) {
  precond_kernel<<<nb(n), kOtThreads, 0, st>>>(r, invd, z, n); count_launch();
}
void axpy(double* y, const double* x, double alpha, uint32_t n, cudaStream_t st) {
  axpy_kernel<<<nb(n), kOtThreads, 0, st>>>(y, x, alpha, n); count_launch();
}
void add_scalar(double* y, double c, uint32_t n, cudaStream_t st) {
  add_scalar_kernel<<<nb(n), kOtThreads, 0, st>>>(y, c, n); count_launch();
}
void scale_copy(double* y, const double* x, double alpha, uint32_t n, cudaStream_t st) {
  scale_copy_kernel<<<nb(n), kOtThreads, 0, st>>>(y, x, alpha, n); count_launch();
}

// ---------------------------------------------------------------------
// Device-resident preconditioned CG
// ---------------------------------------------------------------------
// The last block of a launch to finish: every block has stored its partial
// (thread 0, before the fence) when the ticket reaches gridDim.x - 1.  The
// last block resets the ticket for the next launch.
__device__ __forceinline__ bool last_block(uint32_t* ticket) {
  __shared__ bool am_last;
  __threadfence();
  if (threadIdx.x == 0) am_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  return am_last;
}

// Sum of part[stride * b + off], b < nparts, in a fixed order (thread t adds
// parts t, t + 256, ... then the block tree); result in thread 0.  The
// partials of the other blocks are read from L2.
__device__ __forceinline__ double sum_parts(const double* part, int nparts, int stride, int off) {
  double v = 0.0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += __ldcg(&part[stride * b + off]);
  return block_sum(v);
}

// Rows of one block: a contiguous run of slices, the same in every launch.
struct SliceRange {
  uint32_t lo, hi;
};
__device__ __forceinline__ SliceRange block_slices(uint32_t n) {
  const uint32_t nsl = (n + 31) / 32, ngrp = (nsl + kOtWarps - 1) / kOtWarps;
  const uint32_t per = (ngrp + gridDim.x - 1) / gridDim.x;
  const uint32_t g0 = min(ngrp, blockIdx.x * per), g1 = min(ngrp, g0 + per);
  return {g0 * kOtWarps, min(nsl, g1 * kOtWarps)};
}

// Ap = H p on the sliced-ELL copy, one row per thread (a warp per slice);
// the block's share of p . Ap to part[b]; the last block sets
// alpha = rz / pAp (done if pAp <= 0).
__global__ void __launch_bounds__(kOtThreads)
pcg_spmv_kernel(const uint32_t* __restrict__ sl_off, const uint32_t* __restrict__ s_col,
                const double* __restrict__ s_val, const double* __restrict__ diag,
                const double* __restrict__ p, uint32_t n, double* __restrict__ Ap,
                double* __restrict__ part, CgScalars* __restrict__ sc) {
  if (sc->done) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const SliceRange R = block_slices(n);
  double s = 0.0;
  for (uint32_t sl = R.lo + warp; sl < R.hi; sl += kOtWarps) {
    const uint32_t i = sl * 32 + lane;
    const uint32_t base = sl_off[sl], w = (sl_off[sl + 1] - base) >> 5;
    if (i >= n) continue;
    double acc = 0.0;
    const uint32_t* cp = s_col + base + lane;
    const double* vp = s_val + base + lane;
    for (uint32_t k = 0; k < w; ++k) acc = fma(vp[32 * k], p[cp[32 * k]], acc);
    const double pi = p[i];
    const double yi = fma(diag[i], pi, acc);
    Ap[i] = yi;
    s = fma(pi, yi, s);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (!last_block(&sc->ticket)) return;
  const double pAp = sum_parts(part, gridDim.x, 1, 0);
  if (threadIdx.x == 0) {
    if (pAp > 0.0) sc->alpha = sc->rz / pAp;
    else sc->done = 1;
    sc->ticket = 0;
  }
}

// x += alpha p; r -= alpha Ap; z = r / diag; the block's shares of r . r
// and r . z to part[2 b], part[2 b + 1]; the last block sets beta =
// rz' / rz, rz = rz', counts the iteration and stops at rr <= tol2 b2.
__global__ void __launch_bounds__(kOtThreads)
pcg_xr_kernel(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
              const double* __restrict__ Ap, const double* __restrict__ invd,
              double* __restrict__ z, uint32_t n, double* __restrict__ part,
              CgScalars* __restrict__ sc) {
  if (sc->done) return;
  const double alpha = sc->alpha;
  const SliceRange R = block_slices(n);
  const uint32_t lo = R.lo * 32, hi = min(n, R.hi * 32);
  double rr = 0.0, rz = 0.0;
  for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    const double zi = ri * invd[i];
    z[i] = zi;
    rr = fma(ri, ri, rr);
    rz = fma(ri, zi, rz);
  }
  rr = block_sum(rr);
  rz = block_sum(rz);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = rr;
    part[2 * blockIdx.x + 1] = rz;
  }
  if (!last_block(&sc->ticket)) return;
  const double rr_t = sum_parts(part, gridDim.x, 2, 0);
  const double rz_t = sum_parts(part, gridDim.x, 2, 1);
  if (threadIdx.x == 0) {
    sc->beta = rz_t / sc->rz;
    sc->rz = rz_t;
    sc->k += 1;
    if (rr_t <= sc->tol2 * sc->b2) sc->done = 1;
    sc->ticket = 0;
  }
}

// p = z + beta p.
__global__ void __launch_bounds__(kOtThreads)
pcg_p_kernel(double* __restrict__ p, const double* __restrict__ z, uint32_t n,
             const CgScalars* __restrict__ sc) {
  if (sc->done) return;
  const double beta = sc->beta;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = fma(beta, p[i], z[i]);
}

uint32_t pcg_blocks(uint32_t n) {
  const uint32_t ngrp = ((n + 31) / 32 + kOtWarps - 1) / kOtWarps;
  return ngrp < (uint32_t)kPcgParts ? (ngrp > 0 ? ngrp : 1u) : (uint32_t)kPcgParts;
}

void pcg_iterations(const Hessian& H, double* x, double* r, double* p, double* Ap, double* z,
                    double* part, CgScalars* sc, uint32_t count, cudaStream_t st) {
  const uint32_t G = pcg_blocks(H.n);
  for (uint32_t j = 0; j < count; ++j) {
    pcg_spmv_kernel<<<G, kOtThreads, 0, st>>>(H.sl_off, H.s_col, H.s_val, H.diag, p, H.n, Ap,
                                              part, sc); count_launch();
    pcg_xr_kernel<<<G, kOtThreads, 0, st>>>(x, r, p, Ap, H.invd, z, H.n, part, sc); count_launch();
    pcg_p_kernel<<<nb(H.n), kOtThreads, 0, st>>>(p, z, H.n, sc); count_launch();
  }
}

}  // namespace gbv
