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
// Reductions are deterministic: fixed partition, Neumaier compensated sums.
#include <cfloat>

#include "gbv_common.cuh"
#include "gbv_ot.cuh"

namespace gbv {

constexpr int kOtThreads = 256;

__device__ __forceinline__ void neu_add(double& s, double& c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x)) c += (s - t) + x;
  else c += (x - t) + s;
  s = t;
}

// Block-level combination of per-thread (s, c) pairs into part[2*block].
__device__ __forceinline__ void block_combine(double s, double c, double* part) {
  __shared__ double ss[kOtThreads], sc[kOtThreads];
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0, C = 0.0;
    for (int t = 0; t < kOtThreads; ++t) {
      neu_add(S, C, ss[t]);
      C += sc[t];
    }
    part[2 * blockIdx.x] = S;
    part[2 * blockIdx.x + 1] = C;
  }
}

// ---------------------------------------------------------------------
// Hessian assembly
// ---------------------------------------------------------------------
__global__ void hessian_kernel(const double* __restrict__ xyz, const uint32_t* __restrict__ rowptr,
                               const uint32_t* __restrict__ col, const double* __restrict__ area,
                               uint32_t n, double* __restrict__ val, double* __restrict__ diag) {
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
}

void assemble_hessian(const double* xyz, const uint32_t* rowptr, const uint32_t* col,
                      const double* area, uint32_t n, Hessian& H, cudaStream_t st) {
  H.rowptr = rowptr;
  H.col = col;
  H.n = n;
  hessian_kernel<<<(n + kOtThreads - 1) / kOtThreads, kOtThreads, 0, st>>>(xyz, rowptr, col, area,
                                                                          n, H.val, H.diag); count_launch();
}

// ---------------------------------------------------------------------
// y = H x, 8 lanes per row, with the partial sums of x . y
// ---------------------------------------------------------------------
constexpr int kRowLanes = 8;

__global__ void spmv_dot_kernel(const uint32_t* __restrict__ rowptr,
                                const uint32_t* __restrict__ col, const double* __restrict__ val,
                                const double* __restrict__ diag, const double* __restrict__ x,
                                uint32_t n, double* __restrict__ y, double* __restrict__ part) {
  const int sub = threadIdx.x & (kRowLanes - 1);
  const unsigned FULL = 0xFFFFFFFFu;
  double s = 0.0, cc = 0.0;
  const uint32_t rows_per_block = kOtThreads / kRowLanes;
  for (uint32_t base = blockIdx.x * rows_per_block; base < n; base += gridDim.x * rows_per_block) {
    const uint32_t i = base + threadIdx.x / kRowLanes;
    double acc = 0.0;
    if (i < n)
      for (uint32_t k = rowptr[i] + sub; k < rowptr[i + 1]; k += kRowLanes) acc += val[k] * x[col[k]];
    // fixed reduction tree inside the 8-lane group
#pragma unroll
    for (int o = kRowLanes / 2; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o, kRowLanes);
    if (sub == 0 && i < n) {
      const double yi = diag[i] * x[i] + acc;
      y[i] = yi;
      neu_add(s, cc, x[i] * yi);
    }
  }
  block_combine(s, cc, part);
}

void spmv_dot(const Hessian& H, const double* x, double* y, double* part, int nparts,
              cudaStream_t st) {
  spmv_dot_kernel<<<nparts, kOtThreads, 0, st>>>(H.rowptr, H.col, H.val, H.diag, x, H.n, y,
                                                 part); count_launch();
}

// ---------------------------------------------------------------------
// Reductions and vector steps
// ---------------------------------------------------------------------
__global__ void dot_kernel(const double* __restrict__ a, const double* __restrict__ b, uint32_t n,
                           double* __restrict__ part) {
  double s = 0.0, c = 0.0;
  const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) neu_add(s, c, a[i] * b[i]);
  block_combine(s, c, part);
}

void dot_parts(const double* a, const double* b, uint32_t n, double* part, cudaStream_t st) {
  dot_kernel<<<kOtParts, kOtThreads, 0, st>>>(a, b, n, part); count_launch();
}

// part layout: [2*kOtParts] sum of r^2 (s, c pairs), then per block
// max |r_i|/nu_i at [2*kOtParts + b] and min vol at [3*kOtParts + b].
__global__ void residual_kernel(const double* __restrict__ vol, const double* __restrict__ nu,
                                uint32_t n, double* __restrict__ r, double* __restrict__ part) {
  __shared__ double smax[kOtThreads], smin[kOtThreads];
  double s = 0.0, c = 0.0, mx = 0.0, mn = DBL_MAX;
  const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double ri = vol[i] - nu[i];
    r[i] = ri;
    neu_add(s, c, ri * ri);
    mx = fmax(mx, fabs(ri) / nu[i]);
    mn = fmin(mn, vol[i]);
  }
  smax[threadIdx.x] = mx;
  smin[threadIdx.x] = mn;
  block_combine(s, c, part);
  if (threadIdx.x == 0) {
    double M = 0.0, m = DBL_MAX;
    for (int t = 0; t < kOtThreads; ++t) {
      M = fmax(M, smax[t]);
      m = fmin(m, smin[t]);
    }
    part[2 * kOtParts + blockIdx.x] = M;
    part[3 * kOtParts + blockIdx.x] = m;
  }
}

void residual(const double* vol, const double* nu, uint32_t n, double* r, double* part,
              cudaStream_t st) {
  residual_kernel<<<kOtParts, kOtThreads, 0, st>>>(vol, nu, n, r, part); count_launch();
}

__global__ void cg_xr_kernel(double* __restrict__ x, double* __restrict__ r,
                             const double* __restrict__ p, const double* __restrict__ Ap,
                             double alpha, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = fma(alpha, p[i], x[i]);
  r[i] = fma(-alpha, Ap[i], r[i]);
}

__global__ void cg_precond_kernel(const double* __restrict__ r, const double* __restrict__ diag,
                                  double* __restrict__ z, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = diag[i];
  z[i] = d > 0.0 ? r[i] / d : r[i];
}

__global__ void cg_p_kernel(double* __restrict__ p, const double* __restrict__ z, double beta,
                            uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = fma(beta, p[i], z[i]);
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

void cg_update_xr(double* x, double* r, const double* p, const double* Ap, double alpha,
                  uint32_t n, cudaStream_t st) {
  cg_xr_kernel<<<nb(n), kOtThreads, 0, st>>>(x, r, p, Ap, alpha, n); count_launch();
}
void cg_precond(const double* r, const double* diag, double* z, uint32_t n, cudaStream_t st) {
  cg_precond_kernel<<<nb(n), kOtThreads, 0, st>>>(r, diag, z, n); count_launch();
}
void cg_update_p(double* p, const double* z, double beta, uint32_t n, cudaStream_t st) {
  cg_p_kernel<<<nb(n), kOtThreads, 0, st>>>(p, z, beta, n); count_launch();
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
// (s, c) pairs added in a fixed order: a Neumaier sum of the s parts, the
// c parts summed alongside.
__device__ __forceinline__ void pair_add(double& s, double& c, double s2, double c2) {
  neu_add(s, c, s2);
  c += c2;
}

// Fixed-order tree over the warp, then over the block's warps: the (s, c)
// pair of the whole block in thread 0 (blockDim.x a multiple of 32, <= 1024).
__device__ __forceinline__ void block_pair(double& s, double& c) {
  __shared__ double ws[32], wc[32];
  const unsigned FULL = 0xFFFFFFFFu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double s2 = __shfl_down_sync(FULL, s, o), c2 = __shfl_down_sync(FULL, c, o);
    if (lane < o) pair_add(s, c, s2, c2);
  }
  __syncthreads();  // ws/wc may still be read by a previous call
  if (lane == 0) {
    ws[warp] = s;
    wc[warp] = c;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    s = lane < nw ? ws[lane] : 0.0;
    c = lane < nw ? wc[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double s2 = __shfl_down_sync(FULL, s, o), c2 = __shfl_down_sync(FULL, c, o);
      if (lane < o) pair_add(s, c, s2, c2);
    }
  }
}

// Sum of the partial pairs part[stride * b + off], b < nparts, the same in
// every block: each lane of warp 0 adds a fixed stretch, then a fixed tree;
// the result is broadcast through shared memory.
__device__ __forceinline__ double sum_parts(const double* __restrict__ part, int nparts,
                                            int stride, int off) {
  __shared__ double res;
  __syncthreads();  // res may still be read after a previous call
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int per = (nparts + 31) / 32;
    double s = 0.0, c = 0.0;
    for (int b = lane * per; b < min(nparts, (lane + 1) * per); ++b)
      pair_add(s, c, part[stride * b + off], part[stride * b + off + 1]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double s2 = __shfl_down_sync(0xFFFFFFFFu, s, o);
      const double c2 = __shfl_down_sync(0xFFFFFFFFu, c, o);
      if (lane < o) pair_add(s, c, s2, c2);
    }
    if (lane == 0) res = s + c;
  }
  __syncthreads();
  return res;
}

// Ap = H p, partial pairs of p . Ap to part[2 b]; 8 lanes per row.
__global__ void __launch_bounds__(kOtThreads)
pcg_spmv_kernel(const uint32_t* __restrict__ rowptr, const uint32_t* __restrict__ col,
                const double* __restrict__ val, const double* __restrict__ diag,
                const double* __restrict__ x, uint32_t n, double* __restrict__ y,
                double* __restrict__ part, const CgScalars* __restrict__ sc) {
  if (sc->done) return;
  const int sub = threadIdx.x & (kRowLanes - 1);
  const unsigned FULL = 0xFFFFFFFFu;
  double s = 0.0, cc = 0.0;
  const uint32_t rows_per_block = kOtThreads / kRowLanes;
  const uint32_t nblk = (n + rows_per_block - 1) / rows_per_block;
  const uint32_t per = (nblk + gridDim.x - 1) / gridDim.x;  // contiguous row blocks
  for (uint32_t rb = blockIdx.x * per; rb < min(nblk, (blockIdx.x + 1) * per); ++rb) {
    const uint32_t i = rb * rows_per_block + threadIdx.x / kRowLanes;
    double acc = 0.0;
    if (i < n)
      for (uint32_t k = rowptr[i] + sub; k < rowptr[i + 1]; k += kRowLanes) acc += val[k] * x[col[k]];
#pragma unroll
    for (int o = kRowLanes / 2; o > 0; o >>= 1) acc += __shfl_down_sync(FULL, acc, o, kRowLanes);
    if (sub == 0 && i < n) {
      const double yi = diag[i] * x[i] + acc;
      y[i] = yi;
      neu_add(s, cc, x[i] * yi);
    }
  }
  block_pair(s, cc);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s;
    part[2 * blockIdx.x + 1] = cc;
  }
}

// alpha = rz / pAp; x += alpha p; r -= alpha Ap; z = r / diag; partial
// pairs of r . r and r . z to part_b[4 b .. 4 b + 3].
__global__ void __launch_bounds__(kOtThreads)
pcg_xr_kernel(const double* __restrict__ part_a, double* __restrict__ x, double* __restrict__ r,
              const double* __restrict__ p, const double* __restrict__ Ap,
              const double* __restrict__ diag, double* __restrict__ z, uint32_t n,
              double* __restrict__ part_b, CgScalars* __restrict__ sc, uint32_t k) {
  if (sc->done) return;
  const double pAp = sum_parts(part_a, gridDim.x, 2, 0);
  if (!(pAp > 0.0)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->done = 1;
    return;
  }
  const double alpha = sc->rz[k & 1] / pAp;
  const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  double s1 = 0.0, c1 = 0.0, s2 = 0.0, c2 = 0.0;
  for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    const double d = diag[i];
    const double zi = d > 0.0 ? ri / d : ri;
    z[i] = zi;
    neu_add(s1, c1, ri * ri);
    neu_add(s2, c2, ri * zi);
  }
  block_pair(s1, c1);
  block_pair(s2, c2);
  if (threadIdx.x == 0) {
    part_b[4 * blockIdx.x] = s1;
    part_b[4 * blockIdx.x + 1] = c1;
    part_b[4 * blockIdx.x + 2] = s2;
    part_b[4 * blockIdx.x + 3] = c2;
  }
}

// beta = rz' / rz; p = z + beta p; block 0 records rz', the iteration and
// convergence.
__global__ void __launch_bounds__(kOtThreads)
pcg_p_kernel(const double* __restrict__ part_b, double* __restrict__ p,
             const double* __restrict__ z, uint32_t n, CgScalars* __restrict__ sc, uint32_t k) {
  if (sc->done) return;
  const double rr = sum_parts(part_b, gridDim.x, 4, 0);
  const double rz_new = sum_parts(part_b, gridDim.x, 4, 2);
  const double beta = rz_new / sc->rz[k & 1];
  const uint32_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) p[i] = fma(beta, p[i], z[i]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rz[(k + 1) & 1] = rz_new;
    sc->k = k + 1;
    if (rr <= sc->tol2 * sc->b2) sc->done = 1;
  }
}

void pcg_iterations(const Hessian& H, double* x, double* r, double* p, double* Ap, double* z,
                    double* part_a, double* part_b, CgScalars* sc, uint32_t k0, uint32_t count,
                    cudaStream_t st) {
  for (uint32_t j = 0; j < count; ++j) {
    pcg_spmv_kernel<<<kPcgParts, kOtThreads, 0, st>>>(H.rowptr, H.col, H.val, H.diag, p, H.n,
                                                      Ap, part_a, sc); count_launch();
    pcg_xr_kernel<<<kPcgParts, kOtThreads, 0, st>>>(part_a, x, r, p, Ap, H.diag, z, H.n,
                                                    part_b, sc, k0 + j); count_launch();
    pcg_p_kernel<<<kPcgParts, kOtThreads, 0, st>>>(part_b, p, z, H.n, sc, k0 + j); count_launch();
  }
}

}  // namespace gbv
