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

}  // namespace gbv
