// Semi-discrete optimal transport: Hessian assembly, FP64 conjugate
// gradient and the Newton residual (declarations).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbv {

// Laplacian-form Hessian of the Kantorovich dual, in the caller's seed
// order, with the cells' CSR adjacency as its sparsity pattern:
// H_ij = -A_ij / (2 |p_i - p_j|) (A_ij the shared facet area, averaged over
// the two sides so that H is exactly symmetric), H_ii = -sum_j H_ij.
// Entries whose transposed facet is missing (degenerate facets seen from
// one side only) are dropped from both rows.
struct Hessian {
  const uint32_t* rowptr;  // n + 1
  const uint32_t* col;     // nnz
  double* val;             // nnz (off-diagonal coefficients, <= 0)
  double* diag;            // n (> 0 unless the cell has no seed facet)
  uint32_t n;
};

void assemble_hessian(const double* xyz, const uint32_t* rowptr, const uint32_t* col,
                      const double* area, uint32_t n, Hessian& H, cudaStream_t st);

// y = H x and, into part[block], the partial sums of x . y.
void spmv_dot(const Hessian& H, const double* x, double* y, double* part, int nparts,
              cudaStream_t st);

// Deterministic FP64 reductions to part[0..nparts) (Neumaier sums per block);
// also the grid of the SpMV.  256 blocks: a grid of 8 blocks per SM made the
// dot products twice as slow (their per-block FP64 reduction is serial) and
// did not speed up the SpMV.
constexpr int kOtParts = 256;
void dot_parts(const double* a, const double* b, uint32_t n, double* part, cudaStream_t st);

// r = vol - nu; parts: [0] sum r^2 terms, [1] max |r_i| / nu_i, [2] min vol.
void residual(const double* vol, const double* nu, uint32_t n, double* r, double* part,
              cudaStream_t st);

// Element-wise steps of preconditioned CG (Jacobi).
void cg_update_xr(double* x, double* r, const double* p, const double* Ap, double alpha,
                  uint32_t n, cudaStream_t st);
void cg_precond(const double* r, const double* diag, double* z, uint32_t n, cudaStream_t st);
void cg_update_p(double* p, const double* z, double beta, uint32_t n, cudaStream_t st);
void axpy(double* y, const double* x, double alpha, uint32_t n, cudaStream_t st);

// Preconditioned CG iterations with every scalar on the device: the host
// launches `count` iterations (numbered k0, k0 + 1, ...) without waiting,
// and reads k and done afterwards.  Iteration k: Ap = H p and p . Ap
// (per-block Neumaier partials), alpha = rz / pAp, x += alpha p,
// r -= alpha Ap, z = r / diag, then rr = r . r and rz' = r . z, p = z +
// (rz' / rz) p; done once rr <= tol2 * b2 (or pAp <= 0).  Every block
// combines the same partials in the same order, so the run is
// deterministic; rz alternates between two slots so that no block reads a
// value another block of the same launch is writing.
struct CgScalars {
  double rz[2];
  double b2;     // squared norm of the right-hand side
  double tol2;   // squared relative tolerance
  uint32_t k;    // iterations done
  uint32_t done;
};
constexpr int kPcgParts = 8 * 152;  // blocks of the CG kernels (8 per SM)
void pcg_iterations(const Hessian& H, double* x, double* r, double* p, double* Ap, double* z,
                    double* part_a, double* part_b, CgScalars* sc, uint32_t k0, uint32_t count,
                    cudaStream_t st);
void add_scalar(double* y, double c, uint32_t n, cudaStream_t st);
void scale_copy(double* y, const double* x, double alpha, uint32_t n, cudaStream_t st);

}  // namespace gbv
