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
//
// The CG product reads a sliced-ELL copy (slices of 32 rows, entry k of
// row 32 s + l at sl_off[s] + 32 k + l, rows padded with zeros to the
// longest of their slice): one row per thread with coalesced loads.
struct Hessian {
  const uint32_t* rowptr;  // n + 1
  const uint32_t* col;     // nnz
  double* val;             // nnz (off-diagonal coefficients, <= 0)
  double* diag;            // n (> 0 unless the cell has no seed facet)
  double* invd;            // n: 1 / diag (1 where diag is 0), the preconditioner
  uint32_t n;
  const uint32_t* sl_off = nullptr;  // sell_slices(n) + 1 offsets
  uint32_t* s_col = nullptr;
  double* s_val = nullptr;
};

void assemble_hessian(const double* xyz, const uint32_t* rowptr, const uint32_t* col,
                      const double* area, uint32_t n, Hessian& H, cudaStream_t st);
// The sliced-ELL copy: sell_widths writes 32 x the longest row of each
// slice to sl_off[0 .. sell_slices(n)); an exclusive scan of
// sell_slices(n) + 1 entries turns them into offsets (the last one is the
// entry count); sell_pack fills s_col / s_val of that size.
uint32_t sell_slices(uint32_t n);
void sell_widths(const Hessian& H, uint32_t* sl_off, cudaStream_t st);
void sell_pack(Hessian& H, const uint32_t* sl_off, uint32_t* s_col, double* s_val,
               cudaStream_t st);

// Deterministic FP64 reductions to (s, 0) pairs part[2 b], b < kOtParts,
// added on the host.
constexpr int kOtParts = 256;
void dot_parts(const double* a, const double* b, uint32_t n, double* part, cudaStream_t st);

// r = vol - nu; parts: [0] sum r^2 terms, [1] max |r_i| / nu_i, [2] min vol.
void residual(const double* vol, const double* nu, uint32_t n, double* r, double* part,
              cudaStream_t st);

// z = r * invd (Jacobi), y += alpha x, y += c, y = alpha x.
void cg_precond(const double* r, const double* invd, double* z, uint32_t n, cudaStream_t st);
void axpy(double* y, const double* x, double alpha, uint32_t n, cudaStream_t st);
void add_scalar(double* y, double c, uint32_t n, cudaStream_t st);
void scale_copy(double* y, const double* x, double alpha, uint32_t n, cudaStream_t st);

// Preconditioned CG iterations with every scalar on the device: the host
// launches `count` iterations without waiting and reads k and done
// afterwards.  Iteration: Ap = H p and p . Ap, alpha = rz / pAp, x +=
// alpha p, r -= alpha Ap, z = r / diag, rr = r . r, rz' = r . z, beta =
// rz' / rz, p = z + beta p; done once rr <= tol2 * b2 (or pAp <= 0).  Each
// reduction is finished once, by the last block of its launch, from
// partials of a fixed partition in a fixed order: the run is deterministic.
struct CgScalars {
  double rz;     // r . z of the current iterate (set by the host first)
  double alpha;
  double beta;
  double b2;     // squared norm of the right-hand side
  double tol2;   // squared relative tolerance
  uint32_t k;    // iterations done
  uint32_t done;
  uint32_t ticket;  // blocks finished in the current launch (0 between launches)
  uint32_t pad;
};
constexpr int kPcgParts = 8 * 152;  // at most this many blocks (8 per SM)
uint32_t pcg_blocks(uint32_t n);
// part: 2 * kPcgParts doubles
void pcg_iterations(const Hessian& H, double* x, double* r, double* p, double* Ap, double* z,
                    double* part, CgScalars* sc, uint32_t count, cudaStream_t st);

}  // namespace gbv
