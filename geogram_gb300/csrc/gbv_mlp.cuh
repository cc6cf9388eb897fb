// Learned warm start for the optimal-transport solver: a small MLP that
// predicts, from each seed's position and the distances to its 16 nearest
// seeds, the Laplacian of its Kantorovich weight on the zero-weight cell
// graph (n (H0 w*)_i); the solver integrates it into starting weights
// (declarations).
//
//   input   x (19): seed xyz, then the 16 nearest distances times n^(1/3),
//           standardised per feature, padded with zeros to 32 columns
//   layers  Z1 = X W1^T + b1, H1 = GELU(Z1)       (128)
//           Z2 = H1 W2^T + b2, H2 = GELU(Z2)      (128)
//           Z3 = H2 W3^T + b3, H3 = GELU(Z3)      (128)
//           y  = H3 . W4 + b4                     (1)
//   output  y * out_std + out_mean
//
// Weights are kept in FP32 (the trained parameters) and used in BF16; the
// products run on the tensor cores (mma.sync m16n8k16, BF16 in, FP32
// accumulate); activations between layers are BF16.  Training minimises
// the mean squared error of y against the standardised target with Adam;
// all reductions are deterministic (fixed partitions, fixed order).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbv {

constexpr int kMlpIn = 19, kMlpInPad = 32, kMlpHid = 128;
// parameter vector (FP32)
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHid * kMlpInPad;
constexpr int kOffW2 = kOffB1 + kMlpHid;
constexpr int kOffB2 = kOffW2 + kMlpHid * kMlpHid;
constexpr int kOffW3 = kOffB2 + kMlpHid;
constexpr int kOffB3 = kOffW3 + kMlpHid * kMlpHid;
constexpr int kOffW4 = kOffB3 + kMlpHid;
constexpr int kOffB4 = kOffW4 + kMlpHid;
constexpr int kMlpParams = kOffB4 + 1;
// normalisation vector: in_mean[19], in_std[19], out_mean, out_std
constexpr int kMlpNorm = 2 * kMlpIn + 2;
// rows per pass (buffers are sized for this many rows)
constexpr uint32_t kMlpChunk = 65536;

typedef __nv_bfloat16 bf16;

// Scratch for kMlpChunk rows (device pointers).
struct MlpBuffers {
  bf16 *xn, *h1, *h2, *h3;     // [rows][32] and [rows][128]
  float *z1, *z2, *z3;         // pre-activations [rows][128]
  float* acc;                  // GEMM output [rows][128]
  float *y, *dy;               // [rows]
  float* dz;                   // [rows][128]
  bf16 *dzb, *dzt, *ht;        // [rows][128], [128][rows], [128][rows]
  float* part;                 // split-K / column-sum partials
  bf16 *w1b, *w2b, *w3b;       // weights in BF16 [out][in]
  bf16 *w1t, *w2t, *w3t;       // transposed [in][out]
  double* lpart;               // loss partials
};

size_t mlp_part_floats();

// y (normalised output) of rows [0, rows) of the standardised inputs.
void mlp_forward(const float* params, const float* norm, const float* raw, uint32_t rows,
                 const MlpBuffers& B, bool keep, cudaStream_t st);
// Gradient of the mean squared error over `rows` rows; loss partials in
// B.lpart (kMlpLossParts doubles; the loss is their sum).
constexpr int kMlpLossParts = 64;
void mlp_loss_grad(const float* params, const float* norm, const float* raw, const float* target,
                   uint32_t rows, float* grad, const MlpBuffers& B, cudaStream_t st);
void mlp_adam(float* params, float* m, float* v, const float* grad, uint32_t step, float lr,
              float b1, float b2, float eps, cudaStream_t st);
// w[i] = y[i] * out_std + out_mean (FP64).
void mlp_denorm(const float* y, const float* norm, uint32_t rows, double* w, cudaStream_t st);

// C[M x N] (FP32, ldc) = A[M x K] Bt[N x K]^T (BF16, row-major), on the
// tensor cores; K a multiple of 32, lda and ldb multiples of 8.  splits > 1
// cuts K into `splits` ranges of kchunk, written to C + z * c_split.
void gemm_nt(const bf16* A, int lda, const bf16* Bt, int ldb, float* C, int ldc, int M, int N,
             int K, int splits, size_t c_split, cudaStream_t st);

// Raw features [n][19] from the seeds and the squared distances to their
// 17 nearest stored points (self first), both in the caller's order.
void mlp_features(const double* xyz, const double* knn_d2, uint32_t n, float* raw,
                  cudaStream_t st);

}  // namespace gbv
