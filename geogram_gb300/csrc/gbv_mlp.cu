// Learned warm start: tensor-core MLP forward and backward, Adam, and the
// seed features.  See gbv_mlp.cuh for the network.
//
// The matrix products are one kernel, C = A Bt^T with both operands
// K-contiguous BF16 ("NT"): forward Z = H W^T, backward dH = dZ W (Bt =
// W^T) and dW = dZ^T H (A = dZ^T, Bt = H^T, K = the batch, split over
// CTAs and reduced in a fixed order).  A CTA of four warps computes a
// 64 x 64 tile; each warp a 32 x 32 block with mma.sync.m16n8k16 (BF16
// inputs, FP32 accumulation), operands staged through padded shared
// memory rows (80 bytes: the fragment loads of a warp hit 32 distinct
// banks).
#include <cfloat>

#include "gbv_common.cuh"
#include "gbv_mlp.cuh"

namespace gbv {

namespace {

constexpr int kBM = 64, kBN = 64, kBK = 32, kPad = 8;
constexpr int kMaxSplits = 64;

__device__ __forceinline__ uint32_t ld_pair(const bf16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4],
                                          const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(128) gemm_nt_kernel(const bf16* __restrict__ A, int lda,
                                                      const bf16* __restrict__ Bt, int ldb,
                                                      float* __restrict__ C, int ldc,
                                                      size_t c_split, int M, int N, int K,
                                                      int kchunk) {
  __shared__ __align__(16) bf16 As[kBM][kBK + kPad];
  __shared__ __align__(16) bf16 Bs[kBN][kBK + kPad];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int k_begin = blockIdx.z * kchunk, k_end = min(K, k_begin + kchunk);
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  for (int k0 = k_begin; k0 < k_end; k0 += kBK) {
    // 64 rows x 32 columns per operand: 256 chunks of 8 BF16, two per thread
    for (int c = tid; c < 256; c += 128) {
      const int r = c >> 2, q = (c & 3) * 8;
      uint4 va = make_uint4(0u, 0u, 0u, 0u), vb = make_uint4(0u, 0u, 0u, 0u);
      if (m0 + r < M) va = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * lda + k0 + q);
      if (n0 + r < N) vb = *reinterpret_cast<const uint4*>(Bt + (size_t)(n0 + r) * ldb + k0 + q);
      *reinterpret_cast<uint4*>(&As[r][q]) = va;
      *reinterpret_cast<uint4*>(&Bs[r][q]) = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t af[2][4], bfg[4][2];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
        const int r = wm + mi * 16 + g;
        af[mi][0] = ld_pair(&As[r][kk + 2 * t]);
        af[mi][1] = ld_pair(&As[r + 8][kk + 2 * t]);
        af[mi][2] = ld_pair(&As[r][kk + 2 * t + 8]);
        af[mi][3] = ld_pair(&As[r + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        const int cidx = wn + ni * 8 + g;
        bfg[ni][0] = ld_pair(&Bs[cidx][kk + 2 * t]);
        bfg[ni][1] = ld_pair(&Bs[cidx][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) mma_16816(acc[mi][ni], af[mi], bfg[ni]);
    }
    __syncthreads();
  }
  float* Cz = C + blockIdx.z * c_split;
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni) {
      const int r = m0 + wm + mi * 16 + g;
      const int col = n0 + wn + ni * 8 + 2 * t;
      if (r < M) {
        if (col < N) Cz[(size_t)r * ldc + col] = acc[mi][ni][0];
        if (col + 1 < N) Cz[(size_t)r * ldc + col + 1] = acc[mi][ni][1];
      }
      if (r + 8 < M) {
        if (col < N) Cz[(size_t)(r + 8) * ldc + col] = acc[mi][ni][2];
        if (col + 1 < N) Cz[(size_t)(r + 8) * ldc + col + 1] = acc[mi][ni][3];
      }
    }
}

__device__ __forceinline__ float gelu(float z) {
  return 0.5f * z * (1.f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) +
         z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__global__ void weights_bf16_kernel(const float* __restrict__ p, bf16* __restrict__ w1b,
                                    bf16* __restrict__ w2b, bf16* __restrict__ w3b,
                                    bf16* __restrict__ w1t, bf16* __restrict__ w2t,
                                    bf16* __restrict__ w3t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kMlpHid * kMlpInPad) {
    const int o = i / kMlpInPad, k = i % kMlpInPad;
    const bf16 v = __float2bfloat16_rn(p[kOffW1 + i]);
    w1b[i] = v;
    w1t[k * kMlpHid + o] = v;
  }
  if (i < kMlpHid * kMlpHid) {
    const int o = i / kMlpHid, k = i % kMlpHid;
    const bf16 v2 = __float2bfloat16_rn(p[kOffW2 + i]);
    const bf16 v3 = __float2bfloat16_rn(p[kOffW3 + i]);
    w2b[i] = v2;
    w3b[i] = v3;
    w2t[k * kMlpHid + o] = v2;
    w3t[k * kMlpHid + o] = v3;
  }
}

__global__ void prep_input_kernel(const float* __restrict__ raw, const float* __restrict__ norm,
                                  uint32_t rows, bf16* __restrict__ xn) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * kMlpInPad) return;
  const uint32_t r = i / kMlpInPad, k = i % kMlpInPad;
  float v = 0.f;
  if (k < (uint32_t)kMlpIn) v = (raw[(size_t)r * kMlpIn + k] - norm[k]) / norm[kMlpIn + k];
  xn[i] = __float2bfloat16_rn(v);
}

__global__ void bias_gelu_kernel(const float* __restrict__ acc, const float* __restrict__ bias,
                                 uint32_t rows, float* __restrict__ z, bf16* __restrict__ h) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * kMlpHid) return;
  const float v = acc[i] + bias[i % kMlpHid];
  if (z) z[i] = v;
  h[i] = __float2bfloat16_rn(gelu(v));
}

// y[r] = H3[r] . W4 + b4, one warp per row, fixed lane order.
__global__ void out_kernel(const bf16* __restrict__ h3, const float* __restrict__ p, uint32_t rows,
                           float* __restrict__ y) {
  const uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int k = lane * 4 + q;
    s = fmaf(__bfloat162float(h3[(size_t)r * kMlpHid + k]), p[kOffW4 + k], s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
  if (lane == 0) y[r] = s + p[kOffB4];
}

__global__ void loss_kernel(const float* __restrict__ y, const float* __restrict__ target,
                            const float* __restrict__ norm, uint32_t rows, float* __restrict__ dy,
                            double* __restrict__ lpart) {
  __shared__ double sm[256];
  const float mean = norm[2 * kMlpIn], sd = norm[2 * kMlpIn + 1];
  double s = 0.0;
  const uint32_t chunk = (rows + gridDim.x - 1) / gridDim.x;
  const uint32_t lo = blockIdx.x * chunk, hi = min(rows, lo + chunk);
  for (uint32_t r = lo + threadIdx.x; r < hi; r += blockDim.x) {
    const float e = y[r] - (target[r] - mean) / sd;
    dy[r] = 2.f * e / (float)rows;
    s += (double)e * (double)e / (double)rows;
  }
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) lpart[blockIdx.x] = sm[0];
}

// dZ3 = dy W4 GELU'(Z3)
__global__ void dlast_kernel(const float* __restrict__ dy, const float* __restrict__ p,
                             const float* __restrict__ z3, uint32_t rows, float* __restrict__ dz,
                             bf16* __restrict__ dzb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * kMlpHid) return;
  const float v = dy[i / kMlpHid] * p[kOffW4 + i % kMlpHid] * gelu_grad(z3[i]);
  dz[i] = v;
  dzb[i] = __float2bfloat16_rn(v);
}

// dZ = dH GELU'(Z)
__global__ void gelu_bwd_kernel(const float* __restrict__ dh, const float* __restrict__ z,
                                uint32_t rows, float* __restrict__ dz, bf16* __restrict__ dzb) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * kMlpHid) return;
  const float v = dh[i] * gelu_grad(z[i]);
  dz[i] = v;
  dzb[i] = __float2bfloat16_rn(v);
}

// Column sums of M[rows][ncols] (times rowscale[r] when given): partial
// sums over fixed row ranges, then the ranges added in order.
template <typename T>
__global__ void colsum_part_kernel(const T* __restrict__ M, int ld, const float* __restrict__ scale,
                                   uint32_t rows, int ncols, int nparts, float* __restrict__ part) {
  const int c = threadIdx.x;
  const int pidx = blockIdx.x;
  if (c >= ncols) return;
  const uint32_t chunk = (rows + nparts - 1) / nparts;
  const uint32_t lo = pidx * chunk, hi = min(rows, lo + chunk);
  float s = 0.f;
  for (uint32_t r = lo; r < hi; ++r) {
    float v;
    if constexpr (sizeof(T) == 2) v = __bfloat162float(M[(size_t)r * ld + c]);
    else v = M[(size_t)r * ld + c];
    s += scale ? v * scale[r] : v;
  }
  part[pidx * ncols + c] = s;
}

__global__ void sum_parts_kernel(const float* __restrict__ part, int nparts, int n,
                                 size_t stride, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.f;
  for (int q = 0; q < nparts; ++q) s += part[q * stride + i];
  out[i] = s;
}

// out[c][r] = in[r][c] for c < ncols, r < rows_pad (zero for r >= rows)
__global__ void transpose_kernel(const bf16* __restrict__ in, int ld_in, uint32_t rows,
                                 uint32_t rows_pad, int ncols, bf16* __restrict__ out) {
  __shared__ bf16 tile[32][33];
  const uint32_t r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int k = ty; k < 32; k += 8) {
    const uint32_t r = r0 + k, c = c0 + tx;
    tile[k][tx] = (r < rows && c < (uint32_t)ncols) ? in[(size_t)r * ld_in + c]
                                                    : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const uint32_t c = c0 + k, r = r0 + tx;
    if (c < (uint32_t)ncols && r < rows_pad) out[(size_t)c * rows_pad + r] = tile[tx][k];
  }
}

__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, int n, float lr_t, float b1, float b2,
                            float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr_t * mi / (sqrtf(vi) + eps);
}

__global__ void denorm_kernel(const float* __restrict__ y, const float* __restrict__ norm,
                              uint32_t rows, double* __restrict__ w) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < rows) w[i] = (double)y[i] * (double)norm[2 * kMlpIn + 1] + (double)norm[2 * kMlpIn];
}

__global__ void features_kernel(const double* __restrict__ xyz, const double* __restrict__ d2,
                                uint32_t n, float scale, float* __restrict__ raw) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* o = raw + (size_t)i * kMlpIn;
  o[0] = (float)xyz[3 * (size_t)i];
  o[1] = (float)xyz[3 * (size_t)i + 1];
  o[2] = (float)xyz[3 * (size_t)i + 2];
  for (int m = 0; m < 16; ++m) o[3 + m] = (float)sqrt(d2[(size_t)i * 17 + 1 + m]) * scale;
}

inline unsigned nb(size_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void colsum(const float* M, int ld, const float* scale, uint32_t rows, int ncols, float* out,
            float* part, cudaStream_t st) {
  const int nparts = 64;
  colsum_part_kernel<float><<<nparts, 128, 0, st>>>(M, ld, scale, rows, ncols, nparts, part);
  count_launch();
  sum_parts_kernel<<<1, 128, 0, st>>>(part, nparts, ncols, (size_t)ncols, out);
  count_launch();
}
void colsum_bf16(const bf16* M, int ld, const float* scale, uint32_t rows, int ncols, float* out,
                 float* part, cudaStream_t st) {
  const int nparts = 64;
  colsum_part_kernel<bf16><<<nparts, 128, 0, st>>>(M, ld, scale, rows, ncols, nparts, part);
  count_launch();
  sum_parts_kernel<<<1, 128, 0, st>>>(part, nparts, ncols, (size_t)ncols, out);
  count_launch();
}

void transpose(const bf16* in, int ld_in, uint32_t rows, uint32_t rows_pad, int ncols, bf16* out,
               cudaStream_t st) {
  dim3 grid(nb(rows_pad, 32), nb(ncols, 32));
  transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(in, ld_in, rows, rows_pad, ncols, out);
  count_launch();
}

// dW[M x N] = dZ^T X over the batch (K = rows_pad), split over CTAs and
// reduced in order into out.
void weight_grad(const bf16* dzt, const bf16* xt, uint32_t rows_pad, int M, int N, float* out,
                 float* part, cudaStream_t st) {
  int splits = (int)std::min<uint32_t>(kMaxSplits, std::max<uint32_t>(1, rows_pad / 512));
  const int kchunk = (int)(((rows_pad + splits - 1) / splits + kBK - 1) / kBK * kBK);
  splits = (int)((rows_pad + kchunk - 1) / kchunk);
  gemm_nt(dzt, (int)rows_pad, xt, (int)rows_pad, part, N, M, N, (int)rows_pad, splits,
          (size_t)M * N, st);
  sum_parts_kernel<<<nb((size_t)M * N, 256), 256, 0, st>>>(part, splits, M * N, (size_t)M * N,
                                                           out);
  count_launch();
}

}  // namespace

size_t mlp_part_floats() { return (size_t)kMaxSplits * kMlpHid * kMlpHid; }

void gemm_nt(const bf16* A, int lda, const bf16* Bt, int ldb, float* C, int ldc, int M, int N,
             int K, int splits, size_t c_split, cudaStream_t st) {
  const int kchunk = splits > 1 ? (((K + splits - 1) / splits + kBK - 1) / kBK * kBK) : K;
  dim3 grid(nb(N, kBN), nb(M, kBM), splits);
  gemm_nt_kernel<<<grid, 128, 0, st>>>(A, lda, Bt, ldb, C, ldc, c_split, M, N, K, kchunk);
  count_launch();
}

void mlp_forward(const float* params, const float* norm, const float* raw, uint32_t rows,
                 const MlpBuffers& B, bool keep, cudaStream_t st) {
  weights_bf16_kernel<<<nb(kMlpHid * kMlpHid, 256), 256, 0, st>>>(params, B.w1b, B.w2b, B.w3b,
                                                                  B.w1t, B.w2t, B.w3t);
  count_launch();
  prep_input_kernel<<<nb((size_t)rows * kMlpInPad, 256), 256, 0, st>>>(raw, norm, rows, B.xn);
  count_launch();
  const size_t ne = (size_t)rows * kMlpHid;
  gemm_nt(B.xn, kMlpInPad, B.w1b, kMlpInPad, B.acc, kMlpHid, rows, kMlpHid, kMlpInPad, 1, 0, st);
  bias_gelu_kernel<<<nb(ne, 256), 256, 0, st>>>(B.acc, params + kOffB1, rows, keep ? B.z1 : nullptr,
                                               B.h1);
  count_launch();
  gemm_nt(B.h1, kMlpHid, B.w2b, kMlpHid, B.acc, kMlpHid, rows, kMlpHid, kMlpHid, 1, 0, st);
  bias_gelu_kernel<<<nb(ne, 256), 256, 0, st>>>(B.acc, params + kOffB2, rows, keep ? B.z2 : nullptr,
                                               B.h2);
  count_launch();
  gemm_nt(B.h2, kMlpHid, B.w3b, kMlpHid, B.acc, kMlpHid, rows, kMlpHid, kMlpHid, 1, 0, st);
  bias_gelu_kernel<<<nb(ne, 256), 256, 0, st>>>(B.acc, params + kOffB3, rows, keep ? B.z3 : nullptr,
                                               B.h3);
  count_launch();
  out_kernel<<<nb((size_t)rows * 32, 256), 256, 0, st>>>(B.h3, params, rows, B.y);
  count_launch();
}

void mlp_loss_grad(const float* params, const float* norm, const float* raw, const float* target,
                   uint32_t rows, float* grad, const MlpBuffers& B, cudaStream_t st) {
  mlp_forward(params, norm, raw, rows, B, true, st);
  loss_kernel<<<kMlpLossParts, 256, 0, st>>>(B.y, target, norm, rows, B.dy, B.lpart);
  count_launch();
  const uint32_t rows_pad = (rows + 31) / 32 * 32;
  const size_t ne = (size_t)rows * kMlpHid;
  // output layer
  colsum_bf16(B.h3, kMlpHid, B.dy, rows, kMlpHid, grad + kOffW4, B.part, st);
  colsum(B.dy, 1, nullptr, rows, 1, grad + kOffB4, B.part, st);
  dlast_kernel<<<nb(ne, 256), 256, 0, st>>>(B.dy, params, B.z3, rows, B.dz, B.dzb);
  count_launch();
  // layer 3
  colsum(B.dz, kMlpHid, nullptr, rows, kMlpHid, grad + kOffB3, B.part, st);
  transpose(B.dzb, kMlpHid, rows, rows_pad, kMlpHid, B.dzt, st);
  transpose(B.h2, kMlpHid, rows, rows_pad, kMlpHid, B.ht, st);
  weight_grad(B.dzt, B.ht, rows_pad, kMlpHid, kMlpHid, grad + kOffW3, B.part, st);
  gemm_nt(B.dzb, kMlpHid, B.w3t, kMlpHid, B.acc, kMlpHid, rows, kMlpHid, kMlpHid, 1, 0, st);
  gelu_bwd_kernel<<<nb(ne, 256), 256, 0, st>>>(B.acc, B.z2, rows, B.dz, B.dzb);
  count_launch();
  // layer 2
  colsum(B.dz, kMlpHid, nullptr, rows, kMlpHid, grad + kOffB2, B.part, st);
  transpose(B.dzb, kMlpHid, rows, rows_pad, kMlpHid, B.dzt, st);
  transpose(B.h1, kMlpHid, rows, rows_pad, kMlpHid, B.ht, st);
  weight_grad(B.dzt, B.ht, rows_pad, kMlpHid, kMlpHid, grad + kOffW2, B.part, st);
  gemm_nt(B.dzb, kMlpHid, B.w2t, kMlpHid, B.acc, kMlpHid, rows, kMlpHid, kMlpHid, 1, 0, st);
  gelu_bwd_kernel<<<nb(ne, 256), 256, 0, st>>>(B.acc, B.z1, rows, B.dz, B.dzb);
  count_launch();
  // layer 1 (the padded input columns are zero, so are their gradients)
  colsum(B.dz, kMlpHid, nullptr, rows, kMlpHid, grad + kOffB1, B.part, st);
  transpose(B.dzb, kMlpHid, rows, rows_pad, kMlpHid, B.dzt, st);
  transpose(B.xn, kMlpInPad, rows, rows_pad, kMlpInPad, B.ht, st);
  weight_grad(B.dzt, B.ht, rows_pad, kMlpHid, kMlpInPad, grad + kOffW1, B.part, st);
}

void mlp_adam(float* params, float* m, float* v, const float* grad, uint32_t step, float lr,
              float b1, float b2, float eps, cudaStream_t st) {
  const double c1 = 1.0 - std::pow((double)b1, (double)step);
  const double c2 = 1.0 - std::pow((double)b2, (double)step);
  const float lr_t = (float)(lr * std::sqrt(c2) / c1);
  adam_kernel<<<nb(kMlpParams, 256), 256, 0, st>>>(params, m, v, grad, kMlpParams, lr_t, b1, b2,
                                                  eps);
  count_launch();
}

void mlp_denorm(const float* y, const float* norm, uint32_t rows, double* w, cudaStream_t st) {
  denorm_kernel<<<nb(rows, 256), 256, 0, st>>>(y, norm, rows, w);
  count_launch();
}

void mlp_features(const double* xyz, const double* knn_d2, uint32_t n, float* raw,
                  cudaStream_t st) {
  features_kernel<<<nb(n, 256), 256, 0, st>>>(xyz, knn_d2, n, (float)std::cbrt((double)n), raw);
  count_launch();
}

}  // namespace gbv
