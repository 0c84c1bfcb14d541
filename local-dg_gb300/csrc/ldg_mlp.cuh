// BF16 multilayer-perceptron kernels of the learned closure: tensor-core
// GEMM (BF16 operands, FP32 accumulation), bias + GELU forward/backward,
// loss gradient, Adam.  All hand-written; no library GEMM.
//
// GEMM: C[M x N] (fp32) = op(A)[M x K] * op(B)[K x N] (+ C if accumulate),
// A and B bf16 addressed by (row stride, column stride), so transposed
// operands of the backward pass need no copies.  CTA tile 64 x 64 x 32,
// four warps each owning a 32 x 32 block of m16n8k16 MMA tiles
// (mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32; fragment layout as
// in the PTX ISA's description of that shape).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace ldg {
namespace mlp {

struct Mat {  // bf16 matrix view: element (i, j) at p[i*rs + j*cs]
  const __nv_bfloat16* p;
  long rs, cs;
};

constexpr int kTM = 64, kTN = 64, kTK = 32;

__device__ __forceinline__ unsigned pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], const unsigned b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C = A B (+ C).  grid (ceil(N/64), ceil(M/64)), 128 threads.
__global__ void __launch_bounds__(128) k_gemm_bf16(Mat A, Mat B, float* __restrict__ C, long ldc, int M, int N,
                                                   int K, int accumulate) {
  __shared__ __nv_bfloat16 sA[kTM][kTK + 8];  // row-major M x K tile (padded)
  __shared__ __nv_bfloat16 sB[kTN][kTK + 8];  // N x K tile: B transposed (col operand)
  const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  for (int k0 = 0; k0 < K; k0 += kTK) {
    for (int i = threadIdx.x; i < kTM * kTK; i += 128) {
      const int r = i / kTK, k = i % kTK;
      const int gm = m0 + r, gk = k0 + k;
      sA[r][k] = (gm < M && gk < K) ? A.p[gm * A.rs + gk * A.cs] : zero;
    }
    for (int i = threadIdx.x; i < kTN * kTK; i += 128) {
      const int c = i / kTK, k = i % kTK;
      const int gn = n0 + c, gk = k0 + k;
      sB[c][k] = (gn < N && gk < K) ? B.p[gk * B.rs + gn * B.cs] : zero;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTK; kk += 16) {
      unsigned af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + i * 16 + g;
        af[i][0] = pack2(sA[r][kk + tq * 2], sA[r][kk + tq * 2 + 1]);
        af[i][1] = pack2(sA[r + 8][kk + tq * 2], sA[r + 8][kk + tq * 2 + 1]);
        af[i][2] = pack2(sA[r][kk + tq * 2 + 8], sA[r][kk + tq * 2 + 9]);
        af[i][3] = pack2(sA[r + 8][kk + tq * 2 + 8], sA[r + 8][kk + tq * 2 + 9]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + j * 8 + g;
        bf[j][0] = pack2(sB[c][kk + tq * 2], sB[c][kk + tq * 2 + 1]);
        bf[j][1] = pack2(sB[c][kk + tq * 2 + 8], sB[c][kk + tq * 2 + 9]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int row = m0 + wm + i * 16 + g + (r >> 1) * 8;
        const int col = n0 + wn + j * 8 + tq * 2 + (r & 1);
        if (row < M && col < N) {
          float* dst = C + row * ldc + col;
          *dst = accumulate ? *dst + acc[i][j][r] : acc[i][j][r];
        }
      }
}

// GELU(x) = x * Phi(x) (exact, erf form) and its derivative.
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// Z += b (row broadcast); H = bf16(GELU(Z)) if act, else bf16(Z).
__global__ void k_bias_act(float* __restrict__ Z, const float* __restrict__ b, __nv_bfloat16* __restrict__ H,
                           long rows, int cols, int act) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const float z = Z[i] + b[i % cols];
  Z[i] = z;
  if (H) H[i] = __float2bfloat16(act ? gelu(z) : z);
}

// dZ = dH * GELU'(Z), as bf16 for the next GEMMs (and fp32 for the bias).
__global__ void k_gelu_back(const float* __restrict__ dH, const float* __restrict__ Z, float* __restrict__ dZ,
                            __nv_bfloat16* __restrict__ dZb, long count) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float d = dH[i] * gelu_grad(Z[i]);
  dZ[i] = d;
  dZb[i] = __float2bfloat16(d);
}

// Column sums of an fp32 rows x cols matrix (bias gradients); fixed order.
__global__ void k_colsum(const float* __restrict__ X, long rows, int cols, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (long r = 0; r < rows; ++r) s += X[r * cols + c];
  out[c] = s;
}

// Mean-squared-error gradient: dY = 2 (Y - T) / count (also bf16); per-row
// partial losses for a deterministic sum.
__global__ void k_mse_grad(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY,
                           __nv_bfloat16* __restrict__ dYb, long rows, int cols, float* __restrict__ row_loss) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const float inv = 1.f / (float)(rows * cols);
  float s = 0.f;
  for (int c = 0; c < cols; ++c) {
    const float d = Y[r * cols + c] - T[r * cols + c];
    s += d * d;
    dY[r * cols + c] = 2.f * d * inv;
    dYb[r * cols + c] = __float2bfloat16(2.f * d * inv);
  }
  row_loss[r] = s * inv;
}

// Adam (Kingma & Ba, ICLR 2015) on fp32 master parameters; refreshes the
// bf16 copies (w) and the bf16 transposed copies (wt, optional) used by the
// GEMMs.  Parameter i of a rows x cols weight block lives at w[i].
__global__ void k_adam(float* __restrict__ theta, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt,
                       int rows, int cols, long count, float lr, float b1, float b2, float eps, float c1, float c2) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float t = theta[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  theta[i] = t;
  if (w) w[i] = __float2bfloat16(t);
  if (wt) {
    const long r = i / cols, c = i % cols;
    wt[c * rows + r] = __float2bfloat16(t);
  }
}

}  // namespace mlp
}  // namespace ldg
