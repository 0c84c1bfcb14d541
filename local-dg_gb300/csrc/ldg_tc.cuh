// The sum-factorised volume contraction of the gradient pass,
//   G[e][l][v][q] = sum_r As_l[q_l][r] U[e][v][line_l(q) at r]
// (the element-operator product that the reference evaluates as a dense
// DGEMM, solver.cpp:500), in four arithmetics, to measure whether tensor
// cores pay for it on the mixed-precision path:
//   k_contract_point<N, double>       FP64 FMA chains (the FP64 path)
//   k_contract_point<N, dd>, dot2=0   FP32-pair FMAs renormalised per term
//   k_contract_point<N, dd>, dot2=1   FP32-pair compensated dot product (Acc<dd>)
//   k_contract_tc<5>                  tensor cores, exact integer slices
//
// Tensor-core scheme (the error-free splitting of Ozaki, Ogita, Oishi and
// Rump, "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer.
// Algorithms 59, 2012, with integer slices as in their later work): every
// line of N = 5 values is scaled by a power of two so that its largest
// magnitude is at most 2^9, then cut into three 10-bit signed integer
// slices (X1 + 2^-10 X2 + 2^-20 X3, |Xk| <= 544) that FP16 holds exactly;
// the operator rows are cut the same way on the host.  A slice product
// summed over the K = 5 terms of a line, and all the pairs of one level
// s + t, stay integers below 2^24, so the FP32 accumulation of
// mma.sync.m16n8k8 (f16 in, f32 out) is exact whatever its internal order
// or rounding.  Levels 2..4 (six MMAs per 16 lines) are kept; dropping the
// rest costs ~2^-30 of max|A||x| per line.  The three level sums are
// combined into an FP32 pair and rescaled by the line's power of two.
//
// MMA layout: A (16 x 8, row-major) = 16 lines x their 5 values (K padded
// to 8); B (8 x 8, column-major) = the operator transposed, B[j][i] =
// As[i][j] (N padded to 8); D (16 x 8) = 16 lines x 5 outputs.  Each group
// of 4 lanes holds one line pair, so the per-line power of two is a two-step
// shuffle maximum.  Sets of 16 lines never mix directions, so each set uses
// one direction's operator slices.
#pragma once
#include <cuda_fp16.h>

#include "ldg_kernels.cuh"

namespace ldg {

// Integer slices of the scaled 1-D operators As_l = A / alpha_l:
// As_l = 2^(eA[l] - 9) (S1 + 2^-10 S2 + 2^-20 S3), S[l][k][i*N + j].
struct TcOps {
  float S[3][3][kDevMaxN * kDevMaxN];
  int eA[3];
};

// Host-side slicing of the scaled operators (N = 5).
inline TcOps make_tc_ops(const DevOps& d, int N) {
  TcOps t;
  for (int l = 0; l < 3; ++l) {
    double mx = 0.0;
    for (int i = 0; i < N * N; ++i) mx = std::fmax(mx, std::fabs(d.A[i] * d.ia[l]));
    int e = 0;
    std::frexp(mx, &e);  // mx < 2^e
    t.eA[l] = e;
    for (int i = 0; i < kDevMaxN * kDevMaxN; ++i) {
      double a = i < N * N ? std::ldexp(d.A[i] * d.ia[l], 9 - e) : 0.0;
      for (int k = 0; k < 3; ++k) {
        const double sk = std::nearbyint(a);
        t.S[l][k][i] = (float)sk;
        a = (a - sk) * 1024.0;
      }
    }
  }
  return t;
}

// Modes 0..2: one thread per (element, Gauss point), 15 outputs each.
template <int N, class T>
__global__ void __launch_bounds__(Cfg<N>::T) k_contract_point(const typename Real<T>::S* __restrict__ U,
                                                              typename Real<T>::S* __restrict__ G, int nE,
                                                              const __grid_constant__ OpsT<T> o, int dot2) {
  constexpr int n = Cfg<N>::n, EPC = Cfg<N>::EPC, NT = Cfg<N>::T;
  using R = Real<T>;
  extern __shared__ double smem_raw[];
  T* sU = reinterpret_cast<T*>(smem_raw);
  const long e0 = (long)blockIdx.x * EPC;
  const int ne = (int)min((long)EPC, nE - e0);
  for (int i = threadIdx.x; i < ne * kNS * n; i += NT) sU[i] = R::ld(U + e0 * kNS * n + i);
  __syncthreads();
  const int es = threadIdx.x / n, q = threadIdx.x % n;
  if (es >= ne) return;
  const int c[3] = {q % N, (q / N) % N, q / (N * N)};
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    const int st = stride_of<N>(l);
    const int b = q - c[l] * st;
#pragma unroll
    for (int v = 0; v < kNS; ++v) {
      const T* line = sU + (es * kNS + v) * n + b;
      T g;
      if (dot2) {
        Acc<T> acc;
#pragma unroll
        for (int r = 0; r < N; ++r) acc.add(o.As[l][c[l] * N + r], line[r * st]);
        g = acc.get();
      } else {
        T acc{};
#pragma unroll
        for (int r = 0; r < N; ++r) acc = fma(o.As[l][c[l] * N + r], line[r * st], acc);
        g = acc;
      }
      R::st(G + ((e0 + es) * kNQ + l * kNS + v) * n + q, g);
    }
  }
}

__device__ __forceinline__ unsigned tc_pack(float lo, float hi) {
  __half2 h = __floats2half2_rn(lo, hi);  // integers |x| <= 2048: exact
  return *reinterpret_cast<unsigned*>(&h);
}

__device__ __forceinline__ void tc_mma(float (&d)[4], unsigned a0, unsigned a1, unsigned b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(b0));
}

// 2^e as a float for e in [-126, 127].
__device__ __forceinline__ float tc_pow2(int e) { return __int_as_float((127 + e) << 23); }

// Mode 3: tensor-core slices, N = 5, two elements per CTA, 8 warps.
template <int N>
__global__ void __launch_bounds__(256) k_contract_tc(const float2* __restrict__ U, float2* __restrict__ G, int nE,
                                                     const __grid_constant__ TcOps tc) {
  static_assert(N == 5, "the slice bounds are sized for K = 5");
  constexpr int n = N * N * N, EPC = 2, NT = 256, LINES = EPC * kNS * N * N;  // 250 lines per direction
  constexpr int SETS = (LINES + 15) / 16;
  extern __shared__ double smem_raw[];
  float2* sU = reinterpret_cast<float2*>(smem_raw);  // EPC*5*n
  float2* sG = sU + EPC * kNS * n;                   // EPC*15*n
  const long e0 = (long)blockIdx.x * EPC;
  const int ne = (int)min((long)EPC, nE - e0);
  for (int i = threadIdx.x; i < ne * kNS * n; i += NT) sU[i] = U[e0 * kNS * n + i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const int j0 = 2 * tq, j1 = 2 * tq + 1;
  for (int set = warp; set < 3 * SETS; set += NT / 32) {  // warp-uniform
    const int l = set / SETS, sub = set - l * SETS;
    const int st = stride_of<N>(l);
    unsigned b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      b[k] = tc_pack(g < N && j0 < N ? tc.S[l][k][g * N + j0] : 0.f, g < N && j1 < N ? tc.S[l][k][g * N + j1] : 0.f);
    float X[2][2][3];
    float so[2];
    int lid[2], base[2];
    bool ok[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      lid[h] = sub * 16 + g + 8 * h;
      ok[h] = lid[h] < ne * kNS * N * N;
      const int es = lid[h] / (kNS * N * N), r = lid[h] - es * kNS * N * N;
      const int v = r / (N * N), t = r - v * N * N;
      base[h] = (es * kNS + v) * n + face_point<N>(l, 0, t);
      const float2 x0 = ok[h] && j0 < N ? sU[base[h] + j0 * st] : make_float2(0.f, 0.f);
      const float2 x1 = ok[h] && j1 < N ? sU[base[h] + j1 * st] : make_float2(0.f, 0.f);
      float m = fmaxf(fabsf(x0.x), fabsf(x1.x));
      m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
      m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
      // m < 2^ex; lines below 2^-100 are treated as zero
      const int ex = ((__float_as_int(m) >> 23) & 0xff) - 126;
      const bool live = m > 0x1p-100f;
      const float sc = live ? tc_pow2(9 - ex) : 0.f;
      so[h] = live ? tc_pow2(ex + tc.eA[l] - 18) : 0.f;
      const float2 xs[2] = {x0, x1};
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        const float hh = xs[jj].x * sc, ll = xs[jj].y * sc;
        const float s1 = rintf(hh);
        const float r1 = (hh - s1) * 1024.f;
        const float s2 = rintf(r1);
        const float r2 = __fmaf_rn(ll, 1048576.f, (r1 - s2) * 1024.f);
        X[h][jj][0] = s1;
        X[h][jj][1] = s2;
        X[h][jj][2] = rintf(r2);
      }
    }
    unsigned a0[3], a1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      a0[k] = tc_pack(X[0][0][k], X[0][1][k]);
      a1[k] = tc_pack(X[1][0][k], X[1][1][k]);
    }
    float d2[4] = {0.f, 0.f, 0.f, 0.f}, d3[4] = {0.f, 0.f, 0.f, 0.f}, d4[4] = {0.f, 0.f, 0.f, 0.f};
    tc_mma(d2, a0[0], a1[0], b[0]);
    tc_mma(d3, a0[0], a1[0], b[1]);
    tc_mma(d3, a0[1], a1[1], b[0]);
    tc_mma(d4, a0[0], a1[0], b[2]);
    tc_mma(d4, a0[1], a1[1], b[1]);
    tc_mma(d4, a0[2], a1[2], b[0]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int h = k >> 1, i = 2 * tq + (k & 1);
      if (!ok[h] || i >= N) continue;
      const dd s = dd_two_sum(d2[k], d3[k] * 0x1p-10f);
      const dd w = dd_two_sum(s.h, __fmaf_rn(d4[k], 0x1p-20f, s.l));
      const int es = lid[h] / (kNS * N * N), r = lid[h] - es * kNS * N * N;
      const int v = r / (N * N);
      sG[(es * kNQ + l * kNS + v) * n + base[h] - (es * kNS + v) * n + i * st] =
          make_float2(w.h * so[h], w.l * so[h]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ne * kNQ * n; i += NT) G[e0 * kNQ * n + i] = sG[i];
}

}  // namespace ldg
