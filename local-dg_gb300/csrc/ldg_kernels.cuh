// LDG kernels, templated on N = p + 1 and on the arithmetic type T
// (double: the FP64 path; dd: FP32-pair arithmetic of the mixed path).
//
// State layout in HBM ("Gauss space"): U[e][var][q], q = qx + N qy + N^2 qz,
// the values of the element's polynomial at the tensor Gauss points.  This
// is the reference's polynomial space and quadrature (solver.cpp:74-192)
// written in the Lagrange basis at the Gauss points instead of at the CGL
// nodes, so Interp3D becomes the identity and the mass matrix becomes
// J * diag(w) (it is exact in both bases).  The conversions to and from the
// reference's nodal layout are k_transform below.
//
// Buffers per element (S = double on the FP64 path, float2 pairs on the
// mixed path; 8 bytes per value either way):
//   Un, Uacc [5][n]     state and RK accumulator, always FP64
//   Us   [5][n]  (S)    stage input state
//   Q    [15][n] (S)    LDG gradient q = grad u, c = l*5 + var
//   Tu   [6][5][nf] (S) face traces of the stage state on the six faces
//   Tq   [3][15][nf] (S) traces of Q on the three minus faces (the only ones
//                       the alternating LDG fluxes read)
// with n = N^3, nf = N^2.  Face point t = a + N b over the face's two
// tangential directions in increasing order (mesh.cpp:428-501).
//
// One CTA works on EPC elements with one thread per (element, Gauss
// point); face work is spread over all threads, and the FP64 gradient
// takes one line of Gauss points per item.  The FP64 kernels are FP64-pipe
// bound on GB300, so the layout choices minimise arithmetic: traces are
// written once by the producer of a state and read (not recomputed) by both
// neighbours, the mass matrix inverse is folded into the 1-D operators, and
// the face fluxes of every direction run one code path per warp.
#pragma once
#include <type_traits>

#include "ldg_device.cuh"

namespace ldg {

// Default elements per CTA ("tile") of the solo kernels.
template <int N>
struct DefEPC {
  static constexpr int value = N == 2 ? 32 : N == 3 ? 9 : N == 4 ? 4 : N == 5 ? 2 : 1;
};

template <int N, int E = DefEPC<N>::value>
struct Cfg {
  static constexpr int n = N * N * N;
  static constexpr int nf = N * N;
  static constexpr int EPC = E;
  static constexpr int T = ((EPC * n + 31) / 32) * 32;
};

// Point index of the Gauss point at normal index qn and face point t on a
// face normal to direction l.
template <int N>
__device__ __forceinline__ int face_point(int l, int qn, int t) {
  int a = t % N, b = t / N;
  return l == 0 ? qn + N * a + N * N * b : l == 1 ? a + N * qn + N * N * b : a + N * b + N * N * qn;
}

template <int N>
__device__ __forceinline__ int stride_of(int l) {
  return l == 0 ? 1 : l == 1 ? N : N * N;
}

// Face point index of Gauss point (qx,qy,qz) on a face normal to l.
template <int N>
__device__ __forceinline__ int tangential(int l, int qx, int qy, int qz) {
  return l == 0 ? qy + N * qz : l == 1 ? qx + N * qz : qx + N * qy;
}

// ---------------------------------------------------------------------------
// Tensor transform per element: out = (M x M x M) in for nv components,
// M row major N x N (B: nodal -> Gauss, Bi: Gauss -> nodal).  FP64.
template <int N>
__global__ void __launch_bounds__(Cfg<N>::T) k_transform(const double* __restrict__ in,
                                                         double* __restrict__ out, int nE, int nv,
                                                         const __grid_constant__ DevOps ops, int inverse) {
  constexpr int n = Cfg<N>::n, EPC = Cfg<N>::EPC, T = Cfg<N>::T;
  extern __shared__ double smem[];
  double* s0 = smem;                 // EPC * nv * n
  double* s1 = smem + EPC * nv * n;  // EPC * nv * n
  __shared__ double M[N * N];
  const double* src = inverse ? ops.Bi : ops.B;
  for (int i = threadIdx.x; i < N * N; i += T) M[i] = src[i];
  const long e0 = (long)blockIdx.x * EPC;
  const int ne = (int)min((long)EPC, nE - e0);
  const long base = e0 * nv * n;
  for (int i = threadIdx.x; i < ne * nv * n; i += T) s0[i] = in[base + i];
  __syncthreads();
  const int es = threadIdx.x / n, q = threadIdx.x % n;
  const bool act = es < ne;
  const int c[3] = {q % N, (q / N) % N, q / (N * N)};
  double* bufs[2] = {s0, s1};
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    const double* sin = bufs[l & 1];
    double* sout = bufs[(l + 1) & 1];
    if (act) {
      const int st = stride_of<N>(l);
      const int b = q - c[l] * st;
      for (int v = 0; v < nv; ++v) {
        const double* row = sin + (es * nv + v) * n + b;
        double acc = 0.0;
#pragma unroll
        for (int r = 0; r < N; ++r) acc = fma(M[c[l] * N + r], row[r * st], acc);
        sout[(es * nv + v) * n + q] = acc;
      }
    }
    __syncthreads();
  }
  // three passes: result in s1
  for (int i = threadIdx.x; i < ne * nv * n; i += T) out[base + i] = s1[i];
}

// ---------------------------------------------------------------------------
// Work list shared by a CTA: item i in [0, total) goes to the lane i - base
// of the warp that took the chunk [base, base + 32) from the CTA's counter
// (*next, zeroed and published by a barrier before the first call).  Whole
// warps take chunks, so lanes diverge only in the one chunk that straddles
// two kinds of item; warps that finish early take more, which balances
// items of unequal cost.  Which thread computes an item never changes the
// item's arithmetic.
template <class F>
__device__ __forceinline__ void for_each_item(int* next, int total, F&& f) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(next, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const int i = base + lane;
    if (i < total) f(i);
  }
}

// ---------------------------------------------------------------------------
// Face traces of a state held in shared memory:
// Tu[e][f][v][t] = sum_qn l_{+-}[qn] U[e][v][pt].
template <int N, class T, int E = DefEPC<N>::value>
__device__ __forceinline__ void write_traces(const T* sU, int ne, long e0, typename Real<T>::S* Tu,
                                             const OpsT<T>& o) {
  constexpr int n = Cfg<N, E>::n, nf = Cfg<N, E>::nf, NT = Cfg<N, E>::T;
  for (int i = threadIdx.x; i < ne * 6 * kNS * nf; i += NT) {
    int es = i / (6 * kNS * nf);
    int r = i - es * 6 * kNS * nf;
    int f = r / (kNS * nf);
    int r2 = r - f * kNS * nf;
    int v = r2 / nf, t = r2 - v * nf;
    int l = f >> 1;
    const T* lvec = (f & 1) ? o.lp : o.lm;
    const int st = stride_of<N>(l);
    const T* row = sU + (es * kNS + v) * n + face_point<N>(l, 0, t);
    Acc<T> acc;
#pragma unroll
    for (int qn = 0; qn < N; ++qn) acc.add(lvec[qn], row[qn * st]);
    Real<T>::st(Tu + (e0 + es) * 6 * kNS * nf + r, acc.get());
  }
}

// Traces of an FP64 state; on the mixed path also writes the FP32-pair copy
// of the state (Ucopy) that the stage kernels read.
template <int N, class T>
__global__ void __launch_bounds__(Cfg<N>::T) k_traces(const double* __restrict__ U,
                                                      typename Real<T>::S* __restrict__ Ucopy,
                                                      typename Real<T>::S* __restrict__ Tu, int nE,
                                                      const __grid_constant__ OpsT<T> o) {
  constexpr int n = Cfg<N>::n, EPC = Cfg<N>::EPC, NT = Cfg<N>::T;
  extern __shared__ double smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const long e0 = (long)blockIdx.x * EPC;
  const int ne = (int)min((long)EPC, nE - e0);
  for (int i = threadIdx.x; i < ne * kNS * n; i += NT) {
    T v = Real<T>::from_f64(U[e0 * kNS * n + i]);
    smem[i] = v;
    if (Ucopy) Real<T>::st(Ucopy + e0 * kNS * n + i, v);
  }
  __syncthreads();
  write_traces<N, T>(smem, ne, e0, Tu, o);
}

// ---------------------------------------------------------------------------
// Gradient pass (rk4Rhs solver.cpp:495-508: localDGFlux + -S_l u + Mel\):
//   Q_l = (1/alpha_l) [ -A_l U + Lp (x) tr(+l, own) - Lm (x) tr(+l, -l neighbour) ]
// The one-sided flux numericalFluxL takes u from the element on the minus
// side of every face, so only plus-face traces are read.
// Writes Q and the minus-face traces Tq; on the FP64 path optionally the
// per-element enstrophy.
// Shared memory of grad_body, in 8-byte values per element: U (5n), the +l
// traces of the element and of its -l neighbours (2 x 15 nf), the element's
// own -l traces (15 nf, needed by the Roe phase only) whose space Q (15 n)
// reuses after that phase, and the enstrophy density (n).
template <int N>
constexpr int grad_smem_values_per_element() {
  return kNS * N * N * N + 2 * 3 * kNS * N * N + kNQ * N * N * N + N * N * N;
}

template <int N, class T, int E = DefEPC<N>::value>
__device__ __forceinline__ void grad_body(const typename Real<T>::S* __restrict__ U,
                                          const typename Real<T>::S* __restrict__ Tu,
                                          typename Real<T>::S* __restrict__ Q,
                                          typename Real<T>::S* __restrict__ Tq,
                                          typename Real<T>::S* __restrict__ Fm, double* __restrict__ ens,
                                          const DevOps& ops, const OpsT<T>& o, long e0, int ne,
                                          double* smem_raw) {
  constexpr int n = Cfg<N, E>::n, nf = Cfg<N, E>::nf, EPC = Cfg<N, E>::EPC, NT = Cfg<N, E>::T;
  using R = Real<T>;
  static_assert(kNQ * n >= 3 * kNS * nf, "Q must cover the -l trace space it reuses");
  T* sU = reinterpret_cast<T*>(smem_raw);  // EPC*5*n
  T* sTp = sU + EPC * kNS * n;             // EPC*3*5*nf  own +l traces
  T* sTm = sTp + EPC * 3 * kNS * nf;       // EPC*3*5*nf  (-l neighbour)'s +l traces
  T* sTo = sTm + EPC * 3 * kNS * nf;       // EPC*3*5*nf  own -l traces (Roe phase)
  T* sQ = sTo;                             // EPC*15*n, reuses sTo after the Roe phase
  double* sE = reinterpret_cast<double*>(sQ + EPC * kNQ * n);  // EPC*n enstrophy
  for (int i = threadIdx.x; i < ne * kNS * n; i += NT) sU[i] = R::ld(U + e0 * kNS * n + i);
  for (int i = threadIdx.x; i < ne * 3 * kNS * nf; i += NT) {
    int es = i / (3 * kNS * nf);
    int r = i - es * 3 * kNS * nf;
    int l = r / (kNS * nf);
    int r2 = r - l * kNS * nf;
    long e = e0 + es;
    int en = face_neighbour((int)e, 2 * l, ops.nx, ops.ny, ops.nz);
    sTp[i] = R::ld(Tu + (e * 6 + 2 * l + 1) * kNS * nf + r2);
    sTm[i] = R::ld(Tu + ((long)en * 6 + 2 * l + 1) * kNS * nf + r2);
    sTo[i] = R::ld(Tu + (e * 6 + 2 * l) * kNS * nf + r2);
  }
  __syncthreads();
  // Roe flux on the three minus faces (numericalFluxC, solver.cpp:1194-1374):
  // each face is computed once, here, by the element on its plus side; the
  // element on the minus side uses its negation (the flux is antisymmetric).
  // Every face in the frame where its normal is x (rot_var).
  for (int i = threadIdx.x; i < ne * 3 * nf; i += NT) {
    const int es2 = i / (3 * nf);
    const int r = i - es2 * 3 * nf;
    const int l = r / nf, t = r - l * nf;
    T uK[kNS], uN[kNS], F[kNS];
#pragma unroll
    for (int v = 0; v < kNS; ++v) {
      const int vm = rot_var(v, l);
      uK[v] = sTo[((es2 * 3 + l) * kNS + vm) * nf + t];
      uN[v] = sTm[((es2 * 3 + l) * kNS + vm) * nf + t];
    }
    roe_flux(uN, uK, false, o, F);
#pragma unroll
    for (int v = 0; v < kNS; ++v) R::st(Fm + ((e0 + es2) * 3 + l) * kNS * nf + rot_var(v, l) * nf + t, F[v]);
  }
  __syncthreads();  // the own -l traces are dead: Q takes their space
  if constexpr (std::is_same<T, double>::value) {
    // FP64: one line (element, direction l, variable v, face point t) per
    // item, in the pairwise form of OpsT::gs..gc: 27 FP64 operations for
    // the 5 outputs of a line at p = 4, where per-point sums take 35.
    constexpr int H = N / 2;
    for (int i = threadIdx.x; i < ne * 3 * kNS * nf; i += NT) {
      const int es2 = i / (3 * kNS * nf);
      int r = i - es2 * 3 * kNS * nf;
      const int l = r / (kNS * nf);
      r -= l * kNS * nf;
      const int v = r / nf, t = r - v * nf;
      const int st = stride_of<N>(l);
      const int p0 = face_point<N>(l, 0, t);
      const T* x = sU + (es2 * kNS + v) * n + p0;
      const T tp = sTp[((es2 * 3 + l) * kNS + v) * nf + t];
      const T tm = sTm[((es2 * 3 + l) * kNS + v) * nf + t];
      const T tdif = tp - tm, tsum = tp + tm;
      T ev[H], od[H];
#pragma unroll
      for (int k = 0; k < H; ++k) {
        const T a = x[k * st], b = x[(N - 1 - k) * st];
        ev[k] = a + b;
        od[k] = a - b;
      }
      T* gs_out = sQ + (es2 * kNQ + l * kNS + v) * n + p0;
      auto* gq_out = Q + ((e0 + es2) * kNQ + l * kNS + v) * n + p0;
#pragma unroll
      for (int k = 0; k < H; ++k) {
        T U = o.gs[l][k] * tdif;
#pragma unroll
        for (int j = 0; j < H; ++j) U = fma(-o.gp[l][k][j], od[j], U);
        T V = o.gd[l][k] * tsum;
#pragma unroll
        for (int j = 0; j < H; ++j) V = fma(-o.gm[l][k][j], ev[j], V);
        if constexpr ((N & 1) != 0) V = fma(-o.gm[l][k][H], x[H * st], V);
        const T lo = U + V, hi = U - V;
        gs_out[k * st] = lo;
        gs_out[(N - 1 - k) * st] = hi;
        R::st(gq_out + k * st, lo);
        R::st(gq_out + (N - 1 - k) * st, hi);
      }
      if constexpr ((N & 1) != 0) {
        T g = o.gc[l][H] * tdif;
#pragma unroll
        for (int j = 0; j < H; ++j) g = fma(-o.gc[l][j], od[j], g);
        gs_out[H * st] = g;
        R::st(gq_out + H * st, g);
      }
    }
    if (ens) {
      __syncthreads();
      // enstrophy density rho |curl v|^2 / 2 at each Gauss point
      const int es = threadIdx.x / n, q = threadIdx.x % n;
      if (es < ne) {
        const int c[3] = {q % N, (q / N) % N, q / (N * N)};
        const double* gq = sQ + es * kNQ * n + q;  // component k at gq[k * n]
        const double* u = sU + es * kNS * n + q;
        double ir = 1.0 / u[0];
        double vv[3] = {u[n] * ir, u[2 * n] * ir, u[3 * n] * ir};
        double G[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
          for (int i = 0; i < 3; ++i) G[i][j] = (gq[(j * kNS + 1 + i) * n] - gq[j * kNS * n] * vv[i]) * ir;
        double wx = G[2][1] - G[1][2], wy = G[0][2] - G[2][0], wz = G[1][0] - G[0][1];
        double w3 = ops.w[c[0]] * ops.w[c[1]] * ops.w[c[2]];
        sE[es * n + q] = ops.J * w3 * 0.5 * u[0] * (wx * wx + wy * wy + wz * wz);
      }
    }
  } else {
    // FP32 pairs: one Gauss point per thread, each output one compensated
    // 7-term dot product
    const int es = threadIdx.x / n, q = threadIdx.x % n;
    if (es < ne) {
      const int c[3] = {q % N, (q / N) % N, q / (N * N)};
#pragma unroll
      for (int l = 0; l < 3; ++l) {
        const int qn = c[l];
        const int st = stride_of<N>(l);
        const int b = q - qn * st;
        const int t = tangential<N>(l, c[0], c[1], c[2]);
        T row[N];
#pragma unroll
        for (int r = 0; r < N; ++r) row[r] = o.As[l][qn * N + r];
        const T lp = o.Lps[l][qn], lm = o.Lms[l][qn];
#pragma unroll
        for (int v = 0; v < kNS; ++v) {
          const T* line = sU + (es * kNS + v) * n + b;
          const T tp = sTp[((es * 3 + l) * kNS + v) * nf + t];
          const T tm = sTm[((es * 3 + l) * kNS + v) * nf + t];
          Acc<T> acc;
#pragma unroll
          for (int r = 0; r < N; ++r) acc.add(-row[r], line[r * st]);
          acc.add(lp, tp);
          acc.add(-lm, tm);
          const T g = acc.get();
          sQ[(es * kNQ + l * kNS + v) * n + q] = g;
          R::st(Q + ((e0 + es) * kNQ + l * kNS + v) * n + q, g);
        }
      }
    }
  }
  __syncthreads();
  if constexpr (std::is_same<T, double>::value) {
    if (ens && threadIdx.x < ne) {  // fixed-order per-element sum (deterministic)
      double acc = 0.0;
      for (int k = 0; k < n; ++k) acc += sE[threadIdx.x * n + k];
      ens[e0 + threadIdx.x] = acc;
    }
  }
  // minus-face traces of Q: Tq[e][l][c][t] = sum_qn lm[qn] Q[e][c][pt(l,qn,t)]
  for (int i = threadIdx.x; i < ne * 3 * kNQ * nf; i += NT) {
    int es2 = i / (3 * kNQ * nf);
    int r = i - es2 * 3 * kNQ * nf;
    int l = r / (kNQ * nf);
    int r2 = r - l * kNQ * nf;
    int cc = r2 / nf, t = r2 - cc * nf;
    const int st = stride_of<N>(l);
    const T* row = sQ + (es2 * kNQ + cc) * n + face_point<N>(l, 0, t);
    Acc<T> acc;
#pragma unroll
    for (int qn = 0; qn < N; ++qn) acc.add(o.lm[qn], row[qn * st]);
    R::st(Tq + (e0 + es2) * 3 * kNQ * nf + r, acc.get());
  }
}

template <int N, class T>
__global__ void __launch_bounds__(Cfg<N>::T, Cfg<N>::T == 256 ? 4 : 1) k_grad(const typename Real<T>::S* __restrict__ U,
                                                    const typename Real<T>::S* __restrict__ Tu,
                                                    typename Real<T>::S* __restrict__ Q,
                                                    typename Real<T>::S* __restrict__ Tq,
                                                    typename Real<T>::S* __restrict__ Fm,
                                                    double* __restrict__ ens,
                                                    const __grid_constant__ DevOps ops,
                                                    const __grid_constant__ OpsT<T> o, int ebase, int eend) {
  // elements [ebase, eend), EPC per CTA
  extern __shared__ double smem_raw[];
  const long e0 = ebase + (long)blockIdx.x * Cfg<N>::EPC;
  const int ne = (int)min((long)Cfg<N>::EPC, eend - e0);
  grad_body<N, T>(U, Tu, Q, Tq, Fm, ens, ops, o, e0, ne, smem_raw);
}

// ---------------------------------------------------------------------------
// Kinetic energy of a state held in shared memory (sU: EPC*5*n Gauss values
// in the arithmetic type T; scr: EPC*8*n scratch of T).  Per element:
// diag[2e] = computeKE exactly as the reference evaluates it (nodal values
// weighted by the Gauss weights, solver.cpp:1021-1024, nodal values
// recovered with Bi (x) Bi (x) Bi), and diag[2e+1] = the Gauss-quadrature
// kinetic energy.  On the FP64 path every operation is FP64; on the mixed
// path (T = dd, the FP32-pair copy of the new FP64 state) the nodal
// transform and the point densities run in FP32-pair arithmetic and the
// weights, the densities' products with them and the per-element sums in
// FP64.  Fixed-order sums.
template <int N, class T = double, int E = DefEPC<N>::value>
__device__ __forceinline__ void ke_tail(const T* sU, T* scr, int ne, long e0, double* diag, const DevOps& ops,
                                        const OpsT<T>& o) {
  constexpr int n = Cfg<N, E>::n, EPC = Cfg<N, E>::EPC;
  static_assert(sizeof(T) == sizeof(double), "8-byte values");
  T* s1 = scr;                 // EPC*4*n
  T* s2 = scr + EPC * 4 * n;   // EPC*4*n
  const int es = threadIdx.x / n, q = threadIdx.x % n;
  const bool act = es < ne;
  const int c[3] = {q % N, (q / N) % N, q / (N * N)};
#pragma unroll
  for (int l = 0; l < 3; ++l) {
    const T* sin = l == 0 ? sU : (l == 1 ? s1 : s2);
    T* sout = l == 1 ? s2 : s1;
    const int instride = l == 0 ? kNS : 4;
    if (act) {
      const int st = stride_of<N>(l);
      const int b = q - c[l] * st;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const T* row = sin + (es * instride + v) * n + b;
        Acc<T> acc;
#pragma unroll
        for (int r = 0; r < N; ++r) {
          if constexpr (std::is_same<T, double>::value) acc.add(ops.Bi[c[l] * N + r], row[r * st]);
          else acc.add(o.Bi[c[l] * N + r], row[r * st]);
        }
        sout[(es * 4 + v) * n + q] = acc.get();
      }
    }
    __syncthreads();
  }
  double* d2 = reinterpret_cast<double*>(s2);
  if (act) {
    const T* un = s1 + es * 4 * n + q;    // nodal rho, m at node index q
    const T* ug = sU + es * kNS * n + q;  // Gauss values at point q
    const double w3 = ops.w[c[0]] * ops.w[c[1]] * ops.w[c[2]];
    if constexpr (std::is_same<T, double>::value) {
      d2[es * 2 * n + q] =
          ops.J * w3 * (un[n] * un[n] + un[2 * n] * un[2 * n] + un[3 * n] * un[3 * n]) / (2 * un[0]);
      d2[(es * 2 + 1) * n + q] =
          ops.J * w3 * (ug[n] * ug[n] + ug[2 * n] * ug[2 * n] + ug[3 * n] * ug[3 * n]) / (2 * ug[0]);
    } else {
      const T kn = (un[n] * un[n] + un[2 * n] * un[2 * n] + un[3 * n] * un[3 * n]) * rcp(un[0] + un[0]);
      const T kg = (ug[n] * ug[n] + ug[2 * n] * ug[2 * n] + ug[3 * n] * ug[3 * n]) * rcp(ug[0] + ug[0]);
      d2[es * 2 * n + q] = ops.J * w3 * Real<T>::to_f64(kn);
      d2[(es * 2 + 1) * n + q] = ops.J * w3 * Real<T>::to_f64(kg);
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * ne) {
    const double* src = d2 + threadIdx.x * n;
    double acc = 0.0;
    for (int k = 0; k < n; ++k) acc += src[k];
    diag[(e0 + (threadIdx.x >> 1)) * 2 + (threadIdx.x & 1)] = acc;
  }
}

template <int N>
__global__ void __launch_bounds__(Cfg<N>::T) k_ke(const double* __restrict__ U, double* __restrict__ diag,
                                                  const __grid_constant__ DevOps ops) {
  constexpr int n = Cfg<N>::n, EPC = Cfg<N>::EPC, T = Cfg<N>::T;
  extern __shared__ double smem[];
  const long e0 = (long)blockIdx.x * EPC;
  const int ne = (int)min((long)EPC, ops.nE - e0);
  for (int i = threadIdx.x; i < ne * kNS * n; i += T) smem[i] = U[e0 * kNS * n + i];
  __syncthreads();
  ke_tail<N, double>(smem, smem + EPC * kNS * n, ne, e0, diag, ops, OpsT<double>{});
}

// ---------------------------------------------------------------------------
// RHS pass + RK4 stage update (rk4Rhs solver.cpp:516-533 and the RK glue
// solver.cpp:410-434, 458-480):
//   K = sum_l (1/alpha_l) A_l (Fc_l - Fv_l)
//       - sum_f (1/alpha_l(f)) L_{s(f)} (x) (Fc*_f + Fv*_f)
// Fc* is the Roe flux from this element's side; Fv* = -s Fv_l(u_K, q_win)
// with q from the element on the plus side of the face (numericalFluxV).
// The RK combination is FP64 on both paths.
template <class T>
struct StageArgs {
  using S = typename Real<T>::S;
  const S* Us;        // stage input state
  const S* Q;         // its gradient
  const S* Tu;        // its face traces
  const S* Tq;        // gradient minus-face traces
  const S* Fm;        // Roe fluxes on the minus faces (from the gradient pass)
  const double* Un;   // state at the start of the step
  double* Uacc;       // RK accumulator (u += dt b_s k_s)
  S* Unext;           // next stage input (u + dt a_s k_s); on the last stage
                      // the mixed path's pair copy of the new state
  S* Tu_out;          // traces of Unext (or of Uacc on the last stage)
  double* Kout;       // raw RHS output (rhs-only mode)
  const double* Kadd; // optional additive RHS term (learned closure), same layout as U
  double* diag;       // per-element [ke_ref, ke] on the last stage (FP64 path)
  int* flag;          // nonzero if a non-finite value was produced
  double cacc;        // dt * b_s
  double cnext;       // dt * a_s
  int stage;          // 0..3, or -1 for rhs-only
};

// Numerical flux sum Fc* + Fv* at face point t of face f (direction L) of
// element e, written to out[v*nf].  Evaluated in the frame where the face
// normal is x (rot_var), so faces of all directions share one code path.
template <int N, class T>
__device__ __forceinline__ void face_flux(const StageArgs<T>& a, const DevOps& ops, const OpsT<T>& o, long e,
                                          int f, int t, T* out) {
  constexpr int nf = N * N;
  using R = Real<T>;
  const bool plus = f & 1;
  const int L = f >> 1;
  const long en = face_neighbour((int)e, f, ops.nx, ops.ny, ops.nz);
  int vm[kNS];
#pragma unroll
  for (int v = 0; v < kNS; ++v) vm[v] = rot_var(v, L);
  T uK[kNS], Du[kNQ], F[kNS];
  const auto* tK = a.Tu + (e * 6 + f) * kNS * nf + t;
#pragma unroll
  for (int v = 0; v < kNS; ++v) uK[v] = R::ld(tK + vm[v] * nf);
  // Roe flux: own minus face, or the negated minus-face flux of the plus
  // neighbour
  const auto* fm = a.Fm + ((plus ? en : e) * 3 + L) * kNS * nf + t;
#pragma unroll
  for (int v = 0; v < kNS; ++v) F[v] = sgn(!plus, R::ld(fm + vm[v] * nf));
  // q from the element on the plus side (numericalFluxV kWins switch);
  // gradient direction j of the rotated frame is mesh direction
  // rot_axis(j, L)
  const auto* tq = a.Tq + ((plus ? en : e) * 3 + L) * kNQ * nf + t;
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int v = 0; v < kNS; ++v) Du[j * kNS + v] = R::ld(tq + (rot_axis(j, L) * kNS + vm[v]) * nf);
  ViscPre<T> P;
  visc_pre(uK, Du, P);
  // Fc* + Fv*, Fv* = -s Fv_x: the viscous column enters with -s/Re
  add_visc_column<0>(P, plus ? -o.inv_re : o.inv_re, o, F);
#pragma unroll
  for (int v = 0; v < kNS; ++v) out[vm[v] * nf] = F[v];
}

template <int N, class T, int E = DefEPC<N>::value>
__device__ __forceinline__ void rhs_body(const StageArgs<T>& a, const DevOps& ops, const OpsT<T>& o, long e0,
                                         int ne, double* smem_raw) {
  constexpr int n = Cfg<N, E>::n, nf = Cfg<N, E>::nf, EPC = Cfg<N, E>::EPC;
  using R = Real<T>;
  T* sF = reinterpret_cast<T*>(smem_raw);  // EPC*15*n   volume flux Fc - Fv
  T* sFs = sF + EPC * kNQ * n;             // EPC*6*5*nf face flux sums
  T* sU = sF;                              // EPC*5*n, aliases sF after use
  const int es = threadIdx.x / n, q = threadIdx.x % n;
  const bool act = es < ne;
  const int c[3] = {q % N, (q / N) % N, q / (N * N)};
  // 1-2. The volume fluxes at the Gauss points and the numerical fluxes at
  // the face points (ne*6*nf of them, more than there are threads).
  const int nV = ne * n;
  auto volume_item = [&](int i) {
    const int es2 = i / n, q2 = i - es2 * n;
    const long e = e0 + es2;
    T u[kNS], Du[kNQ];
#pragma unroll
    for (int v = 0; v < kNS; ++v) u[v] = R::ld(a.Us + (e * kNS + v) * n + q2);
#pragma unroll
    for (int k = 0; k < kNQ; ++k) Du[k] = R::ld(a.Q + (e * kNQ + k) * n + q2);
    const T ir = rcp(u[0]);
    ViscPre<T> P;
    visc_pre(u, ir, Du, P);
    const Euler<T> es_ = euler_state(u, ir, P.v, o);
    const T mre = -o.inv_re;
    T F[kNS];
    euler_column<0>(u, P.v, es_, F);
    add_visc_column<0>(P, mre, o, F);
#pragma unroll
    for (int v = 0; v < kNS; ++v) sF[(es2 * kNQ + 0 * kNS + v) * n + q2] = F[v];
    euler_column<1>(u, P.v, es_, F);
    add_visc_column<1>(P, mre, o, F);
#pragma unroll
    for (int v = 0; v < kNS; ++v) sF[(es2 * kNQ + 1 * kNS + v) * n + q2] = F[v];
    euler_column<2>(u, P.v, es_, F);
    add_visc_column<2>(P, mre, o, F);
#pragma unroll
    for (int v = 0; v < kNS; ++v) sF[(es2 * kNQ + 2 * kNS + v) * n + q2] = F[v];
  };
  auto face_item = [&](int j) {
    const int fes = j / (6 * nf);
    const int r = j - fes * 6 * nf;
    const int f = r / nf, t = r - f * nf;
    face_flux<N>(a, ops, o, e0 + fes, f, t, sFs + (fes * 6 + f) * kNS * nf + t);
  };
  if constexpr (std::is_same<T, dd>::value) {
    // The FP32-pair path is latency-bound: one work list over both kinds
    // (volume items, the heavier, first) keeps every warp busy.  Measured
    // at 64^3 p=4: 8.31 -> 8.12 ms per launch.
    __shared__ int s_next;  // the work list's counter
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    for_each_item(&s_next, nV + ne * 6 * nf, [&](int i) {
      if (i < nV) volume_item(i);
      else face_item(i - nV);
    });
  } else {
    // The FP64 path is FP64-pipe bound and gains nothing from the list
    // (measured 22.34 -> 22.47 ms): one volume item per thread, then the
    // face items round-robin.
    if (act) volume_item(threadIdx.x);
    for (int j = threadIdx.x; j < ne * 6 * nf; j += Cfg<N, E>::T) face_item(j);
  }
  __syncthreads();
  // 3. contraction: K at this Gauss point
  T K[kNS];
  if (act) {
#pragma unroll
    for (int v = 0; v < kNS; ++v) K[v] = T{};
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      const int qn = c[l];
      const int st = stride_of<N>(l);
      const int b = q - qn * st;
      const int t = tangential<N>(l, c[0], c[1], c[2]);
      T row[N];
#pragma unroll
      for (int r = 0; r < N; ++r) row[r] = o.As[l][qn * N + r];
      const T lp = -o.Lps[l][qn], lm = -o.Lms[l][qn];
#pragma unroll
      for (int v = 0; v < kNS; ++v) {
        const T* line = sF + (es * kNQ + l * kNS + v) * n + b;
        Acc<T> acc(K[v]);
#pragma unroll
        for (int r = 0; r < N; ++r) acc.add(row[r], line[r * st]);
        acc.add(lm, sFs[((es * 6 + 2 * l) * kNS + v) * nf + t]);
        acc.add(lp, sFs[((es * 6 + 2 * l + 1) * kNS + v) * nf + t]);
        K[v] = acc.get();
      }
    }
  }
  __syncthreads();  // sF is reused as sU below
  // 4. RK4 stage update in FP64 (or raw RHS output)
  if (act) {
    const long e = e0 + es;
    if (a.stage < 0) {
#pragma unroll
      for (int v = 0; v < kNS; ++v) {
        const long idx = (e * kNS + v) * n + q;
        a.Kout[idx] = a.Kadd ? R::to_f64(K[v]) + a.Kadd[idx] : R::to_f64(K[v]);
      }
    } else {
      bool bad = false;
#pragma unroll
      for (int v = 0; v < kNS; ++v) {
        const long idx = (e * kNS + v) * n + q;
        const double kd = a.Kadd ? R::to_f64(K[v]) + a.Kadd[idx] : R::to_f64(K[v]);
        const double un = a.Un[idx];
        const double acc0 = a.stage == 0 ? un : a.Uacc[idx];
        const double uacc = acc0 + a.cacc * kd;
        a.Uacc[idx] = uacc;
        const double nxt = a.stage < 3 ? un + a.cnext * kd : uacc;
        const T nt = R::from_f64(nxt);
        if (a.Unext) R::st(a.Unext + idx, nt);
        bad |= not_finite(nxt);
        sU[(es * kNS + v) * n + q] = nt;
      }
      if (bad && a.flag) atomicOr(a.flag, 1);
    }
  }
  if (a.stage < 0) return;
  __syncthreads();
  // 5. traces of the next stage input for the face fluxes of the next pass
  write_traces<N, T, E>(sU, ne, e0, a.Tu_out, o);
  // 6. diagnostics on the new state (last stage; on the mixed path from
  //    the FP32-pair copy of the new FP64 state)
  if (a.stage == 3 && a.diag) {
    __syncthreads();
    ke_tail<N, T, E>(sU, sF + EPC * kNS * n, ne, e0, a.diag, ops, o);
  }
}

template <int N, class T>
__global__ void __launch_bounds__(Cfg<N>::T, Cfg<N>::T == 256 ? 4 : 1) k_rhs(const __grid_constant__ StageArgs<T> a,
                                                   const __grid_constant__ DevOps ops,
                                                   const __grid_constant__ OpsT<T> o, int ebase, int eend) {
  // elements [ebase, eend), EPC per CTA
  extern __shared__ double smem_raw[];
  const long e0 = ebase + (long)blockIdx.x * Cfg<N>::EPC;
  const int ne = (int)min((long)Cfg<N>::EPC, eend - e0);
  rhs_body<N, T>(a, ops, o, e0, ne, smem_raw);
}

}  // namespace ldg
