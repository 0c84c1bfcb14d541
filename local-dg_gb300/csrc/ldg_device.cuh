// Device-side pieces shared by the LDG kernels: operator blocks, mesh
// neighbour map, pointwise fluxes (templated on the arithmetic type T =
// double or dd, see ldg_real.cuh).
//
// Pointwise physics restated from Local-DG solver.cpp (fluxC 1040-1086,
// fluxV 1089-1188, numericalFluxC 1194-1374, numericalFluxV 891-921,
// numericalFluxL 867-884).  Normals are the mesh's axis unit vectors
// (mesh.cpp:338-353), so the normal dot products reduce to one signed
// component; adding the exact zeros the reference adds changes no bit.
#pragma once
#include <cstdint>

#include "ldg_real.cuh"

namespace ldg {

using ::fabs;
using ::fma;
using ::sqrt;

constexpr int kNS = 5;     // conserved variables (solver.cpp:61)
constexpr int kNQ = 15;    // gradient components: 3 directions x 5 vars
constexpr int kDevMaxN = 8;

// Double-precision operator block and mesh geometry; passed by value.
struct DevOps {
  double A[kDevMaxN * kDevMaxN];   // weak derivative, A[q*N + r]
  double B[kDevMaxN * kDevMaxN];   // CGL nodal -> Gauss, B[q*N + i]
  double Bi[kDevMaxN * kDevMaxN];  // Gauss -> CGL nodal, Bi[i*N + q]
  double lp[kDevMaxN], lm[kDevMaxN];  // Gauss-Lagrange basis at +1 / -1
  double Lp[kDevMaxN], Lm[kDevMaxN];  // lift: basis at +-1 over weight
  double w[kDevMaxN];                 // Gauss weights
  double ia[3];                       // 1 / alpha_l = 2 / dx_l
  double J;                           // alpha_0 alpha_1 alpha_2
  double inv_re;                      // 1 / Re
  double gamma;                       // ratio of specific heats
  double g1;                          // gamma - 1 (the reference's 0.4)
  double kappa;                       // gamma / Pr
  double ke_norm;                     // 1 / (rho0 (2 pi L)^3)
  int nx, ny, nz, nE;
};

// The arithmetic constants of the step kernels in the type they compute in.
template <class T>
struct OpsT {
  T lp[kDevMaxN], lm[kDevMaxN];
  // Per direction l, pre-scaled by 1/alpha_l so the kernels spend no
  // multiplications on the element size: As = A / alpha_l, Lps = Lp /
  // alpha_l, Lms = Lm / alpha_l (gradient pass), and their negations for the
  // RHS lifts.
  T As[3][kDevMaxN * kDevMaxN];
  T Lps[3][kDevMaxN], Lms[3][kDevMaxN];
  T Bi[kDevMaxN * kDevMaxN];  // Gauss -> CGL nodal (the KE quirk), Bi[i*N + q]
  T g1, hg1, gamma, inv_re, kappa, two3, one;
  // The gradient along one line in pairwise form (FP64 gradient pass).  The
  // Gauss points are symmetric, so As is skew-centrosymmetric
  // (As[N-1-q][N-1-r] = -As[q][r]) and the lifts mirror (Lp[N-1-q] =
  // Lm[q]).  With H = N/2, m = H (the middle point of odd N), and along the
  // line e_r = x_r + x_{N-1-r}, o_r = x_r - x_{N-1-r} (r < H), tdif = tp - tm,
  // tsum = tp + tm, the outputs q and N-1-q (q < H) are U + V and U - V:
  //   U = gs[q] tdif - sum_r gp[q][r] o_r,
  //   V = gd[q] tsum - sum_r gm[q][r] e_r - gm[q][H] x_m   (odd N),
  // and the middle output is gc[H] tdif - sum_r gc[r] o_r (odd N), with
  //   gs = (Lps + Lms)[q]/2, gd = (Lps - Lms)[q]/2,
  //   gp[q][r] = (As[q][r] - As[q][N-1-r])/2, gm[q][r] = (As[q][r] + As[q][N-1-r])/2,
  //   gm[q][H] = As[q][m], gc[r] = As[m][r], gc[H] = Lps[m].
  T gs[3][kDevMaxN / 2], gd[3][kDevMaxN / 2];
  T gp[3][kDevMaxN / 2][kDevMaxN / 2], gm[3][kDevMaxN / 2][kDevMaxN / 2 + 1];
  T gc[3][kDevMaxN / 2 + 1];
};

// Host-side conversion of the double block into the arithmetic type T.
inline double host_cast(double v, const double*) { return v; }
inline dd host_cast(double v, const dd*) { return dd_from_host(v); }

template <class T>
inline OpsT<T> make_opst(const DevOps& d, int N) {
  OpsT<T> o;
  const T* tag = nullptr;
  for (int i = 0; i < kDevMaxN; ++i) {
    o.lp[i] = host_cast(d.lp[i], tag);
    o.lm[i] = host_cast(d.lm[i], tag);
  }
  for (int l = 0; l < 3; ++l) {
    for (int i = 0; i < kDevMaxN * kDevMaxN; ++i) o.As[l][i] = host_cast(i < N * N ? d.A[i] * d.ia[l] : 0.0, tag);
    for (int i = 0; i < kDevMaxN; ++i) {
      o.Lps[l][i] = host_cast(d.Lp[i] * d.ia[l], tag);
      o.Lms[l][i] = host_cast(d.Lm[i] * d.ia[l], tag);
    }
  }
  for (int i = 0; i < kDevMaxN * kDevMaxN; ++i) o.Bi[i] = host_cast(i < N * N ? d.Bi[i] : 0.0, tag);
  const int H = N / 2;
  for (int l = 0; l < 3; ++l) {
    const long double ia = d.ia[l];
    for (int q = 0; q < kDevMaxN / 2; ++q) {
      const bool in = q < H;
      o.gs[l][q] = host_cast(in ? (double)(((long double)d.Lp[q] + d.Lm[q]) * ia / 2) : 0.0, tag);
      o.gd[l][q] = host_cast(in ? (double)(((long double)d.Lp[q] - d.Lm[q]) * ia / 2) : 0.0, tag);
      for (int r = 0; r <= kDevMaxN / 2; ++r) {
        double gp = 0.0, gm = 0.0;
        if (in && r < H) {
          gp = (double)(((long double)d.A[q * N + r] - d.A[q * N + N - 1 - r]) * ia / 2);
          gm = (double)(((long double)d.A[q * N + r] + d.A[q * N + N - 1 - r]) * ia / 2);
        } else if (in && r == H && (N & 1)) {
          gm = (double)((long double)d.A[q * N + H] * ia);
        }
        if (r < kDevMaxN / 2) o.gp[l][q][r] = host_cast(gp, tag);
        o.gm[l][q][r] = host_cast(gm, tag);
      }
    }
    for (int r = 0; r <= kDevMaxN / 2; ++r) {
      double gc = 0.0;
      if ((N & 1) && r < H) gc = (double)((long double)d.A[H * N + r] * ia);
      if ((N & 1) && r == H) gc = (double)((long double)d.Lp[H] * ia);
      o.gc[l][r] = host_cast(gc, tag);
    }
  }
  o.g1 = host_cast(d.g1, tag);
  o.hg1 = host_cast(0.5 * d.g1, tag);
  o.gamma = host_cast(d.gamma, tag);
  o.inv_re = host_cast(d.inv_re, tag);
  o.kappa = host_cast(d.kappa, tag);
  o.two3 = host_cast(2.0 / 3.0, tag);
  o.one = host_cast(1.0, tag);
  return o;
}

// Periodic face neighbour: element numbering e = ix + nx (iy + ny iz)
// (mesh.cpp:162); faces -x,+x,-y,+y,-z,+z.  On one rank the reference's
// ghost slots hold exactly the wrapped neighbour's trace (MPIUtil.cpp:23-28,
// solver.cpp:929-998), so the wrap is computed directly.
__device__ __forceinline__ int face_neighbour(int e, int f, int nx, int ny, int nz) {
  int ix = e % nx;
  int r = e / nx;
  int iy = r % ny;
  int iz = r / ny;
  switch (f) {
    case 0: ix = (ix == 0) ? nx - 1 : ix - 1; break;
    case 1: ix = (ix == nx - 1) ? 0 : ix + 1; break;
    case 2: iy = (iy == 0) ? ny - 1 : iy - 1; break;
    case 3: iy = (iy == ny - 1) ? 0 : iy + 1; break;
    case 4: iz = (iz == 0) ? nz - 1 : iz - 1; break;
    default: iz = (iz == nz - 1) ? 0 : iz + 1; break;
  }
  return ix + nx * (iy + ny * iz);
}

// Cyclic relabelling of the axes that takes direction l to x: axis k of the
// rotated frame is axis (k + l) mod 3 of the mesh.  The face kernels
// evaluate the Roe and viscous face fluxes of every face in the rotated
// frame, with the x-direction form of the flux, and apply the relabelling
// to the load and store addresses.  A warp's threads hold faces of
// different directions; with one code path for all of them the warp does
// not diverge (per-direction code paths ran one after the other).  The
// fluxes are invariant under the rotation: only the order of the terms of a
// few three-term sums (|v|^2, v.dm, tau_i v_i) changes.
__device__ __forceinline__ int rot_axis(int k, int l) { return k + l >= 3 ? k + l - 3 : k + l; }
// variable v of the rotated frame -> the same variable in the mesh frame
__device__ __forceinline__ int rot_var(int v, int l) { return (v == 0 || v == 4) ? v : 1 + rot_axis(v - 1, l); }

// Non-finite test on the exponent bits (integer pipe, not the FP64 pipe).
__device__ __forceinline__ bool not_finite(double x) {
  return (__double_as_longlong(x) & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
}

// FP64 reciprocal of the flux formulas, faithful (within one ulp;
// ldg_probe_recip measures it against 1.0/x).  The flux kernels are FP64-pipe
// bound, so it spends as few FP64 instructions as it can:
//   * seed: the FP32 special-function approximation, applied to x truncated
//     to 23 mantissa bits.  The operand goes into and the seed y0 comes out
//     of FP32 by rebiasing the exponent field with integer instructions
//     (an exact change of format, no FP64 or conversion instruction);
//     relative error below 2^-21;
//   * one third-order (Householder) correction with e = 1 - x y0, the
//     seed's residual: y = y0 (1 + e + e^2), three DFMA, leaving e^3
//     (below 2^-60) plus the last rounding.
// Outside [2^-125, 2^126) (zero, negative, non-finite, FP32-subnormal or
// huge operands) CUDA's 1.0/x takes over, so every special case keeps IEEE
// behaviour.  Measured at 64^3 p=4: the RHS pass 20.30 -> 20.04 ms against
// 1.0/x.  The same construction for 1/sqrt(x) (the series 1 + e/2 + 3e^2/8,
// three DFMA and two DMUL) was 1.4 % slower in the gradient pass than
// CUDA's rsqrt, which the flux code keeps.
namespace recip_detail {
constexpr unsigned kRebias = (1023u - 127u) << 20;  // exponent bias difference in the high word

// x's biased exponent with the sign in bit 11: in range iff E in [898, 1148]
__device__ __forceinline__ bool in_range(int hi) { return ((unsigned)hi >> 20) - 898u <= 250u; }

__device__ __forceinline__ float to_f32(int hi, int lo) {
  return __uint_as_float((((unsigned)hi - kRebias) << 3) | ((unsigned)lo >> 29));
}

__device__ __forceinline__ double to_f64(float y) {
  const unsigned b = __float_as_uint(y);
  return __hiloint2double((int)((b >> 3) + kRebias), (int)(b << 29));
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
}  // namespace recip_detail

__device__ __forceinline__ double rcp(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  if (__builtin_expect(!recip_detail::in_range(hi), 0)) return 1.0 / x;
  const double y0 = recip_detail::to_f64(recip_detail::rcp_approx(recip_detail::to_f32(hi, lo)));
  const double e = fma(-x, y0, 1.0);
  return fma(y0, fma(e, e, e), y0);
}

// 1/sqrt(x): CUDA's double rsqrt; on the FP32-pair path the pair reciprocal
// of the pair square root.
__device__ __forceinline__ double rsqrt_(double x) { return ::rsqrt(x); }

// helpers that are exact in both types
__device__ __forceinline__ double half_(double x) { return 0.5 * x; }
__device__ __forceinline__ dd rsqrt_(dd x) { return rcp(sqrt(x)); }
__device__ __forceinline__ dd half_(dd x) { return scale2(x, 0.5f); }
template <class T>
__device__ __forceinline__ T sgn(bool plus, T x) { return plus ? x : -x; }

// a*b rounded on its own, never fused into a neighbouring sum.  A product
// that several sums use must round the same way in every kernel that
// inlines this code (the solo kernels and the ensemble's tiles are
// separate instantiations, and results must agree bit for bit); whether
// the compiler fuses such a product into one of its sums is its own choice
// per instantiation, so those products are pinned.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ dd mul_rn(dd a, dd b) { return a * b; }
__device__ __forceinline__ double half_rn(double x) { return __dmul_rn(0.5, x); }
__device__ __forceinline__ dd half_rn(dd x) { return half_(x); }

// Euler flux, column l of F(u): components (rho, m_x, m_y, m_z, E) of the
// flux in direction l (solver.cpp:1060-1084 with fluxes[iS + 5 l]).
// p = g1 (E - |m|^2/(2 rho)); energy flux m_l (E + p)/rho, with E + p
// written gamma E - g1|m|^2/(2rho) as the reference does.  With v = m/rho
// given: |m|^2/rho = m.v, the diagonal momentum flux plus pressure is one
// FMA m_l v_l + p, and the momentum flux m_i v_l is symmetric in (i, l)
// (both equal rho v_i v_l), so three products give its six off-diagonal
// entries.  Every sum is an explicit FMA or takes unfused operands.
template <class T>
struct Euler {
  T p, h;  // pressure, (E+p)/rho
  T M[3];  // off-diagonal m_i v_l: xy, xz, yz
};

template <class T>
__device__ __forceinline__ Euler<T> euler_state(const T u[kNS], T ir, const T v[3], const OpsT<T>& o) {
  Euler<T> s;
  s.M[0] = u[2] * v[0];
  s.M[1] = u[3] * v[0];
  s.M[2] = u[3] * v[1];
  const T k = o.hg1 * fma(u[3], v[2], fma(u[2], v[1], u[1] * v[0]));
  s.p = fma(o.g1, u[4], -k);
  s.h = fma(o.gamma, u[4], -k) * ir;
  return s;
}

template <int l, class T>
__device__ __forceinline__ void euler_column(const T u[kNS], const T v[3], const Euler<T>& s, T F[kNS]) {
  F[0] = u[1 + l];
  if constexpr (l == 0) {
    F[1] = fma(u[1], v[0], s.p);
    F[2] = s.M[0];
    F[3] = s.M[1];
  } else if constexpr (l == 1) {
    F[1] = s.M[0];
    F[2] = fma(u[2], v[1], s.p);
    F[3] = s.M[2];
  } else {
    F[1] = s.M[1];
    F[2] = s.M[2];
    F[3] = fma(u[3], v[2], s.p);
  }
  F[4] = u[1 + l] * s.h;
}

// Velocity gradient G[i][j] = d_j v_i from u and Du[c], c = j*5 + var
// (the chain rule of solver.cpp:1137-1170), plus d_j e with
// e = E/rho - |v|^2/2 the specific internal energy.
template <class T>
struct ViscPre {
  T v[3];
  T G[3][3];
  T de[3];
  T div;
};

// ir = 1/rho, when the caller has it already
template <class T>
__device__ __forceinline__ void visc_pre(const T u[kNS], const T ir, const T* Du, ViscPre<T>& P) {
  P.v[0] = u[1] * ir;
  P.v[1] = u[2] * ir;
  P.v[2] = u[3] * ir;
  T eo = u[4] * ir;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    T dr = Du[j * kNS + 0];
#pragma unroll
    for (int i = 0; i < 3; ++i) P.G[i][j] = mul_rn(Du[j * kNS + 1 + i] - dr * P.v[i], ir);
    P.de[j] = (Du[j * kNS + 4] - dr * eo) * ir -
              (P.v[0] * P.G[0][j] + P.v[1] * P.G[1][j] + P.v[2] * P.G[2][j]);
  }
  P.div = P.G[0][0] + P.G[1][1] + P.G[2][2];
}

template <class T>
__device__ __forceinline__ void visc_pre(const T u[kNS], const T* Du, ViscPre<T>& P) {
  visc_pre(u, rcp(u[0]), Du, P);
}

// F += c Re * (column j of the viscous flux) (solver.cpp:1136-1187):
// Newtonian stress with Stokes' hypothesis over Re, heat flux (gamma/Pr)
// grad e / Re; c = -1/Re subtracts it from the Euler column (volume), c =
// +-1/Re adds the signed face flux to the Roe flux (faces).  Fused into
// FMAs; F[0] gets no viscous part.
template <int j, class T>
__device__ __forceinline__ void add_visc_column(const ViscPre<T>& P, const T c, const OpsT<T>& o, T F[kNS]) {
  T tau[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) tau[i] = P.G[i][j] + P.G[j][i];
  tau[j] -= o.two3 * P.div;
  F[1] = fma(tau[0], c, F[1]);
  F[2] = fma(tau[1], c, F[2]);
  F[3] = fma(tau[2], c, F[3]);
  F[4] = fma(tau[0] * P.v[0] + tau[1] * P.v[1] + tau[2] * P.v[2] + o.kappa * P.de[j], c, F[4]);
}

// Roe flux F*(uN, uK, n) seen from element K with n = s e_x
// (numericalFluxC, solver.cpp:1291-1372): central flux minus Roe-averaged
// upwind dissipation; the reference's hard-coded 0.4 is g1.  Faces of the
// other directions are evaluated in the frame where their normal is x
// (rot_var).  The algebra is arranged for few operations: p from m.v, the
// wave-strength combinations t179 = a1 dp/c^2 + a2 dq/c and t186 = a2 dp/c
// + a1 dq with one 1/c, and the pressure term inside F[1]'s halving (a
// scaling by 1/2 is exact, so half(a) + half(b) = half(a + b)).
template <class T>
__device__ __forceinline__ void roe_flux(const T uN[kNS], const T uK[kNS], bool s, const OpsT<T>& o, T F[kNS]) {
  T rN = uN[0], rK = uK[0];
  // One reciprocal square root s2 = 1/sqrt(rho_N rho_K) gives both inverse
  // densities (rho_K s2^2, rho_N s2^2) and the Roe weight sqrt(rho_N/rho_K)
  // = rho_N s2.
  T s2 = rsqrt_(rN * rK);
  T ip = s2 * s2;
  T irN = rK * ip, irK = rN * ip;
  T vN[3] = {uN[1] * irN, uN[2] * irN, uN[3] * irN};
  T vK[3] = {uK[1] * irK, uK[2] * irK, uK[3] * irK};
  T qN = sgn(s, vN[0]), qK = sgn(s, vK[0]);
  // p = g1 E - (g1/2) |m|^2 / rho, with |m|^2 / rho = m.v
  T pN = o.g1 * uN[4] - o.hg1 * (uN[1] * vN[0] + uN[2] * vN[1] + uN[3] * vN[2]);
  T pK = o.g1 * uK[4] - o.hg1 * (uK[1] * vK[0] + uK[2] * vK[1] + uK[3] * vK[2]);
  T EpN = uN[4] + pN, EpK = uK[4] + pK;
  // Products that several sums use are pinned (mul_rn): see mul_rn.
  T sq = mul_rn(rN, s2);
  T is1 = rcp(sq + o.one);
  T vt[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) vt[i] = mul_rn(fma(sq, vN[i], vK[i]), is1);
  T Ht = mul_rn(fma(sq, EpN * irN, EpK * irK), is1);
  T hv2 = half_rn(fma(vt[2], vt[2], fma(vt[1], vt[1], vt[0] * vt[0])));
  T qt = sgn(s, vt[0]);
  T c2 = o.g1 * (Ht - hv2);
  T ic = rsqrt_(c2);  // 1/c
  T c = mul_rn(c2, ic);
  T l0 = fabs(qt);
  // eigenvalue combinations a1 = (|qt+c| + |c-qt|)/2 - |qt|, a2 = (|qt+c| - |c-qt|)/2
  T A = fabs(qt + c), B = fabs(c - qt);
  T a1 = half_(A + B) - l0, a2 = half_(A - B);
  T dr = rN - rK;
  T dm[3] = {uN[1] - uK[1], uN[2] - uK[2], uN[3] - uK[3]};
  T dE = uN[4] - uK[4];
  T dp = o.g1 * (hv2 * dr - (vt[0] * dm[0] + vt[1] * dm[1] + vt[2] * dm[2]) + dE);
  T dq = sgn(s, dm[0]) - qt * dr;
  T dpi = dp * ic;
  T t179 = mul_rn(fma(a1, dpi, a2 * dq), ic);
  T t186 = a2 * dpi + a1 * dq;
  F[0] = half_(rN * qN + rK * qK - l0 * dr - t179);
  F[1] = half_(uN[1] * qN + uK[1] * qK - l0 * dm[0] - t179 * vt[0] + sgn(s, pN + pK - t186));
#pragma unroll
  for (int i = 1; i < 3; ++i) F[1 + i] = half_(uN[1 + i] * qN + uK[1 + i] * qK - l0 * dm[i] - t179 * vt[i]);
  F[4] = half_(EpN * qN + EpK * qK - l0 * dE - t179 * Ht - t186 * qt);
}

}  // namespace ldg
