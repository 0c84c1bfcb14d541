// Device-side pieces shared by the LDG kernels: operator block, mesh
// neighbour map, pointwise fluxes.
//
// Pointwise physics restated from Local-DG solver.cpp (fluxC 1040-1086,
// fluxV 1089-1188, numericalFluxC 1194-1374, numericalFluxV 891-921,
// numericalFluxL 867-884).  Normals are the mesh's axis unit vectors
// (mesh.cpp:338-353), so the normal dot products reduce to one signed
// component; adding the exact zeros the reference adds changes no bit.
#pragma once
#include <cstdint>

namespace ldg {

constexpr int kNS = 5;     // conserved variables (solver.cpp:61)
constexpr int kNQ = 15;    // gradient components: 3 directions x 5 vars
constexpr int kDevMaxN = 8;

// Everything a kernel needs about the discretisation; passed by value.
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

// Non-finite test on the exponent bits (integer pipe, not the FP64 pipe).
__device__ __forceinline__ bool not_finite(double x) {
  return (__double_as_longlong(x) & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
}

// Euler flux, column l of F(u): components (rho, m_x, m_y, m_z, E) of the
// flux in direction l (solver.cpp:1060-1084 with fluxes[iS + 5 l]).
// ir = 1/rho; p = g1 (E - |m|^2/(2 rho)); energy flux m_l (E + p)/rho, with
// E + p written gamma E - g1|m|^2/(2rho) as the reference does.
struct Euler {
  double ir, p, h;  // 1/rho, pressure, (E+p)/rho
};

__device__ __forceinline__ Euler euler_state(const double u[kNS], double g1, double gamma) {
  Euler s;
  s.ir = 1.0 / u[0];
  double k = (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) * s.ir * (0.5 * g1);
  s.p = g1 * u[4] - k;
  s.h = (gamma * u[4] - k) * s.ir;
  return s;
}

__device__ __forceinline__ void euler_column(const double u[kNS], const Euler& s, int l,
                                             double F[kNS]) {
  double ml = u[1 + l];
  double vl = ml * s.ir;
  F[0] = ml;
  F[1] = u[1] * vl;
  F[2] = u[2] * vl;
  F[3] = u[3] * vl;
  F[1 + l] += s.p;
  F[4] = ml * s.h;
}

// Velocity gradient G[i][j] = d_j v_i from u and Du[c], c = j*5 + var
// (the chain rule of solver.cpp:1137-1170), plus d_j e with
// e = E/rho - |v|^2/2 the specific internal energy.
struct ViscPre {
  double v[3];
  double G[3][3];
  double de[3];
  double div;
};

__device__ __forceinline__ void visc_pre(const double u[kNS], const double* Du, ViscPre& P) {
  double ir = 1.0 / u[0];
  P.v[0] = u[1] * ir;
  P.v[1] = u[2] * ir;
  P.v[2] = u[3] * ir;
  double eo = u[4] * ir;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double dr = Du[j * kNS + 0];
#pragma unroll
    for (int i = 0; i < 3; ++i) P.G[i][j] = (Du[j * kNS + 1 + i] - dr * P.v[i]) * ir;
    P.de[j] = (Du[j * kNS + 4] - dr * eo) * ir -
              (P.v[0] * P.G[0][j] + P.v[1] * P.G[1][j] + P.v[2] * P.G[2][j]);
  }
  P.div = P.G[0][0] + P.G[1][1] + P.G[2][2];
}

// Column j of the viscous flux (solver.cpp:1136-1187): Newtonian stress with
// Stokes' hypothesis over Re, heat flux (gamma/Pr) grad e / Re.
template <int j>
__device__ __forceinline__ void visc_column(const ViscPre& P, double inv_re,
                                            double kappa, double F[kNS]) {
  double tau[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) tau[i] = P.G[i][j] + P.G[j][i];
  tau[j] -= (2.0 / 3.0) * P.div;
  F[0] = 0.0;
  F[1] = tau[0] * inv_re;
  F[2] = tau[1] * inv_re;
  F[3] = tau[2] * inv_re;
  F[4] = (tau[0] * P.v[0] + tau[1] * P.v[1] + tau[2] * P.v[2] + kappa * P.de[j]) * inv_re;
}

// Roe flux F*(uN, uK, n) seen from element K with n = s e_l
// (numericalFluxC, solver.cpp:1291-1372): central flux minus Roe-averaged
// upwind dissipation; the reference's hard-coded 0.4 is g1.
template <int l>
__device__ __forceinline__ void roe_flux(const double uN[kNS], const double uK[kNS], double s,
                                         double g1, double F[kNS]) {
  double rN = uN[0], rK = uK[0];
  double irN = 1.0 / rN, irK = 1.0 / rK;
  double vN[3] = {uN[1] * irN, uN[2] * irN, uN[3] * irN};
  double vK[3] = {uK[1] * irK, uK[2] * irK, uK[3] * irK};
  double qN = s * vN[l], qK = s * vK[l];
  double pN = g1 * uN[4] - (0.5 * g1) * rN * (vN[0] * vN[0] + vN[1] * vN[1] + vN[2] * vN[2]);
  double pK = g1 * uK[4] - (0.5 * g1) * rK * (vK[0] * vK[0] + vK[1] * vK[1] + vK[2] * vK[2]);
  double sq = sqrt(rN * irK);
  double is1 = 1.0 / (sq + 1.0);
  double vt[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) vt[i] = (sq * vN[i] + vK[i]) * is1;
  double Ht = (sq * (uN[4] + pN) * irN + (uK[4] + pK) * irK) * is1;
  double vt2 = vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2];
  double qt = s * vt[l];
  double c2 = g1 * (Ht - 0.5 * vt2);
  double ic2 = 1.0 / c2;
  double c = sqrt(c2);
  double ic = c * ic2;  // 1/c
  double l0 = fabs(qt);
  double lp = 0.5 * fabs(qt + c), lm = 0.5 * fabs(c - qt);
  double dr = rN - rK;
  double dm[3] = {uN[1] - uK[1], uN[2] - uK[2], uN[3] - uK[3]};
  double dE = uN[4] - uK[4];
  double a1 = lp + lm - l0, a2 = lp - lm;
  double dp = g1 * (0.5 * vt2 * dr - (vt[0] * dm[0] + vt[1] * dm[1] + vt[2] * dm[2]) + dE);
  double dq = -qt * dr + s * dm[l];
  double t179 = a1 * dp * ic2 + a2 * dq * ic;
  double t186 = a2 * dp * ic + a1 * dq;
  F[0] = 0.5 * (rN * qN + rK * qK - l0 * dr - t179);
#pragma unroll
  for (int i = 0; i < 3; ++i)
    F[1 + i] = 0.5 * (uN[1 + i] * qN + uK[1 + i] * qK - l0 * dm[i] - t179 * vt[i]);
  F[1 + l] += 0.5 * s * (pN + pK - t186);
  F[4] = 0.5 * ((uN[4] + pN) * qN + (uK[4] + pK) * qK - l0 * dE - t179 * Ht - t186 * qt);
}

}  // namespace ldg
