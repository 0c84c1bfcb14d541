// Host-side 1-D operators of the tensor-product LDG discretisation.
//
// The reference builds dense 3-D operators (Interp3D, Mel, Sels, Kels,
// Kels2D; Local-DG solver.cpp:74-192, dgMath.cpp:37-615) on the nodal
// Chebyshev-Gauss-Lobatto (CGL) basis with a (p+1)-point Gauss-Legendre
// rule.  All of them are tensor products of 1-D factors, and the mass matrix
// is exact, so the same discrete operator can be written in the basis of
// Lagrange polynomials at the Gauss points ("Gauss space"), where the mass
// matrix is diagonal (J * w_q).  This header holds the 1-D factors that the
// device kernels apply by sum factorisation:
//
//   B[q][i]   = phi_i(x_q)        CGL nodal basis at Gauss point q
//                                 (the 1-D factor of Interp3D/Interp2D)
//   Bi[i][q]  = L_q(xi_i)         inverse of B (Gauss basis at CGL nodes)
//   A[q][r]   = (w_r/w_q) L_q'(x_r)
//                                 weak derivative W^-1 D^T W: the 1-D factor
//                                 of Mel^-1 * Sels / Mel^-1 * Kels^T
//   lp/lm[q]  = L_q(+1) / L_q(-1) face trace (the 1-D factor of Interp2D on
//                                 a face, seen from the Gauss values)
//   Lp/Lm[q]  = L_q(+-1) / w_q    face lift (the 1-D factor of
//                                 Mel^-1 * Kels2D^T scattered to a face)
//
// Everything is evaluated in long double from product-form Lagrange
// formulas and rounded once to double.
#pragma once
#include <vector>

namespace ldg {

constexpr int kMaxN = 8;  // p <= 7

struct Ops1D {
  int N = 0;
  double xi[kMaxN];        // CGL nodes cos((p-i)pi/p), ascending
  double x[kMaxN];         // Gauss-Legendre points, ascending
  double w[kMaxN];         // Gauss-Legendre weights
  double B[kMaxN * kMaxN];
  double Bi[kMaxN * kMaxN];
  double A[kMaxN * kMaxN];
  double lp[kMaxN], lm[kMaxN];
  double Lp[kMaxN], Lm[kMaxN];
  double D[kMaxN * kMaxN];  // D[q][r] = L_r'(x_q): Gauss differentiation
};

// Builds the 1-D operators for order p (1 <= p <= 7). Returns false on a
// bad order.
bool build_ops1d(int p, Ops1D* out);

}  // namespace ldg
