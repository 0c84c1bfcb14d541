#include "ldg_ops.hpp"

#include <cmath>

namespace ldg {
namespace {

typedef long double ld;

const ld kPi = 3.141592653589793238462643383279502884L;

// Legendre P_n(x) and P_n'(x) by the three-term recurrence.
void legendre_pn(int n, ld x, ld* P, ld* dP) {
  ld p0 = 1, p1 = x;
  if (n == 0) { *P = 1; *dP = 0; return; }
  for (int k = 2; k <= n; ++k) {
    ld p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  *P = p1;
  *dP = n * (x * p1 - p0) / (x * x - 1);
}

// Gauss-Legendre nodes/weights by Newton iteration on P_N (the rule the
// reference obtains from the Golub-Welsch eigenproblem, dgMath.cpp:91-114).
void gauss_legendre(int N, ld* x, ld* w) {
  for (int i = 0; i < N; ++i) {
    ld z = cosl(kPi * (i + 0.75L) / (N + 0.5L));
    for (int it = 0; it < 100; ++it) {
      ld P, dP;
      legendre_pn(N, z, &P, &dP);
      ld dz = P / dP;
      z -= dz;
      if (fabsl(dz) < 1e-30L) break;
    }
    ld P, dP;
    legendre_pn(N, z, &P, &dP);
    x[N - 1 - i] = z;  // ascending
    w[N - 1 - i] = 2 / ((1 - z * z) * dP * dP);
  }
}

// Lagrange basis polynomial j on nodes[0..N) evaluated at t (product form).
ld lagrange(int N, const ld* nodes, int j, ld t) {
  ld v = 1;
  for (int k = 0; k < N; ++k)
    if (k != j) v *= (t - nodes[k]) / (nodes[j] - nodes[k]);
  return v;
}

// Derivative of Lagrange basis polynomial j at t.
ld dlagrange(int N, const ld* nodes, int j, ld t) {
  ld s = 0;
  for (int m = 0; m < N; ++m) {
    if (m == j) continue;
    ld v = 1 / (nodes[j] - nodes[m]);
    for (int k = 0; k < N; ++k)
      if (k != j && k != m) v *= (t - nodes[k]) / (nodes[j] - nodes[k]);
    s += v;
  }
  return s;
}

}  // namespace

bool build_ops1d(int p, Ops1D* o) {
  if (p < 1 || p > kMaxN - 1) return false;
  const int N = p + 1;
  o->N = N;
  ld xi[kMaxN], x[kMaxN], w[kMaxN];
  for (int i = 0; i <= p; ++i) xi[i] = cosl((p - i) * kPi / p);  // dgMath.cpp:37-45
  gauss_legendre(N, x, w);
  ld D[kMaxN][kMaxN];
  for (int q = 0; q < N; ++q)
    for (int r = 0; r < N; ++r) D[q][r] = dlagrange(N, x, r, x[q]);
  for (int i = 0; i < N; ++i) {
    o->xi[i] = (double)xi[i];
    o->x[i] = (double)x[i];
    o->w[i] = (double)w[i];
  }
  for (int q = 0; q < N; ++q) {
    for (int i = 0; i < N; ++i) {
      o->B[q * N + i] = (double)lagrange(N, xi, i, x[q]);
      o->Bi[i * N + q] = (double)lagrange(N, x, q, xi[i]);
    }
    for (int r = 0; r < N; ++r) {
      o->A[q * N + r] = (double)((w[r] / w[q]) * D[r][q]);
      o->D[q * N + r] = (double)D[q][r];
    }
    ld lpq = lagrange(N, x, q, 1.0L), lmq = lagrange(N, x, q, -1.0L);
    o->lp[q] = (double)lpq;
    o->lm[q] = (double)lmq;
    o->Lp[q] = (double)(lpq / w[q]);
    o->Lm[q] = (double)(lmq / w[q]);
  }
  return true;
}

}  // namespace ldg
