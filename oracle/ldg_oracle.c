/*
 * ldg_oracle.c -- CPU restatement of the Local-DG reference hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests/, the smoke check in
 * __graft_entry__.py and bench.py's CPU-baseline leg call it as the checker
 * or as the timed CPU baseline.  The product path (local-dg_gb300/) never
 * links, loads or falls back to it.
 *
 * It restates, in plain C with the reference's dense-operator structure,
 * the RK4 right-hand side of the LDG discretisation of 3-D compressible
 * Navier-Stokes on a periodic uniform hex mesh (Local-DG solver.cpp).  Each
 * function names the reference lines it follows.  Layout is the reference's
 * column-major darray: u(node, var, elem), node = ix + N*iy + N*N*iz.
 *
 * Dense GEMMs and the mass-matrix LDL^T solve run on project-written loops
 * (OpenMP over columns).  Optionally ldgo_use_openblas() routes them to an
 * OpenBLAS shared library (the same BLAS/LAPACK calls the reference makes,
 * solver.cpp:500-506,532-533,560-572,736-738,859-861), which is how the CPU
 * baseline reproduces the reference's threaded-BLAS cost profile.
 *
 * Parity pin: outputs are checked against golden vectors produced by the
 * unmodified reference sources (oracle/build_ref.sh + oracle/ref_driver.cpp)
 * in tests/golden/.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define NS 5    /* conserved variables (solver.cpp:61) */
#define DIM 3
#define NF 6    /* faces per element, ordered -x,+x,-y,+y,-z,+z (mesh.h:143-147) */

typedef void (*dgemm_fn)(int, int, int, int, int, int, double, const double*, int, const double*,
                         int, double, double*, int);
typedef int (*dsytrf_fn)(int, char, int, double*, int, int*);
typedef int (*dsytrs_fn)(int, char, int, int, const double*, int, const int*, double*, int);
typedef void (*setthreads_fn)(int);

typedef struct ldgo {
  int p, N, n, nf, nx, ny, nz, nE;
  double L, minDX, minDY, minDZ, alpha[DIM], J;
  /* physics (solver.cpp:30-43) */
  double Re, Pr, gamma, M0, R, rho0, V0, c0, p0, T0;
  double dt;
  long timesteps;
  /* operators (solver.cpp:74-192) */
  double *Interp2D; /* nf x nf   */
  double *Interp3D; /* n x n     */
  double *Mel;      /* n x n, factored in place */
  int *Mipiv;
  double *Sels;     /* n x n x 3 */
  double *Kels;     /* n x n x 3 */
  double *Kels2D;   /* nf x nf x 3 */
  double *wQ3;      /* n */
  int *efToN;       /* nf x 6 */
  int *eToE;        /* 6 x nE, periodic neighbour (ghost slots resolved) */
  /* work arrays (solver.cpp:318-325) */
  double *uCurr, *uInterp2D, *uInterp3D, *ks, *Dus, *DuInterp2D, *DuInterp3D, *onFaces, *flx;
  /* 1-D factors (N x N, row-major out x in) of the dense operators above;
   * on a uniform hex mesh every one of them is a Kronecker product of
   * these (see ldgo_set_factored). */
  double I1[64], IWt[64], DWt[64], M1[64], S1[64], M1i[64];
  int factored;
  /* optional OpenBLAS */
  void *blas;
  dgemm_fn dgemm;
  dsytrf_fn dsytrf;
  dsytrs_fn dsytrs;
  int threads;
} ldgo;

/* ---------------------------------------------------------------- BLAS-like */

/* C = alpha*op(A)*B + beta*C, column-major; op(A) = A (ta=0) or A^T (ta=1). */
static void gemm(const ldgo* o, int ta, int M, int Ncol, int K, double alpha, const double* A,
                 int lda, const double* B, int ldb, double beta, double* C, int ldc) {
  if (o && o->dgemm) {
    o->dgemm(102, ta ? 112 : 111, 111, M, Ncol, K, alpha, A, lda, B, ldb, beta, C, ldc);
    return;
  }
  long j;
#pragma omp parallel for schedule(static) if (Ncol > 64)
  for (j = 0; j < Ncol; ++j) {
    double* c = C + (long)j * ldc;
    const double* b = B + (long)j * ldb;
    if (beta == 0.0) {
      for (int i = 0; i < M; ++i) c[i] = 0.0;
    } else if (beta != 1.0) {
      for (int i = 0; i < M; ++i) c[i] *= beta;
    }
    if (!ta) {
      for (int k = 0; k < K; ++k) {
        double bk = alpha * b[k];
        const double* a = A + (long)k * lda;
        for (int i = 0; i < M; ++i) c[i] += a[i] * bk;
      }
    } else {
      for (int i = 0; i < M; ++i) {
        const double* a = A + (long)i * lda;
        double s = 0.0;
        for (int k = 0; k < K; ++k) s += a[k] * b[k];
        c[i] += alpha * s;
      }
    }
  }
}

/* LU with partial pivoting; solves A X = B in place (B: n x nrhs).  Used for
 * the Vandermonde inverses the reference obtains from LAPACKE_dgesv
 * (solver.cpp:109-111, dgMath.cpp:522-524,560-562,600-602). */
static int lu_solve(int n, double* A, int nrhs, double* B) {
  int* piv = (int*)malloc(sizeof(int) * n);
  for (int k = 0; k < n; ++k) {
    int pr = k;
    double mx = fabs(A[k + k * n]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[i + k * n]) > mx) { mx = fabs(A[i + k * n]); pr = i; }
    piv[k] = pr;
    if (mx == 0.0) { free(piv); return -1; }
    if (pr != k) {
      for (int j = 0; j < n; ++j) { double t = A[k + j * n]; A[k + j * n] = A[pr + j * n]; A[pr + j * n] = t; }
      for (int j = 0; j < nrhs; ++j) { double t = B[k + j * n]; B[k + j * n] = B[pr + j * n]; B[pr + j * n] = t; }
    }
    for (int i = k + 1; i < n; ++i) {
      double f = A[i + k * n] / A[k + k * n];
      A[i + k * n] = f;
      for (int j = k + 1; j < n; ++j) A[i + j * n] -= f * A[k + j * n];
      for (int j = 0; j < nrhs; ++j) B[i + j * n] -= f * B[k + j * n];
    }
  }
  for (int j = 0; j < nrhs; ++j) {
    double* b = B + (long)j * n;
    for (int i = n - 1; i >= 0; --i) {
      double s = b[i];
      for (int k = i + 1; k < n; ++k) s -= A[i + k * n] * b[k];
      b[i] = s / A[i + i * n];
    }
  }
  free(piv);
  return 0;
}

/* Mass-matrix factorisation.  The reference uses Bunch-Kaufman LDL^T
 * (LAPACKE_dsytrf 'U', solver.cpp:155-156).  Mel is symmetric positive
 * definite, so the restatement uses LDL^T without pivoting, M = U^T D U
 * with U unit upper triangular (stored above the diagonal, D on it). */
static void ldl_factor(int n, double* A) {
  for (int j = 0; j < n; ++j) {
    double d = A[j + j * n];
    for (int k = 0; k < j; ++k) d -= A[k + j * n] * A[k + j * n] * A[k + k * n];
    A[j + j * n] = d;
    for (int i = j + 1; i < n; ++i) {
      double s = A[j + i * n];
      for (int k = 0; k < j; ++k) s -= A[k + j * n] * A[k + i * n] * A[k + k * n];
      A[j + i * n] = s / d;
    }
  }
}

/* Solve M X = B for nrhs columns (LAPACKE_dsytrs, solver.cpp:505-506,532-533). */
static void mass_solve(const ldgo* o, double* B, long nrhs) {
  int n = o->n;
  if (o->dsytrs) {
    o->dsytrs(102, 'U', n, (int)nrhs, o->Mel, n, o->Mipiv, B, n);
    return;
  }
  const double* A = o->Mel;
  long j;
#pragma omp parallel for schedule(static)
  for (j = 0; j < nrhs; ++j) {
    double* b = B + j * n;
    for (int i = 0; i < n; ++i) { /* U^T y = b */
      double s = b[i];
      for (int k = 0; k < i; ++k) s -= A[k + i * n] * b[k];
      b[i] = s;
    }
    for (int i = 0; i < n; ++i) b[i] /= A[i + i * n];
    for (int i = n - 1; i >= 0; --i) { /* U x = z */
      double s = b[i];
      for (int k = i + 1; k < n; ++k) s -= A[i + k * n] * b[k];
      b[i] = s;
    }
  }
}

/* ---------------------------------------------------------- dgMath restated */

/* Chebyshev-Gauss-Lobatto points cos((p-i)pi/p) (dgMath.cpp:37-45). */
static void chebyshev(int p, double* x) {
  for (int i = 0; i <= p; ++i) x[i] = cos((p - i) * M_PI / p);
}

/* Cyclic Jacobi eigenvalue iteration on a small symmetric matrix (Jacobi
 * 1846; Golub & Van Loan sec. 8.5).  A is n x n column-major, destroyed;
 * V receives eigenvectors in columns; eigenvalues sorted ascending. */
static void sym_eig(int n, double* A, double* V, double* lam) {
  for (int i = 0; i < n * n; ++i) V[i] = 0.0;
  for (int i = 0; i < n; ++i) V[i + i * n] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int q = 0; q < n; ++q)
      for (int pp = 0; pp < q; ++pp) off += A[pp + q * n] * A[pp + q * n];
    if (off < 1e-300) break;
    for (int pp = 0; pp < n; ++pp)
      for (int q = pp + 1; q < n; ++q) {
        double apq = A[pp + q * n];
        if (apq == 0.0) continue;
        double app = A[pp + pp * n], aqq = A[q + q * n];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) { /* A <- A J */
          double akp = A[k + pp * n], akq = A[k + q * n];
          A[k + pp * n] = c * akp - s * akq;
          A[k + q * n] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) { /* A <- J^T A */
          double apk = A[pp + k * n], aqk = A[q + k * n];
          A[pp + k * n] = c * apk - s * aqk;
          A[q + k * n] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k + pp * n], vkq = V[k + q * n];
          V[k + pp * n] = c * vkp - s * vkq;
          V[k + q * n] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) lam[i] = A[i + i * n];
  for (int i = 0; i < n; ++i) /* selection sort ascending, carrying vectors */
    for (int j = i + 1; j < n; ++j)
      if (lam[j] < lam[i]) {
        double t = lam[i]; lam[i] = lam[j]; lam[j] = t;
        for (int k = 0; k < n; ++k) { t = V[k + i * n]; V[k + i * n] = V[k + j * n]; V[k + j * n] = t; }
      }
}

/* Gauss-Legendre rule exact to degree p via the Golub-Welsch eigenproblem of
 * the Jacobi matrix (dgMath.cpp:91-114): n = ceil((p+1)/2) points. */
static int gauss_quad(int p, double* x, double* w) {
  int n = (int)ceil((p + 1) / 2.0);
  double* T = (double*)calloc((size_t)n * n, sizeof(double));
  double* V = (double*)calloc((size_t)n * n, sizeof(double));
  for (int i = 0; i < n - 1; ++i) {
    double b = (i + 1) / sqrt(4.0 * (i + 1) * (i + 1) - 1);
    T[i + (i + 1) * n] = b;
    T[(i + 1) + i * n] = b;
  }
  sym_eig(n, T, V, x);
  for (int i = 0; i < n; ++i) w[i] = 2 * V[0 + i * n] * V[0 + i * n];
  free(T);
  free(V);
  return n;
}

/* Legendre polynomials 0..p and derivatives at nx points, (nx, p+1) column
 * major, by the three-term recurrences of dgMath.cpp:177-248. */
static void legendre(int p, int nx, const double* x, double* P, double* dP) {
  for (int i = 0; i < nx; ++i) { P[i] = 1.0; if (dP) dP[i] = 0.0; }
  if (p == 0) return;
  for (int i = 0; i < nx; ++i) { P[i + nx] = x[i]; if (dP) dP[i + nx] = 1.0; }
  for (int ip = 0; ip < p - 1; ++ip)
    for (int i = 0; i < nx; ++i) {
      P[i + (ip + 2) * nx] = ((2 * ip + 3) * x[i] * P[i + (ip + 1) * nx] - (ip + 1) * P[i + ip * nx]) / (ip + 2);
      if (dP)
        dP[i + (ip + 2) * nx] = ((2 * ip + 3) * (x[i] * dP[i + (ip + 1) * nx] + P[i + (ip + 1) * nx]) -
                                 (ip + 1) * dP[i + ip * nx]) / (ip + 2);
    }
}

/* Tensor-product Legendre basis on a tensor grid of 1-D points x (m per
 * direction), d = 2 or 3 dimensions: out(pt, mode) with pt and mode both
 * x-fastest (dgMath.cpp:254-294, 361-411).  deriv = -1 for values, or the
 * differentiated direction (dgMath.cpp:300-355, 417-501). */
static void legendre_nd(int p, int d, int m, const double* x, int deriv, double* out) {
  int N = p + 1;
  double* P = (double*)malloc(sizeof(double) * m * N);
  double* dP = (double*)malloc(sizeof(double) * m * N);
  legendre(p, m, x, P, dP);
  int npts = d == 2 ? m * m : m * m * m;
  int nmod = d == 2 ? N * N : N * N * N;
  for (int md = 0; md < nmod; ++md) {
    int mi[3] = {md % N, (md / N) % N, md / (N * N)};
    for (int pt = 0; pt < npts; ++pt) {
      int pi[3] = {pt % m, (pt / m) % m, pt / (m * m)};
      double v = 1.0;
      for (int l = 0; l < d; ++l) v *= (l == deriv ? dP : P)[pi[l] + mi[l] * m];
      out[pt + (long)md * npts] = v;
    }
  }
  free(P);
  free(dP);
}

/* Interpolation matrix from the tensor CGL nodes to the tensor Gauss points
 * in d dimensions: lTo * inv(lFrom) (dgMath.cpp:545-615). */
static void interp_matrix(int p, int d, const double* xFrom, int mTo, const double* xTo, double* I) {
  int N = p + 1;
  int nFrom = d == 2 ? N * N : N * N * N;
  int nTo = d == 2 ? mTo * mTo : mTo * mTo * mTo;
  double* lFrom = (double*)malloc(sizeof(double) * nFrom * nFrom);
  double* coeffs = (double*)calloc((size_t)nFrom * nFrom, sizeof(double));
  double* lTo = (double*)malloc(sizeof(double) * nTo * nFrom);
  legendre_nd(p, d, N, xFrom, -1, lFrom);
  for (int i = 0; i < nFrom; ++i) coeffs[i + i * nFrom] = 1.0;
  lu_solve(nFrom, lFrom, nFrom, coeffs);
  legendre_nd(p, d, mTo, xTo, -1, lTo);
  gemm(NULL, 0, nTo, nFrom, nFrom, 1.0, lTo, nTo, coeffs, nFrom, 0.0, I, nTo);
  free(lFrom);
  free(coeffs);
  free(lTo);
}

/* Face-node map (mesh.cpp:428-501): face f of every element, point
 * j = a + m*b over its two tangential directions in increasing order. */
static void face_map(int m, int* ef) {
  int nf = m * m;
  for (int f = 0; f < NF; ++f) {
    int l = f / 2, end = (f % 2) ? m - 1 : 0;
    for (int b = 0; b < m; ++b)
      for (int a = 0; a < m; ++a) {
        int c[3];
        c[l] = end;
        c[l == 0 ? 1 : 0] = a;
        c[l == 2 ? 1 : 2] = b;
        ef[a + m * b + nf * f] = c[0] + m * c[1] + m * m * c[2];
      }
  }
}

/* ----------------------------------------------------------------- setup */

/* 1-D factors of the reference operators.  The basis is the tensor product
 * of the 1-D Lagrange polynomials l_a on the CGL nodes (the reference builds
 * it as Legendre modes times the inverse Vandermonde, dgMath.cpp:545-615),
 * and the quadrature is the tensor Gauss rule, so on a uniform hex
 * (constant diagonal Jacobian) every dense operator of solver.cpp:74-192 is
 * a Kronecker product of
 *   I1[q][a]  = l_a(x_q)                      (Interp3D = I1^3, Interp2D = I1^2)
 *   IWt[a][q] = l_a(x_q) w_q                  (Kels_l, Kels2D_l: test side)
 *   DWt[a][q] = l_a'(x_q) w_q                 (Kels_l along l)
 *   M1 = I1^T W I1                            (Mel = J M1^3)
 *   S1 = D1^T W I1                            (Sels_l = J/alpha_l S1 (x) M1 (x) M1, S1 along l)
 * with M1i = M1^-1.  Row-major out x in. */
static void setup_factors(ldgo* o, const double* cheb, const double* xq, const double* wq) {
  int p = o->p, N = p + 1;
  double P[64], Pq[64], dPq[64], C[64], D1[64];
  legendre(p, N, cheb, P, NULL);
  legendre(p, N, xq, Pq, dPq);
  for (int i = 0; i < N * N; ++i) C[i] = 0.0;
  for (int i = 0; i < N; ++i) C[i + i * N] = 1.0;
  lu_solve(N, P, N, C); /* C = inverse Vandermonde, column-major */
  for (int q = 0; q < N; ++q)
    for (int a = 0; a < N; ++a) {
      double v = 0.0, d = 0.0;
      for (int m = 0; m < N; ++m) {
        v += Pq[q + m * N] * C[m + a * N];
        d += dPq[q + m * N] * C[m + a * N];
      }
      o->I1[q * N + a] = v;
      D1[q * N + a] = d;
    }
  for (int a = 0; a < N; ++a)
    for (int q = 0; q < N; ++q) {
      o->IWt[a * N + q] = o->I1[q * N + a] * wq[q];
      o->DWt[a * N + q] = D1[q * N + a] * wq[q];
    }
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b) {
      double m = 0.0, sd = 0.0;
      for (int q = 0; q < N; ++q) {
        m += o->I1[q * N + a] * wq[q] * o->I1[q * N + b];
        sd += D1[q * N + a] * wq[q] * o->I1[q * N + b];
      }
      o->M1[a * N + b] = m;
      o->S1[a * N + b] = sd;
    }
  double Mc[64], Mi[64];
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b) { Mc[a + b * N] = o->M1[a * N + b]; Mi[a + b * N] = a == b; }
  lu_solve(N, Mc, N, Mi);
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b) o->M1i[a * N + b] = Mi[a + b * N];
}

void ldgo_destroy(ldgo* o);

static int ldgo_setup(ldgo* o) {
  int p = o->p, N = p + 1, n = N * N * N, nf = N * N, nE = o->nE;
  o->N = N; o->n = n; o->nf = nf;
  double cheb[16], xq[16], wq[16];
  chebyshev(p, cheb);
  int nq = gauss_quad(2 * p, xq, wq);
  if (nq != N) return -2;
  /* Interp2D, Interp3D (solver.cpp:74-92) */
  o->Interp2D = (double*)malloc(sizeof(double) * nf * nf);
  o->Interp3D = (double*)malloc(sizeof(double) * n * n);
  interp_matrix(p, 2, cheb, N, xq, o->Interp2D);
  interp_matrix(p, 3, cheb, N, xq, o->Interp3D);
  /* precomputeLocalMatrices (solver.cpp:95-192) */
  double* l3D = (double*)malloc(sizeof(double) * n * n);
  double* coeffs = (double*)calloc((size_t)n * n, sizeof(double));
  legendre_nd(p, 3, N, cheb, -1, l3D);
  for (int i = 0; i < n; ++i) coeffs[i + i * n] = 1.0;
  lu_solve(n, l3D, n, coeffs);
  double* polyQ = (double*)malloc(sizeof(double) * n * n);
  double* dpolyQ = (double*)malloc(sizeof(double) * n * n * DIM);
  legendre_nd(p, 3, N, xq, -1, polyQ);
  for (int l = 0; l < DIM; ++l) legendre_nd(p, 3, N, xq, l, dpolyQ + (long)l * n * n);
  double* phiQ = (double*)malloc(sizeof(double) * n * n);
  double* dphiQ = (double*)malloc(sizeof(double) * n * n * DIM);
  gemm(NULL, 0, n, n, n, 1.0, polyQ, n, coeffs, n, 0.0, phiQ, n);
  for (int l = 0; l < DIM; ++l)
    gemm(NULL, 0, n, n, n, 1.0, dpolyQ + (long)l * n * n, n, coeffs, n, 0.0, dphiQ + (long)l * n * n, n);
  o->wQ3 = (double*)malloc(sizeof(double) * n);
  for (int iz = 0; iz < N; ++iz)
    for (int iy = 0; iy < N; ++iy)
      for (int ix = 0; ix < N; ++ix) o->wQ3[ix + N * iy + N * N * iz] = wq[ix] * wq[iy] * wq[iz];
  for (int j = 0; j < n; ++j)
    for (int q = 0; q < n; ++q) polyQ[q + j * n] = phiQ[q + j * n] * o->wQ3[q];
  o->alpha[0] = o->minDX / 2.0;
  o->alpha[1] = o->minDY / 2.0;
  o->alpha[2] = o->minDZ / 2.0;
  o->J = o->alpha[0] * o->alpha[1] * o->alpha[2];
  o->Mel = (double*)malloc(sizeof(double) * n * n);
  o->Mipiv = (int*)calloc(n, sizeof(int));
  gemm(NULL, 1, n, n, n, o->J, polyQ, n, phiQ, n, 0.0, o->Mel, n);
  if (o->dsytrf)
    o->dsytrf(102, 'U', n, o->Mel, n, o->Mipiv);
  else
    ldl_factor(n, o->Mel);
  o->Sels = (double*)malloc(sizeof(double) * n * n * DIM);
  o->Kels = (double*)malloc(sizeof(double) * n * n * DIM);
  o->Kels2D = (double*)malloc(sizeof(double) * nf * nf * DIM);
  double w2[64];
  for (int b = 0; b < N; ++b)
    for (int a = 0; a < N; ++a) w2[a + N * b] = wq[a] * wq[b];
  for (int l = 0; l < DIM; ++l) {
    double scaleL = o->J / o->alpha[l];
    gemm(NULL, 1, n, n, n, scaleL, dphiQ + (long)l * n * n, n, polyQ, n, 0.0, o->Sels + (long)l * n * n, n);
    for (int i = 0; i < n; ++i)
      for (int q = 0; q < n; ++q)
        o->Kels[q + (long)i * n + (long)l * n * n] = dphiQ[q + (long)i * n + (long)l * n * n] * o->wQ3[q] * scaleL;
    for (int i = 0; i < nf; ++i)
      for (int q = 0; q < nf; ++q)
        o->Kels2D[q + i * nf + l * nf * nf] = o->Interp2D[q + i * nf] * w2[q] * scaleL;
  }
  free(l3D); free(coeffs); free(polyQ); free(dpolyQ); free(phiQ); free(dphiQ);
  setup_factors(o, cheb, xq, wq);
  /* Mesh connectivity (mesh.cpp:201-353): periodic neighbours directly. */
  o->efToN = (int*)malloc(sizeof(int) * nf * NF);
  face_map(N, o->efToN);
  o->eToE = (int*)malloc(sizeof(int) * NF * nE);
  for (int iz = 0; iz < o->nz; ++iz)
    for (int iy = 0; iy < o->ny; ++iy)
      for (int ix = 0; ix < o->nx; ++ix) {
        int e = ix + o->nx * (iy + o->ny * iz);
        int c[3] = {ix, iy, iz}, dims[3] = {o->nx, o->ny, o->nz};
        for (int f = 0; f < NF; ++f) {
          int cc[3] = {c[0], c[1], c[2]};
          int l = f / 2;
          cc[l] = (c[l] + ((f % 2) ? 1 : dims[l] - 1)) % dims[l];
          o->eToE[f + NF * e] = cc[0] + o->nx * (cc[1] + o->ny * cc[2]);
        }
      }
  long nU = (long)n * NS * nE;
  o->uCurr = (double*)calloc(nU, sizeof(double));
  o->uInterp2D = (double*)calloc((long)nf * NS * NF * nE, sizeof(double));
  o->uInterp3D = (double*)calloc(nU, sizeof(double));
  o->ks = (double*)calloc(nU * 4, sizeof(double));
  o->Dus = (double*)calloc(nU * DIM, sizeof(double));
  o->DuInterp2D = (double*)calloc((long)nf * NS * NF * nE * DIM, sizeof(double));
  o->DuInterp3D = (double*)calloc(nU * DIM, sizeof(double));
  o->onFaces = (double*)calloc((long)nf * NS * NF * nE * DIM, sizeof(double));
  o->flx = (double*)calloc(nU * DIM, sizeof(double));
  if (!o->uCurr || !o->ks || !o->Dus || !o->DuInterp2D || !o->DuInterp3D || !o->onFaces || !o->flx)
    return -3;
  return 0;
}

/* Solver constructor essentials (solver.cpp:7-71): physics, CFL dt rule. */
ldgo* ldgo_create(int nx, int ny, int nz, int p, double L, double tf, double Re, int threads) {
  if (nx < 3 || ny < 3 || nz < 3 || p < 1 || p > 7) return NULL; /* mesh.cpp:102-107 */
  ldgo* o = (ldgo*)calloc(1, sizeof(ldgo));
  o->p = p; o->nx = nx; o->ny = ny; o->nz = nz; o->nE = nx * ny * nz; o->L = L;
  o->threads = threads > 0 ? threads : 1;
#ifdef _OPENMP
  omp_set_num_threads(o->threads);
#endif
  o->Re = Re; o->Pr = .71; o->gamma = 1.4; o->M0 = 0.1; o->R = 8.314; o->rho0 = 1.0; o->V0 = 1.0;
  o->c0 = o->V0 / o->M0;
  o->p0 = o->rho0 * o->c0 * o->c0 / o->gamma;
  o->T0 = o->p0 / (o->R * o->rho0);
  double size = M_PI * L;
  o->minDX = (size - (-size)) / nx;
  o->minDY = (size - (-size)) / ny;
  o->minDZ = (size - (-size)) / nz;
  double maxVel = o->V0;
  double m = o->minDX < o->minDY ? o->minDX : o->minDY;
  m = m < o->minDZ ? m : o->minDZ;
  o->dt = 0.01 * m / (maxVel * (2 * p + 1));
  o->timesteps = (long)ceil(tf / o->dt);
  if (o->timesteps < 1) o->timesteps = 1;
  o->dt = tf / o->timesteps;
  if (ldgo_setup(o) != 0) { ldgo_destroy(o); return NULL; }
  return o;
}

/* Route GEMM and the mass solve to an OpenBLAS library (scipy's bundled
 * build exports scipy_-prefixed names).  Must be called before ldgo_create
 * of the solvers that should use it; returns 0 on success. */
static void* g_blas = NULL;
static dgemm_fn g_dgemm = NULL;
static dsytrf_fn g_dsytrf = NULL;
static dsytrs_fn g_dsytrs = NULL;
int ldgo_use_openblas(const char* path, int threads) {
  if (!path) { g_dgemm = NULL; g_dsytrf = NULL; g_dsytrs = NULL; return 0; }
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  const char* pre[2] = {"scipy_", ""};
  for (int i = 0; i < 2; ++i) {
    char b1[64], b2[64], b3[64], b4[64];
    snprintf(b1, 64, "%scblas_dgemm", pre[i]);
    snprintf(b2, 64, "%sLAPACKE_dsytrf", pre[i]);
    snprintf(b3, 64, "%sLAPACKE_dsytrs", pre[i]);
    snprintf(b4, 64, "%sopenblas_set_num_threads", pre[i]);
    dgemm_fn g = (dgemm_fn)dlsym(h, b1);
    dsytrf_fn f = (dsytrf_fn)dlsym(h, b2);
    dsytrs_fn s = (dsytrs_fn)dlsym(h, b3);
    setthreads_fn t = (setthreads_fn)dlsym(h, b4);
    if (g && f && s) {
      if (t) t(threads > 0 ? threads : 1);
      g_blas = h; g_dgemm = g; g_dsytrf = f; g_dsytrs = s;
      return 0;
    }
  }
  dlclose(h);
  return -2;
}

ldgo* ldgo_create_blas(int nx, int ny, int nz, int p, double L, double tf, double Re, int threads) {
  /* Same as ldgo_create but picks up the OpenBLAS routes (if loaded) before
   * the mass matrix is factored. */
  if (nx < 3 || ny < 3 || nz < 3 || p < 1 || p > 7) return NULL;
  ldgo* o = (ldgo*)calloc(1, sizeof(ldgo));
  o->p = p; o->nx = nx; o->ny = ny; o->nz = nz; o->nE = nx * ny * nz; o->L = L;
  o->threads = threads > 0 ? threads : 1;
#ifdef _OPENMP
  omp_set_num_threads(o->threads);
#endif
  o->dgemm = g_dgemm; o->dsytrf = g_dsytrf; o->dsytrs = g_dsytrs;
  o->Re = Re; o->Pr = .71; o->gamma = 1.4; o->M0 = 0.1; o->R = 8.314; o->rho0 = 1.0; o->V0 = 1.0;
  o->c0 = o->V0 / o->M0;
  o->p0 = o->rho0 * o->c0 * o->c0 / o->gamma;
  o->T0 = o->p0 / (o->R * o->rho0);
  double size = M_PI * L;
  o->minDX = (size - (-size)) / nx;
  o->minDY = (size - (-size)) / ny;
  o->minDZ = (size - (-size)) / nz;
  double m = o->minDX < o->minDY ? o->minDX : o->minDY;
  m = m < o->minDZ ? m : o->minDZ;
  o->dt = 0.01 * m / (o->V0 * (2 * p + 1));
  o->timesteps = (long)ceil(tf / o->dt);
  if (o->timesteps < 1) o->timesteps = 1;
  o->dt = tf / o->timesteps;
  if (ldgo_setup(o) != 0) { ldgo_destroy(o); return NULL; }
  return o;
}

void ldgo_destroy(ldgo* o) {
  if (!o) return;
  free(o->Interp2D); free(o->Interp3D); free(o->Mel); free(o->Mipiv); free(o->Sels);
  free(o->Kels); free(o->Kels2D); free(o->wQ3); free(o->efToN); free(o->eToE);
  free(o->uCurr); free(o->uInterp2D); free(o->uInterp3D); free(o->ks); free(o->Dus);
  free(o->DuInterp2D); free(o->DuInterp3D); free(o->onFaces); free(o->flx);
  free(o);
}

double ldgo_dt(const ldgo* o) { return o->dt; }
long ldgo_timesteps(const ldgo* o) { return o->timesteps; }
int ldgo_dofs(const ldgo* o) { return o->n; }
int ldgo_nelements(const ldgo* o) { return o->nE; }
void ldgo_set_dt(ldgo* o, double dt) { o->dt = dt; }

/* Copies the reference operators out for white-box tests:
 * which 0 Interp2D (nf*nf), 1 Interp3D (n*n), 2 Kels (n*n*3), 3 Kels2D
 * (nf*nf*3), 4 Sels (n*n*3), 5 wQ3 (n). */
int ldgo_get_operator(const ldgo* o, int which, double* out) {
  long n = o->n, nf = o->nf;
  switch (which) {
    case 0: memcpy(out, o->Interp2D, sizeof(double) * nf * nf); return 0;
    case 1: memcpy(out, o->Interp3D, sizeof(double) * n * n); return 0;
    case 2: memcpy(out, o->Kels, sizeof(double) * n * n * 3); return 0;
    case 3: memcpy(out, o->Kels2D, sizeof(double) * nf * nf * 3); return 0;
    case 4: memcpy(out, o->Sels, sizeof(double) * n * n * 3); return 0;
    case 5: memcpy(out, o->wQ3, sizeof(double) * n); return 0;
  }
  return -1;
}

/* Taylor-Green initial condition at the element nodes (solver.cpp:194-236,
 * node coordinates mesh.cpp:127-151,389-408), plus an optional velocity
 * perturbation amp * sum_{k=1..4} sum_d sin(k x_d / L + phi[c][k-1][d])
 * (ensemble inputs; phi as 36 doubles, amp = 0 for none). */
static void initial_condition_impl(const ldgo* o, double* u, double amp, const double* phi);
void ldgo_initial_condition(const ldgo* o, double* u) { initial_condition_impl(o, u, 0.0, NULL); }
void ldgo_initial_condition_perturbed(const ldgo* o, double* u, double amp, const double* phi) {
  initial_condition_impl(o, u, amp, phi);
}
static void initial_condition_impl(const ldgo* o, double* u, double amp, const double* phi) {
  int N = o->N, n = o->n, p = o->p;
  double cheb[16];
  chebyshev(p, cheb);
  double size = M_PI * o->L;
  double bl = -size, tr = size;
  for (int iz = 0; iz < o->nz; ++iz)
    for (int iy = 0; iy < o->ny; ++iy)
      for (int ix = 0; ix < o->nx; ++ix) {
        int k = ix + o->nx * (iy + o->ny * iz);
        double x0 = ix * (tr - bl) / o->nx + bl, x1 = (ix + 1) * (tr - bl) / o->nx + bl;
        double y0 = iy * (tr - bl) / o->ny + bl, y1 = (iy + 1) * (tr - bl) / o->ny + bl;
        double z0 = iz * (tr - bl) / o->nz + bl, z1 = (iz + 1) * (tr - bl) / o->nz + bl;
        for (int c = 0; c < N; ++c)
          for (int b = 0; b < N; ++b)
            for (int a = 0; a < N; ++a) {
              int v = a + N * b + N * N * c;
              double x = x0 + .5 * (cheb[a] + 1.0) * (x1 - x0);
              double y = y0 + .5 * (cheb[b] + 1.0) * (y1 - y0);
              double z = z0 + .5 * (cheb[c] + 1.0) * (z1 - z0);
              double L = o->L;
              double pr = o->p0 + (o->rho0 * o->V0 * o->V0 / 16.0) * (cos(2 * x / L) + cos(2 * y / L)) *
                                      (cos(2 * z / L) + 2);
              double* uk = u + (long)k * n * NS;
              uk[v + 0 * n] = pr / (o->R * o->T0);
              uk[v + 1 * n] = o->rho0 * o->V0 * sin(x / L) * cos(y / L) * cos(z / L);
              uk[v + 2 * n] = -o->rho0 * o->V0 * cos(x / L) * sin(y / L) * cos(z / L);
              uk[v + 3 * n] = 0 * o->rho0;
              if (amp != 0.0) {
                double X[3] = {x / L, y / L, z / L}, dv[3] = {0, 0, 0};
                for (int cpt = 0; cpt < 3; ++cpt)
                  for (int k = 1; k <= 4; ++k)
                    for (int d = 0; d < 3; ++d) dv[cpt] += sin(k * X[d] + phi[cpt * 12 + (k - 1) * 3 + d]);
                for (int cpt = 0; cpt < 3; ++cpt) uk[v + (1 + cpt) * n] += o->rho0 * amp * dv[cpt];
              }
              uk[v + 4 * n] = pr / (o->gamma - 1) + (uk[v + 1 * n] * uk[v + 1 * n] + uk[v + 2 * n] * uk[v + 2 * n] +
                                                     uk[v + 3 * n] * uk[v + 3 * n]) / (2.0 * uk[v + 0 * n]);
            }
      }
}

/* --------------------------------------------------------- pointwise fluxes */

/* Euler flux, fluxes[iS + 5*l] (solver.cpp:1040-1086). */
static void flux_c(const ldgo* o, const double* u, double* f) {
  double ir = 1.0 / u[0];
  double mx = u[1], my = u[2], mz = u[3], E = u[4];
  double pr4 = 0.2e1 / 0.5e1 * E;                   /* (gamma-1) E */
  double ke4 = (mx * mx + my * my + mz * mz) * ir / 0.5e1; /* (gamma-1)|m|^2/(2 rho) */
  double H = o->gamma * E - ke4;
  f[0] = mx; f[1] = mx * mx * ir + pr4 - ke4; f[2] = mx * my * ir; f[3] = mx * mz * ir; f[4] = mx * H * ir;
  f[5] = my; f[6] = f[2]; f[7] = my * my * ir + pr4 - ke4; f[8] = my * mz * ir; f[9] = my * H * ir;
  f[10] = mz; f[11] = f[3]; f[12] = f[8]; f[13] = mz * mz * ir + pr4 - ke4; f[14] = mz * H * ir;
}

/* Navier-Stokes viscous flux from u and its gradient Du[iS + 5*l]
 * (solver.cpp:1089-1188): Newtonian stress with Stokes' hypothesis scaled
 * by 1/Re, heat flux gamma/Pr * grad(e)/Re. */
static void flux_v(const ldgo* o, const double* u, const double* Du, double* f) {
  double ir = 1.0 / u[0];
  double v[3] = {u[1] * ir, u[2] * ir, u[3] * ir};
  double G[3][3]; /* G[i][j] = d_j v_i */
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) G[i][j] = (Du[(1 + i) + 5 * j] - Du[0 + 5 * j] * v[i]) * ir;
  double div = G[0][0] + G[1][1] + G[2][2];
  double iRe = 1.0 / o->Re, kap = o->gamma / o->Pr;
  double tau[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) tau[i][j] = (G[i][j] + G[j][i] - (i == j ? 2.0 / 3.0 * div : 0.0));
  double e = u[4] * ir;
  for (int j = 0; j < 3; ++j) {
    double de = (Du[4 + 5 * j] - Du[0 + 5 * j] * e) * ir - (v[0] * G[0][j] + v[1] * G[1][j] + v[2] * G[2][j]);
    f[0 + 5 * j] = 0.0;
    for (int i = 0; i < 3; ++i) f[1 + i + 5 * j] = tau[i][j] * iRe;
    f[4 + 5 * j] = (tau[0][j] * v[0] + tau[1][j] * v[1] + tau[2][j] * v[2] + kap * de) * iRe;
  }
}

/* Roe flux F(uN, uK, n) from element K's side (solver.cpp:1194-1374),
 * gamma = 1.4 hard-coded as in the reference. */
static void flux_roe(const double* uN, const double* uK, const double* nrm, double* f) {
  const double g1 = 0.4;
  double rN = uN[0], rK = uK[0], irN = 1.0 / rN, irK = 1.0 / rK;
  double vN[3] = {uN[1] * irN, uN[2] * irN, uN[3] * irN};
  double vK[3] = {uK[1] * irK, uK[2] * irK, uK[3] * irK};
  double qN = vN[0] * nrm[0] + vN[1] * nrm[1] + vN[2] * nrm[2];
  double qK = vK[0] * nrm[0] + vK[1] * nrm[1] + vK[2] * nrm[2];
  double pN = g1 * uN[4] - 0.5 * g1 * rN * (vN[0] * vN[0] + vN[1] * vN[1] + vN[2] * vN[2]);
  double pK = g1 * uK[4] - 0.5 * g1 * rK * (vK[0] * vK[0] + vK[1] * vK[1] + vK[2] * vK[2]);
  double s = sqrt(rN * irK); /* sqrt(rhoN/rhoK) */
  double is1 = 1.0 / (s + 1.0);
  double vt[3];
  for (int i = 0; i < 3; ++i) vt[i] = (s * vN[i] + vK[i]) * is1;
  double Ht = (s * (uN[4] + pN) * irN + (uK[4] + pK) * irK) * is1;
  double vt2 = vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2];
  double qt = vt[0] * nrm[0] + vt[1] * nrm[1] + vt[2] * nrm[2];
  double c2 = g1 * (Ht - 0.5 * vt2), c = sqrt(c2);
  double l0 = fabs(qt), lp = 0.5 * fabs(qt + c), lm = 0.5 * fabs(-qt + c);
  double dr = rN - rK, dm[3] = {uN[1] - uK[1], uN[2] - uK[2], uN[3] - uK[3]}, dE = uN[4] - uK[4];
  double a1 = lp + lm - l0;
  double dp = g1 * (0.5 * vt2 * dr - (vt[0] * dm[0] + vt[1] * dm[1] + vt[2] * dm[2]) + dE);
  double dq = -qt * dr + dm[0] * nrm[0] + dm[1] * nrm[1] + dm[2] * nrm[2];
  double a2 = lp - lm;
  double t158 = a1 * dp / c2, t168 = a2 * dq / c;
  double t179 = t158 + t168, t186 = a2 * dp / c + a1 * dq;
  f[0] = 0.5 * rN * qN + 0.5 * rK * qK - 0.5 * l0 * dr - 0.5 * t179;
  for (int i = 0; i < 3; ++i)
    f[1 + i] = 0.5 * uN[1 + i] * qN + 0.5 * uK[1 + i] * qK + 0.5 * nrm[i] * (pN + pK) - 0.5 * l0 * dm[i] -
               0.5 * t179 * vt[i] - 0.5 * t186 * nrm[i];
  f[4] = 0.5 * (uN[4] + pN) * qN + 0.5 * (uK[4] + pK) * qK - 0.5 * l0 * dE - 0.5 * t179 * Ht - 0.5 * t186 * qt;
}

/* ------------------------------------------------------------------ RHS */

/* Gather face nodes and interpolate to face/volume quadrature points
 * (solver.cpp:541-577); periodic neighbours replace the ghost exchange
 * (solver.cpp:929-998). dim = 1 (u) or 3 (Du). */
static void interpolate(ldgo* o, const double* curr, double* i2d, double* i3d, int dim, long e0, long e1) {
  int n = o->n, nf = o->nf, nE = o->nE;
  long blk = (long)nf * NS * NF * nE, nU = (long)n * NS * nE, ne = e1 - e0;
  for (int l = 0; l < dim; ++l) {
    long k;
#pragma omp parallel for schedule(static)
    for (k = e0; k < e1; ++k)
      for (int f = 0; f < NF; ++f)
        for (int s = 0; s < NS; ++s)
          for (int j = 0; j < nf; ++j)
            o->onFaces[j + nf * (s + NS * (f + NF * k)) + l * blk] =
                curr[o->efToN[j + nf * f] + n * (s + NS * k) + (long)l * nU];
    long off = (long)nf * NS * NF * e0 + l * blk;
    gemm(o, 0, nf, (int)(NS * NF * ne), nf, 1.0, o->Interp2D, nf, o->onFaces + off, nf, 0.0, i2d + off, nf);
    long voff = (long)n * NS * e0 + l * nU;
    gemm(o, 0, n, (int)(NS * ne), n, 1.0, o->Interp3D, n, curr + voff, n, 0.0, i3d + voff, n);
  }
}

/* Adds Kels2D(:,:,f/2)^T * fstar into the face nodes of res (the per-face
 * DGEMM + scatter of solver.cpp:618-629). */
static void face_lift(const ldgo* o, int f, const double* fstar, double* res) {
  int n = o->n, nf = o->nf;
  const double* K2 = o->Kels2D + (long)(f / 2) * nf * nf;
  for (int s = 0; s < NS; ++s)
    for (int j = 0; j < nf; ++j) {
      double acc = 0.0;
      for (int q = 0; q < nf; ++q) acc += K2[q + j * nf] * fstar[q + nf * s];
      res[o->efToN[j + nf * f] + n * s] += acc;
    }
}

static const double kNormals[NF][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};

/* ------------------------------------------------- sum-factorised RHS */

/* out = (A2 (x) A1 (x) A0) in on an N^3 block, index a + N b + N^2 c, each
 * A row-major N x N (out x in): three 1-D passes, x then y then z. */
static inline __attribute__((always_inline)) void apply3_n(const int N, const double* A0, const double* A1,
                                                           const double* A2, const double* in, double* out) {
  double t1[512], t2[512];
  int N2 = N * N;
  for (int c = 0; c < N; ++c)
    for (int b = 0; b < N; ++b)
      for (int a = 0; a < N; ++a) {
        double acc = 0.0;
        for (int r = 0; r < N; ++r) acc += A0[a * N + r] * in[r + N * b + N2 * c];
        t1[a + N * b + N2 * c] = acc;
      }
  for (int c = 0; c < N; ++c)
    for (int b = 0; b < N; ++b)
      for (int a = 0; a < N; ++a) {
        double acc = 0.0;
        for (int r = 0; r < N; ++r) acc += A1[b * N + r] * t1[a + N * r + N2 * c];
        t2[a + N * b + N2 * c] = acc;
      }
  for (int c = 0; c < N; ++c)
    for (int b = 0; b < N; ++b)
      for (int a = 0; a < N; ++a) {
        double acc = 0.0;
        for (int r = 0; r < N; ++r) acc += A2[c * N + r] * t2[a + N * b + N2 * r];
        out[a + N * b + N2 * c] = acc;
      }
}

/* apply3_n with N a compile-time constant for the common orders, so the
 * 1-D loops unroll. */
static void apply3(int N, const double* A0, const double* A1, const double* A2, const double* in, double* out) {
  switch (N) {
    case 2: apply3_n(2, A0, A1, A2, in, out); return;
    case 3: apply3_n(3, A0, A1, A2, in, out); return;
    case 4: apply3_n(4, A0, A1, A2, in, out); return;
    case 5: apply3_n(5, A0, A1, A2, in, out); return;
    case 6: apply3_n(6, A0, A1, A2, in, out); return;
    default: apply3_n(N, A0, A1, A2, in, out); return;
  }
}

/* out = (A1 (x) A0) in on an N^2 face block, index a + N b. */
static inline __attribute__((always_inline)) void apply2_n(const int N, const double* A0, const double* A1,
                                                           const double* in, double* out) {
  double t1[64];
  for (int b = 0; b < N; ++b)
    for (int a = 0; a < N; ++a) {
      double acc = 0.0;
      for (int r = 0; r < N; ++r) acc += A0[a * N + r] * in[r + N * b];
      t1[a + N * b] = acc;
    }
  for (int b = 0; b < N; ++b)
    for (int a = 0; a < N; ++a) {
      double acc = 0.0;
      for (int r = 0; r < N; ++r) acc += A1[b * N + r] * t1[a + N * r];
      out[a + N * b] = acc;
    }
}

static void apply2(int N, const double* A0, const double* A1, const double* in, double* out) {
  switch (N) {
    case 2: apply2_n(2, A0, A1, in, out); return;
    case 3: apply2_n(3, A0, A1, in, out); return;
    case 4: apply2_n(4, A0, A1, in, out); return;
    case 5: apply2_n(5, A0, A1, in, out); return;
    case 6: apply2_n(6, A0, A1, in, out); return;
    default: apply2_n(N, A0, A1, in, out); return;
  }
}

/* Interp3D / Interp2D applications of interpolate() (solver.cpp:541-577)
 * in factored form: volume values I1^3 u and face values I1^2 u|face for
 * dim consecutive fields of (n,5,nE) each. */
static void interpolate_factored(ldgo* o, const double* curr, double* i2d, double* i3d, int dim) {
  int N = o->N, n = o->n, nf = o->nf, nE = o->nE;
  long nU = (long)n * NS * nE, blk = (long)nf * NS * NF * nE;
  for (int l = 0; l < dim; ++l) {
    long e;
#pragma omp parallel for schedule(static)
    for (e = 0; e < nE; ++e) {
      double face[64];
      for (int s = 0; s < NS; ++s) {
        const double* ue = curr + l * nU + (long)n * (s + NS * e);
        apply3(N, o->I1, o->I1, o->I1, ue, i3d + l * nU + (long)n * (s + NS * e));
        for (int f = 0; f < NF; ++f) {
          for (int j = 0; j < nf; ++j) face[j] = ue[o->efToN[j + nf * f]];
          apply2(N, o->I1, o->I1, face, i2d + l * blk + nf * (s + NS * (f + NF * e)));
        }
      }
    }
  }
}

/* Kels2D(:,:,f/2)^T fstar scattered to the face nodes (face_lift) as
 * J/alpha_l (IWt (x) IWt) fstar. */
static void face_lift_factored(const ldgo* o, int f, const double* fstar, double* res) {
  int N = o->N, n = o->n, nf = o->nf;
  double scaleL = o->J / o->alpha[f / 2], out[64];
  for (int s = 0; s < NS; ++s) {
    apply2(N, o->IWt, o->IWt, fstar + nf * s, out);
    for (int j = 0; j < nf; ++j) res[o->efToN[j + nf * f] + n * s] += scaleL * out[j];
  }
}

/* Mel \ x for one element's 5 blocks: (1/J) M1i^3 x, in place. */
static void mass_solve_factored(const ldgo* o, double* x) {
  int N = o->N, n = o->n;
  double tmp[512];
  for (int s = 0; s < NS; ++s) {
    apply3(N, o->M1i, o->M1i, o->M1i, x + n * s, tmp);
    for (int i = 0; i < n; ++i) x[i + n * s] = tmp[i] / o->J;
  }
}

/* The gradient half of rk4Rhs (solver.cpp:495-508) in factored form:
 * Dus_l = Mel \ (F_l(u) - Sels_l u), with uInterp2D/uInterp3D of uCurr
 * already computed. */
static void gradient_factored(ldgo* o, const double* uCurr) {
  int N = o->N, n = o->n, nf = o->nf, nE = o->nE;
  long nU = (long)n * NS * nE;
  long e;
#pragma omp parallel for schedule(static)
  for (e = 0; e < nE; ++e) {
    double fstar[NS * 64], tmp[512];
    for (int l = 0; l < DIM; ++l) {
      double* D = o->Dus + l * nU + (long)e * n * NS;
      for (int i = 0; i < n * NS; ++i) D[i] = 0.0;
      for (int f = 0; f < NF; ++f) { /* localDGFlux (solver.cpp:585-635) */
        int nK = o->eToE[f + NF * e], nF = f ^ 1;
        double nl = kNormals[f][l];
        for (int s = 0; s < NS; ++s)
          for (int q = 0; q < nf; ++q) {
            double uK = o->uInterp2D[q + nf * (s + NS * (f + NF * e))];
            double uN = o->uInterp2D[q + nf * (s + NS * (nF + NF * (long)nK))];
            fstar[q + nf * s] = ((nl > 0) ? uK : uN) * nl; /* numericalFluxL */
          }
        face_lift_factored(o, f, fstar, D);
      }
      const double* A[3] = {o->M1, o->M1, o->M1};
      A[l] = o->S1;
      double scaleL = o->J / o->alpha[l];
      for (int s = 0; s < NS; ++s) { /* -Sels_l u, solver.cpp:500 */
        apply3(N, A[0], A[1], A[2], uCurr + (long)n * (s + NS * e), tmp);
        for (int i = 0; i < n; ++i) D[i + n * s] += -scaleL * tmp[i];
      }
      mass_solve_factored(o, D);
    }
  }
}

/* rk4Rhs (solver.cpp:486-535) with every dense operator applied in its
 * Kronecker-factored form: the same discrete operator and the same flux
 * functions, O(N^4) instead of O(N^6) work per element and variable. */
static void rhs_factored(ldgo* o, const double* uCurr, double* k) {
  int N = o->N, n = o->n, nf = o->nf, nE = o->nE;
  long nU = (long)n * NS * nE;
  long fblk = (long)nf * NS * NF * nE;
  interpolate_factored(o, uCurr, o->uInterp2D, o->uInterp3D, 1);
  gradient_factored(o, uCurr);
  interpolate_factored(o, o->Dus, o->DuInterp2D, o->DuInterp3D, DIM);
  long e;
#pragma omp parallel for schedule(static)
  for (e = 0; e < nE; ++e) {
    double fstar[NS * 64], fl[NS], uK[NS], uN[NS], DuK[NS * DIM], DuN[NS * DIM], Fv[NS * DIM];
    double flx[DIM][NS][512], tmp[512];
    double* ke = k + (long)e * n * NS;
    for (int i = 0; i < n * NS; ++i) ke[i] = 0.0;
    for (int f = 0; f < NF; ++f) { /* convectDGFlux (solver.cpp:643-698) */
      int nK = o->eToE[f + NF * e], nF = f ^ 1;
      for (int q = 0; q < nf; ++q) {
        for (int s = 0; s < NS; ++s) {
          uK[s] = o->uInterp2D[q + nf * (s + NS * (f + NF * e))];
          uN[s] = o->uInterp2D[q + nf * (s + NS * (nF + NF * (long)nK))];
        }
        flux_roe(uN, uK, kNormals[f], fl);
        for (int s = 0; s < NS; ++s) fstar[q + nf * s] = fl[s];
      }
      face_lift_factored(o, f, fstar, ke);
    }
    for (int f = 0; f < NF; ++f) { /* viscousDGFlux (solver.cpp:750-814) */
      int nK = o->eToE[f + NF * e], nF = f ^ 1;
      const double* nrm = kNormals[f];
      int kWins = (nrm[0] + nrm[1] + nrm[2]) > 0; /* numericalFluxV */
      for (int q = 0; q < nf; ++q) {
        for (int s = 0; s < NS; ++s) {
          uK[s] = o->uInterp2D[q + nf * (s + NS * (f + NF * e))];
          uN[s] = o->uInterp2D[q + nf * (s + NS * (nF + NF * (long)nK))];
        }
        for (int l = 0; l < DIM; ++l)
          for (int s = 0; s < NS; ++s) {
            DuK[s + NS * l] = o->DuInterp2D[q + nf * (s + NS * (f + NF * e)) + l * fblk];
            DuN[s + NS * l] = o->DuInterp2D[q + nf * (s + NS * (nF + NF * (long)nK)) + l * fblk];
          }
        flux_v(o, uK, kWins ? DuN : DuK, Fv);
        for (int s = 0; s < NS; ++s) {
          double acc = 0.0;
          for (int l = 0; l < DIM; ++l) acc -= Fv[s + NS * l] * nrm[l];
          fstar[q + nf * s] = acc;
        }
      }
      face_lift_factored(o, f, fstar, ke);
    }
    for (int i = 0; i < n * NS; ++i) ke[i] = -ke[i]; /* dscal -1 */
    for (int q = 0; q < n; ++q) { /* volume fluxes (solver.cpp:701-741, 817-864) */
      double u[NS], Du[NS * DIM], Fc[NS * DIM];
      for (int s = 0; s < NS; ++s) u[s] = o->uInterp3D[q + n * (s + NS * e)];
      for (int l = 0; l < DIM; ++l)
        for (int s = 0; s < NS; ++s) Du[s + NS * l] = o->DuInterp3D[q + n * (s + NS * e) + l * nU];
      flux_c(o, u, Fc);
      flux_v(o, u, Du, Fv);
      for (int l = 0; l < DIM; ++l)
        for (int s = 0; s < NS; ++s) flx[l][s][q] = Fc[s + NS * l] - Fv[s + NS * l];
    }
    for (int l = 0; l < DIM; ++l) { /* Kels_l^T (fc - fv), solver.cpp:736-738, 859-861 */
      const double* A[3] = {o->IWt, o->IWt, o->IWt};
      A[l] = o->DWt;
      double scaleL = o->J / o->alpha[l];
      for (int s = 0; s < NS; ++s) {
        apply3(N, A[0], A[1], A[2], flx[l][s], tmp);
        for (int i = 0; i < n; ++i) ke[i + n * s] += scaleL * tmp[i];
      }
    }
    mass_solve_factored(o, ke);
  }
}

/* Switches a handle between the dense operator chain (0, the reference's
 * GEMM structure) and the Kronecker-factored one (1).  Both evaluate the
 * same discrete operator; they differ in rounding only.  The factored form
 * makes long runs at the benchmark meshes affordable on a CPU. */
void ldgo_set_factored(ldgo* o, int on) { o->factored = on ? 1 : 0; }

/* One RHS evaluation k = rhs(uCurr) (rk4Rhs, solver.cpp:486-535). */
/* rk4Rhs (solver.cpp:486-535) with the reference's dense operator chain,
 * for the residual of elements [r0, r1).  The full mesh is r0 = 0, r1 =
 * nE.  A z-slab of whole planes (r0, r1 multiples of nx*ny, at least two
 * planes from either end of the numbering) needs the gradient one plane
 * beyond it and the face values of u two planes beyond it; only those
 * halos are evaluated, which makes a bounded sample of the workload of a
 * large mesh.  k receives the slab's columns only. */
static void rhs_dense(ldgo* o, const double* uCurr, double* k, long r0, long r1) {
  int n = o->n, nf = o->nf, nE = o->nE;
  long nU = (long)n * NS * nE;
  long fblk = (long)nf * NS * NF * nE;
  long plane = (long)o->nx * o->ny;
  long g0 = 0, g1 = nE, i0 = 0, i1 = nE; /* gradient and u-interpolation ranges */
  if (!(r0 == 0 && r1 == nE)) {
    g0 = r0 - plane; g1 = r1 + plane; i0 = r0 - 2 * plane; i1 = r1 + 2 * plane;
  }
  interpolate(o, uCurr, o->uInterp2D, o->uInterp3D, 1, i0, i1);
  /* Gradient pass: Dus_l = Mel \ (-S_l u + F_l(u))  (solver.cpp:495-508) */
  long e;
  for (int l = 0; l < DIM; ++l) memset(o->Dus + l * nU + (long)n * NS * g0, 0, sizeof(double) * n * NS * (g1 - g0));
#pragma omp parallel for schedule(static)
  for (e = g0; e < g1; ++e) { /* localDGFlux (solver.cpp:585-635) */
    double fstar[NS * 64];
    for (int l = 0; l < DIM; ++l)
      for (int f = 0; f < NF; ++f) {
        int nK = o->eToE[f + NF * e], nF = f ^ 1;
        double nl = kNormals[f][l];
        for (int s = 0; s < NS; ++s)
          for (int q = 0; q < nf; ++q) {
            double uK = o->uInterp2D[q + nf * (s + NS * (f + NF * e))];
            double uN = o->uInterp2D[q + nf * (s + NS * (nF + NF * (long)nK))];
            fstar[q + nf * s] = ((nl > 0) ? uK : uN) * nl; /* numericalFluxL, solver.cpp:867-884 */
          }
        face_lift(o, f, fstar, o->Dus + l * nU + (long)e * n * NS);
      }
  }
  long gc = (long)n * NS * g0;
  for (int l = 0; l < DIM; ++l) {
    gemm(o, 0, n, (int)(NS * (g1 - g0)), n, -1.0, o->Sels + (long)l * n * n, n, uCurr + gc, n, 1.0,
         o->Dus + l * nU + gc, n);
    mass_solve(o, o->Dus + l * nU + gc, (long)NS * (g1 - g0));
  }
  interpolate(o, o->Dus, o->DuInterp2D, o->DuInterp3D, DIM, g0, g1);
  /* Residual: faces, negate, volumes, mass solve (solver.cpp:516-533) */
  long rc = (long)n * NS * r0;
  memset(k + rc, 0, sizeof(double) * n * NS * (r1 - r0));
#pragma omp parallel for schedule(static)
  for (e = r0; e < r1; ++e) {
    double fstar[NS * 64];
    double uK[NS], uN[NS], DuK[NS * DIM], DuN[NS * DIM], fl[NS], Fv[NS * DIM];
    for (int f = 0; f < NF; ++f) { /* convectDGFlux (solver.cpp:643-698) */
      int nK = o->eToE[f + NF * e], nF = f ^ 1;
      for (int q = 0; q < nf; ++q) {
        for (int s = 0; s < NS; ++s) {
          uK[s] = o->uInterp2D[q + nf * (s + NS * (f + NF * e))];
          uN[s] = o->uInterp2D[q + nf * (s + NS * (nF + NF * (long)nK))];
        }
        flux_roe(uN, uK, kNormals[f], fl);
        for (int s = 0; s < NS; ++s) fstar[q + nf * s] = fl[s];
      }
      face_lift(o, f, fstar, k + (long)e * n * NS);
    }
    for (int f = 0; f < NF; ++f) { /* viscousDGFlux (solver.cpp:750-814) */
      int nK = o->eToE[f + NF * e], nF = f ^ 1;
      const double* nrm = kNormals[f];
      int kWins = (nrm[0] + nrm[1] + nrm[2]) > 0; /* numericalFluxV, solver.cpp:891-921 */
      for (int q = 0; q < nf; ++q) {
        for (int s = 0; s < NS; ++s) {
          uK[s] = o->uInterp2D[q + nf * (s + NS * (f + NF * e))];
          uN[s] = o->uInterp2D[q + nf * (s + NS * (nF + NF * (long)nK))];
        }
        for (int l = 0; l < DIM; ++l)
          for (int s = 0; s < NS; ++s) {
            DuK[s + NS * l] = o->DuInterp2D[q + nf * (s + NS * (f + NF * e)) + l * fblk];
            DuN[s + NS * l] = o->DuInterp2D[q + nf * (s + NS * (nF + NF * (long)nK)) + l * fblk];
          }
        flux_v(o, uK, kWins ? DuN : DuK, Fv);
        for (int s = 0; s < NS; ++s) {
          double acc = 0.0;
          for (int l = 0; l < DIM; ++l) acc -= Fv[s + NS * l] * nrm[l];
          fstar[q + nf * s] = acc;
        }
      }
      face_lift(o, f, fstar, k + (long)e * n * NS);
    }
    for (long i = 0; i < (long)n * NS; ++i) k[(long)e * n * NS + i] = -k[(long)e * n * NS + i]; /* dscal -1 */
    /* Volume fluxes at quadrature points (solver.cpp:701-741, 817-864),
     * stored as (fc - fv) per direction in flx(n,5,nE,3). */
    for (int q = 0; q < n; ++q) {
      double u[NS], Du[NS * DIM], Fc[NS * DIM];
      for (int s = 0; s < NS; ++s) u[s] = o->uInterp3D[q + n * (s + NS * e)];
      for (int l = 0; l < DIM; ++l)
        for (int s = 0; s < NS; ++s) Du[s + NS * l] = o->DuInterp3D[q + n * (s + NS * e) + l * nU];
      flux_c(o, u, Fc);
      flux_v(o, u, Du, Fv);
      for (int l = 0; l < DIM; ++l)
        for (int s = 0; s < NS; ++s) o->flx[q + n * (s + NS * e) + l * nU] = Fc[s + NS * l] - Fv[s + NS * l];
    }
  }
  for (int l = 0; l < DIM; ++l)
    gemm(o, 1, n, (int)(NS * (r1 - r0)), n, 1.0, o->Kels + (long)l * n * n, n, o->flx + l * nU + rc, n, 1.0,
         k + rc, n);
  mass_solve(o, k + rc, (long)NS * (r1 - r0));
}

/* One RHS evaluation k = rhs(uCurr) (rk4Rhs, solver.cpp:486-535). */
void ldgo_rhs(ldgo* o, const double* uCurr, double* k) {
  if (o->factored) {
    rhs_factored(o, uCurr, k);
    return;
  }
  rhs_dense(o, uCurr, k, 0, o->nE);
}

/* One rk4Rhs stage restricted to the residual of the z-planes [z0, z0 +
 * planes) with the dense chain (see rhs_dense): a bounded sample of the
 * work of a full-mesh stage.  Needs 2 <= z0 and z0 + planes <= nz - 2.
 * Returns 0, or -1 for a slab too close to the ends of the numbering. */
int ldgo_rhs_slab(ldgo* o, const double* uCurr, double* k, int z0, int planes) {
  if (z0 < 2 || planes < 1 || z0 + planes > o->nz - 2) return -1;
  long plane = (long)o->nx * o->ny;
  rhs_dense(o, uCurr, k, z0 * plane, (z0 + planes) * plane);
  return 0;
}

/* Kinetic energy exactly as computeKE (solver.cpp:1007-1034): nodal values
 * weighted by the Gauss weights (the reference quirk; nQ3D == dofs). */
double ldgo_compute_ke(const ldgo* o, const double* u) {
  int n = o->n, nE = o->nE;
  double total = 0.0;
  for (int e = 0; e < nE; ++e) {
    double ke = 0.0;
    const double* uk = u + (long)e * n * NS;
    for (int q = 0; q < n; ++q)
      ke += o->J * o->wQ3[q] *
            (uk[q + n] * uk[q + n] + uk[q + 2 * n] * uk[q + 2 * n] + uk[q + 3 * n] * uk[q + 3 * n]) / (2 * uk[q]);
    total += ke;
  }
  return total / (o->rho0 * pow(2 * M_PI * o->L, 3.0));
}

/* Enstrophy of a state: the Gauss quadrature of rho |curl v|^2 / 2 from
 * the LDG gradient Dus of u (the first half of rk4Rhs, solver.cpp:495-508)
 * and the interpolants Interp3D u, Interp3D Dus, normalised like computeKE
 * (solver.cpp:1007-1034) by rho0 (2 pi L)^3.  The reference prints no
 * enstrophy; this is the functional the CUDA path reports, on the
 * reference's own gradient. */
double ldgo_enstrophy(ldgo* o, const double* u) {
  int n = o->n, nE = o->nE;
  long nU = (long)n * NS * nE;
  if (o->factored) {
    interpolate_factored(o, u, o->uInterp2D, o->uInterp3D, 1);
    gradient_factored(o, u);
    interpolate_factored(o, o->Dus, o->DuInterp2D, o->DuInterp3D, DIM);
  } else {
    double* k = (double*)malloc(sizeof(double) * nU);
    ldgo_rhs(o, u, k); /* leaves uInterp3D, DuInterp3D of u behind */
    free(k);
  }
  double total = 0.0;
  long e;
#pragma omp parallel for schedule(static) reduction(+ : total)
  for (e = 0; e < nE; ++e) {
    double el = 0.0;
    for (int q = 0; q < n; ++q) {
      double rho = o->uInterp3D[q + n * (NS * e)], v[3], G[3][3];
      for (int i = 0; i < 3; ++i) v[i] = o->uInterp3D[q + n * (1 + i + NS * e)] / rho;
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
          G[i][j] = (o->DuInterp3D[q + n * (1 + i + NS * e) + j * nU] - o->DuInterp3D[q + n * (NS * e) + j * nU] * v[i]) / rho;
      double wx = G[2][1] - G[1][2], wy = G[0][2] - G[2][0], wz = G[1][0] - G[0][1];
      el += o->J * o->wQ3[q] * 0.5 * rho * (wx * wx + wy * wy + wz * wz);
    }
    total += el;
  }
  return total / (o->rho0 * pow(2 * M_PI * o->L, 3.0));
}

/* nsteps classical RK4 steps in place (solver.cpp:298-315, 410-440);
 * ke[i] (if given) receives computeKE after step i. */
void ldgo_step(ldgo* o, double* u, int nsteps, double* ke) {
  const double b[4] = {1 / 6.0, 1 / 3.0, 1 / 3.0, 1 / 6.0};
  const double a[3] = {0.5, 0.5, 1.0};
  long nU = (long)o->n * NS * o->nE;
  for (int it = 0; it < nsteps; ++it) {
    for (int s = 0; s < 4; ++s) {
      long i;
      if (s == 0) {
        memcpy(o->uCurr, u, sizeof(double) * nU);
      } else {
        const double* kp = o->ks + (long)(s - 1) * nU;
#pragma omp parallel for schedule(static)
        for (i = 0; i < nU; ++i) o->uCurr[i] = u[i] + o->dt * a[s - 1] * kp[i];
      }
      ldgo_rhs(o, o->uCurr, o->ks + (long)s * nU);
    }
    for (int s = 0; s < 4; ++s) {
      const double* kp = o->ks + (long)s * nU;
      long i;
#pragma omp parallel for schedule(static)
      for (i = 0; i < nU; ++i) u[i] += o->dt * b[s] * kp[i];
    }
    if (ke) ke[it] = ldgo_compute_ke(o, u);
  }
}
