"""The 1-D element operators as the library builds them (ldg_operators_1d,
host only; csrc/ldg_ops.cpp), for every supported order p = 1..7:

* the Gauss rule, the weak derivative A[q, r] = (w_r/w_q) L_q'(x_r) and the
  face lifts Lp/Lm[q] = L_q(+-1)/w_q against their definitions, evaluated
  here with barycentric Lagrange formulas;
* the two symmetries the FP64 gradient pass relies on: A is
  skew-centrosymmetric (A[N-1-q, N-1-r] = -A[q, r]) and the lifts mirror
  (Lp[N-1-q] = Lm[q]);
* the pairwise line form of the gradient that the FP64 gradient pass
  evaluates (OpsT::gs..gc in ldg_device.cuh), restated here, against the
  direct per-point sums g[q] = Lp[q] tp - Lm[q] tm - sum_r A[q, r] x[r].

These are the 1-D factors of the reference's Sels, Kels and Kels2D with its
mass matrix (solver.cpp:74-192) in the Gauss-point basis."""
import numpy as np
import pytest

import ldg

ORDERS = range(1, 8)
EPS = np.finfo(float).eps


def barycentric(x):
    """Weights b_r = 1 / prod_{k != r} (x_r - x_k)."""
    N = len(x)
    return np.array([1.0 / np.prod([x[r] - x[k] for k in range(N) if k != r]) for r in range(N)])


def lagrange_at(x, b, t):
    """L_q(t) for all q (t not a node)."""
    c = b / (t - x)
    return c / c.sum()


def weak_derivative(x, w):
    N = len(x)
    b = barycentric(x)
    D = np.zeros((N, N))  # D[q, r] = L_r'(x_q)
    for q in range(N):
        for r in range(N):
            if r != q:
                D[q, r] = (b[r] / b[q]) / (x[q] - x[r])
        D[q, q] = -D[q].sum()
    return (w[None, :] / w[:, None]) * D.T  # A[q, r] = (w_r / w_q) D[r, q]


@pytest.mark.parametrize("p", ORDERS)
def test_operators_match_their_definitions(p):
    o = ldg.operators_1d(p)
    N = p + 1
    xg, wg = np.polynomial.legendre.leggauss(N)
    assert np.max(np.abs(o["x"] - xg)) <= 4 * EPS and np.max(np.abs(o["w"] - wg)) <= 4 * EPS
    A = weak_derivative(xg, wg)
    assert np.max(np.abs(o["A"] - A)) <= 1e-13 * np.max(np.abs(A))
    b = barycentric(xg)
    Lp = lagrange_at(xg, b, 1.0) / wg
    Lm = lagrange_at(xg, b, -1.0) / wg
    assert np.max(np.abs(o["Lp"] - Lp)) <= 1e-13 * np.max(np.abs(Lp))
    assert np.max(np.abs(o["Lm"] - Lm)) <= 1e-13 * np.max(np.abs(Lm))


@pytest.mark.parametrize("p", ORDERS)
def test_symmetries_of_the_operators(p):
    """Each entry is rounded once from long double, so the symmetries hold
    to an ulp of the largest entry."""
    o = ldg.operators_1d(p)
    A, Lp, Lm = o["A"], o["Lp"], o["Lm"]
    assert np.max(np.abs(A + A[::-1, ::-1])) <= 2 * EPS * np.max(np.abs(A))
    assert np.max(np.abs(Lp[::-1] - Lm)) <= 2 * EPS * np.max(np.abs(Lp))
    if (p + 1) % 2:
        assert abs(A[p // 2, p // 2]) <= 2 * EPS * np.max(np.abs(A))


def pairwise_gradient(A, Lp, Lm, x, tp, tm):
    """The FP64 gradient pass's line form (coefficients as make_opst builds
    them, operations in the kernel's order)."""
    N = len(x)
    H = N // 2
    odd = N % 2 == 1
    gs = [(Lp[k] + Lm[k]) / 2 for k in range(H)]
    gd = [(Lp[k] - Lm[k]) / 2 for k in range(H)]
    gp = [[(A[k, j] - A[k, N - 1 - j]) / 2 for j in range(H)] for k in range(H)]
    gm = [[(A[k, j] + A[k, N - 1 - j]) / 2 for j in range(H)] + ([A[k, H]] if odd else []) for k in range(H)]
    ev = [x[k] + x[N - 1 - k] for k in range(H)]
    od = [x[k] - x[N - 1 - k] for k in range(H)]
    tdif, tsum = tp - tm, tp + tm
    g = np.zeros(N)
    for k in range(H):
        U = gs[k] * tdif
        for j in range(H):
            U -= gp[k][j] * od[j]
        V = gd[k] * tsum
        for j in range(H):
            V -= gm[k][j] * ev[j]
        if odd:
            V -= gm[k][H] * x[H]
        g[k], g[N - 1 - k] = U + V, U - V
    if odd:
        v = Lp[H] * tdif
        for j in range(H):
            v -= A[H, j] * od[j]
        g[H] = v
    return g


@pytest.mark.parametrize("p", ORDERS)
def test_pairwise_line_gradient_equals_the_direct_sums(p):
    o = ldg.operators_1d(p)
    ia = 1.0 / 0.29  # 1/alpha: the kernels use the operators pre-scaled
    A, Lp, Lm = o["A"] * ia, o["Lp"] * ia, o["Lm"] * ia
    rng = np.random.default_rng(p)
    worst = 0.0
    for _ in range(500):
        # Taylor-Green-like magnitudes: energy ~178 with O(1) variation
        x = 178.0 + rng.standard_normal(p + 1)
        tp, tm = 178.0 + rng.standard_normal(2)
        direct = Lp * tp - Lm * tm - A @ x
        got = pairwise_gradient(A, Lp, Lm, x, tp, tm)
        worst = max(worst, np.max(np.abs(got - direct)) / (np.max(np.abs(A)) * 180.0))
    assert worst <= 1e-14, worst


def test_invalid_orders_are_rejected():
    for p in (0, 8):
        with pytest.raises(ldg.LdgError):
            ldg.operators_1d(p)
