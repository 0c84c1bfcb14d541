"""Precision study of the element-operator contraction on low-precision
arithmetics (CPU, numpy emulation): which arithmetic could carry the mixed
path's contractions.

The contraction is the gradient pass's volume product along x, out = As x
with As = W^-1 D^T W / alpha (the 1-D weak derivative at the Gauss points),
applied to Taylor-Green states at p=4:
  K = 5    the sum-factorised 1-D product that the kernels evaluate;
  K = 125  the reference's own dense operator Sels_x (nodal CGL basis, a
           genuinely dense 125 x 125 matrix) on nodal states, the shape in
           which the reference evaluates it (a DGEMM over all elements,
           solver.cpp:500).
Arithmetics, each against FP64:
  fp32          operands rounded to FP32, FP32 products and sums;
  bf16x3        split-BF16x3: each operand as three BF16 parts, the six
                leading part products, FP32 accumulation (the tensor-core
                recipe with FP32 accumulators);
  int10x3       the exact-slice scheme of k_contract_tc: per-line power of
                two, three 10-bit integer slices per operand, level sums
                2..4 exact, recombined in FP64.
The error is max |out - out64| over max |As| max |x| per line (what the
rounding of one contraction can cost), and over max |out64| (what it costs
relative to the result).  The findings the assertions pin:
  * FP32 and split-BF16x3 with FP32 accumulation lose ~3e-7 (K = 5) and
    ~6e-7 to 9e-7 (K = 125) of max|A||x|.  Relative to the result they
    lose far more on the energy lines (E ~ 178, derivative ~1e-2).  The
    FP32-pair path keeps ~1e-14 (measured on the GPU,
    tests/test_gpu_mixed.py).
  * Exact slices lose ~10 * 2^-30 ~ 1.5e-8 for K = 5: every partial sum is
    an integer below 2^24, so only the slices' truncation counts.  For
    K = 125 the same slices would need level sums up to 125 * 2^20 > 2^24,
    so the FP32 accumulator is no longer exact.
"""
import math

import numpy as np
import pytest

import oracle

N = 5  # p = 4


def weak_derivative(alpha):
    """As = W^-1 D^T W / alpha at the N Gauss points (D[q][r] = l_r'(x_q))."""
    x, w = np.polynomial.legendre.leggauss(N)
    D = np.zeros((N, N))
    for r in range(N):
        c = np.zeros(N)
        c[r] = 1.0
        # Lagrange basis l_r through the Gauss points, as a polynomial
        V = np.vander(x, N, increasing=True)
        coef = np.linalg.solve(V, c)
        dcoef = np.polynomial.polynomial.polyder(coef)
        D[:, r] = np.polynomial.polynomial.polyval(x, dcoef)
    return (np.diag(1.0 / w) @ D.T @ np.diag(w)) / alpha


def gauss_states(nx=6, amp=1e-2):
    """Perturbed Taylor-Green states at p=4 in the Gauss basis, (nE, 5, N^3)."""
    o = oracle.Oracle(nx, N - 1)
    u = o.initial_condition(amp, 11, 3)
    n = N ** 3
    I3 = o.operator(1).reshape(n, n, order="F")
    return np.einsum("qi,evi->evq", I3, u), 2 * math.pi / nx / 2


def bf16(a):
    """Round to BF16 (nearest even), as float64."""
    b = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def split3(a, rnd):
    parts, r = [], np.asarray(a, dtype=np.float64)
    for _ in range(3):
        p = rnd(r)
        parts.append(p)
        r = r - p
    return parts


def contract_fp32(A, X):
    return (A.astype(np.float32) @ X.astype(np.float32)).astype(np.float64)


def contract_bf16x3(A, X):
    a, x = split3(A, bf16), split3(X, bf16)
    acc = np.zeros((A.shape[0], X.shape[1]), dtype=np.float32)
    for i, j in [(0, 0), (0, 1), (1, 0), (0, 2), (1, 1), (2, 0)]:
        acc += a[i].astype(np.float32) @ x[j].astype(np.float32)  # exact products, FP32 sums
    return acc.astype(np.float64)


def int_slices(v, e):
    """Three 10-bit integer slices of v scaled by 2^(9-e) (rounded to
    nearest), as the kernel cuts them."""
    a = np.ldexp(v, 9 - e)
    out = []
    for _ in range(3):
        s = np.rint(a)
        out.append(s)
        a = (a - s) * 1024.0
    return out


def contract_int10x3(A, X):
    """Columns of X are lines; per-line power of two, per-matrix power of two
    for A; level sums 2..4 formed exactly (float64 holds them)."""
    eA = math.frexp(np.max(np.abs(A)))[1]
    S = int_slices(A, eA)
    mx = np.max(np.abs(X), axis=0)
    ex = np.array([math.frexp(m)[1] if m > 0 else 0 for m in mx])
    Xs = int_slices(X, ex[None, :])
    levels = []
    for k in (2, 3, 4):
        d = sum(S[s] @ Xs[t] for s in range(3) for t in range(3) if s + t + 2 == k)
        assert np.max(np.abs(d)) < 2 ** 24  # the FP32 accumulator holds it exactly
        levels.append(d)
    val = levels[0] + levels[1] * 2.0 ** -10 + levels[2] * 2.0 ** -20
    return val * np.ldexp(1.0, eA + ex - 18)[None, :]


def lines_x(U):
    """x-lines of every element and variable: (N, lines)."""
    nE = U.shape[0]
    return U.reshape(nE, 5, N, N, N).transpose(4, 0, 1, 2, 3).reshape(N, -1)  # index order z,y,x -> x first


def errors(fn, A, X):
    ref = A @ X
    got = fn(A, X)
    scale = np.max(np.abs(A)) * np.max(np.abs(X), axis=0)  # per line
    return float(np.max(np.abs(got - ref) / scale[None, :])), float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))


@pytest.fixture(scope="module")
def setup():
    U, alpha = gauss_states()
    A = weak_derivative(alpha)
    return U, A


def test_weak_derivative_row_sums_are_the_lifts(setup):
    """On a constant, As gives (Lp - Lm)/alpha (Lp, Lm: the Lagrange basis
    at +1 and -1 over the weights): the weak derivative's rows do not sum to
    zero, which is why a large constant (the energy) costs the low-precision
    contractions accuracy relative to the result."""
    _, A = setup
    x, w = np.polynomial.legendre.leggauss(N)
    lag = [np.polynomial.polynomial.polyval(s, np.linalg.solve(np.vander(x, N, increasing=True), np.eye(N)[r]))
           for r in range(N) for s in (1.0, -1.0)]
    lp = np.array(lag[0::2]) / w
    lm = np.array(lag[1::2]) / w
    alpha = np.pi / 6
    assert np.allclose(A @ np.ones(N) * alpha, lp - lm, rtol=0, atol=1e-12)


def test_k5_low_precision_errors(setup):
    U, A = setup
    X = lines_x(U)
    e32, r32 = errors(contract_fp32, A, X)
    e3, r3 = errors(contract_bf16x3, A, X)
    e10, r10 = errors(contract_int10x3, A, X)
    # FP32-class arithmetic: ~1e-7 of max|A||x| per line
    assert 1e-9 < e32 < 1e-6 and 1e-9 < e3 < 1e-6, (e32, e3)
    # exact slices: each of the 5 terms loses at most 2^-30 of max|A| max|x|
    # through each operand's truncation, so ~10 * 2^-30 ~ 1e-8 per line
    assert e10 < 3e-8, e10
    assert e10 < e32 / 10


def test_k125_dense_low_precision_errors(setup):
    """The reference's own dense operator: Sels_x (125 x 125, nodal CGL
    basis, solver.cpp:95-192) on the nodal states, as the DGEMM of
    solver.cpp:500 applies it."""
    U, A = setup
    o = oracle.Oracle(6, N - 1)
    n = N ** 3
    S = o.operator(4)[: n * n].reshape(n, n, order="F")
    u = o.initial_condition(1e-2, 11, 3)
    X = u.reshape(-1, n).T  # (125, nE*5) columns = element-variable blocks
    e32, _ = errors(contract_fp32, S, X)
    e3, _ = errors(contract_bf16x3, S, X)
    assert 1e-9 < e32 < 1e-5 and 1e-9 < e3 < 1e-5, (e32, e3)
    # over 125 terms the FP32 accumulation loses more than over 5
    e32_1d, _ = errors(contract_fp32, A, lines_x(U))
    assert e32 > e32_1d
    # exact 10-bit slices would overflow the FP32 accumulator's 24 bits at K = 125
    assert 125 * 544 * 512 * 3 > 2 ** 24
