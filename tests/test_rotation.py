"""Rotation equivariance of the discretisation.  On a periodic cubic mesh,
relabelling the axes cyclically (x' = y, y' = z, z' = x) maps a state to
another state, and the LDG right-hand side commutes with it:
rhs(rot u) = rot rhs(u), up to rounding.  The permutation keeps the axes'
orientation, so the alternating LDG fluxes (u from the minus side, q from the
plus side, numericalFluxL/numericalFluxV, solver.cpp:867-921) map onto
themselves, and the Roe and viscous fluxes are rotation invariant
(solver.cpp:1040-1374).

The step kernels rely on this: they evaluate every face's fluxes in the
frame where its normal is x.  The CPU test checks the oracle (the
reference's algorithm); the GPU tests check the CUDA path through the C ABI.

Layout: u[e][var][q], e = ix + nx (iy + nx iz), q = i + N (j + N k)."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2


def rotate(u, nx, N):
    """The state relabelled by x' = y, y' = z, z' = x: the value at new
    indices (a, b, c) along (z', y', x') is the old value at (b, c, a) along
    (z, y, x), and the new momentum components are (m_y, m_z, m_x)."""
    nE, nv, n = u.shape
    g = u.reshape(nx, nx, nx, nv, N, N, N)  # (EZ, EY, EX, var, NZ, NY, NX)
    g = np.transpose(g, (2, 0, 1, 3, 6, 4, 5))
    g = g[:, :, :, [0, 2, 3, 1, 4], :, :, :]
    return np.ascontiguousarray(g).reshape(nE, nv, n)


def perturbed(o, seed):
    """A non-symmetric state: Taylor-Green plus random perturbations."""
    u = o.initial_condition()
    rng = np.random.default_rng(seed)
    r = rng.standard_normal(u.shape)
    u[:, 0, :] *= 1.0 + 0.05 * r[:, 0, :]
    u[:, 1:4, :] += 0.1 * r[:, 1:4, :]
    u[:, 4, :] += 0.5 * r[:, 4, :]
    return u


def test_rotation_is_a_cyclic_relabelling():
    nx, N = 3, 3
    u = np.random.default_rng(0).standard_normal((nx ** 3, 5, N ** 3))
    r3 = rotate(rotate(rotate(u, nx, N), nx, N), nx, N)
    assert np.array_equal(r3, u)
    assert not np.array_equal(rotate(u, nx, N), u)


@pytest.mark.parametrize("nx,p", [(3, 2), (3, 3)])
def test_oracle_rhs_is_rotation_equivariant(nx, p):
    o = oracle.Oracle(nx, p)
    u = perturbed(o, 5)
    N = p + 1
    lhs = o.rhs(rotate(u, nx, N))
    rhs = rotate(o.rhs(u), nx, N)
    # rounding only (1e-14 at p=2, 1e-13 at p=3); a wrong relabelling of the
    # momentum components gives O(1)
    assert rel_l2(lhs, rhs) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nx,p", [(3, 2), (4, 4)])
def test_cuda_rhs_is_rotation_equivariant(nx, p, precision):
    import ldg
    o = oracle.Oracle(nx, p)
    u = perturbed(o, 6)
    N = p + 1
    with ldg.Solver(p, nx, steps=1, precision=precision) as s:
        lhs = s.rhs(rotate(u, nx, N))
        rhs = rotate(s.rhs(u), nx, N)
    assert rel_l2(lhs, rhs) <= 1e-11
