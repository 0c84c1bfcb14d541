"""CPU tests of the oracle (oracle/ldg_oracle.c) against the golden vectors
produced by the unmodified reference (tests/golden/make_golden.py), plus
known-answer checks of the discretisation it restates."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, rel_l2

TOL = 1e-12  # relative L2, the FP64 parity bar


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_tgv_initial_condition_bitwise():
    z = load("tgv_n8_p2.npz")
    o = oracle.Oracle(8, 2, steps=100)
    assert o.dt == float(z["dt"])
    u0 = o.initial_condition()
    assert np.array_equal(u0, z["u0"])


def test_tgv_100_steps_matches_reference():
    """Configuration: 8^3 p=2 Taylor-Green, 100 RK4 steps, per-step KE."""
    z = load("tgv_n8_p2.npz")
    o = oracle.Oracle(8, 2, steps=100, threads=4)
    u = z["u0"].copy()
    u, ke = o.step(u, 1)
    assert rel_l2(u, z["u1"]) <= TOL
    u, ke2 = o.step(u, 9)
    assert rel_l2(u, z["u10"]) <= TOL
    u, ke3 = o.step(u, 90)
    assert rel_l2(u, z["u100"]) <= TOL
    kes = np.concatenate([ke, ke2, ke3])
    assert np.max(np.abs(kes - z["ke"]) / z["ke"]) <= 1e-13


@pytest.mark.parametrize("name", ["rhs_n3_p1", "rhs_n3_p2", "rhs_n4_p3", "rhs_n3_p4", "rhs_n4_p2"])
def test_rhs_matches_reference(name):
    z = load(name + ".npz")
    nx = int(name.split("_")[1][1:])
    p = int(name.split("_")[2][1:])
    o = oracle.Oracle(nx, p)
    k = o.rhs(z["u0"])
    assert rel_l2(k, z["k"]) <= TOL


@pytest.mark.parametrize("name", ["step_n4_p2", "step_n3_p4", "step_n4_p3"])
def test_steps_match_reference(name):
    z = load(name + ".npz")
    nx = int(name.split("_")[1][1:])
    p = int(name.split("_")[2][1:])
    o = oracle.Oracle(nx, p, steps=int(z["steps"]))
    assert o.dt == float(z["dt"])
    u, ke = o.step(z["u0"], int(z["steps"]))
    assert rel_l2(u, z["u_final"]) <= TOL
    assert np.max(np.abs(ke - z["ke"]) / np.abs(z["ke"])) <= 1e-13


def test_openblas_route_matches_loops():
    lib = oracle.find_openblas()
    if lib is None:
        pytest.skip("scipy's OpenBLAS not available")
    z = load("rhs_n4_p3.npz")
    a = oracle.Oracle(4, 3).rhs(z["u0"])
    b = oracle.Oracle(4, 3, openblas=lib, threads=2).rhs(z["u0"])
    assert rel_l2(b, a) <= 1e-13


# ---------------------------------------------------------- known answers
@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_gauss_rule_is_gauss_legendre(p):
    o = oracle.Oracle(3, p)
    w3 = o.operator(5)
    x, w = np.polynomial.legendre.leggauss(p + 1)
    ref = np.einsum("i,j,k->kji", w, w, w).ravel()
    assert np.allclose(w3, ref, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_interp3d_exact_on_polynomials(p):
    """Interp3D maps nodal values of a degree<=p polynomial to its values at
    the Gauss points (dgMath.cpp:583-615)."""
    o = oracle.Oracle(3, p)
    n = (p + 1) ** 3
    I3 = o.operator(1).reshape(n, n, order="F")
    xi = np.cos((p - np.arange(p + 1)) * np.pi / p)
    xq, _ = np.polynomial.legendre.leggauss(p + 1)
    f = lambda x, y, z: 1 + 2 * x ** p - y * z ** (p - 1) + 0.5 * x * y * z
    X, Y, Z = np.meshgrid(xi, xi, xi, indexing="ij")
    nodal = f(X, Y, Z).transpose(2, 1, 0).ravel()  # x fastest
    Xq, Yq, Zq = np.meshgrid(xq, xq, xq, indexing="ij")
    exact = f(Xq, Yq, Zq).transpose(2, 1, 0).ravel()
    assert np.allclose(I3 @ nodal, exact, rtol=0, atol=1e-13)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_free_stream_preserved(p):
    """A constant state is a steady solution: the RHS vanishes."""
    o = oracle.Oracle(3, p)
    u = np.zeros(o.shape)
    u[:, 0], u[:, 1], u[:, 2], u[:, 3], u[:, 4] = 1.2, 0.3, -0.2, 0.1, 180.0
    k = o.rhs(u)
    assert np.max(np.abs(k)) <= 1e-10


def test_tgv_initial_kinetic_energy():
    o = oracle.Oracle(8, 2)
    ke = o.ke(o.initial_condition())
    assert abs(ke - 0.125) < 1e-3


def test_conservation_of_mass():
    """Periodic DG with the (antisymmetric) Roe flux conserves total mass.
    Momentum and energy are not conserved exactly by the reference scheme:
    its viscous face flux evaluates each side with its own trace of u
    (numericalFluxV, solver.cpp:897-912), so the two sides' fluxes differ."""
    z = load("step_n4_p2.npz")
    o = oracle.Oracle(4, 2, steps=5)
    n = o.dofs
    c = o.operator(1).reshape(n, n, order="F").T @ o.operator(5)  # integrals of the nodal basis
    tot = lambda u: np.einsum("evq,q->v", u, c)
    u, _ = o.step(z["u0"], 5)
    assert abs(tot(u)[0] - tot(z["u0"])[0]) <= 1e-13 * abs(tot(z["u0"])[0])


def test_oracle_matches_reference_series_at_32_cubed_p3():
    """The first two steps of the reference's 32^3 p=3 Taylor-Green run
    (tests/golden/series_n32_p3.npz): KE, per-variable norms and the
    sampled entries."""
    z = np.load(os.path.join(GOLDEN, "series_n32_p3.npz"))
    o = oracle.Oracle(32, 3, steps=int(z["steps"]), threads=os.cpu_count() or 1,
                      openblas=oracle.find_openblas())
    assert o.dt == float(z["dt"])
    u = o.initial_condition()
    for k in range(2):
        u, ke = o.step(u, 1)
        assert abs(ke[0] - z["ke"][k]) <= 1e-12 * z["ke"][k]
        assert rel_l2(u.ravel()[z["idx"]], z["samples"][k]) <= 1e-12
        norms = np.sqrt(np.einsum("evq,evq->v", u, u))
        assert np.max(np.abs(norms - np.sqrt(z["norms"][k]))) <= 1e-12 * np.sqrt(np.sum(z["norms"][k]))


@pytest.mark.parametrize("name", ["rhs_n3_p1", "rhs_n3_p2", "rhs_n4_p3", "rhs_n3_p4", "rhs_n4_p2"])
def test_factored_rhs_matches_reference(name):
    """The Kronecker-factored operator chain (the oracle's mode for long
    runs at the benchmark meshes) against the reference's RHS."""
    z = load(name + ".npz")
    nx, p = int(name.split("_")[1][1:]), int(name.split("_")[2][1:])
    o = oracle.Oracle(nx, p)
    o.set_factored(True)
    assert rel_l2(o.rhs(z["u0"]), z["k"]) <= TOL


def test_factored_oracle_matches_reference_series_at_32_cubed_p3():
    """The first three steps of the reference's 32^3 p=3 run with the
    factored chain (all 200 steps agree to <= 1.3e-14 on the samples; the
    generator of the 64^3 p=4 fixture checks its own 20-step window)."""
    z = np.load(os.path.join(GOLDEN, "series_n32_p3.npz"))
    o = oracle.Oracle(32, 3, steps=int(z["steps"]), threads=os.cpu_count() or 1)
    o.set_factored(True)
    u = o.initial_condition()
    for k in range(3):
        u, ke = o.step(u, 1)
        assert abs(ke[0] - z["ke"][k]) <= 1e-12 * z["ke"][k]
        assert rel_l2(u.ravel()[z["idx"]], z["samples"][k]) <= 1e-12


def test_factored_enstrophy_equals_dense():
    """Enstrophy from the factored gradient equals the dense chain's."""
    z = load("rhs_n4_p3.npz")
    a = oracle.Oracle(4, 3)
    b = oracle.Oracle(4, 3)
    b.set_factored(True)
    ea, eb = a.enstrophy(z["u0"]), b.enstrophy(z["u0"])
    assert abs(ea - eb) <= 1e-12 * abs(ea)


def test_series_64_fixture_is_pinned_to_the_reference_window():
    """tests/golden/series_n64_p4.npz holds the reference's own first 20
    steps at 64^3 p=4 beside the factored oracle's 200: on the common steps
    and entries they agree (samples and KE at 1e-12; the enstrophy of step
    20 at 1e-12)."""
    z = load("series_n64_p4.npz")
    R = int(z["ref_steps"])
    assert int(z["steps"]) == 200 and R >= 20
    pos = np.searchsorted(z["ref_idx"], z["idx"])
    assert np.array_equal(z["ref_idx"][pos], z["idx"])
    for k in range(R):
        assert abs(z["ke"][k] - z["ref_ke"][k]) <= 1e-12 * z["ref_ke"][k]
        assert rel_l2(z["samples"][k], z["ref_samples"][k][pos]) <= 1e-12
    ens = dict(zip(z["enst_steps"].tolist(), z["enst"].tolist()))
    ref = dict(zip(z["ref_enst_steps"].tolist(), z["ref_enst"].tolist()))
    common = sorted(set(ens) & set(ref))
    assert common
    for k in common:
        assert abs(ens[k] - ref[k]) <= 1e-12 * abs(ref[k])
