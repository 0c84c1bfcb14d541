"""GPU parity: the CUDA FP64 path (through the C ABI) against the golden
vectors of the unmodified reference and against the oracle on seeded
inputs.  Bar: relative L2 <= 1e-12 per step (FP64 parity)."""
import os

import numpy as np
import pytest

import ldg
import oracle
from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def perturbed(nx, p, seed, amp=1.0):
    o = oracle.Oracle(nx, p)
    u = o.initial_condition()
    rng = np.random.default_rng(seed)
    r = rng.standard_normal(u.shape)
    u[:, 0, :] *= 1.0 + 0.05 * amp * r[:, 0, :]
    u[:, 1:4, :] += 0.1 * amp * r[:, 1:4, :]
    u[:, 4, :] += 0.5 * amp * r[:, 4, :]
    return u


def test_initial_condition_matches_reference():
    z = load("tgv_n8_p2.npz")
    with ldg.Solver(2, 8, steps=100) as s:
        assert s.dt == float(z["dt"])
        u0 = s.get_state()
    assert rel_l2(u0, z["u0"]) <= 1e-14


@pytest.mark.parametrize("name", ["rhs_n3_p1", "rhs_n3_p2", "rhs_n4_p3", "rhs_n3_p4", "rhs_n4_p2"])
def test_rhs_matches_reference(name):
    z = load(name + ".npz")
    nx = int(name.split("_")[1][1:])
    p = int(name.split("_")[2][1:])
    with ldg.Solver(p, nx) as s:
        k = s.rhs(z["u0"])
    assert rel_l2(k, z["k"]) <= TOL


@pytest.mark.parametrize("name", ["step_n4_p2", "step_n3_p4", "step_n4_p3"])
def test_steps_match_reference(name):
    z = load(name + ".npz")
    nx = int(name.split("_")[1][1:])
    p = int(name.split("_")[2][1:])
    steps = int(z["steps"])
    with ldg.Solver(p, nx, steps=steps) as s:
        assert s.dt == float(z["dt"])
        s.set_state(z["u0"])
        s.step(steps)
        u = s.get_state()
        ke = s.ke_history()
    assert rel_l2(u, z["u_final"]) <= TOL
    assert np.max(np.abs(ke - z["ke"]) / np.abs(z["ke"])) <= 1e-12


def test_tgv_8_p2_100_steps_per_step_parity():
    """Configuration 8^3 p=2 Taylor-Green, 100 RK4 steps: the states at
    steps 1, 10, 100 and every step's computeKE against the reference."""
    z = load("tgv_n8_p2.npz")
    with ldg.Solver(2, 8, steps=100) as s:
        s.step(1)
        assert rel_l2(s.get_state(), z["u1"]) <= TOL
        s.step(9)
        assert rel_l2(s.get_state(), z["u10"]) <= TOL
        s.step(90)
        assert rel_l2(s.get_state(), z["u100"]) <= TOL
        ke = s.ke_history()
        eps = s.ke_dissipation()
    assert ke.shape == (100,)
    assert np.max(np.abs(ke - z["ke"]) / z["ke"]) <= 1e-12
    ref_eps = -(z["ke"][2:] - z["ke"][:-2]) / (2 * float(z["dt"]))
    assert eps.shape == ref_eps.shape
    assert np.max(np.abs(eps - ref_eps)) <= 1e-9 * np.max(np.abs(ref_eps)) + 1e-12


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_rhs_matches_oracle_seeded(p):
    nx = 3 if p >= 4 else 4
    u = perturbed(nx, p, 100 + p)
    k_ref = oracle.Oracle(nx, p).rhs(u)
    with ldg.Solver(p, nx) as s:
        k = s.rhs(u)
    assert rel_l2(k, k_ref) <= TOL


@pytest.mark.parametrize("p,nx,steps", [(2, 5, 4), (3, 4, 3), (4, 3, 3), (5, 3, 2)])
def test_steps_match_oracle_seeded(p, nx, steps):
    u0 = perturbed(nx, p, 200 + p, amp=0.3)
    o = oracle.Oracle(nx, p, steps=steps)
    u_ref, ke_ref = o.step(u0, steps)
    with ldg.Solver(p, nx, steps=steps) as s:
        s.set_state(u0)
        s.step(steps)
        u = s.get_state()
        ke = s.ke_history()
    assert rel_l2(u, u_ref) <= TOL
    assert np.max(np.abs(ke - ke_ref) / np.abs(ke_ref)) <= 1e-12


def test_non_cubic_mesh_matches_oracle():
    """nx != ny != nz exercises the element numbering and neighbour wrap."""
    import ctypes
    p, dims = 2, (3, 4, 5)
    L_ = oracle.lib()
    tf = oracle.tf_for_steps(3, p, 1.0, 1)
    h = L_.ldgo_create(dims[0], dims[1], dims[2], p, 1.0, tf, 1600.0, 1)
    n = (p + 1) ** 3
    nE = dims[0] * dims[1] * dims[2]
    u = np.zeros((nE, 5, n))
    L_.ldgo_initial_condition(h, u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    rng = np.random.default_rng(7)
    u[:, 1:4] += 0.05 * rng.standard_normal(u[:, 1:4].shape)
    k_ref = np.zeros_like(u)
    L_.ldgo_rhs(h, u.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                k_ref.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    L_.ldgo_destroy(h)
    with ldg.Solver(p, dims[0], dims[1], dims[2], tf=tf) as s:
        k = s.rhs(u)
    assert rel_l2(k, k_ref) <= TOL


def test_state_roundtrip_and_device_pointers():
    import torch
    u = perturbed(4, 3, 5)
    with ldg.Solver(3, 4) as s:
        s.set_state(u)
        back = s.get_state()
        assert rel_l2(back, u) <= 1e-14
        du = torch.from_numpy(u).cuda()
        k_dev = s.rhs(du)
        k_host = s.rhs(u)
        assert rel_l2(k_dev.cpu().numpy(), k_host) == 0.0


def test_diagnostics_match_reference_ke():
    z = load("tgv_n8_p2.npz")
    o = oracle.Oracle(8, 2)
    with ldg.Solver(2, 8, steps=100) as s:
        ke_ref, ke, ens = s.diagnostics()
        assert abs(ke_ref - o.ke(z["u0"])) <= 1e-13
        s.set_state(z["u10"])
        ke_ref10, ke10, ens10 = s.diagnostics()
        assert abs(ke_ref10 - o.ke(z["u10"])) <= 1e-13
    # quadrature KE and enstrophy of the TGV at t=0: 1/8 and 3/8 (analytic;
    # discretisation error at 8^3 p=2 is a few percent)
    assert abs(ke - 0.125) < 2e-3
    assert abs(ens - 0.375) < 0.03


def test_nonfinite_state_is_reported():
    """Host-made fault: a NaN in the uploaded state; no device fault."""
    u = perturbed(3, 2, 9)
    u[5, 4, 3] = np.nan
    with ldg.Solver(2, 3) as s:
        s.set_state(u)
        with pytest.raises(ldg.LdgError) as ei:
            s.step(1)
        assert ei.value.status == -4


def test_deterministic_bitwise():
    u = perturbed(4, 3, 11, amp=0.3)
    outs = []
    for _ in range(2):
        with ldg.Solver(3, 4, steps=3) as s:
            s.set_state(u)
            s.step(3)
            outs.append((s.get_state(), s.ke_history()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_free_stream_preserved(p):
    with ldg.Solver(p, 3) as s:
        u = np.zeros(s.shape)
        u[:, 0], u[:, 1], u[:, 2], u[:, 3], u[:, 4] = 1.2, 0.3, -0.2, 0.1, 180.0
        k = s.rhs(u)
    assert np.max(np.abs(k)) <= 1e-10


def test_time_step_runs_to_tf():
    with ldg.Solver(2, 4, steps=6) as s:
        s.dg_time_step()
        info = s.info()
        assert info.step == 6 == s.timesteps
        assert s.ke_history().shape == (6,)


@pytest.mark.gpu
def test_transfer_chunking_changes_no_bit():
    """Host transfers overlapped with the basis transforms in element chunks
    (ldg_set_transfer_chunks) give the same bits as one whole copy: the
    state round trip, a step, and an RHS through host buffers, for 1, 3, 8
    and 64 chunks on a mesh whose element count 64 does not divide evenly."""
    rng = np.random.default_rng(4)
    with ldg.Solver(3, 4, 4, 5, steps=3) as s:  # 80 elements
        u0 = s.get_state()
        u0[:, 1:4] += 0.01 * rng.standard_normal(u0[:, 1:4].shape)
        outs = []
        for chunks in (1, 3, 8, 64):
            s.set_transfer_chunks(chunks)
            s.set_state(u0)
            back = s.get_state()
            k = s.rhs(u0)
            s.step(1)
            outs.append((back, k, s.get_state()))
    for back, k, u1 in outs[1:]:
        assert np.array_equal(back, outs[0][0])
        assert np.array_equal(k, outs[0][1])
        assert np.array_equal(u1, outs[0][2])
    with pytest.raises(ldg.LdgError):
        with ldg.Solver(2, 3) as s:
            s.set_transfer_chunks(0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_advance_host_equals_set_step_get(precision):
    """ldg_advance_host overlaps the transfers with the first and last
    passes of the steps; it must give the bits of ldg_set_state +
    ldg_step + ldg_get_state, including the KE series, for several chunk
    counts (z-plane chunks; 7 planes of 4 x 5 elements here) and in place."""
    rng = np.random.default_rng(7)
    with ldg.Solver(3, 4, 5, 7, steps=6, precision=precision) as s:
        u0 = s.get_state()
    u0[:, 1:4] += 0.01 * rng.standard_normal(u0[:, 1:4].shape)
    for chunks in (1, 3, 8):
        with ldg.Solver(3, 4, 5, 7, steps=6, precision=precision) as s:
            s.set_transfer_chunks(chunks)
            s.set_state(u0)
            s.step(3)
            want = s.get_state()
            ke_want = s.ke_history()
            s.set_state(want)  # the fused call below also restarts from the host copy
            s.step(1)
            want2 = s.get_state()
        with ldg.Solver(3, 4, 5, 7, steps=6, precision=precision) as s:
            s.set_transfer_chunks(chunks)
            out = np.empty_like(u0)
            s.advance_host(u0, out, 3)
            assert np.array_equal(out, want), chunks
            assert np.array_equal(s.ke_history(), ke_want), chunks
            buf = out.copy()
            s.advance_host(buf, buf, 1)  # in place
            assert np.array_equal(buf, want2), chunks
