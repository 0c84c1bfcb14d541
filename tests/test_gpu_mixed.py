"""GPU tests of the mixed-precision path (LDG_MIXED_F32X2): the RHS in
FP32-pair arithmetic on the FP32 pipe, FP64 state / RK4 accumulation /
reductions.  Its bar: relative L2 state error <= 1e-9 against the FP64
result after 100 RK4 steps (here checked at 8^3 p2 against the reference's
golden run, at 16^3 p4 and at the full 64^3 p4 workload against the FP64
path)."""
import os

import numpy as np
import pytest

import ldg
import oracle
from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-9


def perturbed(nx, p, seed, amp=1.0):
    o = oracle.Oracle(nx, p)
    u = o.initial_condition()
    rng = np.random.default_rng(seed)
    r = rng.standard_normal(u.shape)
    u[:, 0, :] *= 1.0 + 0.05 * amp * r[:, 0, :]
    u[:, 1:4, :] += 0.1 * amp * r[:, 1:4, :]
    u[:, 4, :] += 0.5 * amp * r[:, 4, :]
    return u


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_mixed_rhs_close_to_oracle(p):
    nx = 3 if p >= 4 else 4
    u = perturbed(nx, p, 300 + p)
    k_ref = oracle.Oracle(nx, p).rhs(u)
    with ldg.Solver(p, nx, precision="mixed") as s:
        k = s.rhs(u)
    # random-noise states are ill-conditioned; the RHS itself carries the
    # pair arithmetic's ~1e-14 relative error amplified by the cancellation
    assert rel_l2(k, k_ref) <= 1e-10


def test_mixed_tgv_8_p2_100_steps_vs_reference():
    z = np.load(os.path.join(GOLDEN, "tgv_n8_p2.npz"))
    with ldg.Solver(2, 8, steps=100, precision="mixed") as s:
        s.step(100)
        u = s.get_state()
        ke = s.ke_history()
    assert rel_l2(u, z["u100"]) <= MIXED_TOL
    assert np.max(np.abs(ke - z["ke"]) / z["ke"]) <= 1e-10


def run(p, nx, steps, precision):
    with ldg.Solver(p, nx, steps=steps, precision=precision) as s:
        s.step(steps)
        return s.get_state(), s.ke_history()


def test_mixed_vs_fp64_16_p4_100_steps():
    u64, ke64 = run(4, 16, 100, "fp64")
    umx, kemx = run(4, 16, 100, "mixed")
    assert rel_l2(umx, u64) <= MIXED_TOL
    assert np.max(np.abs(kemx - ke64) / ke64) <= 1e-10


@pytest.mark.slow
def test_mixed_vs_fp64_64_p4_100_steps():
    """The configuration of the mixed-precision target: 64^3 hexes, p=4,
    Taylor-Green at Re=1600, 100 RK4 steps, relative L2 vs FP64 <= 1e-9."""
    u64, ke64 = run(4, 64, 100, "fp64")
    umx, kemx = run(4, 64, 100, "mixed")
    err = rel_l2(umx, u64)
    print(f"64^3 p4 mixed vs fp64 after 100 steps: rel-L2 {err:.3e}")
    assert err <= MIXED_TOL
    assert np.max(np.abs(kemx - ke64) / ke64) <= 1e-10


def test_mixed_rhs_api_leaves_state_intact():
    """ldg_rhs borrows the stage buffer on the mixed path and rebuilds it:
    stepping after an rhs call gives the same state as without it."""
    u0 = perturbed(4, 3, 17, amp=0.2)
    outs = []
    for with_rhs in (False, True):
        with ldg.Solver(3, 4, steps=2, precision="mixed") as s:
            s.set_state(u0)
            if with_rhs:
                s.rhs(perturbed(4, 3, 18))
            s.step(2)
            outs.append(s.get_state())
    assert np.array_equal(outs[0], outs[1])


def test_mixed_nonfinite_reported():
    u = perturbed(3, 2, 9)
    u[2, 1, 4] = np.inf
    with ldg.Solver(2, 3, precision="mixed") as s:
        s.set_state(u)
        with pytest.raises(ldg.LdgError) as ei:
            s.step(1)
        assert ei.value.status == -4


@pytest.mark.parametrize("mode,tol", [("pair_fma", 1e-13), ("pair_dot2", 1e-13), ("tensor_core_slices", 1e-7)])
def test_contraction_arithmetics_against_fp64(mode, tol):
    """The gradient pass's volume contraction in the mixed path's candidate
    arithmetics, against FP64 on a perturbed Taylor-Green state at 6^3 p=4,
    relative to the largest output: the FP32 pairs keep ~2^-44; the
    tensor-core scheme (three exact 10-bit slices per operand, levels 2..4)
    keeps ~2^-30 of max|A| max|x| per line, which the energy lines (E ~ 178,
    and the weak derivative's rows do not sum to zero) make ~1e-8 of the
    largest output."""
    with ldg.Solver(4, 6, perturb_amp=1e-2, seed=5) as s:
        ms, err = s.probe_contraction(mode, reps=2)
    assert ms > 0
    assert err <= tol, (mode, err)
    if mode == "tensor_core_slices":
        assert err > 1e-13  # it is the sliced arithmetic that ran, not FP64


def test_mixed_vs_reference_series_32_p3_200_steps():
    """The mixed path against the reference's own Taylor-Green run at 32^3
    p=3 (tests/golden/series_n32_p3.npz): after 200 RK4 steps the sampled
    state entries within the mixed bar, and the KE series within 1e-10."""
    z = np.load(os.path.join(GOLDEN, "series_n32_p3.npz"))
    steps = int(z["steps"])
    with ldg.Solver(3, 32, steps=steps, precision="mixed") as s:
        assert abs(s.dt - float(z["dt"])) <= 1e-15 * float(z["dt"])
        s.step(steps)
        u = s.get_state()
        ke = s.ke_history()
    assert rel_l2(u.ravel()[z["idx"]], z["samples"][-1]) <= MIXED_TOL
    assert np.max(np.abs(ke - z["ke"]) / z["ke"]) <= 1e-10
