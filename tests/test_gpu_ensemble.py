"""Batched ensemble (ldg_ensemble_*): members of different sizes, orders,
Reynolds numbers and seeded perturbations, advanced by one persistent
launch per RK4 stage from a CUDA graph, must equal solo runs bit for bit."""
import numpy as np
import pytest

import ldg
import oracle
from conftest import rel_l2


def small_configs(steps=4):
    spec = [(2, 4, 400.0), (3, 3, 900.0), (4, 3, 3200.0), (2, 5, 1600.0), (3, 4, 2000.0), (4, 4, 700.0)]
    return [ldg.make_config(p, nx, steps=steps, Re=Re, perturb_amp=1e-2, seed=99, instance=i)
            for i, (p, nx, Re) in enumerate(spec)]


def test_ensemble_configs_follow_the_spec():
    cfgs = ldg.ensemble_configs(64, seed=5)
    assert len(cfgs) == 64
    assert {c.nx for c in cfgs} <= {8, 12, 16, 24}
    assert {c.p for c in cfgs} <= {2, 3, 4}
    Re = np.array([c.Re for c in cfgs])
    assert Re.min() >= 400 and Re.max() <= 3200
    assert all(c.Ma == 0.1 and c.perturb_amp == 1e-2 for c in cfgs)
    assert len({c.instance for c in cfgs}) == 64
    # deterministic in the seed
    again = ldg.ensemble_configs(64, seed=5)
    assert [(c.nx, c.p, c.Re) for c in cfgs] == [(c.nx, c.p, c.Re) for c in again]


def test_perturbation_phases_are_uniform():
    phi = np.concatenate([oracle.perturbation_phases(3, i).ravel() for i in range(40)])
    assert phi.min() >= 0 and phi.max() < 2 * np.pi
    assert abs(phi.mean() - np.pi) < 0.2


@pytest.mark.gpu
def test_perturbed_initial_condition_matches_oracle():
    o = oracle.Oracle(4, 3)
    u_ref = o.initial_condition(1e-2, 99, 7)
    with ldg.Solver(3, 4, perturb_amp=1e-2, seed=99, instance=7) as s:
        u = s.get_state()
    assert rel_l2(u, u_ref) <= 1e-14
    assert rel_l2(u, o.initial_condition()) > 1e-5  # the perturbation is there


@pytest.mark.gpu
def test_ensemble_members_equal_solo_runs_bitwise():
    steps = 4
    cfgs = small_configs(steps)
    with ldg.Ensemble(cfgs) as ens:
        ens.step(steps)
        states = [ens.get_state(i) for i in range(len(cfgs))]
        kes = [ens.ke_history(i) for i in range(len(cfgs))]
        tuning = ens.tuning()
    assert tuning["threads_per_cta"] in (128, 256) and tuning["persistent_ctas"] > 0
    for i, c in enumerate(cfgs):
        with ldg.Solver(c.p, c.nx, tf=c.tf, Re=c.Re, perturb_amp=c.perturb_amp, seed=c.seed,
                        instance=c.instance) as s:
            s.step(steps)
            u = s.get_state()
            ke = s.ke_history()
        assert np.array_equal(states[i], u), f"member {i} differs from its solo run"
        assert np.array_equal(kes[i], ke), f"member {i} KE differs from its solo run"


@pytest.mark.gpu
def test_ensemble_member_matches_oracle():
    steps = 3
    cfgs = small_configs(steps)[:3]
    with ldg.Ensemble(cfgs) as ens:
        ens.step(steps)
        got = [ens.get_state(i) for i in range(3)]
    for i, c in enumerate(cfgs):
        o = oracle.Oracle(c.nx, c.p, steps=steps, Re=c.Re)
        u_ref, _ = o.step(o.initial_condition(c.perturb_amp, c.seed, c.instance), steps)
        assert rel_l2(got[i], u_ref) <= 1e-12


@pytest.mark.gpu
def test_ensemble_steps_in_several_calls_equal_one_call():
    cfgs = small_configs(6)[:4]
    with ldg.Ensemble(cfgs) as a:
        a.step(6)
        ua = [a.get_state(i) for i in range(4)]
    with ldg.Ensemble(cfgs) as b:
        b.step(1)
        b.step(2)
        b.step(3)
        ub = [b.get_state(i) for i in range(4)]
        assert len(b.ke_history(0)) == 6
    for x, y in zip(ua, ub):
        assert np.array_equal(x, y)


@pytest.mark.gpu
def test_ensemble_reports_nonfinite():
    cfgs = small_configs(2)[:2]
    cfgs[1].Re = 1e-300  # 1/Re overflows to inf in the viscous flux: a host-made fault
    with ldg.Ensemble(cfgs) as ens:
        with pytest.raises(ldg.LdgError) as ei:
            ens.step(1)
        assert ei.value.status == -4


def solo_run(c, steps):
    with ldg.Solver(c.p, c.nx, tf=c.tf, Re=c.Re, perturb_amp=c.perturb_amp, seed=c.seed,
                    instance=c.instance) as s:
        s.step(steps)
        return s.get_state(), s.ke_history()


@pytest.mark.gpu
def test_ensemble_wait_timeout_is_reported_and_state_kept():
    """A member whose RHS items wait for a gradient item that never comes
    (host-injected): with recovery off, the step returns LDG_ERR_TIMEOUT
    after the short wait limit, the state stays at the step's start, and
    the ensemble steps on normally once the stall is lifted."""
    cfgs = small_configs(4)[:4]
    with ldg.Ensemble(cfgs) as ens:
        ens.step(1)
        before = [ens.get_state(i) for i in range(4)]
        ens.set_wait_limit(1 << 14, recover=False)
        ens.inject_stall(2)
        with pytest.raises(ldg.LdgError) as ei:
            ens.step(2)
        assert ei.value.status == -7  # LDG_ERR_TIMEOUT
        assert ens.info(0).step == 1 and len(ens.ke_history(0)) == 1
        for i in range(4):
            assert np.array_equal(ens.get_state(i), before[i])
        ens.inject_stall(2, on=False)
        ens.set_wait_limit(1 << 22, recover=True)
        ens.step(3)
        assert ens.recovered_steps() == 0
        after = [ens.get_state(i) for i in range(4)]
    for i, c in enumerate(cfgs):
        u, ke = solo_run(c, 4)
        assert np.array_equal(after[i], u), f"member {i} differs from its solo run"


@pytest.mark.gpu
def test_ensemble_recovers_a_stalled_step_member_by_member():
    """With recovery on (the default), each step whose wait runs out is
    re-run member by member with the solo kernels: every member, the
    stalled one included, still equals its solo run bit for bit."""
    steps = 3
    cfgs = small_configs(steps)
    with ldg.Ensemble(cfgs) as ens:
        ens.set_wait_limit(1 << 14, recover=True)
        ens.inject_stall(4)
        ens.step(2)
        assert ens.recovered_steps() == 2
        ens.inject_stall(4, on=False)
        ens.set_wait_limit(1 << 22, recover=True)
        ens.step(1)
        assert ens.recovered_steps() == 2
        states = [ens.get_state(i) for i in range(len(cfgs))]
        kes = [ens.ke_history(i) for i in range(len(cfgs))]
    for i, c in enumerate(cfgs):
        u, ke = solo_run(c, steps)
        assert np.array_equal(states[i], u), f"member {i} differs from its solo run"
        assert np.array_equal(kes[i], ke), f"member {i} KE differs from its solo run"


@pytest.mark.gpu
def test_full_ensemble_members_equal_solo_runs_bitwise():
    """The 64-member batched configuration (element counts from
    {8^3,12^3,16^3,24^3}, p from {2,3,4}, Re log-uniform in [400,3200],
    seeded perturbations): after 2 steps, one member of each order equals
    its solo run bit for bit."""
    steps = 2
    cfgs = ldg.ensemble_configs(64, seed=2024, steps=1000)
    pick = {}
    for i, c in enumerate(cfgs):
        pick.setdefault(c.p, i)
    with ldg.Ensemble(cfgs) as ens:
        ens.step(steps)
        got = {i: (ens.get_state(i), ens.ke_history(i)) for i in pick.values()}
    assert sorted(pick) == [2, 3, 4]
    for i, (u_e, ke_e) in got.items():
        u, ke = solo_run(cfgs[i], steps)
        assert np.array_equal(u_e, u), f"member {i} (p={cfgs[i].p}) differs from its solo run"
        assert np.array_equal(ke_e, ke)
