"""Learned closure: the MLP kernels against the numpy restatement
(oracle/mlp_oracle.py), the oracle's own gradients against finite
differences, the fine-to-coarse projection, and a small end-to-end run
(data from fine runs, on-GPU training, held-out error reduction, attached
to a coarse solver)."""
import numpy as np
import pytest

import ldg
import mlp_oracle as M
import oracle
from conftest import rel_l2


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    I, H, O, B = 7, 5, 3, 4
    n = H * I + H + H * H + H + O * H + O
    theta = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((B, I))
    dy = rng.standard_normal((B, O))
    g = M.backward(theta, x, dy, I, H, O, rounding=False)
    eps = 1e-6
    for k in rng.choice(n, 25, replace=False):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += eps
        tm[k] -= eps
        fp = np.sum(M.forward(tp, x, I, H, O, rounding=False)[0] * dy)
        fm = np.sum(M.forward(tm, x, I, H, O, rounding=False)[0] * dy)
        assert abs((fp - fm) / (2 * eps) - g[k]) <= 1e-6 * max(1.0, abs(g[k]))


def test_bf16_rounding_is_nearest_even():
    assert M.bf16(1.0 + 2 ** -9)[()] == 1.0          # halfway to 1+2^-8 -> even (1.0)
    assert M.bf16(1.0 + 3 * 2 ** -9)[()] == 1.0 + 2 ** -7
    assert M.bf16(-2.5)[()] == -2.5


@pytest.mark.gpu
def test_mlp_forward_and_gradients_match_oracle():
    with ldg.Closure(p=2, hidden=128, seed=3) as c:
        I, H, O = c.in_dim, c.hidden, c.out_dim
        theta = c.get_params().astype(np.float64)
        rng = np.random.default_rng(1)
        B = 300  # not a multiple of the 64-row tile
        x = rng.standard_normal((B, I)).astype(np.float32)
        dy = rng.standard_normal((B, O)).astype(np.float32)
        y = c.forward(x)
        g = c.backward(x, dy)
    y_ref, _ = M.forward(theta, x, I, H, O)
    assert rel_l2(y, y_ref) <= 5e-3
    g_ref = M.backward(theta, x, dy, I, H, O)
    gb, rb = M.blocks(g, I, H, O), M.blocks(g_ref, I, H, O)
    for name in gb:
        assert rel_l2(gb[name], rb[name]) <= 2e-2, name


def fine_coarse_pair(seed, instance, steps_fine, nxc=4):
    fine = ldg.Solver(4, 2 * nxc, steps=1000, perturb_amp=0.05, seed=seed, instance=instance)
    coarse = ldg.Solver(2, nxc, steps=1000)
    return fine, coarse


@pytest.mark.gpu
def test_projection_conserves_mass():
    """The L2 projection of the fine (8^3, p=4) state onto the coarse
    (4^3, p=2) mesh keeps the total mass: sum J_c w_q rho_c(q) over the
    coarse samples equals the fine integral of rho."""
    fine, coarse = fine_coarse_pair(1, 0, 0)
    with fine, coarse, ldg.Closure(p=2) as c:
        c.add_samples(fine, coarse)
        X, _ = c.get_samples(0, c.samples)
        u_fine = fine.get_state()
    o_f = oracle.Oracle(8, 4)
    nf = o_f.dofs
    basis_integrals = o_f.operator(1).reshape(nf, nf, order="F").T @ o_f.operator(5)
    mass_fine = np.einsum("eq,q->", u_fine[:, 0, :], basis_integrals) * jacobian(8)
    w = np.polynomial.legendre.leggauss(3)[1]
    w3 = np.einsum("i,j,k->kji", w, w, w).ravel()
    mass_coarse = np.einsum("eq,q->", X[:, :27].astype(np.float64), w3) * jacobian(4)
    # features are stored as float32
    assert abs(mass_coarse - mass_fine) <= 1e-6 * abs(mass_fine)


def jacobian(nx):
    a = (2 * np.pi / nx) / 2
    return a ** 3


@pytest.mark.gpu
def test_closure_end_to_end_reduces_heldout_rhs_error():
    """Training data from fine (8^3, p=4) runs of two seeds, held-out data
    from a third seed; the trained network must cut the coarse (4^3, p=2)
    RHS error on the held-out samples, and a coarse solver with the closure
    attached must step with finite states and differ from the plain one."""
    with ldg.Closure(p=2, hidden=64, seed=11) as c:
        for inst in (0, 1, 2):
            fine, coarse = fine_coarse_pair(7, inst, 0)
            with fine, coarse:
                for _ in range(4):
                    c.add_samples(fine, coarse)
                    fine.step(20)
        per = 64 * 4
        train_n, test_first = 2 * per, 2 * per
        assert c.samples == 3 * per
        c.finalize(0, train_n)
        losses = c.train(0, train_n, iters=400, batch=256, lr=2e-3, seed=5)
        assert np.all(np.isfinite(losses)) and losses[-20:].mean() < losses[:20].mean()
        e_plain, e_cl = c.evaluate(test_first, per)
        assert e_cl < e_plain, (e_plain, e_cl)
        # attach to a coarse solver: a valid run that differs from plain LDG
        with ldg.Solver(2, 4, steps=10, perturb_amp=0.05, seed=7, instance=3) as a, \
                ldg.Solver(2, 4, steps=10, perturb_amp=0.05, seed=7, instance=3) as b:
            a.attach_closure(c)
            a.step(10)
            b.step(10)
            ua, ub = a.get_state(), b.get_state()
            assert np.all(np.isfinite(ua))
            assert rel_l2(ua, ub) > 0
            assert c.fallbacks == 0
            a.attach_closure(None)  # detach: plain operator again
            a.step(1)


@pytest.mark.gpu
def test_attached_correction_never_raises_element_kinetic_energy():
    """Energy stability: with the closure attached, rhs(u) - rhs_plain(u)
    has, in every element, a kinetic-energy production
    sum_q w_q (v . dm - |v|^2/2 drho) <= 0 (up to rounding), evaluated here
    in numpy at the Gauss points (Interp3D of the reference)."""
    with ldg.Closure(p=2, hidden=64, seed=13) as c:
        for inst in (0, 1):
            fine, coarse = fine_coarse_pair(9, inst, 0)
            with fine, coarse:
                for _ in range(3):
                    c.add_samples(fine, coarse)
                    fine.step(15)
        c.finalize(0, c.samples)
        c.train(0, c.samples, iters=200, batch=256, lr=2e-3, seed=1)
        with ldg.Solver(2, 4, steps=10, perturb_amp=0.05, seed=9, instance=5) as a, \
                ldg.Solver(2, 4, steps=10, perturb_amp=0.05, seed=9, instance=5) as b:
            a.step(3)
            u = a.get_state()
            k_plain = b.rhs(u)
            a.attach_closure(c)
            k_cl = a.rhs(u)
            clipped = c.clipped
            c.set_options(energy="neutral")
            k_neutral = a.rhs(u)
            assert c.options()["energy"] == "neutral"
            with pytest.raises(ldg.LdgError):
                c.set_options(scale=-1.0)
            c.set_options(energy="dissipative")
    o = oracle.Oracle(4, 2)
    n = 27
    I3 = o.operator(1).reshape(n, n, order="F")
    w3 = o.operator(5)
    U = np.einsum("qi,evi->evq", I3, u)
    D = np.einsum("qi,evi->evq", I3, k_cl - k_plain)
    assert np.max(np.abs(D)) > 0  # the closure does act
    v = U[:, 1:4] / U[:, 0:1]
    g0 = -0.5 * np.sum(v * v, axis=1)
    prod = np.sum(w3 * (g0 * D[:, 0] + np.sum(v * D[:, 1:4], axis=1)), axis=1)
    scale = np.sum(w3 * (np.abs(g0 * D[:, 0]) + np.sum(np.abs(v * D[:, 1:4]), axis=1)), axis=1)
    assert np.all(prod <= 1e-10 * scale + 1e-300), prod.max()
    assert clipped >= 0
    # the neutral mode removes the KE production entirely
    Dn = np.einsum("qi,evi->evq", I3, k_neutral - k_plain)
    prod_n = np.sum(w3 * (g0 * Dn[:, 0] + np.sum(v * Dn[:, 1:4], axis=1)), axis=1)
    scale_n = np.sum(w3 * (np.abs(g0 * Dn[:, 0]) + np.sum(np.abs(v * Dn[:, 1:4]), axis=1)), axis=1)
    assert np.all(np.abs(prod_n) <= 1e-10 * scale_n + 1e-300)


@pytest.mark.gpu
def test_closure_beats_plain_coarse_ldg_a_posteriori():
    """A posteriori, on the metric the closure is judged by: the coarse 8^3
    p=2 solver with the trained closure attached (energy-stable, dissipative
    projection, fallback beyond 10 sigma) against the plain coarse LDG, both
    judged by the KE-dissipation rate (solver.cpp:438-440) against a fine
    16^3 p=4 run from a seed that the training never saw, to t=10.  The
    closure's rms error (t >= 1, relative to the fine peak rate) must be
    clearly below the plain method's."""
    import closure_study as cs
    variants = [{"name": "n0.3", "input_noise": 0.3, "lr_final": 0.05, "modes": [["dissipative", 1.0, 10.0]]}]
    res, series = cs.run(coarse_nx=8, fine_nx=16, t_end=10.0, iters=4000, data="projected", variants=variants)
    ap = res["a_posteriori"]
    plain = ap["plain"]["rms_err_rel"]
    closure = ap["n0.3/dissipative/x1/ood10"]
    assert closure["status"] == "ok" and np.all(np.isfinite(series["ke_n0.3/dissipative/x1/ood10"]))
    assert closure["rms_err_rel"] < 0.85 * plain, (closure["rms_err_rel"], plain)
    # and the a-priori RHS error on the held-out run drops
    apr = res["a_priori"]["n0.3"]
    assert apr["rhs_err_closure"] < 0.5 * apr["rhs_err_plain"]


def test_dissipation_rate_is_the_reference_central_difference():
    """keDissipation (solver.cpp:438-440): -(KE_{n} - KE_{n-2}) / (2 dt) at
    t_{n-1}; entry i of the KE series is the energy after step i+1."""
    import closure_study as cs
    dt = 0.01
    t = dt * np.arange(1, 101)
    ke = 0.125 - 0.3 * t ** 2  # -dKE/dt = 0.6 t, exact for a central difference
    tt, eps = cs.dissipation(ke, dt)
    assert np.allclose(tt, t[1:-1]) and np.allclose(eps, 0.6 * tt, rtol=0, atol=1e-12)


def test_compare_measures_rms_and_max_after_the_transient():
    import closure_study as cs
    dt = 0.01
    t = dt * np.arange(1, 401)
    ke_ref = 0.125 - 0.01 * t ** 2
    t_ref, e_ref = cs.dissipation(ke_ref, dt)
    scale = float(np.max(e_ref))
    same = cs.compare(ke_ref, dt, t_ref, e_ref, scale)
    assert same["rms_err_rel"] < 1e-9 and same["max_err_rel"] < 1e-9
    off = cs.compare(ke_ref - 0.001 * t, dt, t_ref, e_ref, scale)  # +0.001 dissipation everywhere
    assert abs(off["rms_err_rel"] - 0.001 / scale) < 1e-9 and abs(off["max_err_rel"] - 0.001 / scale) < 1e-9


def test_recorded_closure_beats_plain_on_two_evaluation_seeds():
    """The committed closure-study records: the best variant beats plain
    coarse LDG on the main evaluation seed, and the best variants, re-run
    against a fine run from a seed that neither training nor the choice of
    variant saw, beat it there too (rms and max dissipation-rate error)."""
    import bench
    r = bench.recorded_closure()
    assert r is not None
    assert r["closure_beats_plain"]
    chk = r["second_eval_seed"]
    assert chk["eval_seed"] != r["config"]["seeds"]["eval"][0]
    assert chk["eval_seed"] not in [s for s, _ in r["config"]["seeds"]["train"]]
    assert chk["closures"] and chk["closure_beats_plain"]
