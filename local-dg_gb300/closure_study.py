"""Training and judging the learned closure on the Taylor-Green vortex.

A coarse FP64 LDG solver (order 2) gets a per-element correction learned
from fine runs (order 4 on a mesh r times finer), and is judged a posteriori
on the kinetic-energy dissipation rate -dKE/dt (the reference's
keDissipation, Local-DG solver.cpp:438-440) against a fine run from a seed
that the training never saw.

Data, from fine runs sampled every `sample_dt`:
  projected  the fine state and RHS L2-projected onto the coarse mesh, with
             the coarse RHS of the projected state (ldg_closure_add_samples);
  loop       solver in the loop: at each sample time a coarse solver starts
             from the projected fine state (ldg_closure_project_state) and
             runs on its own until the next sample time, where its state
             gives the features and P(K_f) - K_c(u_c) the target
             (ldg_closure_add_samples_coarse); these are the states the
             coarse solver produces itself, which is what an attached
             closure sees;
  both       the two sets together.
The fine runs may use the mixed-precision path (fine_precision="mixed",
within ~1e-14 of FP64, 2.7x faster at p=4); samples are taken from an FP64
copy of their state.

Each variant trains the network from the same initial parameters (options
input_noise, lr_final) and runs the coarse solver with the closure attached
in one or more inference modes (energy projection, output scale, fallback
range).  run() returns a JSON-able summary.
"""
from __future__ import annotations

import math
import time

import numpy as np

import ldg

SEED_TRAIN = 1001
SEED_EVAL = 2002
P_COARSE, P_FINE = 2, 4


def dt_for(nx: int, p: int, cfl: float) -> float:
    """The reference's time step rule (solver.cpp:47-52) at CFL `cfl`."""
    return cfl * (2 * math.pi / nx) / (2 * p + 1)


def dissipation(ke, dt):
    """-(KE_n - KE_{n-2}) / (2 dt) at t_{n-1} (solver.cpp:438-440); entry i
    of the KE series is the energy after step i+1."""
    ke = np.asarray(ke)
    eps = -(ke[2:] - ke[:-2]) / (2 * dt)
    t = (np.arange(len(eps)) + 2) * dt
    return t, eps


def compare(ke, dt, t_ref, eps_ref, scale, t_from=1.0):
    """Dissipation-rate error of a KE series against the reference rate,
    relative to the reference's peak rate; rms and max over t >= t_from
    (after the acoustic transient of the initial projection)."""
    t, e = dissipation(ke, dt)
    if len(t) == 0:
        return {"steps": len(ke)}
    err = e - np.interp(t, t_ref, eps_ref)
    late = t >= t_from
    return {"steps": len(ke), "t_reached": float(len(ke) * dt),
            "rms_err_rel": float(np.sqrt(np.mean(err[late] ** 2)) / scale) if late.any() else None,
            "max_err_rel": float(np.max(np.abs(err[late])) / scale) if late.any() else None,
            "peak_dissipation": float(np.max(e)), "peak_time": float(t[int(np.argmax(e))]),
            "final_ke": float(ke[-1])}


class _Fine:
    """A fine run, FP64 or mixed, with an FP64 view of its state for the
    closure's sampling."""

    def __init__(self, nx, steps, cfl, amp, seed, instance, precision, view):
        self.s = ldg.Solver(P_FINE, nx, steps=steps, cfl=cfl, perturb_amp=amp, seed=seed, instance=instance,
                            precision=precision)
        self.view = view if precision != "fp64" else None

    def fp64(self):
        if self.view is None:
            return self.s
        self.view.set_state(self.s.get_state())
        return self.view

    def close(self):
        self.s.close()


def run(coarse_nx=16, fine_nx=32, t_end=20.0, sample_dt=0.5, fine_cfl=0.02, iters=10000, batch=4096, lr=1e-3,
        hidden=128, amp=1e-2, data="projected", fine_precision="mixed", variants=None, device=0, log=None,
        eval_seed=SEED_EVAL):
    """The experiment; returns the summary and the KE series.  Each variant
    may name its own data set ("data": projected | loop | both; default the
    `data` argument); every data set needed is collected from the same fine
    runs, in a closure object of its own."""
    variants = variants or [{"name": "noise-0.3", "input_noise": 0.3, "lr_final": 0.05,
                             "modes": [["dissipative", 1.0, 10.0]]}]
    for v in variants:
        v.setdefault("data", data)
    kinds = sorted({v["data"] for v in variants})
    say = log or (lambda *a: None)
    res = {"config": {"coarse": f"{coarse_nx}^3 p={P_COARSE} FP64, CFL 0.01",
                      "fine": f"{fine_nx}^3 p={P_FINE} {fine_precision}, CFL {fine_cfl}",
                      "t_end": t_end, "sample_dt": sample_dt, "iters": iters, "data": kinds,
                      "seeds": {"train": [[SEED_TRAIN, 0], [SEED_TRAIN, 1]], "eval": [eval_seed, 0]}}}
    series = {}
    closures = {k: ldg.Closure(p=P_COARSE, hidden=hidden, seed=7, device=device) for k in kinds}
    theta0 = closures[kinds[0]].get_params()
    coarse_ws = ldg.Solver(P_COARSE, coarse_nx, steps=10, device=device)
    fine_view = ldg.Solver(P_FINE, fine_nx, steps=10, device=device) if fine_precision != "fp64" else None

    dt_f = dt_for(fine_nx, P_FINE, fine_cfl)
    fine_steps = int(math.ceil(t_end / dt_f))
    per_sample = max(1, int(round(sample_dt / dt_f)))
    n_times = fine_steps // per_sample + 1
    dt_c = dt_for(coarse_nx, P_COARSE, 0.01)
    coarse_per_sample = max(1, int(round(per_sample * dt_f / dt_c)))

    # ---- training data: two fine runs (seed SEED_TRAIN, instances 0 and 1)
    t0 = time.perf_counter()
    fines = [_Fine(fine_nx, fine_steps, fine_cfl, amp, SEED_TRAIN, i, fine_precision, fine_view) for i in (0, 1)]
    need_loop = any(k in ("loop", "both") for k in kinds)
    loops = [ldg.Solver(P_COARSE, coarse_nx, steps=10, device=device) for _ in fines] if need_loop else []
    any_c = closures[kinds[0]]
    for k in range(n_times):
        for m, f in enumerate(fines):
            fv = f.fp64()
            for kind, c in closures.items():
                if kind in ("projected", "both"):
                    c.add_samples(fv, coarse_ws)
                if kind in ("loop", "both") and k > 0:
                    c.add_samples_coarse(fv, loops[m])
            if loops:
                any_c.project_state(fv, loops[m])
        if k + 1 < n_times:
            for f in fines:
                f.s.step(per_sample)
            for c in loops:
                c.step(coarse_per_sample)
    for f in fines:
        f.close()
    for c in loops:
        c.close()
    n_train = {kind: c.samples for kind, c in closures.items()}
    res["train_runs"] = {"steps": (n_times - 1) * per_sample, "dt": dt_f, "sample_every_steps": per_sample,
                         "sample_times": n_times, "samples": n_train, "seconds": time.perf_counter() - t0}
    say("training data", res["train_runs"])

    # ---- evaluation run (seed disjoint from training): held-out samples + KE
    t0 = time.perf_counter()
    ev = _Fine(fine_nx, fine_steps, fine_cfl, amp, eval_seed, 0, fine_precision, fine_view)
    for k in range(n_times):
        fv = ev.fp64()
        for c in closures.values():
            c.add_samples(fv, coarse_ws)
        if k + 1 < n_times:
            ev.s.step(per_sample)
    ev.s.step(fine_steps - (n_times - 1) * per_sample)
    series["ke_fine"] = ev.s.ke_history()
    ev.close()
    if fine_view is not None:
        fine_view.close()
    n_held = {kind: c.samples - n_train[kind] for kind, c in closures.items()}
    res["eval_run"] = {"steps": fine_steps, "dt": dt_f, "seconds": time.perf_counter() - t0}
    say("evaluation run", res["eval_run"])

    # ---- a posteriori reference: the plain coarse LDG run
    for kind, c in closures.items():
        c.finalize(0, n_train[kind])
    nc_steps = int(math.ceil(t_end / dt_c))

    def coarse_run(name, closure):
        t0 = time.perf_counter()
        with ldg.Solver(P_COARSE, coarse_nx, steps=nc_steps, perturb_amp=amp, seed=eval_seed, instance=0,
                        device=device) as s:
            if closure is not None:
                s.attach_closure(closure)
            status, done = "ok", 0
            try:
                while done < nc_steps:
                    k = min(1000, nc_steps - done)
                    s.step(k)
                    done += k
            except ldg.LdgError as e:  # a run that blew up keeps its KE so far
                status = f"stopped near step {done + 1}: {e}"
            ke = s.ke_history()
            bad = np.flatnonzero(~np.isfinite(ke))
            series["ke_" + name] = ke[:bad[0]] if bad.size else ke
            return {"status": status, "dt": s.dt, "seconds": time.perf_counter() - t0}

    tf_, ef = dissipation(series["ke_fine"], dt_f)
    scale = float(np.max(ef))
    info = coarse_run("plain", None)
    summary = {"fine": compare(series["ke_fine"], dt_f, tf_, ef, scale),
               "plain": dict(compare(series["ke_plain"], info["dt"], tf_, ef, scale), **info)}
    res["a_posteriori"] = summary
    res["training"], res["a_priori"] = {}, {}
    for var in variants:
        vn, closure = var["name"], closures[var["data"]]
        t0 = time.perf_counter()
        closure.set_params(theta0)
        closure.set_options(input_noise=float(var.get("input_noise", 0.0)), lr_final=float(var.get("lr_final", 1.0)))
        nt = n_train[var["data"]]
        losses = closure.train(0, nt, iters=iters, batch=batch, lr=lr, seed=3)
        e_plain, e_closure = closure.evaluate(nt, n_held[var["data"]])
        res["training"][vn] = {"data": var["data"], "seconds": time.perf_counter() - t0, "samples": nt,
                               "loss_first50": float(np.mean(losses[:50])), "loss_last50": float(np.mean(losses[-50:]))}
        res["a_priori"][vn] = {"heldout_samples": n_held[var["data"]], "rhs_err_plain": e_plain,
                               "rhs_err_closure": e_closure}
        for mode in var["modes"]:
            energy, fac = mode[0], float(mode[1])
            ood = float(mode[2]) if len(mode) > 2 else 10.0
            name = f"{vn}/{energy}/x{fac:g}/ood{ood:g}"
            closure.set_options(energy=energy, scale=fac, ood_sigma=ood)
            f0, c0 = closure.fallbacks, closure.clipped
            info = coarse_run(name, closure)
            summary[name] = dict(compare(series["ke_" + name], info["dt"], tf_, ef, scale), **info)
            summary[name]["data"] = var["data"]
            summary[name]["fallback_element_stages"] = closure.fallbacks - f0
            summary[name]["projected_element_stages"] = closure.clipped - c0
            say(name, summary[name])
    for c in closures.values():
        c.close()
    coarse_ws.close()
    return res, series
