"""Learned-closure experiment on the Taylor-Green vortex at Re=1600.

Coarse model: 16^3 hexes, p=2, FP64 LDG at the reference time step
(CFL 0.01).  Fine runs: 32^3 hexes, p=4, FP64, from the Taylor-Green state
with the seeded 1e-2 V0 velocity perturbation: two training runs (seed 1001,
instances 0 and 1) advanced together by the batched ensemble
(ldg_ensemble_*), then one evaluation run (seed 2002) on a solo solver.
The fine runs use CFL 0.02: RK4 is stable on this mesh up to CFL ~0.027 (the
largest eigenvalues of the linearised LDG operator at 32^3, p=4 are real,
about -4500, from the upwind dissipation of the acoustic modes), and the
fine time-step error stays far below the coarse spatial error that the
closure corrects.

Every --sample-dt the fine states are L2-projected onto the coarse mesh and
paired with the coarse LDG RHS of the projected state
(ldg_closure_add_samples): the training runs give the training set, the
evaluation run the held-out set.  The per-element MLP is trained on the GPU
by the library's kernels and judged against the plain coarse LDG and the
fine FP64 evaluation run:

  a priori      RHS error on the held-out samples, plain vs closure
  a posteriori  KE-dissipation rate -(dKE/dt) (the reference's
                keDissipation, solver.cpp:438-440) of the coarse runs with
                and without the closure, against the fine run, to --t-end;
                the attached closure is energy-stable (its correction never
                raises an element's kinetic energy) and falls back to plain
                LDG outside the training range

One data set can train several closure variants (--variants, a JSON list):
each entry sets the training options (input_noise, lr_final) and lists the
inference modes ([energy, scale] or [energy, scale, ood_sigma]) to run a
posteriori; the network is re-initialised between variants.
--coarse-nx/--fine-nx shrink the meshes for quick studies (defaults: the
16^3 / 32^3 experiment).

Writes a JSON summary after each phase (a partial run still reports) and
the raw KE series to <out>.npz.  Usage:
    python local-dg_gb300/examples/closure_tgv.py --out results.json \
        [--t-end 20] [--sample-dt 0.5] [--iters 10000] [--variants '[...]']
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import ldg  # noqa: E402

SEED_TRAIN = 1001
SEED_EVAL = 2002
P_COARSE, P_FINE = 2, 4
DEFAULT_VARIANTS = [
    {"name": "noise-0.3", "input_noise": 0.3, "lr_final": 0.05,
     "modes": [["dissipative", 1.0, 10.0], ["dissipative", 1.0, 30.0]]},
]


def dt_for(nx, p, cfl):
    return cfl * (2 * math.pi / nx) / (2 * p + 1)


def dissipation(ke, dt):
    """-(KE_n - KE_{n-2}) / (2 dt) at t_{n-1} (solver.cpp:438-440); entry i
    of the KE series is the energy after step i+1."""
    ke = np.asarray(ke)
    eps = -(ke[2:] - ke[:-2]) / (2 * dt)
    t = (np.arange(len(eps)) + 2) * dt
    return t, eps


def compare(name, ke, dt, t_ref, eps_ref, scale):
    t, e = dissipation(ke, dt)
    if len(t) == 0:
        return {"steps": len(ke)}
    err = e - np.interp(t, t_ref, eps_ref)
    late = t >= 1.0  # after the acoustic transient of the initial projection
    return {"steps": len(ke), "t_reached": float((len(ke)) * dt),
            "rms_err_rel": float(np.sqrt(np.mean(err ** 2)) / scale),
            "max_err_rel": float(np.max(np.abs(err)) / scale),
            "rms_err_rel_t_ge_1": float(np.sqrt(np.mean(err[late] ** 2)) / scale) if late.any() else None,
            "max_err_rel_t_ge_1": float(np.max(np.abs(err[late])) / scale) if late.any() else None,
            "peak_dissipation": float(np.max(e)), "peak_time": float(t[int(np.argmax(e))]),
            "final_ke": float(ke[-1])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="closure_tgv.json")
    ap.add_argument("--t-end", type=float, default=20.0)
    ap.add_argument("--sample-dt", type=float, default=0.5)
    ap.add_argument("--fine-cfl", type=float, default=0.02)
    ap.add_argument("--iters", type=int, default=10000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--hidden", type=int, default=128)
    ap.add_argument("--amp", type=float, default=1e-2)
    ap.add_argument("--coarse-nx", type=int, default=16)
    ap.add_argument("--fine-nx", type=int, default=32)
    ap.add_argument("--variants", default=None, help="JSON list of closure variants")
    args = ap.parse_args()
    variants = json.loads(args.variants) if args.variants else DEFAULT_VARIANTS
    res = {"config": vars(args), "coarse": f"{args.coarse_nx}^3 p=2 FP64, CFL 0.01",
           "fine": f"{args.fine_nx}^3 p=4 FP64, CFL {args.fine_cfl}", "variants": variants,
           "seeds": {"train": [[SEED_TRAIN, 0], [SEED_TRAIN, 1]], "eval": [SEED_EVAL, 0]}}
    series = {}

    def save():
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)
        np.savez(os.path.splitext(args.out)[0] + ".npz", **series)

    (ncx, pc), (nfx, pf) = (args.coarse_nx, P_COARSE), (args.fine_nx, P_FINE)
    closure = ldg.Closure(p=pc, hidden=args.hidden, seed=7)
    theta0 = closure.get_params()
    coarse_ws = ldg.Solver(pc, ncx, steps=10)

    dt_f = dt_for(nfx, pf, args.fine_cfl)
    fine_steps = int(math.ceil(args.t_end / dt_f))
    per_sample = max(1, int(round(args.sample_dt / dt_f)))
    n_times = fine_steps // per_sample + 1

    # ---- training data: two fine runs in the batched ensemble
    t0 = time.perf_counter()
    cfgs = [ldg.make_config(pf, nfx, steps=fine_steps, cfl=args.fine_cfl, perturb_amp=args.amp, seed=SEED_TRAIN,
                            instance=i) for i in (0, 1)]
    with ldg.Ensemble(cfgs) as ens, ldg.Solver(pf, nfx, steps=10) as fine_ws:
        for k in range(n_times):
            for m in range(len(cfgs)):
                fine_ws.set_state(ens.get_state(m))
                closure.add_samples(fine_ws, coarse_ws)
            if k + 1 < n_times:
                ens.step(per_sample)
        res["train_runs"] = {"steps": (n_times - 1) * per_sample, "dt": ens.info(0).dt,
                             "sample_every_steps": per_sample, "sample_times": n_times,
                             "seconds": time.perf_counter() - t0, "tuning": ens.tuning()}
    n_train = closure.samples
    save()

    # ---- evaluation run (seed disjoint from training): held-out samples + KE
    t0 = time.perf_counter()
    with ldg.Solver(pf, nfx, steps=fine_steps, cfl=args.fine_cfl, perturb_amp=args.amp, seed=SEED_EVAL,
                    instance=0) as ev:
        for k in range(n_times):
            closure.add_samples(ev, coarse_ws)
            if k + 1 < n_times:
                ev.step(per_sample)
        ev.step(fine_steps - (n_times - 1) * per_sample)
        series["ke_fine"] = ev.ke_history()
        dt_eval = ev.dt
    n_held = closure.samples - n_train
    res["eval_run"] = {"steps": fine_steps, "dt": dt_eval, "seconds": time.perf_counter() - t0}
    save()

    # ---- a posteriori reference: the plain coarse LDG run
    closure.finalize(0, n_train)
    nc_steps = int(math.ceil(args.t_end / dt_for(ncx, pc, 0.01)))

    def coarse_run(name, attach):
        t0 = time.perf_counter()
        with ldg.Solver(pc, ncx, steps=nc_steps, perturb_amp=args.amp, seed=SEED_EVAL, instance=0) as s:
            if attach:
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

    tf_, ef = dissipation(series["ke_fine"], dt_eval)
    scale = float(np.max(ef))
    info = coarse_run("plain", False)
    summary = {"fine": compare("fine", series["ke_fine"], dt_eval, tf_, ef, scale),
               "plain": dict(compare("plain", series["ke_plain"], info["dt"], tf_, ef, scale), **info)}
    res["a_posteriori"] = summary
    save()

    # ---- each variant: train on the GPU, a priori error, a posteriori runs
    res["training"], res["a_priori"] = {}, {}
    per = n_held // n_times
    for var in variants:
        vn = var["name"]
        t0 = time.perf_counter()
        closure.set_params(theta0)
        closure.set_options(input_noise=float(var.get("input_noise", 0.0)),
                            lr_final=float(var.get("lr_final", 1.0)))
        losses = closure.train(0, n_train, iters=args.iters, batch=args.batch, lr=args.lr, seed=3)
        series["losses_" + vn] = losses
        e_plain, e_closure = closure.evaluate(n_train, n_held)
        e_plain_tr, e_closure_tr = closure.evaluate(0, n_train)
        by_time = []
        for k in range(n_times):
            a, b = closure.evaluate(n_train + k * per, per)
            by_time.append([k * per_sample * dt_eval, a, b])
        res["training"][vn] = {"seconds": time.perf_counter() - t0, "samples": n_train,
                               "params": closure.n_params, "loss_first50": float(np.mean(losses[:50])),
                               "loss_last50": float(np.mean(losses[-50:]))}
        res["a_priori"][vn] = {"heldout_samples": n_held, "rhs_err_plain": e_plain, "rhs_err_closure": e_closure,
                               "train_rhs_err_plain": e_plain_tr, "train_rhs_err_closure": e_closure_tr,
                               "heldout_by_time": by_time,
                               "units": "mean squared RHS error over the normalised target channels"}
        for mode in var["modes"]:
            energy, fac = mode[0], float(mode[1])
            ood = float(mode[2]) if len(mode) > 2 else 10.0
            name = f"{vn}/{energy}/x{fac:g}/ood{ood:g}"
            closure.set_options(energy=energy, scale=fac, ood_sigma=ood)
            f0, c0 = closure.fallbacks, closure.clipped
            info = coarse_run(name, True)
            summary[name] = dict(compare(name, series["ke_" + name], info["dt"], tf_, ef, scale), **info)
            summary[name]["fallback_element_stages"] = closure.fallbacks - f0
            summary[name]["projected_element_stages"] = closure.clipped - c0
            save()
    closure.close()
    coarse_ws.close()
    print(json.dumps({k: res[k] for k in ("train_runs", "eval_run", "training", "a_posteriori")}, indent=1))

if __name__ == "__main__":
    main()
