"""Learned-closure experiment on the Taylor-Green vortex at Re=1600 (command
line for closure_study.run).

Coarse model: 16^3 hexes, p=2, FP64 LDG at the reference time step
(CFL 0.01).  Fine runs: 32^3 hexes, p=4, from the Taylor-Green state with
the seeded 1e-2 V0 velocity perturbation: two training runs (seed 1001,
instances 0 and 1) and one evaluation run (seed 2002).  The fine runs use
CFL 0.02: RK4 is stable on this mesh up to CFL ~0.027 (the largest
eigenvalues of the linearised LDG operator at 32^3, p=4 are real, about
-4500, from the upwind dissipation of the acoustic modes), and the fine
time-step error stays far below the coarse spatial error that the closure
corrects.  By default they run on the mixed-precision path (within ~1e-14
of FP64).

Usage:
    python local-dg_gb300/examples/closure_tgv.py --out results.json \\
        [--t-end 20] [--sample-dt 0.5] [--iters 10000] [--data projected|loop|both] \\
        [--variants '[{"name": ..., "data": "loop", "input_noise": 0.3, "lr_final": 0.05,
                       "modes": [["dissipative", 1.0, 10.0]]}]' | --variants @closure_c5_variants.json]

Writes the JSON summary and the KE series (<out>.npz).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import closure_study  # noqa: E402


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
    ap.add_argument("--data", default="projected", choices=["projected", "loop", "both"])
    ap.add_argument("--fine-precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--eval-seed", type=int, default=closure_study.SEED_EVAL,
                    help="seed of the evaluation run and of the coarse runs (never a training seed)")
    ap.add_argument("--variants", default=None,
                    help="JSON list of closure variants, or @file with one (e.g. @closure_c5_variants.json)")
    args = ap.parse_args()
    variants = None
    if args.variants:
        if args.variants.startswith("@"):
            path = args.variants[1:]
            if not os.path.isabs(path) and not os.path.exists(path):
                path = os.path.join(HERE, path)
            with open(path) as f:
                variants = json.load(f)
        else:
            variants = json.loads(args.variants)
    res, series = closure_study.run(
        coarse_nx=args.coarse_nx, fine_nx=args.fine_nx, t_end=args.t_end, sample_dt=args.sample_dt,
        fine_cfl=args.fine_cfl, iters=args.iters, batch=args.batch, lr=args.lr, hidden=args.hidden, amp=args.amp,
        data=args.data, fine_precision=args.fine_precision,
        variants=variants, eval_seed=args.eval_seed,
        log=lambda *a: print(*a, file=sys.stderr, flush=True))
    res["command"] = " ".join(["python", "local-dg_gb300/examples/closure_tgv.py"] + sys.argv[1:])
    with open(args.out, "w") as f:
        json.dump(res, f, indent=1)
    np.savez(os.path.splitext(args.out)[0] + ".npz", **series)
    print(json.dumps(res["a_posteriori"], indent=1))


if __name__ == "__main__":
    main()
