"""Mixed-precision (FP32-pair arithmetic) against FP64 over a long horizon.

Runs the Taylor-Green vortex (Re=1600, Ma=0.1) twice on the same mesh, once
with the FP64 RHS and once with the FP32-pair RHS (FP64 state, RK
accumulation and reductions in both), to --t-end convective times at the
reference's time step, and reports the relative L2 state difference at the
end, the KE series difference and the KE-dissipation-rate difference
(-(KE_n - KE_{n-2})/(2 dt), solver.cpp:438-440) over the whole run,
relative to the peak dissipation, plus the wall time of each run.

    python local-dg_gb300/examples/mixed_tgv.py --nx 32 --p 4 --t-end 10 --out mixed.json
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=32)
    ap.add_argument("--p", type=int, default=4)
    ap.add_argument("--t-end", type=float, default=10.0)
    ap.add_argument("--out", default="mixed_tgv.json")
    args = ap.parse_args()
    dt0 = 0.01 * (2 * math.pi / args.nx) / (2 * args.p + 1)
    steps = int(math.ceil(args.t_end / dt0))
    res = {"nx": args.nx, "p": args.p, "t_end": args.t_end, "steps": steps}
    out = {}
    for prec in ("fp64", "mixed"):
        with ldg.Solver(args.p, args.nx, steps=steps, precision=prec) as s:
            t0 = time.perf_counter()
            done = 0
            while done < steps:
                k = min(2000, steps - done)
                s.step(k)
                done += k
            s.synchronize()
            sec = time.perf_counter() - t0
            out[prec] = (s.get_state(), s.ke_history(), s.dt)
            res[prec + "_seconds"] = sec
            res[prec + "_ms_per_step"] = 1e3 * sec / steps
    (u64, ke64, dt), (umx, kemx, _) = out["fp64"], out["mixed"]
    eps64 = -(ke64[2:] - ke64[:-2]) / (2 * dt)
    epsmx = -(kemx[2:] - kemx[:-2]) / (2 * dt)
    peak = float(np.max(eps64))
    res.update({
        "dt": dt,
        "state_rel_l2_end": float(np.linalg.norm(umx - u64) / np.linalg.norm(u64)),
        "ke_max_rel_err": float(np.max(np.abs(kemx - ke64) / np.abs(ke64))),
        "dissipation_max_err_rel_to_peak": float(np.max(np.abs(epsmx - eps64)) / peak),
        "dissipation_rms_err_rel_to_peak": float(np.sqrt(np.mean((epsmx - eps64) ** 2)) / peak),
        "peak_dissipation": peak,
        "peak_time": float((np.argmax(eps64) + 2) * dt),
        "speedup": res["fp64_seconds"] / res["mixed_seconds"],
    })
    idx = np.linspace(0, len(eps64) - 1, min(400, len(eps64))).astype(int)
    res["curve"] = {"t": ((idx + 2) * dt).tolist(), "eps_fp64": eps64[idx].tolist(), "eps_mixed": epsmx[idx].tolist()}
    with open(args.out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({k: v for k, v in res.items() if k != "curve"}, indent=1))


if __name__ == "__main__":
    main()
