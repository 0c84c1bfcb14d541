"""Generates the golden vectors in this folder from the unmodified reference.

Runs oracle/_ref/ldg_ref (the reference sources compiled by
oracle/build_ref.sh with the project's MPI/BLAS shim headers) and stores
compact .npz fixtures.  Needs the reference checkout, so it runs only where
that exists; the fixtures it writes are committed and travel everywhere.

    python tests/golden/make_golden.py

Fixtures (arrays use the reference layout u(node,var,elem) = numpy (nE,5,dofs)):
  tgv_n8_p2.npz     Taylor-Green 8^3 p=2, 100 RK4 steps: ke[100], dt,
                    u at steps 0, 1, 10, 100, per-step norms are implied.
  rhs_n{nx}_p{p}.npz  one rk4Rhs on a seeded perturbed Taylor-Green state:
                    u0, k, q (the gradient Dus, (3,nE,5,dofs)), dt.
  step_n{nx}_p{p}.npz  a few RK4 steps from a seeded perturbed state:
                    u0, u_final, ke, steps, dt.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402


def perturbed_state(nx: int, p: int, seed: int) -> np.ndarray:
    """Taylor-Green plus seeded node-wise noise (keeps rho, pressure > 0)."""
    o = oracle.Oracle(nx, p)
    u = o.initial_condition()
    rng = np.random.default_rng(seed)
    r = rng.standard_normal(u.shape)
    u[:, 0, :] *= 1.0 + 0.05 * r[:, 0, :]
    u[:, 1:4, :] += 0.1 * r[:, 1:4, :]
    u[:, 4, :] += 0.5 * r[:, 4, :]
    return u


def meta(path):
    out = {}
    for line in open(path):
        k, v = line.split()
        out[k] = float(v)
    return out


def main():
    if not os.path.exists(oracle.REF_BIN):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        # C1: Taylor-Green 8^3 p2, 100 steps.
        oracle.run_reference(["step", 8, 2, 100, "tgv", 1, 1], tmp)
        m = meta(os.path.join(tmp, "tgv.meta"))
        shape = (512, 5, 27)
        us = {s: np.fromfile(os.path.join(tmp, f"tgv.u{s}")).reshape(shape) for s in (0, 1, 10, 100)}
        np.savez_compressed(os.path.join(HERE, "tgv_n8_p2.npz"),
                            ke=np.fromfile(os.path.join(tmp, "tgv.ke")), dt=m["dt"],
                            u0=us[0], u1=us[1], u10=us[10], u100=us[100], steps=100)
        # One RHS on perturbed states, p = 1..4.
        for nx, p, seed in [(3, 1, 11), (3, 2, 12), (4, 3, 13), (3, 4, 14), (4, 2, 15)]:
            u0 = perturbed_state(nx, p, seed)
            u0.tofile(os.path.join(tmp, "in.u"))
            oracle.run_reference(["rhs", nx, p, "in.u", "r", 1], tmp)
            n = (p + 1) ** 3
            nE = nx ** 3
            k = np.fromfile(os.path.join(tmp, "r.k")).reshape(nE, 5, n)
            q = np.fromfile(os.path.join(tmp, "r.q")).reshape(3, nE, 5, n)
            np.savez_compressed(os.path.join(HERE, f"rhs_n{nx}_p{p}.npz"), u0=u0, k=k, q=q,
                                dt=meta(os.path.join(tmp, "r.meta"))["dt"], seed=seed)
        # A few RK4 steps from perturbed states.
        for nx, p, steps, seed in [(4, 2, 5, 21), (3, 4, 3, 22), (4, 3, 4, 23)]:
            u0 = perturbed_state(nx, p, seed)
            u0.tofile(os.path.join(tmp, "in.u"))
            oracle.run_reference(["step", nx, p, steps, "s", steps, 1, "in.u"], tmp)
            n = (p + 1) ** 3
            nE = nx ** 3
            uf = np.fromfile(os.path.join(tmp, f"s.u{steps}")).reshape(nE, 5, n)
            np.savez_compressed(os.path.join(HERE, f"step_n{nx}_p{p}.npz"), u0=u0, u_final=uf,
                                ke=np.fromfile(os.path.join(tmp, "s.ke")), steps=steps,
                                dt=meta(os.path.join(tmp, "s.meta"))["dt"], seed=seed)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
