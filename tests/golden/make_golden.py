"""Generates the golden vectors in this folder from the unmodified reference.

Runs oracle/_ref/ldg_ref (the reference sources compiled by
oracle/build_ref.sh with the project's MPI/BLAS shim headers) and stores
compact .npz fixtures.  Needs the reference checkout, so it runs only where
that exists; the fixtures it writes are committed and travel everywhere.

    REF_DIR=<reference checkout> python tests/golden/make_golden.py          # small fixtures
    REF_DIR=<reference checkout> python tests/golden/make_golden.py series   # large-mesh series

Fixtures (arrays use the reference layout u(node,var,elem) = numpy (nE,5,dofs)):
  tgv_n8_p2.npz     Taylor-Green 8^3 p=2, 100 RK4 steps: ke[100], dt,
                    u at steps 0, 1, 10, 100, per-step norms are implied.
  rhs_n{nx}_p{p}.npz  one rk4Rhs on a seeded perturbed Taylor-Green state:
                    u0, k, q (the gradient Dus, (3,nE,5,dofs)), dt.
  step_n{nx}_p{p}.npz  a few RK4 steps from a seeded perturbed state:
                    u0, u_final, ke, steps, dt.
  xyzv_n{nx}_p{p}_s{steps}.csv.gz  the reference's own X-Y-Z-V snapshot
                    writer (io.cpp:8-72) on the Taylor-Green state after
                    <steps> RK4 steps (gzip of the text file).
  series_n32_p3.npz  the reference's Taylor-Green run at 32^3 p=3 for 200
                    steps, whose states are too large to store per step:
                    after every step the KE, the per-variable sums of
                    squares (norms, steps x 5) and the entries at seeded
                    flat indices of the (dofs,5,nE) column-major state
                    (idx, samples).
  series_n64_p4.npz  Taylor-Green at 64^3 p=4 for 200 steps.  The first 20
                    steps come from the reference itself (ref_ke, ref_norms,
                    ref_samples at 4096 indices ref_idx, and ref_enst, the
                    enstrophy from the reference's own gradient after
                    steps ref_enst_steps).  All 200 steps come from the
                    oracle's Kronecker-factored chain (ke, norms, samples at
                    1024 indices idx, enst at enst_steps), which is first
                    checked against that window at 1e-12 (the reference
                    needs ~200 s a step at this size on 8 cores; the
                    factored oracle ~15 s).
"""
from __future__ import annotations

import gzip
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


SERIES = [(32, 3, 200, 1024, 32)]  # nx, p, steps, samples, seed


def series(threads: int = 8):
    """The large-mesh per-step series (about 40 min for 32^3 p=3 and 7 min
    for 64^3 p=4 on 8 cores)."""
    if not os.path.exists(oracle.REF_BIN):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        for nx, p, steps, count, seed in SERIES:
            nU = (p + 1) ** 3 * 5 * nx ** 3
            idx = np.sort(np.random.default_rng(seed).choice(nU, count, replace=False)).astype(np.int64)
            idx.tofile(os.path.join(tmp, "idx"))
            oracle.run_reference(["series", nx, p, steps, "ser", "idx", threads], tmp)
            m = meta(os.path.join(tmp, "ser.meta"))
            np.savez_compressed(os.path.join(HERE, f"series_n{nx}_p{p}.npz"), idx=idx,
                                ke=np.fromfile(os.path.join(tmp, "ser.ke")),
                                norms=np.fromfile(os.path.join(tmp, "ser.norms")).reshape(steps, 5),
                                samples=np.fromfile(os.path.join(tmp, "ser.samples")).reshape(steps, count),
                                dt=m["dt"], steps=steps, ke0=m["ke0"], seconds=m["seconds"], threads=threads)
            print(f"series_n{nx}_p{p}: {m['seconds']:.1f} s", flush=True)


SERIES64 = dict(nx=64, p=4, count=4096, seed=64, ref_steps=20, steps=200, ens_every_ref=4, ens_every=10)


def series64_indices():
    c = SERIES64
    nU = (c["p"] + 1) ** 3 * 5 * c["nx"] ** 3
    ref_idx = np.sort(np.random.default_rng(c["seed"]).choice(nU, c["count"], replace=False)).astype(np.int64)
    return ref_idx, ref_idx[::4].copy()


def series64_oracle(out_npz: str, threads: int = 8):
    """Phase 1 of the 64^3 p=4 fixture: the oracle's factored chain over all
    steps, recording per step the KE, norms and the entries at the 4096
    reference sample indices, and the enstrophy at every step that the
    reference window or the fixture records it."""
    c = SERIES64
    ref_idx, _ = series64_indices()
    o = oracle.Oracle(c["nx"], c["p"], steps=c["steps"], threads=threads)
    o.set_factored(True)
    u = o.initial_condition()
    ke, norms, samples, enst, enst_steps = [], [], [], [], []
    for k in range(1, c["steps"] + 1):
        u, kk = o.step(u, 1)
        ke.append(kk[0])
        norms.append(np.einsum("evq,evq->v", u, u))
        samples.append(u.ravel()[ref_idx])
        if k % c["ens_every"] == 0 or (k <= c["ref_steps"] and k % c["ens_every_ref"] == 0):
            enst.append(o.enstrophy(u))
            enst_steps.append(k)
        if k % 10 == 0:
            print(f"series_n64_p4 oracle: step {k}", flush=True)
    np.savez(out_npz, ke=np.array(ke), norms=np.array(norms), samples=np.array(samples), enst=np.array(enst),
             enst_steps=np.array(enst_steps), dt=o.dt, threads=threads)


def series_64(threads: int = 8, ref_dir: str | None = None, oracle_npz: str | None = None):
    """The 64^3 p=4 fixture: the reference's first ref_steps steps (run
    here, or read from ref_dir: the output of `ldg_ref series 64 4 20 ser
    idx <threads> 4` with the seeded indices of series64_indices) pin the
    oracle's factored chain (phase 1, run here or read from oracle_npz),
    which then provides all steps."""
    c = SERIES64
    ref_idx, idx = series64_indices()
    with tempfile.TemporaryDirectory() as tmp:
        if ref_dir is None:
            if not os.path.exists(oracle.REF_BIN):
                subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
            ref_idx.tofile(os.path.join(tmp, "idx"))
            oracle.run_reference(["series", c["nx"], c["p"], c["ref_steps"], "ser", "idx", threads,
                                  c["ens_every_ref"]], tmp)
            ref_dir = tmp
        m = meta(os.path.join(ref_dir, "ser.meta"))
        assert int(m["steps"]) == c["ref_steps"] and int(m["nx"]) == c["nx"] and int(m["p"]) == c["p"]
        R = c["ref_steps"]
        ref_ke = np.fromfile(os.path.join(ref_dir, "ser.ke"))
        ref_norms = np.fromfile(os.path.join(ref_dir, "ser.norms")).reshape(R, 5)
        ref_samples = np.fromfile(os.path.join(ref_dir, "ser.samples")).reshape(R, c["count"])
        ref_e = np.fromfile(os.path.join(ref_dir, "ser.enst")).reshape(-1, 2)
        if oracle_npz is None:
            oracle_npz = os.path.join(tmp, "oracle.npz")
            series64_oracle(oracle_npz, threads)
        z = np.load(oracle_npz)
    assert abs(float(z["dt"]) - m["dt"]) <= 1e-15 * m["dt"]
    ens = dict(zip(z["enst_steps"].tolist(), z["enst"].tolist()))
    # The pin: every step of the reference window.  The state samples and
    # the KE at 1e-12.  The per-variable norms at 1e-11: the reference's
    # driver sums the 32.8M squares of a variable in plain order, whose
    # rounding (~sqrt(N) u ~ 6e-13 of the sum, up to ~1e-12 seen) exceeds
    # the states' own difference; numpy sums pairwise.
    NORM_TOL_REF = 1e-11
    for k in range(1, R + 1):
        tot = np.sqrt(np.sum(ref_norms[k - 1]))
        e_ke = abs(z["ke"][k - 1] - ref_ke[k - 1]) / ref_ke[k - 1]
        e_s = np.linalg.norm(z["samples"][k - 1] - ref_samples[k - 1]) / np.linalg.norm(ref_samples[k - 1])
        e_n = np.max(np.abs(np.sqrt(z["norms"][k - 1]) - np.sqrt(ref_norms[k - 1]))) / tot
        assert e_ke <= 1e-12 and e_s <= 1e-12 and e_n <= NORM_TOL_REF, (k, e_ke, e_s, e_n)
    for k, v in ref_e:
        assert abs(ens[int(k)] - v) <= 1e-12 * abs(v), (k, ens[int(k)], v)
    keep = np.searchsorted(ref_idx, idx)
    fix = [k for k in sorted(ens) if k % c["ens_every"] == 0]
    np.savez_compressed(os.path.join(HERE, "series_n64_p4.npz"), idx=idx, ke=z["ke"], norms=z["norms"],
                        samples=z["samples"][:, keep], dt=z["dt"], steps=c["steps"], ke0=m["ke0"],
                        enst=np.array([ens[k] for k in fix]), enst_steps=np.array(fix),
                        ref_idx=ref_idx, ref_ke=ref_ke, ref_norms=ref_norms, ref_samples=ref_samples,
                        ref_enst=ref_e[:, 1], ref_enst_steps=ref_e[:, 0].astype(np.int64),
                        ref_steps=R, ref_seconds=m["seconds"], threads=threads)
    print("series_n64_p4: pinned to the reference's window and written", flush=True)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "series":
        series()
        series_64()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "series64-oracle":  # <out.npz>: phase 1 alone
        series64_oracle(sys.argv[2])
        return
    if len(sys.argv) > 1 and sys.argv[1] == "series64":  # [ref_dir [oracle.npz]]
        series_64(ref_dir=sys.argv[2] if len(sys.argv) > 2 else None,
                  oracle_npz=sys.argv[3] if len(sys.argv) > 3 else None)
        return
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
        # The reference's CSV snapshots.
        for nx, p, steps in [(4, 2, 0), (3, 3, 5)]:
            oracle.run_reference(["csv", nx, p, steps, "snap", 1], tmp)
            with open(os.path.join(tmp, "snap.0"), "rb") as f_in, \
                    open(os.path.join(HERE, f"xyzv_n{nx}_p{p}_s{steps}.csv.gz"), "wb") as f_out:
                f_out.write(gzip.compress(f_in.read(), mtime=0))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz") or f.endswith(".gz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
