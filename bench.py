"""Benchmark: RK4 DOF-stage updates/s of the LDG Navier-Stokes RHS on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--nx 64] [--p 4]

One "step" is one classical RK4 time step (four RHS stages) of the periodic
Taylor-Green vortex, Re=1600, Ma=0.1, on an nx^3 hex mesh of order p (default
64^3, p=4: 262,144 elements, 32.8M nodal DOFs x 5 variables, 1.31 GB of
state, larger than L2).  The metric counts nodal DOF-stage updates:
(p+1)^3 * nE * 4 per step.

  value  device-resident: ldg_step on the solver's stream, CUDA events.
  e2e    through the C ABI with host buffers: every step uploads the state
         from pinned host memory, advances one RK4 step and reads the new
         state back (ldg_advance_host, which overlaps the copies with the
         step's first and last passes; e2e.breakdown_ms times the separate
         ldg_set_state / ldg_step / ldg_get_state calls).

--impl reference times the CPU oracle (the restatement of the reference's
dense BLAS/LAPACK path, with OpenBLAS when available and all host threads)
on the same nx^3 order-p mesh, held whole; each of its steps is one RHS
stage over a slab of z-planes (a bounded sample of the stage work).

Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "local-dg_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "RK4 DOF-stage updates/s (FP64 LDG Navier-Stokes RHS, Taylor-Green)"
UNIT = "DOF-stage/s"

# Algorithmic HBM bytes per nodal DOF-stage (FP64): read U, write q (15),
# read U, read q, write k: 8*(5+15+5+15+5) = 360 B.  Split per pass:
BYTES_GRAD = 8 * (5 + 15)        # read U, write q
BYTES_RHS = 8 * (5 + 15 + 5)     # read U, read q, write k / next stage


# Per element and launch, from one ncu --set full capture of the same
# kernels at 24^3 p=4 (13,824 elements; DRAM traffic and instruction counts
# grow in proportion to the element count): DRAM bytes read + written, and
# FP64 floating-point operations executed (2 per DFMA, 1 per DMUL or DADD;
# k_grad: 13,350 DFMA + 5,250 DMUL + 5,100 DADD; k_rhs: 27,925 + 5,450 +
# 2,650).
NCU_PER_ELEMENT = {
    ("grad", 5, "fp64"): {"dram_bytes": (153.860608e6 + 322.368512e6) / 13824, "fp64_flops": 37050.0,
                          "fp64_pipe_ops": 13350.0 + 5250.0 + 5100.0},
    ("rhs", 5, "fp64"): {"dram_bytes": (649.355776e6 + 189.405952e6) / 13824, "fp64_flops": 63950.0,
                         "fp64_pipe_ops": 27925.0 + 5450.0 + 2650.0},
    ("grad", 5, "mixed"): {"dram_bytes": (152.870400e6 + 312.989952e6) / 13824},
    ("rhs", 5, "mixed"): {"dram_bytes": (649.710080e6 + 189.202176e6) / 13824},
}


def read_peak_field(name):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[name])
    except Exception:
        return None


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, pg=None) -> float:
    """The largest of every rank's x (the slowest replica sets the job's
    time); x itself without a process group.  Works on the nccl backend
    (CUDA tensor) and on gloo (CPU tensor)."""
    if pg is None:
        return x
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def host_memory_bytes() -> int:
    """Available host memory (MemAvailable), or total RAM if unknown."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")


def port_bytes(nx: int, p: int) -> int:
    """Host bytes of the dense port at nx^3 order p: its work arrays (23.4
    states: uCurr, the u and Du interpolants, 4 ks, Dus, the face gather
    and the volume fluxes) plus the caller's u and k."""
    return int((p + 1) ** 3 * 5 * nx ** 3 * 8 * 25.5)


def reference_sample(nx: int, p: int, steps: int, warmup: int, planes: int = 16):
    """The reference's CPU path timed on the host cores on the full nx^3
    order-p Taylor-Green workload.  The oracle's dense port (the reference's
    GEMM + LDL^T chain, solver.cpp:486-535, routed to OpenBLAS when present,
    OpenMP over elements elsewhere) holds the whole mesh; each step is one
    rk4Rhs stage whose residual covers `planes` z-planes of it (the
    gradient and face values it needs one and two planes beyond are
    computed too, and not counted as work), followed by the slab's stage
    update.  Returns (DOF-stage/s, seconds, description), or raises
    MemoryError when the host cannot hold the mesh."""
    import numpy as np
    import oracle
    need = port_bytes(nx, p)
    have = host_memory_bytes()
    if need > 0.9 * have:
        raise MemoryError(f"the dense port needs {need / 2**30:.1f} GiB of host memory at {nx}^3 p={p}; "
                          f"{have / 2**30:.1f} GiB available")
    threads = os.cpu_count() or 1
    blas = oracle.find_openblas()
    o = oracle.Oracle(nx, p, steps=1, threads=threads, openblas=blas)
    planes = min(planes, nx - 4)
    z0 = (nx - planes) // 2
    u = o.initial_condition()
    k = np.zeros_like(u)
    sl = slice(z0 * nx * nx, (z0 + planes) * nx * nx)
    b = o.dt / 6.0
    for _ in range(warmup):
        o.rhs_slab(u, k, z0, planes)
        u[sl] += b * k[sl]
    t0 = time.perf_counter()
    for _ in range(steps):
        o.rhs_slab(u, k, z0, planes)
        u[sl] += b * k[sl]
    el = time.perf_counter() - t0
    assert np.all(np.isfinite(u[sl]))
    units = o.dofs * planes * nx * nx * steps
    desc = (f"{nx}^3 p={p} Taylor-Green held whole (dense port, "
            f"{'OpenBLAS' if blas else 'C loops'} + OpenMP x{threads}); each step one rk4Rhs stage over "
            f"z-planes {z0}..{z0 + planes - 1} ({planes * nx * nx} of {nx ** 3} elements; the halo planes "
            f"it needs are computed and not counted)")
    return units / el, el, desc, threads


def cpu_baseline(nx: int, p: int):
    """The oracle on the host cores: a bounded sample (one warm-up and two
    timed slab stages) of the same workload."""
    try:
        value, el, desc, threads = reference_sample(nx, p, steps=2, warmup=1)
    except MemoryError as e:
        return {"value": None, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                "sample": f"unavailable: {e}"}
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc, "seconds": el}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    workload = f"tgv_{args.nx}^3_p{args.p}_fp64"
    try:
        value, el, desc, threads = reference_sample(args.nx, args.p, args.steps, args.warmup)
    except MemoryError as e:
        print(json.dumps({"impl": "reference", "unavailable": str(e), "config": {"workload": workload}}))
        return 0
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (Taylor-Green initial condition, Re=1600, Ma=0.1)",
        "config": {"workload": workload, "nx": args.nx, "p": args.p, "elements": args.nx ** 3,
                   "dofs_per_element": (args.p + 1) ** 3, "precision": "fp64", "same_config": True},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def time_steps(s, K, W, dev, pg=None, clocks=False):
    """W untimed steps, then K timed steps on the solver's stream (CUDA
    events), per-kernel event timings, optional clock sampling."""
    import torch
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    for _ in range(W):
        s.step(1)
    s.synchronize()
    s.enable_kernel_timing(True)
    s.kernel_times(reset=True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(dev) if clocks else None
    if clk:
        clk.__enter__()
    try:
        e0.record(stream)
        s.step(K)
        e1.record(stream)
        torch.cuda.synchronize()
    finally:
        if clk:
            clk.__exit__(None, None, None)
    ms = max_over_ranks(e0.elapsed_time(e1), pg)
    kt = s.kernel_times(reset=True)
    s.enable_kernel_timing(False)
    return ms, kt, (clk.summary() if clk else None)


def accuracy_vs_fp64(p, nx, steps, dev):
    """Mixed path against the FP64 path from the same Taylor-Green state:
    relative L2 state difference after `steps` RK4 steps and the error of
    the KE-dissipation series (solver.cpp:438-440)."""
    import numpy as np
    import ldg
    out = {}
    for prec in ("fp64", "mixed"):
        s = ldg.Solver(p, nx, steps=steps, device=dev, precision=prec)
        s.step(steps)
        out[prec] = (s.get_state(), s.ke_history(), s.ke_dissipation())
        s.close()
    u64, ke64, eps64 = out["fp64"]
    umx, kemx, epsmx = out["mixed"]
    return {"steps": steps,
            "rel_l2_state": float(np.linalg.norm(umx - u64) / np.linalg.norm(u64)),
            "ke_max_rel_err": float(np.max(np.abs(kemx - ke64) / np.abs(ke64))),
            "ke_dissipation_max_err_rel": float(np.max(np.abs(epsmx - eps64)) / np.max(np.abs(eps64)))
            if len(eps64) else None}


def ensemble_variant(count, K, W, dev):
    """The batched ensemble: `count` Taylor-Green members with element counts
    from {8^3,12^3,16^3,24^3}, p from {2,3,4}, Re log-uniform in [400,3200],
    1e-2 V0 seeded perturbations; one persistent launch per RK4 stage, steps
    replayed from a CUDA graph."""
    import torch
    import ldg
    cfgs = ldg.ensemble_configs(count, seed=2024, device=dev, steps=1000)
    t0 = time.perf_counter()
    ens = ldg.Ensemble(cfgs)
    setup_s = time.perf_counter() - t0
    dof_stage = sum(((c.p + 1) ** 3) * c.nx ** 3 * 4 for c in cfgs)
    stream = torch.cuda.ExternalStream(ens.stream, device=dev)
    ens.step(W)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ens.step(K)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    out = {"members": count, "value": dof_stage * K / (ms * 1e-3), "ms_per_step": ms / K,
           "elements_total": sum(c.nx ** 3 for c in cfgs),
           "orders": {str(p): sum(1 for c in cfgs if c.p == p) for p in (2, 3, 4)},
           "setup_s": setup_s, "tuning": ens.tuning(),
           "launches_per_step": 4 + 2, "graph": True}
    ens.close()
    return out


CLOSURE_RECORDS = [os.path.join(ROOT, "local-dg_gb300", "examples", f)
                   for f in ("closure_c5_result.json", "closure_c5_loop_result.json", "closure_c5_loop2_result.json")]
# The best variants evaluated again against a fine run from an evaluation seed
# that neither training nor the choice of variant saw.
CLOSURE_SEED_CHECK = os.path.join(ROOT, "local-dg_gb300", "examples", "closure_c5_seed3003_result.json")


def learned_variant(K, W, dev):
    """The learned-closure configuration: a coarse 16^3 p=2 FP64 Taylor-Green
    solver timed without and with the closure attached (per-element MLP
    inference, energy projection and fallback in every RK stage).  The
    network is trained briefly here on samples from a 32^3 p=4 state, which
    is enough to time its inference; the accuracy of a fully trained closure
    comes from the committed records of the closure study
    (recorded_closure)."""
    import torch
    import ldg
    out = {"coarse": "16^3 p=2 FP64, CFL 0.01", "network": "540-128-128-135 GELU, BF16 mma.sync"}
    with ldg.Closure(p=2, hidden=128, seed=7, device=dev) as c, \
            ldg.Solver(4, 32, steps=10, perturb_amp=1e-2, seed=1001, device=dev) as fine, \
            ldg.Solver(2, 16, steps=10, device=dev) as ws:
        c.add_samples(fine, ws)
        c.finalize(0, c.samples)
        c.train(0, c.samples, iters=200, batch=1024)
        rates = {}
        for name, attach in (("plain", False), ("closure", True)):
            with ldg.Solver(2, 16, steps=max(K + W, 1) + 8, perturb_amp=1e-2, seed=2002, device=dev) as s:
                if attach:
                    s.attach_closure(c)
                stream = torch.cuda.ExternalStream(s.stream, device=dev)
                s.step(W)
                s.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                s.step(K)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                rates[name] = {"value": s.dofs * s.nE * 4 * K / (ms * 1e-3), "ms_per_step": ms / K}
        out.update(rates)
        out["closure_overhead"] = rates["closure"]["ms_per_step"] / rates["plain"]["ms_per_step"]
    out["recorded_a_posteriori"] = recorded_closure()
    return out


def recorded_closure():
    """The a-posteriori accuracy of the fully trained closure from the
    committed records of the closure study: the best variant over the
    records on the main evaluation seed, against plain LDG on that seed, and
    the best variants evaluated again on a second evaluation seed.  None if a
    record is missing."""
    rec_out = None
    try:
        keys = ("rms_err_rel", "max_err_rel", "final_ke", "peak_time")
        runs, cmds = {}, {}
        for path in CLOSURE_RECORDS:
            with open(path) as f:
                rec = json.load(f)
            ap = rec["a_posteriori"]
            src = os.path.relpath(path, ROOT)
            for k, v in ap.items():
                if k not in ("fine", "plain") and v.get("rms_err_rel") is not None:
                    runs[k] = dict(v, source=src)
            cmds[src] = rec.get("command")
        best = min(runs, key=lambda k: runs[k]["rms_err_rel"])
        rec_out = {
            "sources": cmds, "config": rec.get("config"),
            "metric": "KE-dissipation-rate error (solver.cpp:438-440) vs the fine run, t >= 1, rel. to its peak",
            "fine": {k: ap["fine"].get(k) for k in ("final_ke", "peak_time")},
            "plain": {k: ap["plain"].get(k) for k in keys},
            "best_closure": dict({k: runs[best].get(k) for k in keys}, variant=best, source=runs[best]["source"],
                                 fallback_element_stages=runs[best].get("fallback_element_stages")),
            "closure_beats_plain": runs[best]["rms_err_rel"] < ap["plain"]["rms_err_rel"],
            "variants_tried": len(runs)}
        with open(CLOSURE_SEED_CHECK) as f:
            chk = json.load(f)
        cap = chk["a_posteriori"]
        closures = {k: {m: v.get(m) for m in keys} for k, v in cap.items() if k not in ("fine", "plain")}
        rec_out["second_eval_seed"] = {
            "source": os.path.relpath(CLOSURE_SEED_CHECK, ROOT), "command": chk.get("command"),
            "eval_seed": chk["config"]["seeds"]["eval"][0],
            "plain": {m: cap["plain"].get(m) for m in keys}, "closures": closures,
            "closure_beats_plain": all(v["rms_err_rel"] < cap["plain"]["rms_err_rel"] and
                                       v["max_err_rel"] < cap["plain"]["max_err_rel"] for v in closures.values())}
    except (OSError, KeyError, ValueError):
        return None
    return rec_out


def contraction_probe(s, reps=5):
    """The gradient pass's volume contraction alone (15 sum-factorised 1-D
    products per Gauss point) on the solver's state, in the four candidate
    arithmetics: ms per launch and the largest difference from FP64."""
    out = {}
    for mode in ("fp64", "pair_fma", "pair_dot2", "tensor_core_slices"):
        ms, err = s.probe_contraction(mode, reps=reps)
        out[mode] = {"ms": ms, "max_rel_err_vs_fp64": err}
    return out


def run_contraction_probe(args):
    import torch
    import ldg
    torch.cuda.set_device(0)
    ldg.load()
    with ldg.Solver(args.p, args.nx, device=0, perturb_amp=1e-2, seed=5) as s:
        print(json.dumps({"workload": f"tgv_{args.nx}^3_p{args.p}", "contraction_probe":
                          contraction_probe(s, reps=args.probe_reps)}))
    return 0


def run_ours(args):
    import numpy as np
    import torch
    import ldg

    ws, rank, local = dist_env()
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist
    ldg.load()
    K, W = args.steps, args.warmup
    s = ldg.Solver(args.p, args.nx, steps=max(K + W, 1) * 3 + 8, device=dev, check_finite=True,
                   precision=args.precision)
    n_per_step = s.dofs * s.nE * 4

    # ---- device-resident timed region
    ms, kt, clocks = time_steps(s, K, W, dev, pg, clocks=True)
    value = ws * n_per_step * K / (ms * 1e-3)

    # ---- end to end through the C ABI with host buffers
    state_bytes = s.nE * 5 * s.dofs * 8
    host = torch.empty(s.shape, dtype=torch.float64, pin_memory=True).numpy()
    s.get_state(host)
    s.step(1)
    s.synchronize()
    s.advance_host(host, host, 1)  # one untimed end-to-end iteration warms the path
    Ke = 10
    if pg:
        pg.barrier()
    # The interpreter's cyclic garbage collector stays off in the timed loop
    # (as timeit keeps it off): its occasional full passes over the
    # interpreter's objects took tens of ms inside single iterations.
    import gc
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    its = []
    for _ in range(Ke):
        ti = time.perf_counter()
        s.advance_host(host, host, 1)  # upload, one RK4 step, download, overlapped
        its.append(time.perf_counter() - ti)
    e2e_elapsed = time.perf_counter() - t0
    gc.enable()
    e2e_s = max_over_ranks(e2e_elapsed, pg)
    its_in_order = [round(t * 1e3, 2) for t in its]
    its.sort()
    assert np.all(np.isfinite(host))
    # where an end-to-end step goes (untimed diagnostic: each call waited
    # for), with the transfers overlapped with the transforms in 8 chunks
    # (the default) and copied whole before transforming (1 chunk)
    breakdown = {}
    for chunks in (8, 1):
        s.set_transfer_chunks(chunks)
        parts = {"set_state": [], "step": [], "get_state": []}
        for _ in range(3):
            t = time.perf_counter()
            s.set_state(host)
            s.synchronize()
            parts["set_state"].append(time.perf_counter() - t)
            t = time.perf_counter()
            s.step(1)
            s.synchronize()
            parts["step"].append(time.perf_counter() - t)
            t = time.perf_counter()
            s.get_state(host)
            parts["get_state"].append(time.perf_counter() - t)
        breakdown[f"chunks_{chunks}"] = {k: 1e3 * sorted(v)[1] for k, v in parts.items()}
    s.set_transfer_chunks(8)
    e2e = {"value": ws * n_per_step * Ke / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes, "steps": Ke,
           "ms_per_step": e2e_s * 1e3 / Ke,
           "iteration_ms": {"min": its[0] * 1e3, "median": its[len(its) // 2] * 1e3, "max": its[-1] * 1e3,
                            "in_order": its_in_order},
           "api": "ldg_advance_host (host state in, one RK4 step, host state out)",
           "breakdown_ms": breakdown}

    # ---- roofline of the dominant kernel (live event timings above)
    hbm_peak, peak_kind = read_peaks()
    dom = "rhs" if kt["rhs"][0] >= kt["grad"][0] else "grad"
    dom_ms, dom_n = kt[dom]
    avg_s = dom_ms * 1e-3 / max(dom_n, 1)
    per_dof = BYTES_RHS if dom == "rhs" else BYTES_GRAD
    alg_bytes = per_dof * s.dofs * s.nE
    achieved = alg_bytes / avg_s / 1e9
    N = args.p + 1
    ncu = NCU_PER_ELEMENT.get((dom, N, args.precision), {})
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak,
                "traffic": ncu["dram_bytes"] * s.nE if "dram_bytes" in ncu else None,
                "algorithmic_bytes": alg_bytes,
                "kernel": f"k_{dom}<{N},{'double' if args.precision == 'fp64' else 'dd'}>",
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback"}
    if "fp64_flops" in ncu:
        # The pipe that binds: FP64 operations per launch of the same
        # kernel, against the larger of the probe's measured FP64 rate and
        # the rate derived from SMs x max SM clock x FP64 FMAs per SM per
        # clock (the probe's clock64 reading, rounded up to a whole FMA) x 2.
        import math
        pr = ldg.probe_fp64(dev)
        props = torch.cuda.get_device_properties(dev)
        max_mhz = (clocks or {}).get("sm_max_mhz") or read_peak_field("sm_max_mhz") or pr["sm_mhz"]
        fma_clk = float(math.ceil(pr["fma_per_sm_clk"] - 0.05))
        derived = props.multi_processor_count * max_mhz * 1e6 * fma_clk * 2 / 1e12
        peak, src = (derived, f"derived: {props.multi_processor_count} SMs x {max_mhz:.0f} MHz x "
                              f"{fma_clk:.0f} FP64 FMA/SM/clk x 2") if derived >= pr["tflops"] else \
                    (pr["tflops"], "measured (ldg_probe_fp64 FMA chains)")
        fp64_achieved = ncu["fp64_flops"] * s.nE / avg_s / 1e12
        roofline["binding_roof"] = {"pipe": "fp64", "achieved_tflops": fp64_achieved, "peak_tflops": peak,
                                    "frac": fp64_achieved / peak, "peak_source": src,
                                    "probe": pr, "derived_peak_tflops": derived,
                                    "flops_per_dof": ncu["fp64_flops"] / N ** 3,
                                    "flops_source": "ncu instruction counts, 24^3 p=4 capture"}
        # The same in FP64 pipe instructions: a DMUL or DADD takes a pipe slot
        # as a DFMA does but counts one flop, so flops understate how busy
        # the pipe is.  Instructions per SM per clock (at the sampled SM
        # clock) against the probe's FMAs per SM per clock.
        clk = (clocks or {}).get("sm_mhz") or max_mhz
        per_clk = ncu["fp64_pipe_ops"] * s.nE / avg_s / (props.multi_processor_count * clk * 1e6)
        roofline["binding_roof"]["pipe_issue"] = {
            "fp64_instructions_per_sm_clk": per_clk, "probe_fma_per_sm_clk": pr["fma_per_sm_clk"],
            "frac_of_probe": per_clk / pr["fma_per_sm_clk"], "sm_mhz": clk,
            "instructions_per_element": ncu["fp64_pipe_ops"],
            "source": "DFMA + DMUL + DADD per element from the same ncu capture"}
    kernel_ms = {k: {"total_ms": v[0], "launches": v[1], "avg_ms": v[0] / max(v[1], 1)} for k, v in kt.items()}
    contraction = None
    if args.precision == "fp64" and not args.no_variants and args.p == 4:
        contraction = contraction_probe(s, reps=5)
    s.close()

    # ---- the mixed-precision variant on the same workload, and its error
    variants = {}
    if args.precision == "fp64" and not args.no_variants:
        sm = ldg.Solver(args.p, args.nx, steps=max(K + W, 1) * 3 + 8, device=dev, precision="mixed")
        ms_m, kt_m, _ = time_steps(sm, K, W, dev, pg)
        sm.close()
        mixed = {"value": ws * n_per_step * K / (ms_m * 1e-3), "ms_per_step": ms_m / K,
                 "speedup_vs_fp64": ms / ms_m,
                 "kernels": {k: {"total_ms": v[0], "launches": v[1]} for k, v in kt_m.items()},
                 "arithmetic": "RHS in FP32-pair (double-word) arithmetic; FP64 state, RK4, reductions"}
        if args.accuracy_steps > 0:
            mixed["accuracy_vs_fp64"] = accuracy_vs_fp64(args.p, args.nx, args.accuracy_steps, dev)
        variants["mixed_f32x2"] = mixed

    if contraction:
        variants["contraction_probe"] = contraction
    if args.precision == "fp64" and not args.no_variants and args.ensemble > 0:
        variants["ensemble"] = ensemble_variant(args.ensemble, K, W, dev)
    if args.precision == "fp64" and not args.no_variants:
        variants["learned"] = learned_variant(K, W, dev)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (Taylor-Green initial condition, Re=1600, Ma=0.1)",
        "config": {"workload": f"tgv_{args.nx}^3_p{args.p}_{args.precision}", "nx": args.nx, "p": args.p,
                   "elements": s.nE, "dofs_per_element": s.dofs, "precision": args.precision,
                   "l2": "inputs larger than L2 (state 1.31 GB at 64^3 p4)" if s.nE * s.dofs * 40 > 129e6
                   else "inputs smaller than L2", "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "e2e": e2e,
        "roofline": roofline,
        "kernels": kernel_ms,
        "gpu_launches": int(kt["grad"][1] + kt["rhs"][1] + kt["reduce"][1]),
        "clocks": clocks,
        "variants": variants,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.nx, args.p)
    if rank == 0:
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=64)
    ap.add_argument("--p", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--ensemble", type=int, default=64, help="members of the ensemble variant (0: skip)")
    ap.add_argument("--contraction-probe", action="store_true",
                    help="only time the gradient volume contraction in each arithmetic")
    ap.add_argument("--probe-reps", type=int, default=5)
    args = ap.parse_args()
    if args.contraction_probe:
        return run_contraction_probe(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
