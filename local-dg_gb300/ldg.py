"""Python front end of libldg_gb300.so (the C ABI in include/ldg.h).

Mirrors the reference's Solver interface (Local-DG solver.h:109-113):
``Solver(p, dt_snaps, tf, L, mesh)`` plus ``dg_time_step()``, and exposes the
seam the GPU path replaces: ``rhs(u)`` (Solver::rk4Rhs, solver.cpp:486-535)
and ``step(n)`` (the RK4 loop body of Solver::dgTimeStep,
solver.cpp:410-440).  State arrays use the reference layout
u(node, var, elem) column major == numpy C-order (nE, 5, dofs).

The library is built in-tree by :func:`build` (nvcc, sm_103a).  There is no
CPU fallback: every call goes through the CUDA library, and loading fails
loudly if it is missing.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libldg_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE] + ARCH
SOURCES = ["ldg_capi.cu", "ldg_noalloc.cu", "ldg_ensemble.cu", "ldg_closure.cu", "ldg_ops.cpp", "ldg_io.cpp"]

LDG_OK = 0
LDG_HOST = 0
LDG_DEVICE = 1
LDG_FP64 = 0
LDG_MIXED_F32X2 = 1
PRECISIONS = {"fp64": LDG_FP64, "mixed": LDG_MIXED_F32X2}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles libldg_gb300.so for sm_103a (translation units in parallel)."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc, "-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-c",
                   os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


class LdgConfig(ctypes.Structure):
    _fields_ = [
        ("p", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("L", ctypes.c_double), ("tf", ctypes.c_double), ("dt_snaps", ctypes.c_int),
        ("Re", ctypes.c_double), ("Pr", ctypes.c_double), ("gamma", ctypes.c_double),
        ("Ma", ctypes.c_double), ("cfl", ctypes.c_double), ("precision", ctypes.c_int),
        ("device", ctypes.c_int), ("check_finite", ctypes.c_int), ("use_box", ctypes.c_int),
        ("box_lo", ctypes.c_double * 3), ("box_hi", ctypes.c_double * 3),
        ("perturb_amp", ctypes.c_double), ("seed", ctypes.c_ulonglong), ("instance", ctypes.c_int),
        ("reserved", ctypes.c_int * 7),
    ]


class LdgInfo(ctypes.Structure):
    _fields_ = [
        ("p", ctypes.c_int), ("dofs", ctypes.c_int), ("nf", ctypes.c_int),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nelements", ctypes.c_int),
        ("dt", ctypes.c_double), ("timesteps", ctypes.c_longlong), ("step", ctypes.c_longlong),
        ("time", ctypes.c_double), ("device_bytes", ctypes.c_size_t), ("precision", ctypes.c_int),
    ]


class LdgClosureOptions(ctypes.Structure):
    _fields_ = [("input_noise", ctypes.c_float), ("energy", ctypes.c_int), ("scale", ctypes.c_float),
                ("ood_sigma", ctypes.c_float), ("lr_final", ctypes.c_float), ("reserved", ctypes.c_int * 3)]


CLOSURE_ENERGY = {"none": 0, "dissipative": 1, "neutral": 2}

# Every symbol include/ldg.h declares, with its ctypes signature.
_vp, _i, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
SIGNATURES = {
    "ldg_config_default": (_i, [ctypes.POINTER(LdgConfig)]),
    "ldg_create": (_i, [ctypes.POINTER(LdgConfig), ctypes.POINTER(_vp)]),
    "ldg_destroy": (_i, [_vp]),
    "ldg_get_info": (_i, [_vp, ctypes.POINTER(LdgInfo)]),
    "ldg_set_state": (_i, [_vp, _vp, _i]),
    "ldg_get_state": (_i, [_vp, _vp, _i]),
    "ldg_set_initial_condition": (_i, [_vp]),
    "ldg_rhs": (_i, [_vp, _vp, _vp, _i]),
    "ldg_step": (_i, [_vp, _i]),
    "ldg_time_step": (_i, [_vp]),
    "ldg_diagnostics": (_i, [_vp, _dp, _dp, _dp]),
    "ldg_ke_history": (_i, [_vp, _dp, _i, _ip]),
    "ldg_ke_dissipation": (_i, [_vp, _dp, _i, _ip]),
    "ldg_synchronize": (_i, [_vp]),
    "ldg_write_xyzv": (_i, [_vp, ctypes.c_char_p, _i]),
    "ldg_set_snapshots": (_i, [_vp, ctypes.c_char_p, _i]),
    "ldg_save_checkpoint": (_i, [_vp, ctypes.c_char_p]),
    "ldg_checkpoint_config": (_i, [ctypes.c_char_p, ctypes.POINTER(LdgConfig)]),
    "ldg_load_checkpoint": (_i, [_vp, ctypes.c_char_p]),
    "ldg_stream": (_vp, [_vp]),
    "ldg_enable_kernel_timing": (_i, [_vp, _i]),
    "ldg_kernel_times": (_i, [_vp, _dp, ctypes.POINTER(ctypes.c_longlong), _i, _i]),
    "ldg_probe_fp64_peak": (_i, [_i, _dp]),
    "ldg_probe_fp64": (_i, [_i, _dp, _dp, _dp]),
    "ldg_probe_recip": (_i, [_i, _vp, _vp, _vp, ctypes.c_long]),
    "ldg_operators_1d": (_i, [_i, _vp, _vp, _vp, _vp, _vp]),
    "ldg_probe_contraction": (_i, [_vp, _i, _i, _dp, _dp]),
    "ldg_set_transfer_chunks": (_i, [_vp, _i]),
    "ldg_advance_host": (_i, [_vp, _vp, _vp, _i]),
    "ldg_rhs_noalloc": (_i, [ctypes.POINTER(LdgConfig), _vp, _vp, _vp]),
    "ldg_ensemble_create": (_i, [ctypes.POINTER(LdgConfig), _i, ctypes.POINTER(_vp)]),
    "ldg_ensemble_destroy": (_i, [_vp]),
    "ldg_ensemble_step": (_i, [_vp, _i]),
    "ldg_ensemble_get_state": (_i, [_vp, _i, _vp, _i]),
    "ldg_ensemble_ke_history": (_i, [_vp, _i, _dp, _i, _ip]),
    "ldg_ensemble_member_info": (_i, [_vp, _i, ctypes.POINTER(LdgInfo)]),
    "ldg_ensemble_tuning": (_i, [_vp, _ip, _ip, ctypes.POINTER(ctypes.c_float), _i]),
    "ldg_ensemble_stream": (_vp, [_vp]),
    "ldg_ensemble_set_wait_limit": (_i, [_vp, ctypes.c_longlong, _i]),
    "ldg_ensemble_recovered_steps": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "ldg_ensemble_inject_stall": (_i, [_vp, _i, _i]),
    "ldg_closure_create": (_i, [_i, _i, ctypes.c_ulonglong, _i, ctypes.POINTER(_vp)]),
    "ldg_closure_destroy": (_i, [_vp]),
    "ldg_closure_add_samples": (_i, [_vp, _vp, _vp]),
    "ldg_closure_project_state": (_i, [_vp, _vp, _vp]),
    "ldg_closure_add_samples_coarse": (_i, [_vp, _vp, _vp]),
    "ldg_closure_sample_count": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "ldg_closure_finalize_data": (_i, [_vp, ctypes.c_longlong, ctypes.c_longlong]),
    "ldg_closure_train": (_i, [_vp, ctypes.c_longlong, ctypes.c_longlong, _i, _i, ctypes.c_float,
                               ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_float)]),
    "ldg_closure_evaluate": (_i, [_vp, ctypes.c_longlong, ctypes.c_longlong, _dp, _dp]),
    "ldg_closure_param_count": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "ldg_closure_get_params": (_i, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "ldg_closure_set_params": (_i, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "ldg_closure_get_stats": (_i, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "ldg_closure_mlp_forward": (_i, [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), _i]),
    "ldg_closure_mlp_backward": (_i, [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), _i,
                                      ctypes.POINTER(ctypes.c_float)]),
    "ldg_closure_fallbacks": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "ldg_closure_counters": (_i, [_vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "ldg_closure_get_options": (_i, [_vp, ctypes.POINTER(LdgClosureOptions)]),
    "ldg_closure_set_options": (_i, [_vp, ctypes.POINTER(LdgClosureOptions)]),
    "ldg_closure_get_samples": (_i, [_vp, ctypes.c_longlong, ctypes.c_longlong, ctypes.POINTER(ctypes.c_float),
                                     ctypes.POINTER(ctypes.c_float)]),
    "ldg_solver_attach_closure": (_i, [_vp, _vp]),
    "ldg_error_string": (ctypes.c_char_p, [_i]),
    "ldg_last_error_message": (ctypes.c_char_p, []),
    "ldg_abi_version": (_i, []),
}

_lib = None


def load(path: str | None = None):
    """Loads the CUDA library (building it first if needed)."""
    global _lib
    if _lib is None:
        path = path or build()
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def probe_fp64_peak(device: int = 0) -> float:
    """Measured FP64 FMA rate of the device in TFLOP/s."""
    out = ctypes.c_double()
    _check(load().ldg_probe_fp64_peak(device, ctypes.byref(out)), "ldg_probe_fp64_peak")
    return out.value


def probe_fp64(device: int = 0) -> dict:
    """The FP64 probe's readings: TFLOP/s, FMAs per SM per clock and the SM
    clock (MHz) it ran at."""
    t, r, m = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _check(load().ldg_probe_fp64(device, ctypes.byref(t), ctypes.byref(r), ctypes.byref(m)), "ldg_probe_fp64")
    return {"tflops": t.value, "fma_per_sm_clk": r.value, "sm_mhz": m.value}


def operators_1d(p: int) -> dict:
    """The 1-D element operators of order p as the library builds them (host
    only): Gauss points x, weights w, weak derivative A (N x N, A[q, r]) and
    face lifts Lp, Lm."""
    N = p + 1
    out = {k: np.zeros(N) for k in ("x", "w", "Lp", "Lm")}
    out["A"] = np.zeros((N, N))
    _check(load().ldg_operators_1d(p, out["x"].ctypes.data, out["w"].ctypes.data, out["A"].ctypes.data,
                                    out["Lp"].ctypes.data, out["Lm"].ctypes.data), "ldg_operators_1d")
    return out


def probe_recip(x, device: int = 0):
    """The flux kernels' FP64 reciprocal and reciprocal square root applied
    on the device to the float64 array x: returns (1/x, 1/sqrt(x))."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    r, rs = np.empty_like(x), np.empty_like(x)
    _check(load().ldg_probe_recip(device, x.ctypes.data, r.ctypes.data, rs.ctypes.data, x.size),
           "ldg_probe_recip")
    return r, rs


class LdgError(RuntimeError):
    def __init__(self, status: int, where: str):
        L = load()
        super().__init__(f"{where}: {L.ldg_error_string(status).decode()} "
                         f"({L.ldg_last_error_message().decode()})")
        self.status = status


def _check(status: int, where: str):
    if status != LDG_OK:
        raise LdgError(status, where)


def tf_for_steps(nx: int, p: int, L: float, steps: int, cfl: float = 0.01) -> float:
    """Final time whose CFL step count (solver.cpp:47-52) is exactly steps."""
    size = math.pi * L
    dt0 = cfl * ((size - (-size)) / nx) / (1.0 * (2 * p + 1))
    tf = steps * dt0
    while math.ceil(tf / dt0) > steps:
        tf = float(np.nextafter(tf, 0.0))
    return float(tf)


def _arg(a, where_hint=None):
    """(pointer, where, keepalive) for a numpy array or a CUDA torch tensor."""
    if isinstance(a, np.ndarray):
        a = np.ascontiguousarray(a, dtype=np.float64)
        return a.ctypes.data, LDG_HOST, a
    t = a
    if getattr(t, "is_cuda", False):
        assert t.is_contiguous() and str(t.dtype) == "torch.float64"
        return t.data_ptr(), LDG_DEVICE, t
    raise TypeError("expected a numpy array or a CUDA float64 torch tensor")


class Solver:
    """GPU LDG solver on an nx x ny x nz periodic hex mesh of order p."""

    def __init__(self, p: int, nx: int, ny: int | None = None, nz: int | None = None, *, L: float = 1.0,
                 tf: float | None = None, steps: int | None = None, Re: float = 1600.0, Pr: float = 0.71,
                 gamma: float = 1.4, Ma: float = 0.1, cfl: float = 0.01, device: int = 0,
                 check_finite: bool = True, dt_snaps: int = 0, box=None, precision: str = "fp64",
                 perturb_amp: float = 0.0, seed: int = 0, instance: int = 0):
        L_ = load()
        cfg = LdgConfig()
        _check(L_.ldg_config_default(ctypes.byref(cfg)), "ldg_config_default")
        cfg.p, cfg.nx = p, nx
        cfg.ny = ny if ny is not None else nx
        cfg.nz = nz if nz is not None else nx
        cfg.L = L
        if tf is None:
            tf = tf_for_steps(max(cfg.nx, cfg.ny, cfg.nz), p, L, steps if steps else 1, cfl)
        cfg.tf = tf
        cfg.Re, cfg.Pr, cfg.gamma, cfg.Ma, cfg.cfl = Re, Pr, gamma, Ma, cfl
        cfg.device = device
        cfg.precision = PRECISIONS[precision]
        cfg.perturb_amp, cfg.seed, cfg.instance = perturb_amp, seed, instance
        cfg.check_finite = 1 if check_finite else 0
        cfg.dt_snaps = dt_snaps
        if box is not None:
            cfg.use_box = 1
            for l in range(3):
                cfg.box_lo[l], cfg.box_hi[l] = box[0][l], box[1][l]
        self._open(cfg)

    def _open(self, cfg: "LdgConfig") -> None:
        h = ctypes.c_void_p()
        _check(load().ldg_create(ctypes.byref(cfg), ctypes.byref(h)), "ldg_create")
        self._h = h
        self.cfg = cfg
        info = self.info()
        self.p, self.dofs, self.nE, self.dt = cfg.p, info.dofs, info.nelements, info.dt
        self.timesteps = info.timesteps
        self.shape = (self.nE, 5, self.dofs)

    @classmethod
    def from_config(cls, cfg: "LdgConfig") -> "Solver":
        """A solver for an ldg_config (e.g. one stored in a checkpoint)."""
        self = cls.__new__(cls)
        self._open(cfg)
        return self

    @classmethod
    def from_checkpoint(cls, path: str) -> "Solver":
        """A solver created from a checkpoint's config with its state,
        step count and KE series loaded (ldg_checkpoint_config +
        ldg_load_checkpoint)."""
        cfg = LdgConfig()
        _check(load().ldg_checkpoint_config(os.fsencode(path), ctypes.byref(cfg)), "ldg_checkpoint_config")
        self = cls.from_config(cfg)
        self.load_checkpoint(path)
        return self

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ldg_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def info(self) -> LdgInfo:
        info = LdgInfo()
        _check(load().ldg_get_info(self._h, ctypes.byref(info)), "ldg_get_info")
        return info

    def set_state(self, u) -> None:
        ptr, where, keep = _arg(u)
        _check(load().ldg_set_state(self._h, ptr, where), "ldg_set_state")
        if where == LDG_DEVICE:
            self.synchronize()
        del keep

    def set_transfer_chunks(self, chunks: int) -> None:
        """Host transfers in `chunks` element ranges overlapped with the basis
        transforms (1: copy everything, then transform)."""
        _check(load().ldg_set_transfer_chunks(self._h, chunks), "ldg_set_transfer_chunks")

    def advance_host(self, u_in, u_out, nsteps: int = 1) -> None:
        """set_state(u_in), step(nsteps), get_state(u_out) in one call that
        overlaps the host transfers with the step (host numpy arrays; they
        may be the same array)."""
        a, _, ka = _arg(u_in)
        b, _, kb = _arg(u_out)
        assert isinstance(u_out, np.ndarray) and kb is u_out, "u_out must be a C-contiguous float64 array"
        _check(load().ldg_advance_host(self._h, a, b, nsteps), "ldg_advance_host")
        del ka, kb

    def get_state(self, out=None):
        if out is None:
            out = np.empty(self.shape)
        ptr, where, keep = _arg(out)
        _check(load().ldg_get_state(self._h, ptr, where), "ldg_get_state")
        if where == LDG_DEVICE:
            self.synchronize()
        return keep if where == LDG_DEVICE else out

    def set_initial_condition(self) -> None:
        _check(load().ldg_set_initial_condition(self._h), "ldg_set_initial_condition")

    def rhs(self, u, out=None):
        ptr, where, keep = _arg(u)
        if out is None:
            out = np.empty(self.shape) if where == LDG_HOST else None
            if out is None:
                import torch
                out = torch.empty_like(keep)
        optr, owhere, okeep = _arg(out)
        assert owhere == where, "input and output must live on the same side"
        _check(load().ldg_rhs(self._h, ptr, optr, where), "ldg_rhs")
        if where == LDG_DEVICE:
            self.synchronize()
        return out

    def step(self, nsteps: int = 1) -> None:
        _check(load().ldg_step(self._h, nsteps), "ldg_step")

    def dg_time_step(self) -> None:
        _check(load().ldg_time_step(self._h), "ldg_time_step")

    CONTRACTION_MODES = {"fp64": 0, "pair_fma": 1, "pair_dot2": 2, "tensor_core_slices": 3}

    def probe_contraction(self, mode: str, reps: int = 10):
        """Times the gradient pass's volume contraction in one arithmetic
        (see CONTRACTION_MODES) on the current state: (ms per launch, largest
        difference from FP64 relative to the largest value)."""
        ms, err = ctypes.c_double(), ctypes.c_double()
        _check(load().ldg_probe_contraction(self._h, self.CONTRACTION_MODES[mode], reps, ctypes.byref(ms),
                                            ctypes.byref(err)), "ldg_probe_contraction")
        return ms.value, err.value

    def diagnostics(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _check(load().ldg_diagnostics(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "ldg_diagnostics")
        return a.value, b.value, c.value

    def ke_history(self) -> np.ndarray:
        cnt = ctypes.c_int()
        _check(load().ldg_ke_history(self._h, None, 0, ctypes.byref(cnt)), "ldg_ke_history")
        out = np.zeros(cnt.value)
        if cnt.value:
            _check(load().ldg_ke_history(self._h, out.ctypes.data_as(_dp), cnt.value, ctypes.byref(cnt)),
                   "ldg_ke_history")
        return out

    def ke_dissipation(self) -> np.ndarray:
        cnt = ctypes.c_int()
        _check(load().ldg_ke_dissipation(self._h, None, 0, ctypes.byref(cnt)), "ldg_ke_dissipation")
        out = np.zeros(cnt.value)
        if cnt.value:
            _check(load().ldg_ke_dissipation(self._h, out.ctypes.data_as(_dp), cnt.value, ctypes.byref(cnt)),
                   "ldg_ke_dissipation")
        return out

    def synchronize(self) -> None:
        _check(load().ldg_synchronize(self._h), "ldg_synchronize")

    def write_xyzv(self, filename: str, timeseries: int = -1) -> None:
        """The reference's X-Y-Z-V CSV snapshot (io.cpp:8-72) of the state,
        to <filename>.<timeseries> (or <filename> when timeseries < 0)."""
        _check(load().ldg_write_xyzv(self._h, os.fsencode(filename), timeseries), "ldg_write_xyzv")

    def set_snapshots(self, filename: str | None, every: int | None = None) -> None:
        """dg_time_step writes <filename>.<k> before step k*every
        (solver.cpp:366-381); every defaults to dt_snaps.  None: off."""
        every = self.cfg.dt_snaps if every is None else every
        name = os.fsencode(filename) if filename else None
        _check(load().ldg_set_snapshots(self._h, name, every if filename else 0), "ldg_set_snapshots")

    def save_checkpoint(self, path: str) -> None:
        _check(load().ldg_save_checkpoint(self._h, os.fsencode(path)), "ldg_save_checkpoint")

    def load_checkpoint(self, path: str) -> None:
        _check(load().ldg_load_checkpoint(self._h, os.fsencode(path)), "ldg_load_checkpoint")
        info = self.info()
        self.timesteps = info.timesteps

    def attach_closure(self, closure) -> None:
        """Adds the closure's correction to every RK stage (None: plain LDG)."""
        _check(load().ldg_solver_attach_closure(self._h, closure._h if closure is not None else None),
               "ldg_solver_attach_closure")
        self._closure = closure

    def enable_kernel_timing(self, enable: bool = True) -> None:
        _check(load().ldg_enable_kernel_timing(self._h, 1 if enable else 0), "ldg_enable_kernel_timing")

    def kernel_times(self, reset: bool = False):
        """{class: (total_ms, launches)} for 'grad', 'rhs', 'reduce'."""
        ms = (ctypes.c_double * 3)()
        n = (ctypes.c_longlong * 3)()
        _check(load().ldg_kernel_times(self._h, ms, n, 3, 1 if reset else 0), "ldg_kernel_times")
        return {name: (ms[i], n[i]) for i, name in enumerate(("grad", "rhs", "reduce"))}

    @property
    def stream(self) -> int:
        return load().ldg_stream(self._h)


def make_config(p: int, nx: int, *, steps: int | None = None, tf: float | None = None, L: float = 1.0,
                Re: float = 1600.0, Pr: float = 0.71, gamma: float = 1.4, Ma: float = 0.1, cfl: float = 0.01,
                device: int = 0, precision: str = "fp64", perturb_amp: float = 0.0, seed: int = 0,
                instance: int = 0, check_finite: bool = True) -> LdgConfig:
    """An ldg_config for an nx^3 periodic Taylor-Green problem."""
    cfg = LdgConfig()
    _check(load().ldg_config_default(ctypes.byref(cfg)), "ldg_config_default")
    cfg.p, cfg.nx, cfg.ny, cfg.nz = p, nx, nx, nx
    cfg.L = L
    cfg.tf = tf if tf is not None else tf_for_steps(nx, p, L, steps if steps else 1, cfl)
    cfg.Re, cfg.Pr, cfg.gamma, cfg.Ma, cfg.cfl = Re, Pr, gamma, Ma, cfl
    cfg.device, cfg.precision = device, PRECISIONS[precision]
    cfg.perturb_amp, cfg.seed, cfg.instance = perturb_amp, seed, instance
    cfg.check_finite = 1 if check_finite else 0
    return cfg


def ensemble_configs(count: int = 64, seed: int = 2024, device: int = 0, steps: int = 1000):
    """The batched-ensemble inputs: element counts uniform in {8^3, 12^3,
    16^3, 24^3}, p uniform in {2, 3, 4}, Re log-uniform in [400, 3200],
    Ma = 0.1, velocity perturbation of amplitude 1e-2 V0 over wavenumbers
    1-4 with phases keyed by (seed, member)."""
    rng = np.random.default_rng(seed)
    cfgs = []
    for i in range(count):
        nx = int(rng.choice([8, 12, 16, 24]))
        p = int(rng.choice([2, 3, 4]))
        Re = float(np.exp(rng.uniform(np.log(400.0), np.log(3200.0))))
        cfgs.append(make_config(p, nx, steps=steps, Re=Re, Ma=0.1, device=device, perturb_amp=1e-2,
                                seed=seed, instance=i))
    return cfgs


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class Closure:
    """The learned RHS closure (ldg_closure_*)."""

    def __init__(self, p: int = 2, hidden: int = 128, seed: int = 0, device: int = 0):
        h = ctypes.c_void_p()
        _check(load().ldg_closure_create(p, hidden, seed, device, ctypes.byref(h)), "ldg_closure_create")
        self._h = h
        self.p, self.hidden = p, hidden
        n = (p + 1) ** 3
        self.in_dim, self.out_dim = 20 * n, 5 * n

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ldg_closure_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_samples(self, fine: "Solver", coarse: "Solver") -> None:
        _check(load().ldg_closure_add_samples(self._h, fine._h, coarse._h), "ldg_closure_add_samples")

    def project_state(self, fine: "Solver", coarse: "Solver") -> None:
        """The coarse solver's state becomes the projection of the fine one's."""
        _check(load().ldg_closure_project_state(self._h, fine._h, coarse._h), "ldg_closure_project_state")

    def add_samples_coarse(self, fine: "Solver", coarse: "Solver") -> None:
        """Samples with the coarse solver's own state as features (solver in
        the loop) and P(K_f) - K_c(u_c) as target."""
        _check(load().ldg_closure_add_samples_coarse(self._h, fine._h, coarse._h), "ldg_closure_add_samples_coarse")

    @property
    def samples(self) -> int:
        c = ctypes.c_longlong()
        _check(load().ldg_closure_sample_count(self._h, ctypes.byref(c)), "ldg_closure_sample_count")
        return c.value

    def finalize(self, first: int, count: int) -> None:
        _check(load().ldg_closure_finalize_data(self._h, first, count), "ldg_closure_finalize_data")

    def train(self, first: int, count: int, iters: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0):
        losses = np.zeros(max(iters, 1), dtype=np.float32)
        _check(load().ldg_closure_train(self._h, first, count, iters, batch, lr, seed, _fp(losses)),
               "ldg_closure_train")
        return losses[:iters]

    def evaluate(self, first: int, count: int):
        a, b = ctypes.c_double(), ctypes.c_double()
        _check(load().ldg_closure_evaluate(self._h, first, count, ctypes.byref(a), ctypes.byref(b)),
               "ldg_closure_evaluate")
        return a.value, b.value

    @property
    def n_params(self) -> int:
        c = ctypes.c_longlong()
        _check(load().ldg_closure_param_count(self._h, ctypes.byref(c)), "ldg_closure_param_count")
        return c.value

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.n_params, dtype=np.float32)
        _check(load().ldg_closure_get_params(self._h, _fp(out)), "ldg_closure_get_params")
        return out

    def set_params(self, theta) -> None:
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        _check(load().ldg_closure_set_params(self._h, _fp(theta)), "ldg_closure_set_params")

    def stats(self) -> np.ndarray:
        out = np.zeros(50, dtype=np.float32)
        _check(load().ldg_closure_get_stats(self._h, _fp(out)), "ldg_closure_get_stats")
        return out

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros((x.shape[0], self.out_dim), dtype=np.float32)
        _check(load().ldg_closure_mlp_forward(self._h, _fp(x), _fp(y), x.shape[0]), "ldg_closure_mlp_forward")
        return y

    def backward(self, x, dy) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        dy = np.ascontiguousarray(dy, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        _check(load().ldg_closure_mlp_backward(self._h, _fp(x), _fp(dy), x.shape[0], _fp(g)),
               "ldg_closure_mlp_backward")
        return g

    def get_samples(self, first: int, count: int):
        X = np.zeros((count, self.in_dim), dtype=np.float32)
        Y = np.zeros((count, self.out_dim), dtype=np.float32)
        _check(load().ldg_closure_get_samples(self._h, first, count, _fp(X), _fp(Y)), "ldg_closure_get_samples")
        return X, Y

    def options(self) -> dict:
        o = LdgClosureOptions()
        _check(load().ldg_closure_get_options(self._h, ctypes.byref(o)), "ldg_closure_get_options")
        energy = {v: k for k, v in CLOSURE_ENERGY.items()}[o.energy]
        return {"input_noise": o.input_noise, "energy": energy, "scale": o.scale, "ood_sigma": o.ood_sigma,
                "lr_final": o.lr_final}

    def set_options(self, **kw) -> None:
        """input_noise, energy ('none' | 'dissipative' | 'neutral'), scale,
        ood_sigma, lr_final (ldg_closure_set_options)."""
        cur = self.options()
        unknown = set(kw) - set(cur)
        if unknown:
            raise TypeError(f"unknown closure options {sorted(unknown)}")
        cur.update(kw)
        o = LdgClosureOptions(cur["input_noise"], CLOSURE_ENERGY[cur["energy"]], cur["scale"], cur["ood_sigma"],
                              cur["lr_final"])
        _check(load().ldg_closure_set_options(self._h, ctypes.byref(o)), "ldg_closure_set_options")

    @property
    def clipped(self) -> int:
        """Element-stage corrections whose KE-raising part was removed."""
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        _check(load().ldg_closure_counters(self._h, ctypes.byref(a), ctypes.byref(b)), "ldg_closure_counters")
        return b.value

    @property
    def fallbacks(self) -> int:
        c = ctypes.c_longlong()
        _check(load().ldg_closure_fallbacks(self._h, ctypes.byref(c)), "ldg_closure_fallbacks")
        return c.value


class Ensemble:
    """Members advanced together by ldg_ensemble_* (one persistent launch per
    RK4 stage, CUDA-graph steps)."""

    def __init__(self, cfgs):
        L_ = load()
        arr = (LdgConfig * len(cfgs))(*cfgs)
        h = ctypes.c_void_p()
        _check(L_.ldg_ensemble_create(arr, len(cfgs), ctypes.byref(h)), "ldg_ensemble_create")
        self._h = h
        self.cfgs = list(cfgs)
        self.count = len(cfgs)

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ldg_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def info(self, member: int) -> LdgInfo:
        info = LdgInfo()
        _check(load().ldg_ensemble_member_info(self._h, member, ctypes.byref(info)), "ldg_ensemble_member_info")
        return info

    def step(self, nsteps: int = 1) -> None:
        _check(load().ldg_ensemble_step(self._h, nsteps), "ldg_ensemble_step")

    def get_state(self, member: int) -> np.ndarray:
        info = self.info(member)
        out = np.empty((info.nelements, 5, info.dofs))
        _check(load().ldg_ensemble_get_state(self._h, member, out.ctypes.data, LDG_HOST), "ldg_ensemble_get_state")
        return out

    def ke_history(self, member: int) -> np.ndarray:
        cnt = ctypes.c_int()
        _check(load().ldg_ensemble_ke_history(self._h, member, None, 0, ctypes.byref(cnt)), "ke_history")
        out = np.zeros(cnt.value)
        if cnt.value:
            _check(load().ldg_ensemble_ke_history(self._h, member, out.ctypes.data_as(_dp), cnt.value,
                                                  ctypes.byref(cnt)), "ke_history")
        return out

    def tuning(self):
        t, g = ctypes.c_int(), ctypes.c_int()
        ms = (ctypes.c_float * 8)()
        _check(load().ldg_ensemble_tuning(self._h, ctypes.byref(t), ctypes.byref(g), ms, 8), "ldg_ensemble_tuning")
        return {"threads_per_cta": t.value, "persistent_ctas": g.value,
                "stage_ms": {f"{128 * (1 + k // 4)}x{k % 4}": ms[k] for k in range(8)}}

    @property
    def stream(self) -> int:
        return load().ldg_ensemble_stream(self._h)

    def set_wait_limit(self, polls: int, recover: bool = True) -> None:
        """Bounded-wait limit (polls of ~100 ns) and whether a step whose wait
        ran out is re-run member by member (True) or reported (False)."""
        _check(load().ldg_ensemble_set_wait_limit(self._h, polls, 1 if recover else 0),
               "ldg_ensemble_set_wait_limit")

    def recovered_steps(self) -> int:
        n = ctypes.c_longlong()
        _check(load().ldg_ensemble_recovered_steps(self._h, ctypes.byref(n)), "ldg_ensemble_recovered_steps")
        return n.value

    def inject_stall(self, member: int, on: bool = True) -> None:
        """Test hook: member's RHS items wait for a gradient item that never
        comes (host-side fault injection)."""
        _check(load().ldg_ensemble_inject_stall(self._h, member, 1 if on else 0), "ldg_ensemble_inject_stall")
