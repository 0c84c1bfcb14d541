"""ctypes front end of the CPU oracle (oracle/ldg_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, the smoke check and bench.py's CPU
baseline leg use it as the checker or the timed CPU baseline.  The product
(local-dg_gb300/) never imports it.

State arrays use the reference layout, darray u(node, var, elem) column
major (Local-DG solver.cpp:62), which is a C-order numpy array of shape
(nE, 5, dofs).
"""
from __future__ import annotations

import ctypes
import glob
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libldg_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ldg_ref")

_lib = None


def build(force: bool = False) -> str:
    """Compiles libldg_oracle.so with the Makefile beside this file."""
    src = os.path.join(HERE, "ldg_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-C", HERE, "libldg_oracle.so"], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i, d, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_double)
        L.ldgo_create.restype = vp
        L.ldgo_create.argtypes = [i, i, i, i, d, d, d, i]
        L.ldgo_create_blas.restype = vp
        L.ldgo_create_blas.argtypes = [i, i, i, i, d, d, d, i]
        L.ldgo_use_openblas.restype = i
        L.ldgo_use_openblas.argtypes = [ctypes.c_char_p, i]
        L.ldgo_destroy.argtypes = [vp]
        L.ldgo_dt.restype = d
        L.ldgo_dt.argtypes = [vp]
        L.ldgo_set_dt.argtypes = [vp, d]
        L.ldgo_timesteps.restype = ctypes.c_long
        L.ldgo_timesteps.argtypes = [vp]
        L.ldgo_dofs.restype = i
        L.ldgo_dofs.argtypes = [vp]
        L.ldgo_nelements.restype = i
        L.ldgo_nelements.argtypes = [vp]
        L.ldgo_initial_condition.argtypes = [vp, dp]
        L.ldgo_initial_condition_perturbed.argtypes = [vp, dp, d, dp]
        L.ldgo_rhs.argtypes = [vp, dp, dp]
        L.ldgo_step.argtypes = [vp, dp, i, dp]
        L.ldgo_compute_ke.restype = d
        L.ldgo_compute_ke.argtypes = [vp, dp]
        L.ldgo_set_factored.argtypes = [vp, i]
        L.ldgo_rhs_slab.restype = i
        L.ldgo_rhs_slab.argtypes = [vp, dp, dp, i, i]
        L.ldgo_enstrophy.restype = d
        L.ldgo_enstrophy.argtypes = [vp, dp]
        L.ldgo_get_operator.restype = i
        L.ldgo_get_operator.argtypes = [vp, i, dp]
        _lib = L
    return _lib


def tf_for_steps(nx: int, p: int, L: float, steps: int) -> float:
    """Final time whose CFL step count (solver.cpp:47-52) is exactly `steps`;
    the same rule oracle/ref_driver.cpp uses to produce the golden vectors."""
    size = math.pi * L
    min_dx = (size - (-size)) / nx
    dt0 = 0.01 * min_dx / (1.0 * (2 * p + 1))
    tf = steps * dt0
    while math.ceil(tf / dt0) > steps:
        tf = np.nextafter(tf, 0.0)
    return float(tf)


_MASK = (1 << 64) - 1


def splitmix64(z: int) -> int:
    """SplitMix64 (Steele, Lea & Flood 2014)."""
    z = (z + 0x9E3779B97F4A7C15) & _MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
    return z ^ (z >> 31)


def perturbation_phases(seed: int, instance: int) -> np.ndarray:
    """Phases [component][wavenumber-1][direction] of the seeded velocity
    perturbation of the ensemble inputs."""
    base = splitmix64(seed ^ splitmix64((0x4C44470000000000 + instance) & _MASK))
    phi = np.zeros((3, 4, 3))
    for c in range(3):
        for k in range(4):
            for d in range(3):
                r = splitmix64((base + c * 16 + k * 4 + d) & _MASK)
                phi[c, k, d] = 2.0 * math.pi * (r >> 11) * (1.0 / 9007199254740992.0)
    return phi


def find_openblas() -> str | None:
    """scipy's bundled OpenBLAS, if scipy is installed."""
    try:
        import scipy
    except Exception:
        return None
    libs = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__) + ".libs",
                                         "libscipy_openblas-*.so")))
    return libs[0] if libs else None


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One periodic Taylor-Green problem on an nx^3 mesh of order p."""

    def __init__(self, nx: int, p: int, steps: int = 1, L: float = 1.0, Re: float = 1600.0,
                 threads: int = 1, openblas: str | None = None, tf: float | None = None):
        L_ = lib()
        if tf is None:
            tf = tf_for_steps(nx, p, L, steps)
        if openblas:
            if L_.ldgo_use_openblas(openblas.encode(), threads) != 0:
                raise RuntimeError(f"cannot load OpenBLAS from {openblas}")
            h = L_.ldgo_create_blas(nx, nx, nx, p, L, tf, Re, threads)
            L_.ldgo_use_openblas(None, 0)
        else:
            h = L_.ldgo_create(nx, nx, nx, p, L, tf, Re, threads)
        if not h:
            raise ValueError(f"oracle rejected nx={nx} p={p}")
        self._h = h
        self.nx, self.p, self.L, self.Re = nx, p, L, Re
        self.dofs = L_.ldgo_dofs(h)
        self.nE = L_.ldgo_nelements(h)
        self.dt = L_.ldgo_dt(h)
        self.timesteps = L_.ldgo_timesteps(h)
        self.shape = (self.nE, 5, self.dofs)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.ldgo_destroy(h)
            self._h = None

    def set_factored(self, on: bool = True) -> None:
        """Dense operator chain (the reference's GEMM structure) or the
        Kronecker-factored one: the same discrete operator, different
        rounding, O(N^4) instead of O(N^6) work per element."""
        lib().ldgo_set_factored(self._h, 1 if on else 0)

    def enstrophy(self, u: np.ndarray) -> float:
        """rho |curl v|^2 / 2 integrated with the Gauss rule from the LDG
        gradient of u, normalised like computeKE."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        return lib().ldgo_enstrophy(self._h, _ptr(u))

    def set_dt(self, dt: float) -> None:
        lib().ldgo_set_dt(self._h, dt)
        self.dt = dt

    def initial_condition(self, perturb_amp: float = 0.0, seed: int = 0, instance: int = 0) -> np.ndarray:
        u = np.zeros(self.shape)
        if perturb_amp:
            phi = np.ascontiguousarray(perturbation_phases(seed, instance).ravel())
            lib().ldgo_initial_condition_perturbed(self._h, _ptr(u), perturb_amp / 12.0, _ptr(phi))
        else:
            lib().ldgo_initial_condition(self._h, _ptr(u))
        return u

    def rhs(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        k = np.zeros(self.shape)
        lib().ldgo_rhs(self._h, _ptr(u), _ptr(k))
        return k

    def rhs_slab(self, u: np.ndarray, k: np.ndarray, z0: int, planes: int) -> None:
        """The dense RHS for the residual of z-planes [z0, z0+planes) only
        (with the halo planes it needs), written into k's slab columns: a
        bounded sample of a large mesh's stage work."""
        assert u.shape == self.shape and k.shape == self.shape
        if lib().ldgo_rhs_slab(self._h, _ptr(u), _ptr(k), z0, planes) != 0:
            raise ValueError(f"slab z0={z0} planes={planes} does not fit nz={self.nx}")

    def step(self, u: np.ndarray, nsteps: int = 1):
        u = np.array(u, dtype=np.float64, order="C", copy=True)
        ke = np.zeros(max(nsteps, 1))
        lib().ldgo_step(self._h, _ptr(u), nsteps, _ptr(ke))
        return u, ke[:nsteps]

    def ke(self, u: np.ndarray) -> float:
        u = np.ascontiguousarray(u, dtype=np.float64)
        return lib().ldgo_compute_ke(self._h, _ptr(u))

    def operator(self, which: int) -> np.ndarray:
        sizes = {0: self.dofs ** 0, }
        n, nf = self.dofs, round(self.dofs ** (2 / 3))
        count = {0: nf * nf, 1: n * n, 2: n * n * 3, 3: nf * nf * 3, 4: n * n * 3, 5: n}[which]
        out = np.zeros(count)
        lib().ldgo_get_operator(self._h, which, _ptr(out))
        del sizes
        return out


def run_reference(args, cwd):
    """Runs the reference build (oracle/_ref/ldg_ref); only where the
    reference sources were present to build it."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError(REF_BIN)
    return subprocess.run([REF_BIN] + [str(a) for a in args], cwd=cwd, check=True,
                          capture_output=True, text=True)


if __name__ == "__main__":
    o = Oracle(int(sys.argv[1]), int(sys.argv[2]), steps=int(sys.argv[3]))
    u = o.initial_condition()
    u, ke = o.step(u, int(sys.argv[3]))
    print(o.dt, ke)


def node_coordinates(nx: int, p: int, L: float = 1.0) -> np.ndarray:
    """Coordinates (nE, 3, dofs) of the CGL nodes of a periodic nx^3 mesh on
    [-pi L, pi L]^3: element vertices ix*(hi-lo)/nx + lo (mesh.cpp:128-146),
    nodes lo_e + (xi+1)/2 (hi_e - lo_e) with xi = cos((p-i) pi/p)
    (dgMath.cpp:41, mesh.cpp:396-407), node i = ix + iy N + iz N^2."""
    N = p + 1
    lo, hi = -math.pi * L, math.pi * L
    xi = np.array([math.cos((p - i) * math.pi / p) for i in range(N)])
    out = np.zeros((nx ** 3, 3, N ** 3))
    for k in range(nx ** 3):
        idx = (k % nx, (k // nx) % nx, k // (nx * nx))
        for l in range(3):
            a = idx[l] * (hi - lo) / nx + lo
            b = (idx[l] + 1) * (hi - lo) / nx + lo
            for i in range(N ** 3):
                c = (i % N, (i // N) % N, i // (N * N))
                out[k, l, i] = a + .5 * (xi[c[l]] + 1.0) * (b - a)
    return out


def xyzv_text(coords: np.ndarray, u: np.ndarray) -> str:
    """The reference's X-Y-Z-V CSV (initXYZVFile + exportToXYZVFile,
    io.cpp:8-72) of a state u (nE, 5, dofs): header, then per element and
    node 'x, y, z, u0, ..., u4', each value as a C++ stream prints a double
    by default (%.6g)."""
    lines = ["X, Y, Z, u0, u1, u2, u3, u4"]
    nE, _, n = u.shape
    for k in range(nE):
        for i in range(n):
            vals = list(coords[k, :, i]) + list(u[k, :, i])
            lines.append(", ".join("%.6g" % v for v in vals))
    return "\n".join(lines) + "\n"
