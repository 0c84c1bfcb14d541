"""ldg_rhs_noalloc: the right-hand side for callers that cannot allocate
device memory.

Some applications cannot let a library call cudaMalloc: their GPU memory is
owned by their own arena or by another framework's caching allocator, or
they run a real-time loop in which an allocation (which may synchronise the
device and can fail under fragmentation) is not allowed.  They cannot create
an ldg_solver handle, so ldg_rhs_noalloc takes their input and output device
buffers and keeps its intermediates in a fixed 64 MiB device array that the
library owns.  These tests call it through the C ABI and compare it with the
handle-based ldg_rhs, on two calls in a row (the second call finds the first
call's leftovers in the shared array).

This file sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

import ldg
from conftest import rel_l2

TOL = 1e-12  # the relative-L2 bar of the FP64 parity tests


def seeded_states(solver, seeds):
    """Taylor-Green initial state plus seeded noise, one per seed."""
    u0 = solver.get_state()
    out = []
    for seed in seeds:
        rng = np.random.default_rng(seed)
        u = u0.copy()
        u[:, 0] *= 1.0 + 0.02 * rng.standard_normal(u[:, 0].shape)
        u[:, 1:4] += 0.05 * rng.standard_normal(u[:, 1:4].shape)
        u[:, 4] += 0.2 * rng.standard_normal(u[:, 4].shape)
        out.append(u)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("p,nx", [(3, 4), (4, 3), (2, 5)])
def test_noalloc_rhs_matches_ldg_rhs_on_two_calls(p, nx):
    import torch

    lib = ldg.load()
    with ldg.Solver(p, nx) as s:
        states = seeded_states(s, [31 * p + 1, 31 * p + 2])
        expected = [s.rhs(u) for u in states]
        cfg = s.cfg
    stream = torch.cuda.current_stream()
    for u, k_ref in zip(states, expected):
        du = torch.from_numpy(u).cuda()
        dk = torch.full_like(du, float("nan"))
        torch.cuda.synchronize()
        status = lib.ldg_rhs_noalloc(ctypes.byref(cfg), du.data_ptr(), dk.data_ptr(), stream.cuda_stream)
        assert status == 0, lib.ldg_last_error_message().decode()
        torch.cuda.synchronize()
        assert rel_l2(dk.cpu().numpy(), k_ref) <= TOL


def test_noalloc_rejects_meshes_beyond_the_fixed_scratch():
    """16^3 elements at p=4 need about 140 MB of intermediates, more than the
    64 MiB array; the call is refused before any device work."""
    lib = ldg.load()
    cfg = ldg.LdgConfig()
    lib.ldg_config_default(ctypes.byref(cfg))
    cfg.p, cfg.nx, cfg.ny, cfg.nz = 4, 16, 16, 16
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    status = lib.ldg_rhs_noalloc(ctypes.byref(cfg), dummy, dummy, None)
    assert status == -1
    assert b"scratch" in lib.ldg_last_error_message()
