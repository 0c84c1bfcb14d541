"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports
every symbol include/ldg.h declares, and answers host-only calls."""
import ctypes
import os
import re

import pytest

import ldg
from conftest import ROOT, has_gpu


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ldg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ldg_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = ldg.load()
    names = declared_symbols()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
        assert name in ldg.SIGNATURES, f"{name} has no ctypes signature"


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of ldg_config / ldg_info agree with the C compiler."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "sz.c"
    src.write_text('#include "ldg.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(ldg_config), sizeof(ldg_info),'
                   ' offsetof(ldg_config, box_lo), offsetof(ldg_info, device_bytes),'
                   ' sizeof(ldg_closure_options), offsetof(ldg_closure_options, lr_final));}\n')
    exe = tmp_path / "sz"
    subprocess.run([cc, "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert got == [ctypes.sizeof(ldg.LdgConfig), ctypes.sizeof(ldg.LdgInfo),
                   ldg.LdgConfig.box_lo.offset, ldg.LdgInfo.device_bytes.offset,
                   ctypes.sizeof(ldg.LdgClosureOptions), ldg.LdgClosureOptions.lr_final.offset]


def test_config_defaults_follow_reference():
    lib = ldg.load()
    cfg = ldg.LdgConfig()
    assert lib.ldg_config_default(ctypes.byref(cfg)) == 0
    assert (cfg.p, cfg.nx, cfg.dt_snaps) == (2, 10, 10)  # Solver() defaults, solver.cpp:4
    assert (cfg.Re, cfg.Pr, cfg.gamma, cfg.Ma, cfg.cfl) == (1600.0, 0.71, 1.4, 0.1, 0.01)
    assert lib.ldg_abi_version() == 1


def test_error_strings():
    lib = ldg.load()
    assert lib.ldg_error_string(0) == b"LDG_OK"
    assert lib.ldg_error_string(-4) == b"LDG_ERR_NONFINITE"
    assert lib.ldg_error_string(-99) == b"LDG_ERR_UNKNOWN"


def test_invalid_configs_rejected_before_any_device_work():
    lib = ldg.load()
    cfg = ldg.LdgConfig()
    lib.ldg_config_default(ctypes.byref(cfg))
    h = ctypes.c_void_p()
    cfg.nx = 2  # mesh.cpp:102-107: fewer than 3 elements per direction
    assert lib.ldg_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
    cfg.nx = 10
    cfg.p = 9
    assert lib.ldg_create(ctypes.byref(cfg), ctypes.byref(h)) == -5
    cfg.p = 2
    cfg.Re = -1.0
    assert lib.ldg_create(ctypes.byref(cfg), ctypes.byref(h)) == -1
    assert lib.ldg_create(None, ctypes.byref(h)) == -1
    assert lib.ldg_step(None, 1) == -1


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_reports_nodevice():
    lib = ldg.load()
    cfg = ldg.LdgConfig()
    lib.ldg_config_default(ctypes.byref(cfg))
    h = ctypes.c_void_p()
    assert lib.ldg_create(ctypes.byref(cfg), ctypes.byref(h)) == -6


def test_tf_for_steps_matches_reference_rule():
    import oracle
    for nx, p, steps in [(8, 2, 100), (32, 3, 200), (64, 4, 200), (16, 2, 7)]:
        assert ldg.tf_for_steps(nx, p, 1.0, steps) == oracle.tf_for_steps(nx, p, 1.0, steps)


def test_noalloc_rejects_non_fp64_precision_before_device_work():
    """ldg_rhs_noalloc computes in FP64 only: the mixed mode is refused as
    unsupported and an unknown precision value as invalid, before any CUDA
    call (so this runs without a device)."""
    lib = ldg.load()
    cfg = ldg.LdgConfig()
    lib.ldg_config_default(ctypes.byref(cfg))
    cfg.nx = cfg.ny = cfg.nz = 3
    dummy = ctypes.c_void_p(16)  # never dereferenced: the checks come first
    cfg.precision = 1  # LDG_MIXED_F32X2
    assert lib.ldg_rhs_noalloc(ctypes.byref(cfg), dummy, dummy, None) == -5
    assert b"FP64 only" in lib.ldg_last_error_message()
    cfg.precision = 7
    assert lib.ldg_rhs_noalloc(ctypes.byref(cfg), dummy, dummy, None) == -1
