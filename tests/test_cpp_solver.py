"""The reference-style C++ interface (include/ldg_solver.hpp): the example
driver compiles and links against the CUDA library on any machine, and on a
GPU it reproduces the oracle's Taylor-Green run through Solver::dgTimeStep."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import ldg
import oracle
from conftest import ROOT


def build_driver(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = ldg.build()
    exe = tmp_path / "driver"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "local-dg_gb300", "examples", "driver.cpp"),
                    "-L" + os.path.dirname(lib), "-lldg_gb300", "-Wl,-rpath," + os.path.dirname(lib),
                    "-o", str(exe)], check=True)
    return exe


def test_driver_compiles_and_links(tmp_path):
    assert os.path.exists(build_driver(tmp_path))


@pytest.mark.gpu
def test_driver_dgtimestep_matches_oracle(tmp_path):
    exe = build_driver(tmp_path)
    nx, p, steps = 4, 2, 5
    tf = oracle.tf_for_steps(nx, p, 1.0, steps)
    out = subprocess.run([str(exe), str(nx), str(p), repr(tf)], capture_output=True, text=True, check=True).stdout
    vals = {}
    ke = []
    for line in out.splitlines():
        k, *rest = line.split()
        if k == "ke":
            ke.append(float(rest[1]))
        else:
            vals[k] = float(rest[0])
    o = oracle.Oracle(nx, p, steps=steps)
    assert vals["steps"] == steps and vals["dt"] == o.dt
    u, ke_ref = o.step(o.initial_condition(), steps)
    assert np.max(np.abs(np.array(ke) - ke_ref) / ke_ref) <= 1e-12
    assert abs(vals["u_0_4_0"] - u[0, 4, 0]) <= 1e-12 * abs(u[0, 4, 0])


@pytest.mark.gpu
def test_driver_writes_reference_snapshots(tmp_path):
    """dgTimeStep with snapshots on: <file>.0 before the first step, in the
    reference's CSV format (golden file from the reference's writer)."""
    import gzip
    from conftest import GOLDEN
    exe = build_driver(tmp_path)
    tf = oracle.tf_for_steps(4, 2, 1.0, 5)
    snap = str(tmp_path / "xyzu.txt")
    subprocess.run([str(exe), "4", "2", repr(tf), snap], capture_output=True, text=True, check=True)
    assert sorted(p.name for p in tmp_path.iterdir() if p.name.startswith("xyzu")) == ["xyzu.txt.0"]
    from test_io import assert_same_csv
    with gzip.open(os.path.join(GOLDEN, "xyzv_n4_p2_s0.csv.gz"), "rt") as f:
        ref = f.read()
    assert_same_csv((tmp_path / "xyzu.txt.0").read_text(), ref)
