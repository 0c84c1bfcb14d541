"""Snapshots and checkpoints.

X-Y-Z-V CSV snapshots against the reference's own writer (io.cpp:8-72,
golden files tests/golden/xyzv_*.csv.gz made by the reference build), the
snapshot cadence of dg_time_step (solver.cpp:366-381), and exact
checkpoint/resume (no reference counterpart).  Printed values carry 6
significant digits, so a state that agrees to 1e-12 can still flip the last
printed digit of a value that sits on a rounding boundary: numbers are
compared to the printed precision and the coordinates as text.
"""
import ctypes
import gzip
import os

import numpy as np
import pytest

import ldg
import oracle
from conftest import GOLDEN


def golden_csv(name):
    with gzip.open(os.path.join(GOLDEN, name), "rt") as f:
        return f.read()


def assert_same_csv(text, ref):
    """Same header, line count and separators; coordinates identical as
    text; values equal to the printed precision (6 significant digits, or
    1e-12 absolute for values that are rounding noise around zero, which a
    nodal -> Gauss -> nodal round trip changes at the 1e-16 level)."""
    a, b = text.splitlines(), ref.splitlines()
    assert a[0] == b[0] == "X, Y, Z, u0, u1, u2, u3, u4"
    assert len(a) == len(b)
    ta = [line.split(", ") for line in a[1:]]
    tb = [line.split(", ") for line in b[1:]]
    assert all(len(x) == 8 for x in ta)
    assert [x[:3] for x in ta] == [x[:3] for x in tb]
    va = np.array([[float(v) for v in x[3:]] for x in ta])
    vb = np.array([[float(v) for v in x[3:]] for x in tb])
    assert np.all(np.abs(va - vb) <= 1e-5 * np.abs(vb) + 1e-12)


def test_oracle_csv_restatement_matches_reference_writer():
    o = oracle.Oracle(4, 2)
    text = oracle.xyzv_text(oracle.node_coordinates(4, 2), o.initial_condition())
    assert text == golden_csv("xyzv_n4_p2_s0.csv.gz")
    o = oracle.Oracle(3, 3, steps=5)
    u, _ = o.step(o.initial_condition(), 5)
    assert_same_csv(oracle.xyzv_text(oracle.node_coordinates(3, 3), u), golden_csv("xyzv_n3_p3_s5.csv.gz"))


def test_checkpoint_reader_rejects_missing_and_foreign_files(tmp_path):
    lib = ldg.load()
    cfg = ldg.LdgConfig()
    assert lib.ldg_checkpoint_config(str(tmp_path / "none").encode(), ctypes.byref(cfg)) == -8
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"not a checkpoint" * 64)
    assert lib.ldg_checkpoint_config(str(bad).encode(), ctypes.byref(cfg)) == -8
    assert b"not a checkpoint" in lib.ldg_last_error_message()
    assert lib.ldg_checkpoint_config(None, ctypes.byref(cfg)) == -1
    assert lib.ldg_write_xyzv(None, b"x", 0) == -1
    assert lib.ldg_save_checkpoint(None, b"x") == -1
    assert lib.ldg_load_checkpoint(None, b"x") == -1


@pytest.mark.gpu
def test_write_xyzv_matches_reference_snapshot(tmp_path):
    with ldg.Solver(2, 4) as s:
        s.write_xyzv(str(tmp_path / "ic"), 0)
    assert_same_csv((tmp_path / "ic.0").read_text(), golden_csv("xyzv_n4_p2_s0.csv.gz"))
    with ldg.Solver(3, 3, steps=5) as s:
        s.step(5)
        s.write_xyzv(str(tmp_path / "s5.txt"))  # timeseries < 0: the name as given
    assert_same_csv((tmp_path / "s5.txt").read_text(), golden_csv("xyzv_n3_p3_s5.csv.gz"))


@pytest.mark.gpu
def test_time_step_writes_snapshots_every_dt_snaps(tmp_path):
    base = str(tmp_path / "xyzu.txt")
    with ldg.Solver(2, 4, steps=7, dt_snaps=3) as s:
        s.set_snapshots(base)
        s.dg_time_step()
        assert s.info().step == 7
    # snapshots before steps 0, 3, 6 (solver.cpp:366-381): files .0 .1 .2
    assert sorted(os.listdir(tmp_path)) == ["xyzu.txt.0", "xyzu.txt.1", "xyzu.txt.2"]
    with ldg.Solver(2, 4, steps=7) as r:
        r.write_xyzv(str(tmp_path / "r"), 0)
        r.step(6)
        r.write_xyzv(str(tmp_path / "r"), 2)
    assert (tmp_path / "xyzu.txt.0").read_text() == (tmp_path / "r.0").read_text()
    assert (tmp_path / "xyzu.txt.2").read_text() == (tmp_path / "r.2").read_text()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_checkpoint_resume_is_bitwise(tmp_path, precision):
    kw = dict(steps=20, perturb_amp=0.05, seed=5, instance=1, precision=precision)
    path = str(tmp_path / "run.ckpt")
    with ldg.Solver(3, 4, **kw) as a:
        a.step(8)
        ua, ka = a.get_state(), a.ke_history()
    with ldg.Solver(3, 4, **kw) as b:
        b.step(5)
        b.save_checkpoint(path)
    assert not os.path.exists(path + ".tmp")
    with ldg.Solver.from_checkpoint(path) as c:
        info = c.info()
        assert info.step == 5 and info.precision == ldg.PRECISIONS[precision]
        c.step(3)
        uc, kc = c.get_state(), c.ke_history()
    assert np.array_equal(ua, uc)
    assert np.array_equal(ka, kc)


@pytest.mark.gpu
def test_checkpoint_rejects_other_discretisation_and_corruption(tmp_path):
    path = tmp_path / "a.ckpt"
    with ldg.Solver(2, 4, steps=5) as s:
        s.step(2)
        s.save_checkpoint(str(path))
    with ldg.Solver(3, 4, steps=5) as other, pytest.raises(ldg.LdgError) as e:
        other.load_checkpoint(str(path))
    assert e.value.status == -1
    with ldg.Solver(2, 4, steps=5, cfl=0.02) as other_dt, pytest.raises(ldg.LdgError) as e:
        other_dt.load_checkpoint(str(path))  # same mesh, another time step
    assert e.value.status == -1
    raw = bytearray(path.read_bytes())
    raw[len(raw) // 2] ^= 0x40
    (tmp_path / "flip.ckpt").write_bytes(bytes(raw))
    (tmp_path / "short.ckpt").write_bytes(bytes(raw[:-8]))
    with ldg.Solver(2, 4, steps=5) as s:
        for name in ("flip.ckpt", "short.ckpt"):
            with pytest.raises(ldg.LdgError) as e:
                s.load_checkpoint(str(tmp_path / name))
            assert e.value.status == -8
        s.load_checkpoint(str(path))  # the intact file still loads
        assert s.info().step == 2
