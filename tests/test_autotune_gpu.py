"""The autotuner: at lesgpu_start each ADI sweep class of a case's shape is
timed with every feasible lanes-per-line count and the fastest kept for the
process; LESGPU_AUTOTUNE=0 turns it off.  Any choice gives the same solution
to rounding, so tuned runs keep the parity tolerance."""
import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases, solver

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_tuned_classes_reported_and_reused(monkeypatch):
    monkeypatch.setenv("LESGPU_AUTOTUNE", "1")
    case = cases.channel(32, 32, 16, precision=abi.PREC_MIXED)
    a = leswht_gb300.gpu_solver(case)
    ta = leswht_gb300.tuning(a.lib, a.h)
    assert any(d == 3 and nc == 2 and w in (1, 2, 4, 8, 16, 32) for d, nc, f32, w in ta)   # z FFT lines per block
    ta = [t for t in ta if t[0] < 3]
    dirs = {(d, nc, f32) for d, nc, f32, w in ta}
    # momentum (3 components) and temperature (1) in x, y, z; x/z in FP32, y in FP64
    assert {(0, 3, 1), (1, 3, 0), (2, 3, 1), (0, 1, 1), (1, 1, 0), (2, 1, 1)} <= dirs
    assert all(w & 63 in (1, 8, 16, 32) and (w & 63 > 1 or w < 64) for *_, w in ta)   # + 64: register-capped
    b = leswht_gb300.gpu_solver(case)
    assert sorted(t for t in leswht_gb300.tuning(b.lib, b.h) if t[0] < 3) == sorted(ta)   # the process-wide table
    for _ in range(2):
        a.step(); b.step()
    fa, fb = a.fields(), b.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert np.array_equal(fa[k], fb[k]), k


def test_off_reports_nothing(monkeypatch):
    monkeypatch.setenv("LESGPU_AUTOTUNE", "0")
    s = leswht_gb300.gpu_solver(cases.channel(16, 16, 8))
    assert leswht_gb300.tuning(s.lib, s.h) == []


def test_tuned_step_matches_oracle(oracle_lib, monkeypatch):
    monkeypatch.setenv("LESGPU_AUTOTUNE", "1")
    case = cases.cylinder(64, 48, 8)
    g, r = leswht_gb300.gpu_solver(case), solver.Solver(oracle_lib, "ref_", case)
    mg = [w for d, nc, f32, w in leswht_gb300.tuning(g.lib, g.h) if d == 4]
    assert len(mg) == 1 and mg[0] in (1, 2, 4, 8, 16)                   # z_ft multigrid blocks per cluster
    g.step(); r.step()
    fg, fr = g.fields(), r.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert rel(fg[k], fr[k]) <= 1e-10, k


def test_table_persists_in_a_file(tmp_path, monkeypatch):
    path = tmp_path / "tune.txt"
    monkeypatch.setenv("LESGPU_AUTOTUNE", "1")
    monkeypatch.setenv("LESGPU_TUNE_FILE", str(path))
    s = leswht_gb300.gpu_solver(cases.channel(16, 16, 8))
    lines = [ln.split() for ln in path.read_text().splitlines()]
    mine = [ln for ln in lines if ln[0] == "adi" and ln[1:4] == ["16", "16", "8"]]
    assert mine and all(int(ln[-1]) & 63 in (1, 8, 16, 32) for ln in mine)
    tuned = {(int(ln[4]), int(ln[5]), int(ln[6]), int(ln[-1])) for ln in mine}
    assert {t for t in leswht_gb300.tuning(s.lib, s.h) if t[0] < 3} <= tuned


def test_table_file_choices_are_reused(tmp_path, monkeypatch):
    """A choice read from the file -- here the register-capped 8-lane y sweep
    (code 8 + 64) -- is used as is, not timed again."""
    path = tmp_path / "tune.txt"
    path.write_text("adi 24 20 12 1 3 0 0 20 72\n")
    monkeypatch.setenv("LESGPU_AUTOTUNE", "1")
    monkeypatch.setenv("LESGPU_TUNE_FILE", str(path))
    s = leswht_gb300.gpu_solver(cases.channel(24, 20, 12))
    assert (1, 3, 0, 72) in leswht_gb300.tuning(s.lib, s.h)
    assert "adi 24 20 12 1 3 0 0 20 72" in path.read_text()

