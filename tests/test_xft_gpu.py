"""GPU parity of poiss_x_ft (FFT in x, then per x mode a z-y problem solved
by the z-semicoarsened multigrid or, above IMGSOR, by zebra SOR; one
thread-block cluster per mode) against the CPU oracle, on a periodic channel
and on a duct with walls in z.

Both sides stop on the same max-norm test, so the cycle counts agree and phi
matches to rounding (FMA contraction, FFT summation order): relative L2
<= 1e-10 for the Poisson solve on the oracle's own divergence, and per field
after one full step.
"""
import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases, solver

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


CASES = {
    "channel": lambda: cases.with_poisson(cases.channel(32, 32, 16), abi.POISSON_X_FT, nlev=3),
    "duct": lambda: cases.with_poisson(cases.channel(32, 32, 16, zwalls=True), abi.POISSON_X_FT, nlev=3),
    "channel_sor": lambda: cases.with_poisson(cases.channel(32, 32, 16), abi.POISSON_X_FT, nlev=3),
}


def build(name):
    c = CASES[name]()
    if name == "channel_sor":
        c.settings.update(imgsor=3)          # modes 4..17 by zebra SOR
    return c


@pytest.mark.parametrize("name", sorted(CASES))
def test_poisson_on_the_oracle_divergence(oracle_lib, name):
    c = build(name)
    g, r = leswht_gb300.gpu_solver(c), solver.Solver(oracle_lib, "ref_", c)
    for s in (g, r):
        s.phase(abi.PH_STEPINIT)
        s.phase(abi.PH_SUBSTEPINIT, 1)
    r.phase(abi.PH_SGS, 1)
    r.phase(abi.PH_RHSNLHS, 1)
    r.phase(abi.PH_DIVGS, 1)
    g.set(abi.F_DIVGSUM, r.get(abi.F_DIVGSUM))
    for s in (g, r):
        s.phase(abi.PH_POISSON, 1)
    ig, ir = g.report()["poisson_iters"][0], r.report()["poisson_iters"][0]
    assert 1 <= ir < c.settings["mgitr"] and ig == ir
    assert rel(g.get(abi.F_PHI), r.get(abi.F_PHI)) <= TOL


def test_upper_wall_mean_removed():
    """ICH = 1: phi(:, n2m, 1) has zero f2fx-weighted mean on the GPU too."""
    c = build("channel")
    g = leswht_gb300.gpu_solver(c)
    g.phase(abi.PH_STEPINIT)
    g.phase(abi.PH_SUBSTEPINIT, 1)
    g.phase(abi.PH_SGS, 1)
    g.phase(abi.PH_RHSNLHS, 1)
    g.phase(abi.PH_DIVGS, 1)
    g.phase(abi.PH_POISSON, 1)
    gr = c.grid
    line = g.get(abi.F_PHI)[1, gr.n2m, 1:gr.n1m + 1]
    w = gr.f2fx[1:gr.n1m + 1]
    assert abs((line * w).sum()) <= 1e-13 * (np.abs(line) * w).sum()


@pytest.mark.parametrize("name", ["channel", "duct"])
def test_one_step(oracle_lib, name):
    c = build(name)
    g, r = leswht_gb300.gpu_solver(c), solver.Solver(oracle_lib, "ref_", c)
    rg, rr = g.step(), r.step()
    assert rg["poisson_iters"] == rr["poisson_iters"]
    fg, fr = g.fields(), r.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert rel(fg[k], fr[k]) <= TOL, (k, rel(fg[k], fr[k]))
    assert rg["dvmax"] < 1e-5


def test_graph_replay_matches_eager():
    c = build("duct")
    a, b = leswht_gb300.gpu_solver(c), leswht_gb300.gpu_solver(c)
    b.lib.lesgpu_use_graph(b.h, 0)
    for _ in range(2):
        ra, rb = a.step(), b.step()
        assert ra["poisson_iters"] == rb["poisson_iters"]
    fa, fb = a.fields(), b.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert np.array_equal(fa[k], fb[k]), k


def test_tuned_choices_reported(monkeypatch):
    monkeypatch.setenv("LESGPU_AUTOTUNE", "1")
    s = leswht_gb300.gpu_solver(build("channel"))
    t = leswht_gb300.tuning(s.lib, s.h)
    assert any(d == 3 and nc == 0 and w in (1, 2, 4, 8, 16, 32) for d, nc, f32, w in t)   # x FFT lines per block
    assert [w for d, nc, f32, w in t if d == 4][0] in (1, 2, 4, 8, 16)                      # blocks per mode
