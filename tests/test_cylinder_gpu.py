"""GPU parity on the open-flow cylinder: convective outlet (convbc,
rhsincorpbc and their thermal forms), far-field lateral boundaries, IB
forcing with interpolation, and the poiss_z_ft Poisson solver (z FFT +
x-semi-coarsened multigrid per mode), against the CPU oracle.

The multigrid is iterative; both sides stop on the same max-norm test, so
the cycle counts must agree and the fields then match to rounding.
Tolerance: relative L2 <= 1e-10 per field after one step, 1e-9 after three.
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


@pytest.fixture(scope="module")
def cyl():
    return cases.cylinder(64, 48, 8)


def pair(oracle_lib, case):
    return leswht_gb300.gpu_solver(case), solver.Solver(oracle_lib, "ref_", case)


def test_poisson_after_divergence(oracle_lib, cyl):
    g, r = pair(oracle_lib, cyl)
    for s in (g, r):
        s.phase(abi.PH_STEPINIT)
        s.phase(abi.PH_SUBSTEPINIT, 1)
        s.phase(abi.PH_SGS, 1)
        s.phase(abi.PH_RHSNLHS, 1)
    for f in (abi.F_U, abi.F_V, abi.F_W):
        assert rel(g.get(f), r.get(f)) <= TOL, f
    for s in (g, r):
        s.phase(abi.PH_DIVGS, 1)
    assert rel(g.get(abi.F_DIVGSUM), r.get(abi.F_DIVGSUM)) <= TOL
    for s in (g, r):
        s.phase(abi.PH_POISSON, 1)
    it_g, it_r = g.report()["poisson_iters"][0], r.report()["poisson_iters"][0]
    assert it_g == it_r and it_g > 0
    assert rel(g.get(abi.F_PHI), r.get(abi.F_PHI)) <= TOL


@pytest.mark.parametrize("dims", [(64, 48, 8), (64, 48, 1), (128, 96, 16)])
def test_one_step(oracle_lib, dims):
    case = cases.cylinder(*dims)
    g, r = pair(oracle_lib, case)
    rg, rr = g.step(), r.step()
    assert rg["poisson_iters"] == rr["poisson_iters"]
    fg, fr = g.fields(), r.fields()
    for k in ("u", "v", "w", "p", "t"):
        if k == "w" and dims[2] == 1:
            continue
        assert rel(fg[k], fr[k]) <= TOL, (k, rel(fg[k], fr[k]))
    assert rg["dt"] == pytest.approx(rr["dt"], rel=1e-13)
    for q in range(2):
        assert rg["cd"][q] == pytest.approx(rr["cd"][q], rel=1e-9, abs=1e-12), q
    assert rg["heat_flux"][0] == pytest.approx(rr["heat_flux"][0], rel=1e-9)
    # the thermal forcing's heat rate (the Nusselt number's numerator)
    assert rg["heat_body"] != 0.0
    assert rg["heat_body"] == pytest.approx(rr["heat_body"], rel=1e-9)
    assert rg["poisson_unconverged"] == rr["poisson_unconverged"] == 0
    assert rg["dvmax"] < 1e-5


def test_three_steps(oracle_lib, cyl):
    g, r = pair(oracle_lib, cyl)
    for _ in range(3):
        rg, rr = g.step(), r.step()
        assert rg["poisson_iters"] == rr["poisson_iters"]
    fg, fr = g.fields(), r.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert rel(fg[k], fr[k]) <= 1e-9, (k, rel(fg[k], fr[k]))


def test_graph_replay_matches_eager(cyl):
    a = leswht_gb300.gpu_solver(cyl)
    b = leswht_gb300.gpu_solver(cyl)
    b.lib.lesgpu_use_graph(b.h, 0)
    for _ in range(3):
        a.step(); b.step()
    fa, fb = a.fields(), b.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert np.array_equal(fa[k], fb[k]), k
