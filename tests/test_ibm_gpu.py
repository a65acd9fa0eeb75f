"""GPU parity of the immersed-boundary path: direct forcing with 27-point
interpolation (rhs_ibm, rhs_ibm_t), the divgs mass source/sink, lagforce,
draglift and heatflux, against the CPU oracle on a row of heated cylinders
(periodic x/z, walls in y, constant flow rate, FFT Poisson solver), with
forcing tables produced by leswht_gb300.ibmpre.

Tolerance: relative L2 <= 1e-10 per field after one step, 1e-9 after three;
force and flux scalars (sums over forcing points, different summation
order) to 1e-9 relative.
"""
import ctypes as C

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
    return cases.cylinder_array(48, 40, 8)


def pair(oracle_lib, case):
    return leswht_gb300.gpu_solver(case), solver.Solver(oracle_lib, "ref_", case)


def test_tables_loaded(cyl):
    assert min(cyl.ibm["nintp"][:3]) > 0 and cyl.ibm["nzero"] > 0


def test_one_step(oracle_lib, cyl):
    g, r = pair(oracle_lib, cyl)
    rg, rr = g.step(), r.step()
    fg, fr = g.fields(), r.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert rel(fg[k], fr[k]) <= TOL, (k, rel(fg[k], fr[k]))
    for q in range(3):
        assert rg["cd"][q] == pytest.approx(rr["cd"][q], rel=1e-9, abs=1e-12), q
    assert rg["qmmax"] == pytest.approx(rr["qmmax"], rel=1e-12)
    assert rg["pmi"][0] == pytest.approx(rr["pmi"][0], rel=1e-9)
    assert rg["dvmax"] < 1e-10 and rr["dvmax"] < 1e-10


def test_phases_with_forcing(oracle_lib, cyl):
    g, r = pair(oracle_lib, cyl)
    for s in (g, r):
        s.phase(abi.PH_STEPINIT)
        s.phase(abi.PH_SUBSTEPINIT, 1)
        s.phase(abi.PH_SGS, 1)
    for f in (abi.F_NUSGS, abi.F_NUSGS1, abi.F_ALSGS):
        assert rel(g.get(f), r.get(f)) <= TOL, f
    for s in (g, r):
        s.phase(abi.PH_RHSNLHS, 1)
    for f in (abi.F_U, abi.F_V, abi.F_W):
        assert rel(g.get(f), r.get(f)) <= TOL, f
    for s in (g, r):
        s.phase(abi.PH_DIVGS, 1)
    assert rel(g.get(abi.F_QMASS), r.get(abi.F_QMASS)) <= TOL
    assert rel(g.get(abi.F_DIVGSUM), r.get(abi.F_DIVGSUM)) <= TOL
    for s in (g, r):
        s.phase(abi.PH_POISSON, 1)
        s.phase(abi.PH_UCALC, 1)
        s.phase(abi.PH_MEANPG, 1)
        s.phase(abi.PH_ENERGY, 1)
    for f in (abi.F_U, abi.F_V, abi.F_W, abi.F_P, abi.F_T):
        assert rel(g.get(f), r.get(f)) <= TOL, f


def test_three_steps(oracle_lib, cyl):
    g, r = pair(oracle_lib, cyl)
    for _ in range(3):
        rg, rr = g.step(), r.step()
    fg, fr = g.fields(), r.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert rel(fg[k], fr[k]) <= 1e-9, (k, rel(fg[k], fr[k]))
    for q in range(3):
        assert rg["cd"][q] == pytest.approx(rr["cd"][q], rel=1e-8, abs=1e-11), q


def test_graph_replay_matches_eager(cyl):
    a = leswht_gb300.gpu_solver(cyl)
    b = leswht_gb300.gpu_solver(cyl)
    b.lib.lesgpu_use_graph(b.h, 0)
    for _ in range(3):
        a.step(); b.step()
    fa, fb = a.fields(), b.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert np.array_equal(fa[k], fb[k]), k


def test_load_ibm_rejects_bad_indices(cyl):
    s = leswht_gb300.gpu_solver(cyl)
    t = dict(cyl.ibm)
    fc = [a.copy() for a in t["fc"]]
    fc[0][0, 0] = cyl.grid.n1m + 5                     # outside the grid
    t["fc"] = fc
    pk = abi.pack_ibm(t, cyl.grid.n1m, cyl.grid.n2m, cyl.grid.n3m)
    assert s.lib.lesgpu_load_ibm(s.h, C.byref(pk.struct)) == abi.ERR_ARG
    t = dict(cyl.ibm)
    ix = [a.copy() for a in t["intpindx"]]
    ix[1][0, 1] = 2                                    # not a unit direction
    t["intpindx"] = ix
    pk = abi.pack_ibm(t, cyl.grid.n1m, cyl.grid.n2m, cyl.grid.n3m)
    assert s.lib.lesgpu_load_ibm(s.h, C.byref(pk.struct)) == abi.ERR_ARG
