"""IB pre-processing on the GPU (lesgpu_ibmpre_run) gives exactly the tables
of the host restatement (ibmpre.build_tables) -- the forcing points in the
same order, the same interpolation directions, geomfac bit for bit after its
8-decimal rounding, the same zero-viscosity list and wall mask -- and a step
run with them equals a step run with the host tables."""
import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases, gridgen, ibmpre, serving

pytestmark = pytest.mark.gpu

CASES = {
    "cylinder_64x48x8": (lambda: cases.cylinder(64, 48, 8), (False, False, True)),
    "cylinder_128x96x16": (lambda: cases.cylinder(128, 96, 16), (False, False, True)),
    "cylinder_row": (lambda: cases.cylinder_array(48, 40, 8), (True, False, True)),
    "sphere": (lambda: serving.build_case(dict(grid=(96, 64, 16), body=abi.BODY_SPHERE, center=(0.1, 0.4, 1.5),
                                                re=60.0, pr=0.71, seed=3), abi.PREC_FP64), (False, False, True)),
    "square": (lambda: serving.build_case(dict(grid=(64, 48, 8), body=abi.BODY_SQUARE, center=(-0.3, 0.25, 1.5),
                                                re=300.0, pr=7.0, seed=2), abi.PREC_FP64), (False, False, True)),
}


def host_and_gpu(name):
    build, prd = CASES[name]
    c = build()
    axes = gridgen.axis_vectors(c.grid_dat, *prd)
    return c, ibmpre.build_tables(c.grid, c.settings, axes), ibmpre.build_tables_gpu(
        leswht_gb300.load_library(), c.settings, c.grid, axes)


@pytest.mark.parametrize("name", sorted(CASES))
def test_tables_match_host(name):
    c, h, d = host_and_gpu(name)
    nl = 4 if c.settings.get("ihtrans", 0) == 1 else 3
    for l in range(nl):
        assert d["nintp"][l] == h["nintp"][l] and d["nbody"][l] == h["nbody"][l], l
        assert np.array_equal(np.asarray(d["fc"][l]), np.asarray(h["fc"][l])), l
        assert np.array_equal(np.asarray(d["intpindx"][l]), np.asarray(h["intpindx"][l])), l
        assert np.array_equal(np.asarray(d["geomfac"][l]).view(np.int64),
                              np.asarray(h["geomfac"][l]).reshape(-1, 27).view(np.int64)), l
    assert d["nzero"] == h["nzero"]
    for k in ("inz", "jnz", "knz", "nwall_dvm"):
        assert np.array_equal(np.asarray(d[k]), np.asarray(h[k])), k


def test_step_with_gpu_tables_equals_host_tables():
    c, h, d = host_and_gpu("cylinder_64x48x8")
    a = leswht_gb300.gpu_solver(c)
    c2 = cases.Case(c.name, c.settings, c.grid, c.grid_dat, c.grid_bin, c.fields, time=c.time, dt=c.dt,
                    ihist=c.ihist, m=c.m, ibm=d)
    b = leswht_gb300.gpu_solver(c2)
    for _ in range(2):
        a.step(); b.step()
    fa, fb = a.fields(), b.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert np.array_equal(fa[k], fb[k]), k


@pytest.mark.parametrize("name", ["cylinder_64x48x8", "cylinder_row", "sphere", "square"])
def test_conjugate_tables_match_host(name):
    """conjg_intp on the GPU (lesgpu_conjg_run) equals the host restatement
    bit for bit: c*, the six face k* and the fluid mask."""
    build, prd = CASES[name]
    c = build()
    axes = gridgen.axis_vectors(c.grid_dat, *prd)
    flags = tuple(int(v) for v in prd)
    s = dict(c.settings, xprdic=flags[0], yprdic=flags[1], zprdic=flags[2])
    cs, ks, om = ibmpre.conjg_intp(s["body"], 0.4, 25.0, axes, flags)
    gc, gk, go = ibmpre.conjg_tables_gpu(leswht_gb300.load_library(), s, c.grid, axes, 0.4, 25.0)
    assert np.array_equal(gc.view(np.int64), cs.reshape(-1).view(np.int64))
    assert np.array_equal(gk.view(np.int64), ks.reshape(-1).view(np.int64))
    assert np.array_equal(go, om.reshape(-1))
    assert 0 < int(om.sum()) < om.size and np.unique(ks).size > 3      # a real interface
