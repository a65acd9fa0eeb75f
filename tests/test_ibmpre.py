"""Immersed-boundary pre-processing tables (leswht_gb300.ibmpre) on CPU.

The reference builds these tables with f2py-compiled Fortran
(02_solver/f90/lib/ibm_body.f90), which cannot be compiled here, so the
tables are checked through the properties the solver relies on:
  * every forcing point lies in the body, interpolated points first;
  * an interpolated point has a fluid neighbour in each direction its
    intpindx marks, an inner point has none along an unfixed direction;
  * the 27 weights reproduce a constant (they sum to 1, up to the 8-decimal
    rounding of the table file);
  * the zero-eddy-viscosity list and the wall mask agree.
"""
import numpy as np
import pytest

from leswht_gb300 import abi, cases, ibmpre
from leswht_gb300.gridgen import Segment, axis_vectors, make_grid


def _sphere_case():
    n = 24
    g, gdat, _ = make_grid(n + 1, n + 1, n + 1, 4.0, 4.0, 4.0,
                           [Segment("X", -2.0, 2.0, 1, n + 1, "U")],
                           [Segment("Y", -2.0, 2.0, 1, n + 1, "U")],
                           [Segment("Z", -2.0, 2.0, 1, n + 1, "U")],
                           xprdic=False, zprdic=True)
    s = cases.base_settings()
    s.update(ihtrans=1, body=dict(kind=abi.BODY_SPHERE, cx=0.1, cy=-0.05, cz=0.0, r=0.7, p0=0.0))
    ax = axis_vectors(gdat, False, False, True)
    return g, s, ax, ibmpre.build_tables(g, s, ax)


@pytest.fixture(scope="module", params=["cylinder", "sphere"])
def tables(request):
    if request.param == "cylinder":
        c = cases.cylinder_array(48, 40, 8)
        return c.grid, c.settings, axis_vectors(c.grid_dat, True, False, True), c.ibm
    return _sphere_case()


def _locs(ax, d):
    X, XM = ax["x"]; Y, YM = ax["y"]; Z, ZM = ax["z"]
    return {1: (X, YM, ZM), 2: (XM, Y, ZM), 3: (XM, YM, Z), 4: (XM, YM, ZM)}[d]


def test_forcing_points_in_body(tables):
    g, s, ax, t = tables
    for d in range(1, 5):
        xc, yc, zc = _locs(ax, d)
        fc = t["fc"][d - 1]
        assert len(fc) == t["nbody"][d - 1] > 0
        val = ibmpre.funcbody(s["body"], xc[fc[:, 0]], yc[fc[:, 1]], zc[fc[:, 2]])
        assert np.all(val <= 1.0e-10)
        assert len(np.unique(fc, axis=0)) == len(fc)


def test_interpolation_directions_point_to_fluid(tables):
    g, s, ax, t = tables
    for d in range(1, 5):
        xc, yc, zc = _locs(ax, d)
        fc, ix, ni = t["fc"][d - 1], t["intpindx"][d - 1], t["nintp"][d - 1]
        assert ni > 0 and np.all(np.abs(ix).sum(axis=1) > 0)
        for q in range(3):
            m = ix[:, q] != 0
            p = fc[:ni][m].copy()
            p[:, q] += ix[m, q]
            val = ibmpre.funcbody(s["body"], xc[p[:, 0]], yc[p[:, 1]], zc[p[:, 2]])
            assert np.all(val > 1.0e-10), (d, q)


def test_weights_reproduce_a_constant(tables):
    g, s, ax, t = tables
    for d in range(4):
        gf = t["geomfac"][d]
        assert np.abs(gf.sum(axis=1) - 1.0).max() <= 27 * 5.0e-9
        # written with 8 decimals
        assert np.array_equal(gf, np.round(gf, 8))


def test_zero_viscosity_list_matches_mask(tables):
    g, s, ax, t = tables
    mask = t["nwall_dvm"].reshape(g.n3m, g.n2m, g.n1m)
    assert t["nzero"] == int((mask == 0).sum())
    # indices are the 0-based positions of the zeros, i-major
    z = np.argwhere(mask.transpose(2, 1, 0) == 0)
    assert np.array_equal(z[:, 0], t["inz"]) and np.array_equal(z[:, 1], t["jnz"])
    assert np.array_equal(z[:, 2], t["knz"])
    # a cell whose centre is solid is always in the list
    X, XM = ax["x"]; Y, YM = ax["y"]; Z, ZM = ax["z"]
    sol = ibmpre.funcbody(s["body"], XM[None, None, 1:-1], YM[None, 1:-1, None], ZM[1:-1, None, None]) <= 1e-10
    assert np.all(mask[sol] == 0)


def test_geomfac_preset_keeps_the_unset_periodic_ghosts():
    coord = np.linspace(0.0, 1.0, 6)
    center = np.concatenate([[coord[0]], 0.5 * (coord[1:-1] + coord[2:]), [coord[-1]]])
    a = ibmpre.geomfac_preset(coord, center)
    assert a.shape == (len(coord) + 2, 3)
    assert np.all(a[0] == 0.0) and np.all(a[-1] == 0.0)


@pytest.mark.parametrize("kind, z", [(abi.BODY_CYLINDER, (0.0, 0.3)), (abi.BODY_SPHERE, None), (abi.BODY_SQUARE, (0.0, 0.2))])
def test_fluid_portion_is_the_reference_flood_fill(kind, z):
    """fluid_portion (the start sub-cell's same-phase component) equals the
    reference's stack flood fill with its fill-then-assign rule, on boxes
    cut by the surface."""
    rng = np.random.default_rng(11)
    body = dict(kind=kind, cx=0.05, cy=-0.1, cz=0.02, r=0.45, p0=0.0)
    n = 120
    cx, cy = rng.uniform(-0.7, 0.7, n), rng.uniform(-0.7, 0.7, n)
    w, h = rng.uniform(0.05, 0.7, n), rng.uniform(0.05, 0.7, n)
    if z is None:
        z1 = rng.uniform(-0.6, 0.4, n)
        z2 = z1 + rng.uniform(0.05, 0.6, n)
    else:
        z1, z2 = np.full(n, z[0]), np.full(n, z[1])
    box = (cx - w / 2, cx + w / 2, cy - h / 2, cy + h / 2, z1, z2)
    fast = ibmpre.fluid_portion(body, *box)
    fill = np.array([ibmpre.fluid_portion_fill(body, *(v[q] for v in box)) for q in range(n)])
    assert np.array_equal(fast, fill)
    assert np.unique(fast[(fast > 0.0) & (fast < 1.0)]).size > 10     # many boxes cut by the surface


def test_conjugate_tables_on_a_cylinder():
    """c* and k* are the fluid values (1) away from the body, the solid ratios
    inside, and the harmonic mean across the interface; omega marks the cells
    entirely in the fluid."""
    c = cases.cylinder(32, 24, 4, nlev=2)
    axes = axis_vectors(c.grid_dat, False, False, True)
    cs, ks, om = ibmpre.conjg_intp(c.settings["body"], 0.5, 4.0, axes, (0, 0, 1))
    assert set(np.unique(om)) == {0, 1}
    assert np.all(cs[om == 1] == 1.0) and cs.min() == 0.5
    assert np.all((ks >= 1.0) & (ks <= 4.0)) and ks.max() == 4.0
    assert np.all(ks[:, om == 1][0] >= 1.0)
