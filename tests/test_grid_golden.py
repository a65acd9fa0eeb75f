"""The grid pipeline against fixtures made by the reference's own
pre-processor (tests/golden/make_grid_golden.py): gridlines (grid.py), the
metrics of lib_setgrid.py and the %f-rounded grid.bin of
lib_preprocessing.grid_preprocessing_data must match byte for byte."""
from pathlib import Path

import numpy as np
import pytest

from leswht_gb300 import gridgen
from tests.golden.make_grid_golden import CASES

GOLD = Path(__file__).resolve().parent / "golden"


def _segments(segs):
    return [gridgen.Segment(*s) for s in segs]


@pytest.mark.parametrize("name", sorted(CASES))
def test_grid_files_match_reference(name):
    n, l, segs, (xp, zp) = CASES[name]
    segs = _segments(segs)
    xs = [s for s in segs if s.direction == "X"]
    ys = [s for s in segs if s.direction == "Y"]
    zs = [s for s in segs if s.direction == "Z"]
    g, gdat, gbin = gridgen.make_grid(n[0], n[1], n[2], l[0], l[1], l[2], xs, ys, zs, xprdic=xp, zprdic=zp)
    assert gdat == (GOLD / f"{name}.grid.dat").read_text()
    assert gbin == (GOLD / f"{name}.grid.bin").read_text()


@pytest.mark.parametrize("name", sorted(CASES))
def test_readgeom_of_golden(name):
    g = gridgen.read_grid_bin((GOLD / f"{name}.grid.bin").read_text())
    n, l, segs, (xp, zp) = CASES[name]
    assert (g.n1, g.n2, g.n3) == n
    assert g.c2cx.shape == (g.n1 + 1,) and g.ipv.shape == (g.n1m,)
    # periodic neighbour maps wrap, non-periodic ones run to the ghost
    assert g.imv[0] == (g.n1m if xp else 0)
    assert g.kpv[-1] == (1 if zp else g.n3)
    assert g.fixjl[0] == 1 and g.fixju[-1] == 1
    assert np.all(g.f2fy[1:g.n2] > 0)


def test_channel_preset_uses_golden_grid():
    from leswht_gb300 import cases
    c = cases.channel(16, 16, 8)
    assert c.grid_bin == (GOLD / "channel_16x16x8.grid.bin").read_text()
