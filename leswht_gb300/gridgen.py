"""Stretched staggered grids in the reference's formats.

Restates, in this package's own code, the grid pipeline the solver consumes:
  * gridline distributions of 01_pre_processor/lib/lib_gridfunc.py
    (uniform :3, geometric :22, hyperbolic tangent :50), written to grid.dat
    with 15 decimals as grid.py:83-95 does;
  * cell metrics of 01_pre_processor/lib/lib_setgrid.py (readcoord :1,
    setindex :24, setmesh :38, physcenter :72);
  * the text file grid.bin of lib_preprocessing.py:112-170, every real
    written with '%f' (6 decimals) -- the solver reads these rounded values;
  * the reader readgeom of 02_solver/f90/lib/misc_init.f90:204-251.

`make_grid(...)` returns the metrics exactly as the Fortran solver holds them
after readgeom, i.e. after the 15- and 6-decimal text round trips.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Dict, List, Sequence, Tuple

import numpy as np


@dataclass
class Segment:
    """One gridline segment: a line of grid.input."""
    direction: str          # 'X', 'Y' or 'Z'
    coord_i: float
    coord_f: float
    index_i: int
    index_f: int
    opt: str                # 'U', 'G' or 'H'
    factor1: float = 0.0
    factor2: float = 0.0


def _fill_segment(xyz: Dict[int, float], s: Segment) -> None:
    ii, jf = s.index_i, s.index_f
    if s.opt.upper() == "U":
        delta = (s.coord_f - s.coord_i) / (jf - ii)
        for i in range(ii, jf + 1):
            xyz[i] = s.coord_i + (i - ii) * delta
    elif s.opt.upper() == "G":
        f1, r = s.factor1, s.factor2
        if r <= 1:
            raise ValueError("geometric ratio must be larger than 1")
        if f1 != 1:
            r = 1 / r
        d0 = (s.coord_f - s.coord_i) * (1 - r) / (1 - r ** (jf - ii))
        for i in range(ii, jf + 1):
            xyz[i] = s.coord_i + d0 * (1 - r ** (i - ii)) / (1 - r)
    elif s.opt.upper() == "H":
        f1, g = s.factor1, s.factor2
        if f1 != 0:
            for i in range(ii, jf + 1):
                prop = (i - ii) / (jf - ii)
                xyz[i] = s.coord_i + (s.coord_f - s.coord_i) * f1 * \
                    (1 - np.tanh(g * (f1 - prop)) / np.tanh(g * f1))
        else:
            f1 = 1
            for i in range(ii, jf + 1):
                prop = (i - ii) / (jf - ii)
                xyz[i] = s.coord_i + (s.coord_f - s.coord_i) * f1 * \
                    (1 - np.tanh(g * prop) / np.tanh(g * f1))
    else:
        raise ValueError(f"unknown grid option {s.opt!r}")


def gridlines(n: int, segments: Sequence[Segment]) -> List[float]:
    xyz: Dict[int, float] = {}
    for s in segments:
        _fill_segment(xyz, s)
    missing = [i for i in range(1, n + 1) if i not in xyz]
    if missing:
        raise ValueError(f"gridlines {missing[:5]}... not covered by any segment")
    return [xyz[i] for i in range(1, n + 1)]


def grid_dat_text(nx: int, ny: int, nz: int, lx: float, ly: float, lz: float,
                  xs: Sequence[float], ys: Sequence[float], zs: Sequence[float]) -> str:
    """The grid.dat file of grid.py:83-95."""
    out = ["%23d %22d %22d\n" % (nx, ny, nz), "%23.15f %22.15f %22.15f\n" % (lx, ly, lz)]
    out.append("".join("%23.15f" % v for v in xs) + "\n")
    out.append("".join("%23.15f" % v for v in ys) + "\n")
    out.append("".join("%23.15f" % v for v in zs))
    return "".join(out)


def _axis_info(coords_text: Sequence[str], prdic: bool) -> List[dict]:
    """readcoord + setindex + setmesh + physcenter for one direction."""
    n = len(coords_text)
    coord = [float(v) for v in coords_text]
    coord = [coord[0]] + coord               # coord[0] duplicates coord[1]
    info = [dict() for _ in range(n + 1)]
    cells = n - 1
    for i in range(1, cells + 1):
        info[i]["idxplus"] = i + 1
        info[i]["idxminus"] = i - 1
        if i == 1:
            info[i]["lowerfix"], info[i]["upperfix"] = 1, 0
        elif i == cells:
            info[i]["lowerfix"], info[i]["upperfix"] = 0, 1
        else:
            info[i]["lowerfix"], info[i]["upperfix"] = 0, 0
    if prdic:
        info[1]["lowerfix"] = 0
        info[1]["idxminus"] = cells
        info[cells]["upperfix"] = 0
        info[cells]["idxplus"] = 1
    if cells != 1:
        for i in range(1, cells + 1):
            info[i]["f2fd"] = coord[i + 1] - coord[i]
            if i != 1:
                info[i]["c2cd"] = 0.5 * (info[i]["f2fd"] + info[i - 1]["f2fd"])
        info[1]["c2cd"] = 0.5 * info[1]["f2fd"]
        info[cells + 1]["c2cd"] = 0.5 * info[cells]["f2fd"]
        for i in range(1, cells + 1):
            info[i]["1/f2fd"] = 1 / info[i]["f2fd"]
            info[i]["1/c2cd"] = 1 / info[i]["c2cd"]
        info[cells + 1]["1/c2cd"] = 1 / info[cells + 1]["c2cd"]
    else:
        coord[2] = coord[1] + 1.
        for q in (1, 2):
            info[q].update({"f2fd": 1.0, "c2cd": 1.0, "1/f2fd": 1.0, "1/c2cd": 1.0})
    info[0].update({"f2fd": 0, "c2cd": 0, "1/c2cd": 0, "1/f2fd": 0})
    info[cells + 1].update({"f2fd": 0, "1/f2fd": 0})
    if prdic:
        coord[0] = coord[1] - info[cells]["f2fd"]
        info[0].update({"f2fd": info[cells]["f2fd"], "1/f2fd": info[cells]["1/f2fd"]})
        info[1]["c2cd"] = 0.5 * (info[1]["f2fd"] + info[cells]["f2fd"])
        info[cells + 1].update({"f2fd": info[1]["f2fd"], "1/f2fd": info[1]["1/f2fd"]})
        info[cells + 1]["c2cd"] = 0.5 * (info[1]["f2fd"] + info[cells]["f2fd"])
        for i in range(1, cells + 2):
            info[i]["1/c2cd"] = 1 / info[i]["c2cd"]
    for i in range(0, cells + 2):
        info[i]["coord"] = coord[i]
    for i in range(1, cells + 1):
        info[i]["center"] = coord[i] + 0.5 * info[i]["f2fd"]
    info[cells + 1]["center"] = coord[cells + 1]
    info[0]["center"] = coord[0]
    return info


def grid_bin_text(grid_dat: str, xprdic: bool, yprdic: bool, zprdic: bool) -> str:
    """grid.dat text -> grid.bin text (lib_setgrid.setgrid + grid_preprocessing_data)."""
    lines = grid_dat.split("\n")
    nx, ny, nz = (int(v) for v in lines[0].split())
    lx, ly, lz = (float(v) for v in lines[1].split())
    ax = _axis_info(lines[2].split(), xprdic)
    ay = _axis_info(lines[3].split(), yprdic)
    az = _axis_info(lines[4].split(), zprdic)
    cx, cy, cz = nx - 1, ny - 1, nz - 1
    out = []

    def ints(vals):
        out.append("".join(" %d " % int(v) for v in vals) + "\n")

    def reals(vals, newline=True):
        out.append("".join(" %f " % v for v in vals) + ("\n" if newline else ""))

    out.append("%d %d %d\n" % (nx, ny, nz))
    out.append("%d %d %d\n" % (cx, cy, cz))
    out.append("%f %f %f\n" % (lx, ly, lz))
    for a, n in ((ax, nx), (ay, ny), (az, nz)):
        reals([a[i]["coord"] for i in range(1, n + 1)])
    for key in ("idxplus", "idxminus", "lowerfix", "upperfix"):
        for a, cn in ((ax, cx), (ay, cy), (az, cz)):
            ints([a[i][key] for i in range(1, cn + 1)])
    for key in ("c2cd", "1/c2cd", "f2fd", "1/f2fd"):
        for a, n in ((ax, nx), (ay, ny), (az, nz)):
            reals([a[i][key] for i in range(n + 1)])
    reals([ax[i]["center"] for i in range(nx + 1)])
    reals([ay[i]["center"] for i in range(ny + 1)])
    reals([az[i]["center"] for i in range(nz + 1)], newline=False)
    return "".join(out)


@dataclass
class GridMetrics:
    """The grid as the solver holds it after readgeom (misc_init.f90:204)."""
    n1: int
    n2: int
    n3: int
    n1m: int
    n2m: int
    n3m: int
    xl: float
    yl: float
    zl: float
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    ipv: np.ndarray
    jpv: np.ndarray
    kpv: np.ndarray
    imv: np.ndarray
    jmv: np.ndarray
    kmv: np.ndarray
    fixil: np.ndarray
    fixjl: np.ndarray
    fixkl: np.ndarray
    fixiu: np.ndarray
    fixju: np.ndarray
    fixku: np.ndarray
    c2cx: np.ndarray
    c2cy: np.ndarray
    c2cz: np.ndarray
    c2cxi: np.ndarray
    c2cyi: np.ndarray
    c2czi: np.ndarray
    f2fx: np.ndarray
    f2fy: np.ndarray
    f2fz: np.ndarray
    f2fxi: np.ndarray
    f2fyi: np.ndarray
    f2fzi: np.ndarray
    xmp: np.ndarray
    ymp: np.ndarray
    zmp: np.ndarray

    @property
    def shape(self) -> Tuple[int, int, int]:
        """numpy shape of a (0:n1,0:n2,0:n3) array in C order (k, j, i)."""
        return (self.n3 + 1, self.n2 + 1, self.n1 + 1)


def read_grid_bin(text: str) -> GridMetrics:
    """readgeom, misc_init.f90:204-251 (list-directed reads of grid.bin)."""
    tok = text.split()
    pos = 0

    def take(n, conv):
        nonlocal pos
        vals = [conv(t) for t in tok[pos:pos + n]]
        if len(vals) != n:
            raise ValueError("grid.bin is truncated")
        pos += n
        return vals

    n1, n2, n3 = take(3, int)
    n1m, n2m, n3m = take(3, int)
    xl, yl, zl = take(3, float)
    d = {}
    d["x"], d["y"], d["z"] = (np.array(take(n, float)) for n in (n1, n2, n3))
    for key in ("pv", "mv"):
        for ax, n in (("i", n1m), ("j", n2m), ("k", n3m)):
            d[ax + key] = np.array(take(n, int), dtype=np.int64)
    for key in ("l", "u"):
        for ax, n in (("i", n1m), ("j", n2m), ("k", n3m)):
            d["fix" + ax + key] = np.array(take(n, int), dtype=np.int64)
    for key in ("c2c", "c2ci", "f2f", "f2fi"):
        for ax, n in (("x", n1), ("y", n2), ("z", n3)):
            name = key[:3] + ax + key[3:]
            d[name] = np.array(take(n + 1, float))
    for ax, n in (("x", n1), ("y", n2), ("z", n3)):
        d[ax + "mp"] = np.array(take(n + 1, float))
    return GridMetrics(n1=n1, n2=n2, n3=n3, n1m=n1m, n2m=n2m, n3m=n3m, xl=xl, yl=yl, zl=zl, **d)


def axis_vectors(grid_dat: str, xprdic: bool, yprdic: bool, zprdic: bool) -> Dict[str, Tuple[np.ndarray, np.ndarray]]:
    """Per-axis (coord, center) vectors, indices 0..N, as lib_setgrid holds
    them in full precision before grid.bin is written (the pre-processor's
    X/XM, Y/YM, Z/ZM of preprocessing.py:102-113)."""
    lines = grid_dat.split("\n")
    out = {}
    for name, line, prd in (("x", lines[2], xprdic), ("y", lines[3], yprdic), ("z", lines[4], zprdic)):
        info = _axis_info(line.split(), prd)
        n = len(info) - 1
        out[name] = (np.array([info[i]["coord"] for i in range(n + 1)]),
                     np.array([info[i]["center"] for i in range(n + 1)]))
    return out


def clustered_lines(x0: float, x1: float, xc: float, n_cells: int, dmin: float) -> List[float]:
    """n_cells + 1 gridlines on [x0, x1] clustered at xc (x0 <= xc <= x1):
    on each side a sinh distribution x = xc +- L sinh(b s) / sinh(b), s in
    [0, 1], whose first spacing at xc is dmin (uniform where the side's
    plain spacing is already finer).  The cells are split between the sides
    in proportion to their lengths."""
    la, lb = xc - x0, x1 - xc
    na = int(round(n_cells * la / (la + lb))) if la > 0 else 0
    nb = n_cells - na

    def side(length, n):
        if n == 0:
            return np.zeros(1)
        s = np.arange(n + 1) / n
        target = dmin * n / length          # b / sinh(b) for a first spacing of dmin
        if target >= 1.0:
            return length * s
        lo, hi = 1.0e-6, 60.0
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            if mid / math.sinh(mid) > target:
                lo = mid
            else:
                hi = mid
        b = 0.5 * (lo + hi)
        return length * np.sinh(b * s) / math.sinh(b)

    left = xc - side(la, na)[::-1]
    right = xc + side(lb, nb)
    xs = np.concatenate([left, right[1:]])
    xs[0], xs[-1] = x0, x1
    return [float(v) for v in xs]


def make_grid_lines(xs: Sequence[float], ys: Sequence[float], zs: Sequence[float],
                    xprdic: bool, zprdic: bool, yprdic: bool = False) -> Tuple[GridMetrics, str, str]:
    """Explicit gridlines -> grid.dat -> grid.bin -> metrics."""
    nx, ny, nz = len(xs), len(ys), len(zs)
    lx, ly, lz = xs[-1] - xs[0], ys[-1] - ys[0], zs[-1] - zs[0]
    gdat = grid_dat_text(nx, ny, nz, lx, ly, lz, xs, ys, zs)
    gbin = grid_bin_text(gdat, xprdic, yprdic, zprdic)
    return read_grid_bin(gbin), gdat, gbin


def make_grid(nx: int, ny: int, nz: int, lx: float, ly: float, lz: float,
              xseg: Sequence[Segment], yseg: Sequence[Segment], zseg: Sequence[Segment],
              xprdic: bool, zprdic: bool, yprdic: bool = False) -> Tuple[GridMetrics, str, str]:
    """Gridlines -> grid.dat -> grid.bin -> metrics.  Returns (metrics, grid.dat, grid.bin)."""
    xs, ys, zs = gridlines(nx, xseg), gridlines(ny, yseg), gridlines(nz, zseg)
    gdat = grid_dat_text(nx, ny, nz, lx, ly, lz, xs, ys, zs)
    gbin = grid_bin_text(gdat, xprdic, yprdic, zprdic)
    return read_grid_bin(gbin), gdat, gbin
