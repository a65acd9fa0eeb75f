"""Immersed-boundary pre-processing tables: the host restatement (numpy)
and, in build_tables_gpu, the same tables from the GPU kernels of
k_ibmpre.cu (lesgpu_ibmpre_run).

Restates the geometry routines the reference compiles with f2py for its
pre-processor (02_solver/f90/lib/ibm_body.f90, driven by
01_pre_processor/preprocessing.py) so a case can be built without a Fortran
compiler:
  find_inout       ibm_body.f90:14-46    solid/fluid mask at a staggered location
  findbdy_intp     ibm_body.f90:49-123   forcing points (interpolated first, inner after)
  geomfac_preset   ibm_body.f90:126-157  coordinate tables with one ghost on each side
  geomfac_intp     ibm_body.f90:160-322  3x3x3 interpolation weights from the surface point
  find_zero_nu_sgs ibm_body.f90:357-399  zero-eddy-viscosity cells (7-point test)
  conjg_intp       ibm_body.f90:402-550  conjugate heat transfer: c*, k* on the six
                                         faces and the fluid mask omega, from
  fluid_portion    ibm_body.f90:553-667  the fluid fraction of a box by a flood fill
                                         on 6x6x6 sub-cells
and the way preprocessing.py writes them (lib_preprocessing.py:223-328):
geomfac rounded to '%15.8f', the zero-viscosity list written 0-based and read
back by the solver as if 1-based (kept, the solver's behaviour depends on it).

Quirk kept: geomfac_preset compares its periodicity argument with 'on' while
preprocessing.py passes 'ON', so the periodic ghost coordinates are never set
(they stay 0).
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

from . import abi


def funcbody(body: Dict, x, y, z):
    """Vectorised body function (geometry/funcbody*.f90); >0 fluid, <=0 solid."""
    k = body.get("kind", abi.BODY_NONE)
    if k == abi.BODY_CHANNEL:
        return (1.0 + body.get("p0", 0.0)) - np.abs(y) + 0.0 * x + 0.0 * z
    if k == abi.BODY_CYLINDER:
        dx = x - body.get("cx", 0.0)
        dy = y - body.get("cy", 0.0)
        return np.sqrt(dx * dx + dy * dy) - body.get("r", 0.5) + 0.0 * z
    if k == abi.BODY_SPHERE:
        dx = x - body.get("cx", 0.0)
        dy = y - body.get("cy", 0.0)
        dz = z - body.get("cz", 0.0)
        return np.sqrt(dx * dx + dy * dy + dz * dz) - body.get("r", 0.5)
    if k == abi.BODY_SQUARE:
        return np.maximum(np.abs(x - body.get("cx", 0.0)), np.abs(y - body.get("cy", 0.0))) - body.get("r", 0.5) + 0.0 * z
    return np.ones(np.broadcast(x, y, z).shape)


def find_inout(body, xc, yc, zc):
    """inout[k, j, i] = 0 inside the body (funcbody <= 1e-10), 1 outside."""
    X = xc[None, None, :]
    Y = yc[None, :, None]
    Z = zc[:, None, None]
    val = funcbody(body, X, Y, Z)
    return np.where(val <= 1.0e-10, 0, 1).astype(np.int64)


def findbdy_intp(direction: int, inout, ufix, lfix):
    """Forcing points of one variable.  ufix/lfix: (x, y, z) tuples of the
    upper/lower fix flags of cells 1..n-1.  Returns (nintp, fcp, intpindx)
    with fcp = interpolated points first (in the k, j, i loop order of the
    reference), inner points after."""
    nz1, ny1, nx1 = inout.shape
    nx, ny, nz = nx1 - 1, ny1 - 1, nz1 - 1
    ist = 2 if direction == 1 else 1
    jst = 2 if direction == 2 else 1
    kst = 2 if direction == 3 else 1
    c = inout
    ks, js, is_ = slice(kst, nz), slice(jst, ny), slice(ist, nx)
    ctr = c[ks, js, is_]
    ux = np.asarray(ufix[0])[ist - 1:nx - 1][None, None, :]
    lx = np.asarray(lfix[0])[ist - 1:nx - 1][None, None, :]
    uy = np.asarray(ufix[1])[jst - 1:ny - 1][None, :, None]
    ly = np.asarray(lfix[1])[jst - 1:ny - 1][None, :, None]
    uz = np.asarray(ufix[2])[kst - 1:nz - 1][:, None, None]
    lz = np.asarray(lfix[2])[kst - 1:nz - 1][:, None, None]
    dxi = c[ks, js, ist + 1:nx + 1] - c[ks, js, ist - 1:nx - 1]
    dyi = c[ks, jst + 1:ny + 1, is_] - c[ks, jst - 1:ny - 1, is_]
    dzi = c[kst + 1:nz + 1, js, is_] - c[kst - 1:nz - 1, js, is_]
    s = (np.abs(dxi) * (1 - ux) * (1 - lx) + np.abs(dyi) * (1 - uy) * (1 - ly)
         + np.abs(dzi) * (1 - uz) * (1 - lz))
    intp = (ctr == 0) & (s > 0)
    inner = (ctr == 0) & (s == 0)
    pi = np.argwhere(intp)      # (k, j, i) lexicographic = the reference's k, j, i loop order
    pn = np.argwhere(inner)
    off = np.array([kst, jst, ist])
    pi_abs = pi + off
    pn_abs = pn + off
    fcp = np.concatenate([pi_abs[:, ::-1], pn_abs[:, ::-1]]).astype(np.int64)   # (i, j, k)
    indx = np.stack([dxi[intp], dyi[intp], dzi[intp]], axis=1).astype(np.int64)
    return len(pi), fcp, indx


def geomfac_preset(coord, center):
    """i_adj(-1:n+1, 3) of geomfac_preset with the periodic branch never taken."""
    n = len(coord) - 1
    a = np.zeros((n + 3, 3))
    a[1:n + 2, 0] = coord
    a[1:n + 2, 1] = center
    a[1:n + 2, 2] = center
    return a            # row r corresponds to index r - 1


def geomfac_intp(body, xpre, ypre, zpre, fcp, indx):
    """Weights geomfac(l, 1:3, 1:3, 1:3) of geomfac_intp for the interpolated points."""
    n = len(indx)
    gf = np.zeros((n, 3, 3, 3))
    if n == 0:
        return gf
    fi, fj, fk = fcp[:n, 0], fcp[:n, 1], fcp[:n, 2]
    di, dj, dk = indx[:, 0], indx[:, 1], indx[:, 2]
    X = lambda idx: xpre[idx + 1]
    Y = lambda idx: ypre[idx + 1]
    Z = lambda idx: zpre[idx + 1]
    x1, y1, z1 = X(fi), Y(fj), Z(fk)
    x2, y2, z2 = X(fi + di), Y(fj + dj), Z(fk + dk)
    ffs = funcbody(body, x1, y1, z1)
    ffe = funcbody(body, x2, y2, z2)
    bad = ffs * ffe > 0.0
    x0, y0, z0 = x1.copy(), y1.copy(), z1.copy()
    done = bad.copy()
    t1 = [x1.copy(), y1.copy(), z1.copy()]
    t2 = [x2.copy(), y2.copy(), z2.copy()]
    xx1 = [x1.copy(), y1.copy(), z1.copy()]
    xx2 = [x2.copy(), y2.copy(), z2.copy()]
    for m in range(1, 4):
        if m > 1:
            t1 = [a.copy() for a in xx1]
            t2 = [a.copy() for a in xx2]
        found = np.zeros(n, bool)
        for s in range(20):
            act = ~done & ~found
            if not act.any():
                break
            d = [t2[q] - t1[q] for q in range(3)]
            a1 = [t1[q] + d[q] * float(s) / 20.0 for q in range(3)]
            a2 = [t1[q] + d[q] * float(s + 1) / 20.0 for q in range(3)]
            for q in range(3):
                xx1[q] = np.where(act, a1[q], xx1[q])
                xx2[q] = np.where(act, a2[q], xx2[q])
            ff1 = funcbody(body, a1[0], a1[1], a1[2])
            ff2 = funcbody(body, a2[0], a2[1], a2[2])
            h1 = act & (ff1 == 0.0)
            h2 = act & ~h1 & (ff2 == 0.0)
            h3 = act & ~h1 & ~h2 & (ff1 * ff2 < 0.0)
            x0 = np.where(h1, a1[0], np.where(h2, a2[0], np.where(h3, 0.5 * (a1[0] + a2[0]), x0)))
            y0 = np.where(h1, a1[1], np.where(h2, a2[1], np.where(h3, 0.5 * (a1[1] + a2[1]), y0)))
            z0 = np.where(h1, a1[2], np.where(h2, a2[2], np.where(h3, 0.5 * (a1[2] + a2[2]), z0)))
            done |= h1 | h2
            if m == 3:
                done |= h3
            else:
                found |= h3
    x3, y3, z3 = X(fi + 2 * di), Y(fj + 2 * dj), Z(fk + 2 * dk)
    dx1, dx2, dx3 = np.abs(x1 - x0), np.abs(x2 - x0), np.abs(x3 - x0)
    dy1, dy2, dy3 = np.abs(y1 - y0), np.abs(y2 - y0), np.abs(y3 - y0)
    dz1, dz2, dz3 = np.abs(z1 - z0), np.abs(z2 - z0), np.abs(z3 - z0)

    def w(ind, d1, d2, d3):
        c0 = np.where(ind == 0, 1.0, np.where(d2 >= d1, d2 / np.where(d1 + d2 == 0, 1.0, d1 + d2), 0.5))
        den = d3 - d2
        c1 = np.where(ind == 0, 1.0, np.where(d2 >= d1, 1.0, (d3 - d1) / np.where(den == 0, 1.0, den)))
        return c0, c1

    with np.errstate(divide="ignore", invalid="ignore"):
        a0, a1 = w(di, dx1, dx2, dx3)
        b0, b1 = w(dj, dy1, dy2, dy3)
        c0, c1 = w(dk, dz1, dz2, dz3)
        # the reference multiplies left to right: -1/(a0 b0 c0), then the
        # first-level factors of x, y, z, then the second-level ones
        inv = 1.0 / (a0 * b0 * c0)
        F = [[a0, 1.0 - a0, 1.0 - a0], [b0, 1.0 - b0, 1.0 - b0], [c0, 1.0 - c0, 1.0 - c0]]
        G = [[None, a1, 1.0 - a1], [None, b1, 1.0 - b1], [None, c1, 1.0 - c1]]
        for p in range(3):
            for q in range(3):
                for r in range(3):
                    v = -inv * F[0][p] * F[1][q] * F[2][r]
                    for ax, e in ((0, p), (1, q), (2, r)):
                        if e > 0:
                            v = v * G[ax][e]
                    gf[:, p, q, r] = v
        gf[:, 0, 0, 0] = inv
    gf[bad] = 0.0
    gf[bad, 0, 0, 0] = 1.0
    return gf


def find_zero_nu_sgs(body, xm, ym, zm):
    """iszero(1:nx-1,1:ny-1,1:nz-1) as [k, j, i]: 0 where the cell or one of its
    six neighbours is solid."""
    sol = funcbody(body, xm[None, None, :], ym[None, :, None], zm[:, None, None]) <= 1.0e-10
    c = sol[1:-1, 1:-1, 1:-1] | sol[1:-1, 1:-1, :-2] | sol[1:-1, 1:-1, 2:] | sol[1:-1, :-2, 1:-1] \
        | sol[1:-1, 2:, 1:-1] | sol[:-2, 1:-1, 1:-1] | sol[2:, 1:-1, 1:-1]
    return np.where(c, 0, 1).astype(np.int64)


_SUBC = 6   # sub-cells per direction of fluid_portion (ibm_body.f90:425)


def fluid_portion(body, x1, x2, y1, y2, z1, z2):
    """fluid_portion (ibm_body.f90:553-667) of the boxes [x1,x2]x[y1,y2]x[z1,z2]
    (arrays of one shape).  The reference flood-fills from sub-cell (1,1,1)
    through 6-connected sub-cells of its phase, stops at sub-cells of the other
    phase, and gives every sub-cell it never reached the opposite phase; so the
    start sub-cell's 6-connected same-phase component keeps the start phase and
    every other sub-cell takes the opposite one, whatever the order of the
    fill.  Returns 1 - (solid sub-cells) / 216."""
    d = _SUBC
    x1, x2, y1, y2, z1, z2 = (np.asarray(v, dtype=np.float64).reshape(-1) for v in (x1, x2, y1, y2, z1, z2))
    f = (2.0 * np.arange(1, d + 1) - 1.0) / 2.0                  # dble(2 ii - 1) / 2
    xs = x1[:, None] + ((x2 - x1) / float(d))[:, None] * f[None, :]
    ys = y1[:, None] + ((y2 - y1) / float(d))[:, None] * f[None, :]
    zs = z1[:, None] + ((z2 - z1) / float(d))[:, None] * f[None, :]
    solid = funcbody(body, xs[:, None, None, :], ys[:, None, :, None], zs[:, :, None, None]) <= 1.0e-10   # [p, k, j, i]
    start_solid = solid[:, 0, 0, 0]
    same = solid == start_solid[:, None, None, None]
    reach = np.zeros_like(same)
    reach[:, 0, 0, 0] = True
    while True:
        grow = reach.copy()
        grow[:, 1:] |= reach[:, :-1]
        grow[:, :-1] |= reach[:, 1:]
        grow[:, :, 1:] |= reach[:, :, :-1]
        grow[:, :, :-1] |= reach[:, :, 1:]
        grow[:, :, :, 1:] |= reach[:, :, :, :-1]
        grow[:, :, :, :-1] |= reach[:, :, :, 1:]
        grow &= same
        if np.array_equal(grow, reach):
            break
        reach = grow
    comp = reach.reshape(reach.shape[0], -1).sum(axis=1)
    nsolid = np.where(start_solid, comp, d ** 3 - comp)
    return 1.0 - nsolid.astype(np.float64) / float(d ** 3)


def fluid_portion_fill(body, x1, x2, y1, y2, z1, z2):
    """fluid_portion of one box by the reference's own stack flood fill (a
    literal restatement for small checks of fluid_portion)."""
    d = _SUBC
    def solid_at(ii, jj, kk):
        xc = x1 + (x2 - x1) / float(d) * (float(2 * ii - 1) / 2.0)
        yc = y1 + (y2 - y1) / float(d) * (float(2 * jj - 1) / 2.0)
        zc = z1 + (z2 - z1) / float(d) * (float(2 * kk - 1) / 2.0)
        return bool(funcbody(body, np.float64(xc), np.float64(yc), np.float64(zc)) <= 1.0e-10)
    phase = {}
    start = 0 if solid_at(1, 1, 1) else 1
    phase[(1, 1, 1)] = start
    stack = [(1, 1, 1)]
    while stack:
        i, j, k = stack.pop()
        for kk in (k - 1, k, k + 1):
            for jj in (j - 1, j, j + 1):
                for ii in (i - 1, i, i + 1):
                    if abs(ii - i) + abs(jj - j) + abs(kk - k) != 1:
                        continue
                    if not (1 <= ii <= d and 1 <= jj <= d and 1 <= kk <= d) or (ii, jj, kk) in phase:
                        continue
                    phase[(ii, jj, kk)] = 0 if solid_at(ii, jj, kk) else 1
                    if phase[(ii, jj, kk)] == start:
                        stack.append((ii, jj, kk))
    nsolid = sum(1 for k in range(1, d + 1) for j in range(1, d + 1) for i in range(1, d + 1)
                 if phase.get((i, j, k), 1 - start) == 0)
    return 1.0 - float(nsolid) / float(d ** 3)


def conjg_intp(body, cratio: float, kratio: float, gdat_axes, prdic, chunk: int = 4096):
    """conjg_intp (ibm_body.f90:402-550) on the cells 1..n-1 of each
    direction: c* = (1 - fp) cratio + fp for the cell's fluid fraction fp;
    omega = 1 where fp >= 1 - 1e-12; k* of the six faces (east, west, north,
    south, top, bottom) from the fluid fraction of the box between the two
    cell centres -- (1 - fp) kratio + fp when the centres share a phase, else
    the harmonic mean kratio / (kratio fp + (1 - fp)) -- with periodic wraps
    shifted by the domain length.  Returns (cstar[k, j, i], kstar[6, k, j, i],
    omega[k, j, i])."""
    X, XM = (np.asarray(v, dtype=np.float64) for v in gdat_axes["x"])
    Y, YM = (np.asarray(v, dtype=np.float64) for v in gdat_axes["y"])
    Z, ZM = (np.asarray(v, dtype=np.float64) for v in gdat_axes["z"])
    nx, ny, nz = len(X) - 1, len(Y) - 1, len(Z) - 1
    xpr, ypr, zpr = (int(v) for v in prdic)
    lx, ly, lz = X[nx] - X[1], Y[ny] - Y[1], Z[nz] - Z[1]
    kk, jj, ii = np.meshgrid(np.arange(1, nz), np.arange(1, ny), np.arange(1, nx), indexing="ij")
    i, j, k = ii.reshape(-1), jj.reshape(-1), kk.reshape(-1)
    xm, ym, zm = XM[i], YM[j], ZM[k]
    aa = funcbody(body, xm, ym, zm)
    xmp = np.where((xpr == 1) & (i == nx - 1), XM[1] + lx, XM[np.minimum(i + 1, nx)])
    xmm = np.where((xpr == 1) & (i == 1), XM[nx - 1] - lx, XM[i - 1])
    ymp = np.where((ypr == 1) & (j == ny - 1), YM[1] + ly, YM[np.minimum(j + 1, ny)])
    ymm = np.where((ypr == 1) & (j == 1), YM[ny - 1] - ly, YM[j - 1])
    zmp = np.where((zpr == 1) & (k == nz - 1), ZM[1] + lz, ZM[np.minimum(k + 1, nz)])
    zmm = np.where((zpr == 1) & (k == 1), ZM[nz - 1] - lz, ZM[k - 1])
    boxes = [  # (x1, x2, y1, y2, z1, z2), neighbour centre for the phase test
        ((X[i], X[i + 1], Y[j], Y[j + 1], Z[k], Z[k + 1]), None),
        ((xm, xmp, Y[j], Y[j + 1], Z[k], Z[k + 1]), (xmp, ym, zm)),
        ((xmm, xm, Y[j], Y[j + 1], Z[k], Z[k + 1]), (xmm, ym, zm)),
        ((X[i], X[i + 1], ym, ymp, Z[k], Z[k + 1]), (xm, ymp, zm)),
        ((X[i], X[i + 1], ymm, ym, Z[k], Z[k + 1]), (xm, ymm, zm)),
        ((X[i], X[i + 1], Y[j], Y[j + 1], zm, zmp), (xm, ym, zmp)),
        ((X[i], X[i + 1], Y[j], Y[j + 1], zmm, zm), (xm, ym, zmm)),
    ]
    n = i.size
    shape = (nz - 1, ny - 1, nx - 1)
    kstar = np.empty((6, n))
    cstar = None
    omega = None
    for f, (box, nbr) in enumerate(boxes):
        fp = np.concatenate([fluid_portion(body, *(b[s:s + chunk] for b in box)) for s in range(0, n, chunk)]) \
            if n else np.zeros(0)
        if nbr is None:
            cstar = (1.0 - fp) * cratio + fp * 1.0
            omega = np.where(fp >= (1.0 - 1.0e-12), 1, 0).astype(np.int64)
        else:
            same = aa * funcbody(body, *nbr) >= 0.0
            kstar[f - 1] = np.where(same, (1.0 - fp) * kratio + fp * 1.0,
                                    kratio / (kratio * fp + 1.0 * (1.0 - fp)))
    return cstar.reshape(shape), kstar.reshape((6,) + shape), omega.reshape(shape)


def _round8(gf):
    """geomfac as the solver reads it back from '%15.8f' text."""
    return np.array([float("%15.8f" % v) for v in gf.reshape(-1)]).reshape(gf.shape)


def build_tables(grid, settings, gdat_axes) -> Dict:
    """All IB/LES tables of one case.  gdat_axes: dict with the coord/center
    vectors (0..N) per axis exactly as lib_setgrid builds them (gridgen
    provides them); fix flags come from the grid metrics."""
    body = settings["body"]
    X, XM = gdat_axes["x"]
    Y, YM = gdat_axes["y"]
    Z, ZM = gdat_axes["z"]
    ufix = (grid.fixiu, grid.fixju, grid.fixku)
    lfix = (grid.fixil, grid.fixjl, grid.fixkl)
    locs = {1: (X, YM, ZM), 2: (XM, Y, ZM), 3: (XM, YM, Z), 4: (XM, YM, ZM)}
    XX, YY, ZZ = geomfac_preset(X, XM), geomfac_preset(Y, YM), geomfac_preset(Z, ZM)
    pre = {1: (XX[:, 0], YY[:, 2], ZZ[:, 1]), 2: (XX[:, 1], YY[:, 0], ZZ[:, 2]),
           3: (XX[:, 2], YY[:, 1], ZZ[:, 0]), 4: (XX[:, 2], YY[:, 2], ZZ[:, 2])}
    nl = 4 if settings.get("ihtrans", 0) == 1 else 3
    out = dict(nintp=[0] * 4, nbody=[0] * 4, fc=[np.zeros((0, 3), np.int64)] * 4,
               intpindx=[np.zeros((0, 3), np.int64)] * 4, geomfac=[np.zeros((0, 27))] * 4)
    for d in range(1, nl + 1):
        inout = find_inout(body, *locs[d])
        nintp, fcp, indx = findbdy_intp(d, inout, ufix, lfix)
        gf = geomfac_intp(body, *pre[d], fcp, indx)
        out["nintp"][d - 1] = nintp
        out["nbody"][d - 1] = len(fcp)
        out["fc"][d - 1] = fcp
        out["intpindx"][d - 1] = indx
        out["geomfac"][d - 1] = _round8(gf).reshape(nintp, 27)
    isz = find_zero_nu_sgs(body, XM, YM, ZM)
    # les_preprocessing_data: indices of iszero == 0 in i, j, k loop order, 0-based
    ii, jj, kk = np.nonzero(isz.transpose(2, 1, 0) == 0)
    out["nzero"] = len(ii)
    out["inz"], out["jnz"], out["knz"] = ii.astype(np.int64), jj.astype(np.int64), kk.astype(np.int64)
    out["nwall_dvm"] = isz.reshape(-1).astype(np.int64)           # (i fastest) = Fortran order of (k,j,i) C array
    n = grid.n1m * grid.n2m * grid.n3m
    out["cstar"] = np.ones(n)
    out["kstar"] = np.ones(6 * n)
    out["omega"] = np.ones(n, np.int64)
    return out


def build_tables_gpu(lib, settings, grid, gdat_axes) -> Dict:
    """The same tables as build_tables, computed on the GPU by
    lesgpu_ibmpre_run (the compute path; build_tables is the host
    restatement it is tested against)."""
    import ctypes as C
    P = C.c_void_p
    lib.lesgpu_ibmpre_run.argtypes = [C.POINTER(abi.Config), C.POINTER(abi.Grid), C.POINTER(abi.PD), C.POINTER(P)]
    lib.lesgpu_ibmpre_tables.argtypes = [P, C.POINTER(abi.Ibm)]
    lib.lesgpu_ibmpre_free.argtypes = [P]
    for f in ("lesgpu_ibmpre_run", "lesgpu_ibmpre_tables", "lesgpu_ibmpre_free"):
        getattr(lib, f).restype = C.c_int
    cfg = abi.pack_config(settings)
    gr = abi.pack_grid(grid)
    vecs = [np.ascontiguousarray(v, dtype=np.float64) for ax in ("x", "y", "z") for v in gdat_axes[ax]]
    arr = (abi.PD * 6)(*[v.ctypes.data_as(abi.PD) for v in vecs])
    h = P()
    rc = lib.lesgpu_ibmpre_run(C.byref(cfg), C.byref(gr.struct), arr, C.byref(h))
    if rc != 0:
        raise RuntimeError(f"lesgpu_ibmpre_run: {abi.ERR_NAMES.get(rc, rc)}")
    try:
        t = abi.Ibm()
        lib.lesgpu_ibmpre_tables(h, C.byref(t))
        nl = 4 if settings.get("ihtrans", 0) == 1 else 3
        out = dict(nintp=[0] * 4, nbody=[0] * 4, fc=[np.zeros((0, 3), np.int64)] * 4,
                   intpindx=[np.zeros((0, 3), np.int64)] * 4, geomfac=[np.zeros((0, 27))] * 4)
        for l in range(nl):
            ni, nb = int(t.nintp[l]), int(t.nbody[l])
            out["nintp"][l], out["nbody"][l] = ni, nb
            if nb:
                out["fc"][l] = np.ctypeslib.as_array(t.fc[l], shape=(nb * 3,)).reshape(nb, 3).copy()
            if ni:
                out["intpindx"][l] = np.ctypeslib.as_array(t.intpindx[l], shape=(ni * 3,)).reshape(ni, 3).copy()
                out["geomfac"][l] = np.ctypeslib.as_array(t.geomfac[l], shape=(ni * 27,)).reshape(ni, 27).copy()
        nz = int(t.nzero)
        out["nzero"] = nz
        for name in ("inz", "jnz", "knz"):
            out[name] = np.ctypeslib.as_array(getattr(t, name), shape=(nz,)).copy() if nz else np.zeros(0, np.int64)
        ncell = grid.n1m * grid.n2m * grid.n3m
        out["nwall_dvm"] = np.ctypeslib.as_array(t.nwall_dvm, shape=(ncell,)).copy()
        out["cstar"] = np.ones(ncell)
        out["kstar"] = np.ones(6 * ncell)
        out["omega"] = np.ones(ncell, np.int64)
        return out
    finally:
        lib.lesgpu_ibmpre_free(h)


def conjg_tables_gpu(lib, settings, grid, gdat_axes, cratio: float, kratio: float):
    """conjg_intp computed on the GPU (lesgpu_conjg_run): (cstar, kstar,
    omega) flattened as lesgpu_ibm holds them (cells i fastest; kstar face by
    face), the layout conjg_intp's arrays take under reshape(-1)."""
    import ctypes as C
    fn = lib.lesgpu_conjg_run
    fn.argtypes = [C.POINTER(abi.Config), C.POINTER(abi.Grid), C.POINTER(abi.PD), C.c_double, C.c_double,
                   C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    cfg = abi.pack_config(settings)
    gr = abi.pack_grid(grid)
    vecs = [np.ascontiguousarray(v, dtype=np.float64) for ax in ("x", "y", "z") for v in gdat_axes[ax]]
    arr = (abi.PD * 6)(*[v.ctypes.data_as(abi.PD) for v in vecs])
    n = grid.n1m * grid.n2m * grid.n3m
    cs, ks, om = np.empty(n), np.empty(6 * n), np.empty(n, np.int64)
    rc = fn(C.byref(cfg), C.byref(gr.struct), arr, float(cratio), float(kratio),
            cs.ctypes.data, ks.ctypes.data, om.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"lesgpu_conjg_run: {abi.ERR_NAMES.get(rc, rc)}")
    return cs, ks, om

