"""Synthetic LES cases with the shapes of the benchmark configurations.

A case = settings (settings.input + boundary.input + periodicity flags, as a
dict matching lesgpu_config), a grid (gridgen.GridMetrics) and an initial
field in the state prefld (misc_init.f90:610-786) leaves after reading a
field file with IREAD = 1.  No dataset is involved: grids come from the
gridline recipes below and the initial fields from a seeded PCG64 stream.

Presets
  channel(...)  : turbulent channel, periodic x/z, walls at y = +-1, tanh
                  wall-normal stretching, constant flow rate (ICH = 1),
                  passive temperature with the decomposition source
                  (IDECOMP = 1), dynamic SGS.  64^3 is the Re_tau = 180
                  configuration; 384x256x384 the Re_tau = 590 one.
  cylinder_array(...)  : a row of heated circular cylinders, periodic in x
                  and z, between no-slip isothermal walls, constant flow
                  rate, direct-forcing IB with interpolation (the IB path
                  with the FFT Poisson solver).
  cylinder(...) : flow past a heated circular cylinder (D = 1) in a
                  30D x 20D x pi D box: uniform inflow, convective outlet,
                  far-field (slip) lateral boundaries, periodic z, grid
                  clustered at the body, direct-forcing IB, FFT-z +
                  multigrid-xy Poisson solver.  128x96x16 at Re = 100 and
                  256x192x64 at Re = 3900 are the benchmark sizes.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any, Dict, Optional

import numpy as np

from . import abi
from .gridgen import GridMetrics, Segment, axis_vectors, clustered_lines, make_grid, make_grid_lines
from . import ibmpre


def base_settings() -> Dict[str, Any]:
    """Defaults of 02_solver/settings.input and boundary.input."""
    return dict(
        re=180.0, pr=0.71, gr=0.0, grdir=2, tflu_i=0.0, tsol_i=0.0,
        ireset=0, iread=1, iavg=0, ipzero=0, eps_ptr=0.0, udrv_i=1.0,
        nend=999999, nprint=10000, npriavg=50000, npin=1,
        tend=1.0e9, ptb_tst=-1.0, avg_tst=1.0e9,
        idtopt=1, dt_size=0.005, cflfac=0.5,
        resid1=1.0e-6, nlev=5, nbli=3, ioldv=0, mgitr=500, imgsor=170, wwsor=1.8,
        iles=1, insmdl=1, itemdl=0, idvmon=1, csgsts=0.025, csgshf=0.003, filter=3,
        ibmon=0, masson=0, imovingon=0, ihtrans=1, idecomp=0,
        bc_ybtm=0, bc_ytop=0, bc_zbtm=0, bc_ztop=0,
        bc_t_ybtm=0, bc_t_ytop=0, val_t_ybtm=0.0, val_t_ytop=0.0,
        bc_t_zbtm=1, bc_t_ztop=1, val_t_zbtm=0.0, val_t_ztop=0.0,
        ich=0, iconjg=0,
        xprdic=0, yprdic=0, zprdic=0, iintp=0,
        poisson=abi.POISSON_FTFT, precision=abi.PREC_FP64,
        body=dict(kind=abi.BODY_NONE, cx=0.0, cy=0.0, cz=0.0, r=0.5, p0=0.0),
    )


def readbcs_overrides(s: Dict[str, Any]) -> Dict[str, Any]:
    """What readbcs (misc_init.f90:95-160) does to the boundary.input flags
    once the periodicity flags are known: a periodic direction's momentum
    flags become 4 (periodic), so no wall term is evaluated there."""
    if s.get("yprdic", 0) == 1:
        s["bc_ybtm"] = s["bc_ytop"] = 4
    if s.get("zprdic", 0) == 1:
        s["bc_zbtm"] = s["bc_ztop"] = 4
    return s


@dataclass
class Case:
    name: str
    settings: Dict[str, Any]
    grid: GridMetrics
    grid_dat: str
    grid_bin: str
    fields: Dict[str, np.ndarray]          # u, v, w, p, t in (n3+1, n2+1, n1+1) C order
    time: float = 0.0
    dt: float = 0.0
    ihist: int = 0
    m: int = 0
    ibm: Optional[Dict[str, Any]] = None   # pack_ibm tables, or None

    @property
    def cells(self) -> int:
        g = self.grid
        return g.n1m * g.n2m * g.n3m


def prefld_apply(s: Dict[str, Any], g: GridMetrics, u, v, w, p, t):
    """Leave the arrays the way prefld (misc_init.f90:610-786) does after an
    IREAD = 1 read: only the record ranges are kept, T's unread cells are
    TSOL_I, then the periodic ghost copies."""
    n1, n2, n3, n1m, n2m, n3m = g.n1, g.n2, g.n3, g.n1m, g.n2m, g.n3m
    U = np.zeros(g.shape); U[0:n3 + 1, 0:n2 + 1, 1:n1 + 1] = u[0:n3 + 1, 0:n2 + 1, 1:n1 + 1]
    V = np.zeros(g.shape); V[0:n3 + 1, 1:n2 + 1, 0:n1 + 1] = v[0:n3 + 1, 1:n2 + 1, 0:n1 + 1]
    W = np.zeros(g.shape); W[1:n3 + 1, 0:n2 + 1, 0:n1 + 1] = w[1:n3 + 1, 0:n2 + 1, 0:n1 + 1]
    P = np.zeros(g.shape); P[1:n3m + 1, 1:n2m + 1, 1:n1m + 1] = p[1:n3m + 1, 1:n2m + 1, 1:n1m + 1]
    T = np.full(g.shape, float(s["tsol_i"]))
    T[1:n3m + 1, 1:n2m + 1, 1:n1m + 1] = t[1:n3m + 1, 1:n2m + 1, 1:n1m + 1]
    if s.get("ipzero", 0) == 1:
        P[:] = 0.0
    if s["xprdic"] == 1:
        U[:, :, 0] = U[:, :, n1m]; U[:, :, n1] = U[:, :, 1]
        V[:, 1:, 0] = V[:, 1:, n1m]; V[:, 1:, n1] = V[:, 1:, 1]
        W[1:, :, 0] = W[1:, :, n1m]; W[1:, :, n1] = W[1:, :, 1]
        T[:, :, 0] = T[:, :, n1m]; T[:, :, n1] = T[:, :, 1]
    if s["yprdic"] == 1:
        U[:, 0, 1:] = U[:, n2m, 1:]; U[:, n2, 1:] = U[:, 1, 1:]
        V[:, 0, :] = V[:, n2m, :]; V[:, n2, :] = V[:, 1, :]
        W[1:, 0, :] = W[1:, n2m, :]; W[1:, n2, :] = W[1:, 1, :]
        T[:, 0, :] = T[:, n2m, :]; T[:, n2, :] = T[:, 1, :]
    if s["zprdic"] == 1:
        U[0, :, 1:] = U[n3m, :, 1:]; U[n3, :, 1:] = U[1, :, 1:]
        V[0, 1:, :] = V[n3m, 1:, :]; V[n3, 1:, :] = V[1, 1:, :]
        W[0, :, :] = W[n3m, :, :]; W[n3, :, :] = W[1, :, :]
        T[0, :, :] = T[n3m, :, :]; T[n3, :, :] = T[1, :, :]
    return U, V, W, P, T


def _plane_mean_correct(f, mask, weight, axis):
    """Subtract the weighted mean of the perturbation over each plane normal
    to `axis` (the correction of addperturb_isotropic, misc_init.f90:900-926)."""
    num = (f * mask * weight).sum(axis=tuple(a for a in range(3) if a != axis), keepdims=True)
    den = (mask * weight).sum(axis=tuple(a for a in range(3) if a != axis), keepdims=True)
    adj = np.where(den > 0, num / np.where(den > 0, den, 1.0), 0.0)
    return f - adj * mask


def channel(n1m: int = 64, n2m: int = 64, n3m: int = 64,
            lx: float = 4.0 * math.pi, ly: float = 2.0, lz: float = 4.0 * math.pi / 3.0,
            gamma: float = 2.75, re: float = 2800.0, pr: float = 0.71,
            amp: float = 0.1, seed: int = 20261203, precision: int = abi.PREC_FP64,
            zwalls: bool = False, name: Optional[str] = None) -> Case:
    """Channel with passive heat transfer (temperature decomposition source).

    Re is the bulk Reynolds number on the half height (Re_b = 2800 gives
    Re_tau ~ 180 for the 4pi x 2 x 4pi/3 box); the initial field is the
    laminar profile 1.5(1 - y^2) plus a seeded uniform perturbation of
    relative amplitude `amp`, mean-corrected plane by plane.  `zwalls`
    closes z with no-slip adiabatic walls (a duct; ZPRDIC = 0, the z grid
    clustered at both walls as y is)."""
    s = base_settings()
    s.update(re=re, pr=pr, ich=1, iconjg=1, idecomp=1, ihtrans=1, iles=1, idvmon=1,
             xprdic=1, zprdic=0 if zwalls else 1, yprdic=0, udrv_i=1.0, cflfac=0.5, idtopt=1, dt_size=0.002,
             bc_ybtm=0, bc_ytop=0, bc_t_ybtm=0, bc_t_ytop=0, poisson=abi.POISSON_FTFT,
             precision=precision,
             body=dict(kind=abi.BODY_CHANNEL, cx=0.0, cy=0.0, cz=0.0, r=0.0, p0=1.0e-6))
    if zwalls:
        s.update(bc_zbtm=0, bc_ztop=0, bc_t_zbtm=1, bc_t_ztop=1)
    readbcs_overrides(s)
    n1, n2, n3 = n1m + 1, n2m + 1, n3m + 1
    zseg = (Segment("Z", 0.0, lz, 1, n3, "H", 0.5, gamma) if zwalls else Segment("Z", 0.0, lz, 1, n3, "U"))
    g, gdat, gbin = make_grid(
        n1, n2, n3, lx, ly, lz,
        [Segment("X", 0.0, lx, 1, n1, "U")],
        [Segment("Y", -1.0, 1.0, 1, n2, "H", 0.5, gamma)],
        [zseg],
        xprdic=True, zprdic=not zwalls)
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = g.shape
    u = np.zeros(sh); v = np.zeros(sh); w = np.zeros(sh); p = np.zeros(sh); t = np.zeros(sh)
    ymp = g.ymp[None, :, None]
    u[:] = 1.5 * s["udrv_i"] * (1.0 - ymp ** 2)
    # walls: no-slip ghosts (the ghost centre ymp(0), ymp(n2) lies on the wall)
    u[:, 0, :] = 0.0; u[:, n2, :] = 0.0
    # perturbations on the interior unknowns
    def pert():
        return (rng.random(sh) - 0.5) * 2.0 * amp * s["udrv_i"]
    fl = np.zeros(sh); fl[1:n3m + 1, 1:n2m + 1, 1:n1m + 1] = 1.0
    dy = g.f2fy[None, :, None]; dz = g.f2fz[:, None, None]; dx = g.f2fx[None, None, :]
    fv = np.zeros(sh); fv[1:n3m + 1, 2:n2m + 1, 1:n1m + 1] = 1.0   # v unknowns: j = 2..n2m
    u += _plane_mean_correct(pert(), fl, dy * dz, axis=2)
    v += _plane_mean_correct(pert(), fv, dz * dx, axis=1)
    w += _plane_mean_correct(pert(), fl, dx * dy, axis=0)
    u *= fl; v *= fv; w *= fl
    u[:, 0, :] = 0.0; u[:, n2, :] = 0.0
    if zwalls:                                   # w(k = 1) lies on the wall
        w[1, :, :] = 0.0
    # temperature of the decomposition form: t = u / Pr in the fluid (makefld :529-541)
    t[:] = 0.0
    t[1:n3m + 1, 1:n2m + 1, 1:n1m + 1] = (0.5 * (u[1:n3m + 1, 1:n2m + 1, 1:n1m + 1]
                                              + u[1:n3m + 1, 1:n2m + 1, 2:n1m + 2])) / pr
    U, V, W, P, T = prefld_apply(s, g, u, v, w, p, t)
    nm = name or f"channel_{n1m}x{n2m}x{n3m}"
    return Case(nm, s, g, gdat, gbin, dict(u=U, v=V, w=W, p=P, t=T), time=0.0, dt=s["dt_size"],
                ihist=0, m=0, ibm=channel_ibm_tables(g))


def channel_ibm_tables(g: GridMetrics) -> Dict[str, Any]:
    """The placeholder pre-processing outputs of write_ibmpre_placeholders
    (lib_preprocessing.py:172-221): no forcing points, no zero-viscosity
    points, nwall = 1, c* = k* = 1."""
    z3 = np.zeros((0, 3), np.int64)
    return dict(nintp=[0, 0, 0, 0], nbody=[0, 0, 0, 0], fc=[z3] * 4, intpindx=[z3] * 4,
                geomfac=[np.zeros((0, 27))] * 4, nzero=0,
                inz=np.zeros(0, np.int64), jnz=np.zeros(0, np.int64), knz=np.zeros(0, np.int64),
                nwall_dvm=np.ones(g.n1m * g.n2m * g.n3m, np.int64),
                cstar=np.ones(g.n1m * g.n2m * g.n3m), kstar=np.ones(6 * g.n1m * g.n2m * g.n3m),
                omega=np.ones(g.n1m * g.n2m * g.n3m, np.int64))


def cylinder_array(n1m: int = 48, n2m: int = 40, n3m: int = 8,
                   lx: float = 6.0, ly: float = 4.0, lz: float = math.pi,
                   re: float = 200.0, pr: float = 0.71, amp: float = 0.05,
                   seed: int = 20261203, precision: int = abi.PREC_FP64,
                   name: Optional[str] = None) -> Case:
    """Cylinders of diameter 1 on a pitch lx, centred between no-slip walls
    at y = -ly/2 and +ly/2, periodic in x and z, constant flow rate.  The
    temperature uses the decomposition source (IDECOMP = 1) with T = 0 on the
    walls and, through thermal IB forcing (ICONJG = 0), on the cylinder.
    IB tables come from ibmpre (forcing points with interpolation, zero-eddy-
    viscosity list, wall-function mask).  Initial field: plane Poiseuille
    profile outside the body plus a seeded uniform perturbation."""
    s = base_settings()
    s.update(re=re, pr=pr, ich=1, iconjg=0, idecomp=1, ihtrans=1, iles=1, idvmon=1,
             ibmon=1, masson=1, iintp=1,
             xprdic=1, zprdic=1, yprdic=0, udrv_i=1.0, cflfac=0.5, idtopt=1, dt_size=0.002,
             bc_ybtm=0, bc_ytop=0, bc_t_ybtm=0, bc_t_ytop=0, poisson=abi.POISSON_FTFT,
             precision=precision,
             body=dict(kind=abi.BODY_CYLINDER, cx=0.5 * lx, cy=0.0, cz=0.0, r=0.5, p0=0.0))
    readbcs_overrides(s)
    n1, n2, n3 = n1m + 1, n2m + 1, n3m + 1
    h = 0.5 * ly
    g, gdat, gbin = make_grid(
        n1, n2, n3, lx, ly, lz,
        [Segment("X", 0.0, lx, 1, n1, "U")],
        [Segment("Y", -h, h, 1, n2, "U")],
        [Segment("Z", 0.0, lz, 1, n3, "U")],
        xprdic=True, zprdic=True)
    tables = ibmpre.build_tables(g, s, axis_vectors(gdat, True, False, True))
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = g.shape
    body = s["body"]
    X = np.concatenate([[0.0], g.x])[None, None, :]
    fl_u = ibmpre.funcbody(body, X, g.ymp[None, :, None], g.zmp[:, None, None]) > 1.0e-10
    u = np.where(fl_u, 1.5 * (1.0 - (g.ymp[None, :, None] / h) ** 2), 0.0) * np.ones(sh)
    v = np.zeros(sh); w = np.zeros(sh); p = np.zeros(sh); t = np.zeros(sh)
    inner = np.zeros(sh); inner[1:n3m + 1, 1:n2m + 1, 1:n1m + 1] = 1.0
    fv = np.zeros(sh); fv[1:n3m + 1, 2:n2m + 1, 1:n1m + 1] = 1.0
    u += (rng.random(sh) - 0.5) * 2.0 * amp * inner * fl_u
    v += (rng.random(sh) - 0.5) * 2.0 * amp * fv
    w += (rng.random(sh) - 0.5) * 2.0 * amp * inner
    u *= inner; v *= fv; w *= inner
    t[1:n3m + 1, 1:n2m + 1, 1:n1m + 1] = (0.5 * (u[1:n3m + 1, 1:n2m + 1, 1:n1m + 1]
                                              + u[1:n3m + 1, 1:n2m + 1, 2:n1m + 2])) / pr
    U, V, W, P, T = prefld_apply(s, g, u, v, w, p, t)
    nm = name or f"cylinder_array_{n1m}x{n2m}x{n3m}"
    return Case(nm, s, g, gdat, gbin, dict(u=U, v=V, w=W, p=P, t=T), time=0.0, dt=s["dt_size"],
                ihist=0, m=0, ibm=tables)


def cylinder(n1m: int = 128, n2m: int = 96, n3m: int = 16, re: float = 100.0, pr: float = 0.71,
             dmin: float = 0.02, amp: float = 1.0e-3, body_kind: int = abi.BODY_CYLINDER,
             center=(0.0, 0.0, 0.5 * math.pi), seed: int = 20261203, nlev: Optional[int] = None,
             precision: int = abi.PREC_FP64, name: Optional[str] = None) -> Case:
    """Heated body (wall T = 0 through the thermal forcing) in a free stream
    (U = 1, T = TFLU_I = -1) on x in [-10, 20], y in [-10, 10], z in [0, pi],
    gridlines clustered at the body with a first spacing of `dmin`.  The
    initial field is the one makefld (misc_init.f90:442-560) builds for
    ICH = 0 -- U = 1 in the fluid, 0 in the body -- plus a seeded uniform
    perturbation of amplitude `amp` on the interior unknowns, in the state
    prefld leaves after reading it back."""
    s = base_settings()
    s.update(re=re, pr=pr, ich=0, iconjg=0, idecomp=0, ihtrans=1, iles=1, idvmon=1,
             ibmon=1, masson=1, iintp=1, tflu_i=-1.0, tsol_i=0.0,
             xprdic=0, yprdic=0, zprdic=1, udrv_i=1.0, cflfac=0.5, idtopt=1, dt_size=0.005,
             bc_ybtm=1, bc_ytop=1, bc_t_ybtm=1, bc_t_ytop=1, val_t_ybtm=0.0, val_t_ytop=0.0,
             poisson=abi.POISSON_Z_FT, precision=precision,
             body=dict(kind=body_kind, cx=float(center[0]), cy=float(center[1]), cz=float(center[2]),
                       r=0.5, p0=0.0))
    if nlev is None:
        nlev = 1
        while nlev < 5 and n1m % (2 ** (nlev + 1)) == 0 and n1m // (2 ** (nlev + 1)) >= 2:
            nlev += 1
    s["nlev"] = nlev
    readbcs_overrides(s)
    xs = clustered_lines(-10.0, 20.0, float(center[0]), n1m, dmin)
    ys = clustered_lines(-10.0, 10.0, float(center[1]), n2m, dmin)
    zs = [math.pi * k / n3m for k in range(n3m + 1)]
    g, gdat, gbin = make_grid_lines(xs, ys, zs, xprdic=False, zprdic=True)
    tables = ibmpre.build_tables(g, s, axis_vectors(gdat, False, False, True))
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = g.shape
    body = s["body"]
    X = np.concatenate([[g.x[0]], g.x])[None, None, :]
    fl_u = ibmpre.funcbody(body, X, g.ymp[None, :, None], g.zmp[:, None, None]) >= 1.0e-10
    fl_c = ibmpre.funcbody(body, g.xmp[None, None, :], g.ymp[None, :, None], g.zmp[:, None, None]) >= 1.0e-10
    u = np.where(fl_u, s["udrv_i"], 0.0) * np.ones(sh)
    v = np.zeros(sh); w = np.zeros(sh); p = np.zeros(sh)
    t = np.where(fl_c, s["tflu_i"], s["tsol_i"]) * np.ones(sh)
    inner = np.zeros(sh); inner[1:n3m + 1, 1:n2m + 1, 2:n1m + 1] = 1.0     # u unknowns i = 2..n1m
    fv = np.zeros(sh); fv[1:n3m + 1, 2:n2m + 1, 1:n1m + 1] = 1.0
    fw = np.zeros(sh); fw[1:n3m + 1, 1:n2m + 1, 1:n1m + 1] = 1.0
    u += (rng.random(sh) - 0.5) * 2.0 * amp * inner * fl_u
    v += (rng.random(sh) - 0.5) * 2.0 * amp * fv
    w += (rng.random(sh) - 0.5) * 2.0 * amp * fw
    U, V, W, P, T = prefld_apply(s, g, u, v, w, p, t)
    nm = name or f"cylinder_{n1m}x{n2m}x{n3m}"
    return Case(nm, s, g, gdat, gbin, dict(u=U, v=V, w=W, p=P, t=T), time=0.0, dt=s["dt_size"],
                ihist=0, m=0, ibm=tables)


def with_conjugate(case: Case, cratio: float, kratio: float) -> Case:
    """The same case with conjugate heat transfer (ICONJG = 1): the body
    conducts heat, with solid/fluid heat-capacity ratio cratio and
    conductivity ratio kratio; c*, k* and the fluid mask omega come from
    conjg_intp (the pre-processor's CONJG-HTRANS tables) instead of the
    placeholders, and the body gets no thermal direct forcing."""
    from .gridgen import axis_vectors
    s = dict(case.settings)
    s["iconjg"] = 1
    axes = axis_vectors(case.grid_dat, s.get("xprdic", 0) == 1, s.get("yprdic", 0) == 1, s.get("zprdic", 0) == 1)
    cs, ks, om = ibmpre.conjg_intp(s["body"], cratio, kratio, axes,
                                   (s.get("xprdic", 0), s.get("yprdic", 0), s.get("zprdic", 0)))
    ibm = dict(case.ibm)
    ibm["cstar"], ibm["kstar"], ibm["omega"] = cs.reshape(-1), ks.reshape(-1), om.reshape(-1)
    return Case(case.name + "_conjg", s, case.grid, case.grid_dat, case.grid_bin, case.fields, time=case.time,
                dt=case.dt, ihist=case.ihist, m=case.m, ibm=ibm)


def with_poisson(case: Case, poisson: int, nlev: Optional[int] = None) -> Case:
    """The same case solved with another of the reference's Poisson solvers.
    For poiss_mgrd (x and z coarsened together) the default NLEV is the
    deepest with n1m and n3m divisible by 2^NLEV and at least two cells per
    direction on the coarsest level."""
    s = dict(case.settings)
    s["poisson"] = int(poisson)
    if nlev is None and poisson == abi.POISSON_MGRD:
        g = case.grid
        nlev = 0
        while nlev < 5 and all(n % (2 ** (nlev + 1)) == 0 and n // (2 ** (nlev + 1)) >= 2 for n in (g.n1m, g.n3m)):
            nlev += 1
    if nlev is not None:
        s["nlev"] = int(nlev)
    return Case(case.name + f"_p{poisson}", s, case.grid, case.grid_dat, case.grid_bin, case.fields, time=case.time,
                dt=case.dt, ihist=case.ihist, m=case.m, ibm=case.ibm)


PRESETS = {
    "channel64": lambda **kw: channel(64, 64, 64, **kw),
    "channel590": lambda **kw: channel(384, 256, 384, lx=2 * math.pi, lz=math.pi, re=10950.0, **kw),
    "cylinder100": lambda **kw: cylinder(128, 96, 16, re=100.0, **kw),
    "cylinder3900": lambda **kw: cylinder(256, 192, 64, re=3900.0, **kw),
}
