"""The reference's on-disk formats, for cases built here.

* settings.input / boundary.input (read by readsettings / readbcs,
  misc_init.f90:19-92 and :95-158): a header line, then a line of values, per group;
* output/grid/grid.bin: the text file of gridgen.grid_bin_text;
* output/ibmpre/*.bin: the text tables of the pre-processor
  (lib_preprocessing.py:172-345): ibmpre_prdic, ibmpre_fcpts(_t),
  ibmpre_nutzero, ibmpre_wallfdvm, ibmpre_conjg, ibmpre_omega;
* output/field/fld%07d: Fortran unformatted sequential records (4-byte
  length markers before and after each record) in the order writefield
  (misc_hist.f90:212-252) writes and prefld (misc_init.f90:610-700) reads;
* output/field_avg/fav%07d-%07d: field_avg's records (misc_hist.f90:468-490).

`write_case_dir` lays out a case as 02_solver/ + output/ so the compiled
driver (lesgpu_exec) or the reference's solver_exec can run it.
"""
from __future__ import annotations

import os
import struct
from typing import Dict, List, Sequence

import numpy as np

from . import abi


# ------------------------------------------------------ Fortran records
def write_records(path: str, records: Sequence[bytes]) -> None:
    with open(path, "wb") as f:
        for r in records:
            n = struct.pack("<i", len(r))
            f.write(n); f.write(r); f.write(n)


def read_records(path: str) -> List[bytes]:
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        pos += 4
        out.append(data[pos:pos + n])
        pos += n
        (n2,) = struct.unpack_from("<i", data, pos)
        if n2 != n:
            raise ValueError(f"{path}: record markers {n} / {n2} differ")
        pos += 4
    return out


def _i8(*v) -> bytes:
    return np.asarray(v, dtype="<i8").tobytes()


def _f8(*v) -> bytes:
    return np.asarray(v, dtype="<f8").tobytes()


def _fort(a: np.ndarray) -> bytes:
    """A C-ordered (k, j, i) numpy block as the Fortran (i fastest) record."""
    return np.ascontiguousarray(a, dtype="<f8").tobytes()


def write_field(path: str, settings: Dict, g, fields: Dict[str, np.ndarray], ihist: int, m: int,
                time: float, dt: float) -> None:
    """writefield, misc_hist.f90:230-243."""
    n1, n2, n3, n1m, n2m, n3m = g.n1, g.n2, g.n3, g.n1m, g.n2m, g.n3m
    xp, yp, zp = (int(settings.get(k, 0)) for k in ("xprdic", "yprdic", "zprdic"))
    bcx = (4, 4) if xp == 1 else (2, 3)
    recs = [
        _i8(n1, n2, n3) + _f8(settings["re"], settings["pr"], settings["gr"]),
        _i8(ihist, m) + _f8(time, dt),
        _i8(xp, yp, zp),
        _i8(bcx[0], bcx[1], settings["bc_ybtm"], settings["bc_ytop"], settings["bc_zbtm"], settings["bc_ztop"]),
        _i8(settings["ich"], settings["iconjg"]),
        _fort(fields["u"][0:n3 + 1, 0:n2 + 1, 1:n1 + 1]),
        _fort(fields["v"][0:n3 + 1, 1:n2 + 1, 0:n1 + 1]),
        _fort(fields["w"][1:n3 + 1, 0:n2 + 1, 0:n1 + 1]),
        _fort(fields["p"][1:n3m + 1, 1:n2m + 1, 1:n1m + 1]),
    ]
    if settings.get("ihtrans", 0) == 1:
        recs.append(_fort(fields["t"][1:n3m + 1, 1:n2m + 1, 1:n1m + 1]))
    write_records(path, recs)


def read_field(path: str, g, ihtrans: int, tsol_i: float = 0.0) -> Dict:
    """prefld's read (misc_init.f90:622-645): arrays in the full layout,
    unread cells 0 (T: TSOL_I); the periodic ghost copies are the caller's."""
    r = read_records(path)
    n1, n2, n3 = np.frombuffer(r[0][:24], "<i8")
    if (n1, n2, n3) != (g.n1, g.n2, g.n3):
        raise ValueError("field does not match the grid")
    re, pr, gr = np.frombuffer(r[0][24:48], "<f8")
    ihist, m = np.frombuffer(r[1][:16], "<i8")
    time, dt = np.frombuffer(r[1][16:32], "<f8")
    sh = g.shape
    u = np.zeros(sh); v = np.zeros(sh); w = np.zeros(sh); p = np.zeros(sh)
    t = np.full(sh, float(tsol_i))
    u[0:n3 + 1, 0:n2 + 1, 1:n1 + 1] = np.frombuffer(r[5], "<f8").reshape(n3 + 1, n2 + 1, n1)
    v[0:n3 + 1, 1:n2 + 1, 0:n1 + 1] = np.frombuffer(r[6], "<f8").reshape(n3 + 1, n2, n1 + 1)
    w[1:n3 + 1, 0:n2 + 1, 0:n1 + 1] = np.frombuffer(r[7], "<f8").reshape(n3, n2 + 1, n1 + 1)
    p[1:g.n3m + 1, 1:g.n2m + 1, 1:g.n1m + 1] = np.frombuffer(r[8], "<f8").reshape(g.n3m, g.n2m, g.n1m)
    if ihtrans == 1:
        t[1:g.n3m + 1, 1:g.n2m + 1, 1:g.n1m + 1] = np.frombuffer(r[9], "<f8").reshape(g.n3m, g.n2m, g.n1m)
    return dict(u=u, v=v, w=w, p=p, t=t, ihist=int(ihist), m=int(m), time=float(time), dt=float(dt),
                re=float(re), pr=float(pr), gr=float(gr))


def read_fav(path: str, ihtrans: int) -> Dict:
    """The fav records of field_avg (misc_hist.f90:475-489)."""
    r = read_records(path)
    n1m, n2m, n3m = np.frombuffer(r[0][:24], "<i8")
    sh = (int(n3m), int(n2m), int(n1m))
    head = np.frombuffer(r[1], "<f8")
    out = {"n": (int(n1m), int(n2m), int(n3m)), "re": float(np.frombuffer(r[0][24:32], "<f8")[0]),
           "timeinit": head[0], "timeend": head[1], "ihistinit": head[2], "ihistend": head[3]}
    names = ["uavg", "vavg", "wavg", "uiujavg", "pavg", "p2avg", "voravg", "vor2avg", "ssavg"]
    counts = [1, 1, 1, 6, 1, 1, 3, 6, 1]
    if ihtrans == 1:
        names += ["tavg", "t2avg"]; counts += [1, 1]
    for q, (nm, c) in enumerate(zip(names, counts)):
        a = np.frombuffer(r[2 + q], "<f8")
        out[nm] = a.reshape((c,) + sh) if c > 1 else a.reshape(sh)
    return out


FAV_NAMES = ["uavg", "vavg", "wavg", "uiujavg", "pavg", "p2avg", "voravg", "vor2avg", "ssavg", "tavg", "t2avg"]
FAV_COUNTS = [1, 1, 1, 6, 1, 1, 3, 6, 1, 1, 1]


def write_fav(path: str, re: float, n: Sequence[int], sums: np.ndarray, timeinit: float, timeend: float,
              ihistinit: int, ihistend: int, ihtrans: int) -> None:
    """A fav file as field_avg writes it (misc_hist.f90:468-490) and the
    compiled driver's write_fav writes it: (n1m, n2m, n3m, re), the window
    (timeinit, timeend, ihistinit, ihistend as reals), then the dt-weighted
    sums, one record per group (u, v, w, uiuj(6), p, p2, vor(3), vorvor(6),
    ss, and t, t2 with heat transfer).  `sums` holds the LESGPU_NAVG (or
    LESGPU_NAVG - 2) arrays of n1m*n2m*n3m values in that order, i fastest."""
    n1m, n2m, n3m = (int(x) for x in n)
    ncell = n1m * n2m * n3m
    a = np.ascontiguousarray(sums, dtype="<f8").reshape(-1)
    ng = 11 if ihtrans == 1 else 9
    recs = [_i8(n1m, n2m, n3m) + _f8(re), _f8(timeinit, timeend, float(ihistinit), float(ihistend))]
    a0 = 0
    for q in range(ng):
        c = FAV_COUNTS[q]
        recs.append(a[a0 * ncell:(a0 + c) * ncell].tobytes())
        a0 += c
    if a0 * ncell != a.size:
        raise ValueError("fav sums do not match the grid and ihtrans")
    write_records(path, recs)


# ---------------------------------------------------------- text inputs
def _fmt(v) -> str:
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return repr(float(v))


def settings_text(s: Dict, gridfile: str, prev_fld: str) -> str:
    """settings.input in the layout readsettings reads (misc_init.f90:19-92)."""
    rows = [
        ("RE#     PR#     GR#     GRDIR   TFLU_I  TSOL_I", ["re", "pr", "gr", "grdir", "tflu_i", "tsol_i"]),
        ("IRESET  IREAD   IAVG    IPZERO  EPS_PTR UDRV_I", ["ireset", "iread", "iavg", "ipzero", "eps_ptr", "udrv_i"]),
        ("NEND    NPRINT  NPRIAVG NPIN", ["nend", "nprint", "npriavg", "npin"]),
        ("TEND    PTB_TST AVG_TST", ["tend", "ptb_tst", "avg_tst"]),
        ("IDTOPT  DT_SIZE CFLFAC", ["idtopt", "dt_size", "cflfac"]),
        ("RESID1  NLEV    NBLI    IOLDV   MGITR   IMGSOR  WWSOR", ["resid1", "nlev", "nbli", "ioldv", "mgitr", "imgsor", "wwsor"]),
        ("ILES    INSMDL  ITEMDL  IDVMON  CSGSTS  CSGSHF  FILTER", ["iles", "insmdl", "itemdl", "idvmon", "csgsts", "csgshf", "filter"]),
        ("IBMON   MASSON  IMOVING IHTRANS IDECOMP", ["ibmon", "masson", "imovingon", "ihtrans", "idecomp"]),
    ]
    ints = {"grdir", "ireset", "iread", "iavg", "ipzero", "nend", "nprint", "npriavg", "npin", "idtopt", "nlev",
            "nbli", "ioldv", "mgitr", "imgsor", "iles", "insmdl", "itemdl", "idvmon", "filter", "ibmon", "masson",
            "imovingon", "ihtrans", "idecomp"}
    out = []
    for head, keys in rows:
        out.append(head)
        out.append("  ".join(str(int(s[k])) if k in ints else repr(float(s[k])) for k in keys))
    out += ["FILES", f'"{gridfile}"', f'"{prev_fld}"', "TRACE   NTR", "0       1"]
    return "\n".join(out) + "\n"


def boundary_text(s: Dict) -> str:
    """boundary.input in the layout readbcs reads (misc_init.f90:95-158).
    A periodic direction is written as a wall; readbcs overrides it."""
    def bc(k, prd):
        return 0 if s.get(prd, 0) == 1 else int(s[k])
    lines = ["BC_YBTM    BC_YTOP", f"{bc('bc_ybtm', 'yprdic')} {bc('bc_ytop', 'yprdic')}",
             "BC_ZBTM    BC_ZTOP", f"{bc('bc_zbtm', 'zprdic')} {bc('bc_ztop', 'zprdic')}",
             "BC_T_YBTM  BC_T_YTOP", f"{int(s['bc_t_ybtm'])} {int(s['bc_t_ytop'])}",
             "VAL_T_YBTM VAL_T_YTOP", f"{float(s['val_t_ybtm'])!r} {float(s['val_t_ytop'])!r}",
             "BC_T_ZBTM  BC_T_ZTOP", f"{int(s['bc_t_zbtm'])} {int(s['bc_t_ztop'])}",
             "VAL_T_ZBTM VAL_T_ZTOP", f"{float(s['val_t_zbtm'])!r} {float(s['val_t_ztop'])!r}",
             "ICH        ICONJG", f"{int(s['ich'])} {int(s['iconjg'])}"]
    return "\n".join(lines) + "\n"


def write_ibmpre(dirpath: str, case) -> None:
    """The pre-processor's table files for `case` (lib_preprocessing.py:172-345)."""
    s, g, t = case.settings, case.grid, case.ibm
    os.makedirs(dirpath, exist_ok=True)
    with open(os.path.join(dirpath, "ibmpre_prdic.bin"), "w") as f:
        f.write("%d %d %d %d\n" % (s.get("xprdic", 0), s.get("yprdic", 0), s.get("zprdic", 0), s.get("iintp", 0)))
    nintp, nbody = list(t["nintp"]), list(t["nbody"])
    with open(os.path.join(dirpath, "ibmpre_fcpts.bin"), "w") as f:
        f.write("%d %d %d\n" % tuple(nintp[:3]))
        f.write("%d %d %d\n" % tuple(nbody[l] - nintp[l] for l in range(3)))
        for l in range(3):
            for r in np.asarray(t["fc"][l]).reshape(-1, 3):
                f.write("%d %d %d\n" % tuple(r))
        for l in range(3):
            for r in np.asarray(t["intpindx"][l]).reshape(-1, 3)[:nintp[l]]:
                f.write("%d %d %d\n" % tuple(r))
        for l in range(3):
            for r in np.asarray(t["geomfac"][l]).reshape(-1, 27)[:nintp[l]]:
                f.write("".join(" %15.8f " % v for v in r) + "\n")
    if s.get("ihtrans", 0) == 1:
        with open(os.path.join(dirpath, "ibmpre_fcpts_t.bin"), "w") as f:
            f.write("%d\n%d\n" % (nintp[3], nbody[3] - nintp[3]))
            for r in np.asarray(t["fc"][3]).reshape(-1, 3):
                f.write("%d %d %d\n" % tuple(r))
            for r in np.asarray(t["intpindx"][3]).reshape(-1, 3)[:nintp[3]]:
                f.write("%d %d %d\n" % tuple(r))
            for r in np.asarray(t["geomfac"][3]).reshape(-1, 27)[:nintp[3]]:
                f.write("".join(" %15.8f " % v for v in r) + "\n")
    ncell = g.n1m * g.n2m * g.n3m
    if s.get("iles", 0) == 1:
        nz = int(t.get("nzero", 0))
        with open(os.path.join(dirpath, "ibmpre_nutzero.bin"), "w") as f:
            f.write("%d \n" % nz)
            for key in ("inz", "jnz", "knz"):
                f.write("".join(" %d " % v for v in np.asarray(t[key])[:nz]) + "\n")
        nw = t.get("nwall_dvm")
        nw = np.ones(ncell, np.int64) if nw is None else np.asarray(nw)
        with open(os.path.join(dirpath, "ibmpre_wallfdvm.bin"), "w") as f:
            f.write("".join(" %d " % v for v in nw))
    if s.get("iconjg", 0) == 1:
        cs = t.get("cstar"); ks = t.get("kstar"); om = t.get("omega")
        cs = np.ones(ncell) if cs is None else np.asarray(cs)
        ks = np.ones(6 * ncell) if ks is None else np.asarray(ks)
        with open(os.path.join(dirpath, "ibmpre_conjg.bin"), "w") as f:
            f.write("".join(" %r " % float(v) for v in cs) + "\n")
            f.write("".join(" %r " % float(v) for v in ks))
        if om is not None:
            with open(os.path.join(dirpath, "ibmpre_omega.bin"), "w") as f:
                f.write("".join(" %d " % v for v in np.asarray(om)))


def write_case_dir(root: str, case, nend: int, nprint: int = 10 ** 6, npin: int = 1) -> str:
    """root/02_solver/{settings,boundary}.input + root/output/{grid,ibmpre,field,...}
    with the case's initial field as output/field/fld0000000 (IREAD = 1).
    Returns the solver directory (the working directory of a run)."""
    sdir = os.path.join(root, "02_solver")
    for d in (sdir, os.path.join(root, "output", "grid"), os.path.join(root, "output", "ibmpre"),
              os.path.join(root, "output", "field"), os.path.join(root, "output", "field_avg"),
              os.path.join(root, "output", "ftr")):
        os.makedirs(d, exist_ok=True)
    s = dict(case.settings)
    s.update(iread=1, ireset=0, nend=int(nend), nprint=int(nprint), npin=int(npin))
    with open(os.path.join(root, "output", "grid", "grid.bin"), "w") as f:
        f.write(case.grid_bin)
    write_ibmpre(os.path.join(root, "output", "ibmpre"), case)
    write_field(os.path.join(root, "output", "field", "fld0000000"), s, case.grid, case.fields,
                case.ihist, case.m, case.time, case.dt)
    with open(os.path.join(sdir, "settings.input"), "w") as f:
        f.write(settings_text(s, "../output/grid/grid.bin", "../output/field/fld0000000"))
    with open(os.path.join(sdir, "boundary.input"), "w") as f:
        f.write(boundary_text(s))
    with open(os.path.join(sdir, "body.input"), "w") as f:
        f.write(body_text(s))
    return sdir


def body_text(s: Dict) -> str:
    """body.input: the reference links its body function at compile time
    (geometry/funcbody.f90); the compiled driver of this library reads the
    body, the Poisson solver and the arithmetic form from this file instead."""
    b = s.get("body", {})
    return ("KIND CX CY CZ R P0 POISSON PRECISION\n"
            f"{int(b.get('kind', 0))} {float(b.get('cx', 0.0))!r} {float(b.get('cy', 0.0))!r} "
            f"{float(b.get('cz', 0.0))!r} {float(b.get('r', 0.5))!r} {float(b.get('p0', 0.0))!r} "
            f"{int(s.get('poisson', 0))} {int(s.get('precision', 0))}\n")
