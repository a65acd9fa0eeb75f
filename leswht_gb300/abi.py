"""ctypes mirror of include/lesgpu.h.

The structs here are byte-for-byte the C structs of the library ABI; both the
GPU library (liblesgpu.so) and any other implementation of the same ABI take
them.  `pack_*` helpers build them from numpy arrays and keep the arrays
alive for as long as the returned holder object lives.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional

import numpy as np

i64 = C.c_int64
f64 = C.c_double
PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int64)

# ---- constants (lesgpu.h) ------------------------------------------------
OK = 0
ERR_ARG, ERR_CONFIG, ERR_CUDA, ERR_OOM, ERR_NOT_CONVERGED, ERR_NAN, ERR_STATE, ERR_UNSUPPORTED = (
    -1, -2, -3, -4, -5, -6, -7, -8)
ERR_TOO_LARGE = -9
ERR_NAMES = {0: "OK", -1: "ERR_ARG", -2: "ERR_CONFIG", -3: "ERR_CUDA", -4: "ERR_OOM",
             -5: "ERR_NOT_CONVERGED", -6: "ERR_NAN", -7: "ERR_STATE", -8: "ERR_UNSUPPORTED",
             -9: "ERR_TOO_LARGE"}

POISSON_FTFT, POISSON_Z_FT, POISSON_MGRD, POISSON_X_FT = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1
BODY_NONE, BODY_CHANNEL, BODY_CYLINDER, BODY_SPHERE, BODY_SQUARE = 0, 1, 2, 3, 4

F_U, F_V, F_W, F_P, F_T = 0, 1, 2, 3, 4
F_NUSGS, F_NUSGS1, F_ALSGS, F_ALSGS1 = 5, 6, 7, 8
F_RHS1, F_RK3O, F_RK3OO, F_DIVGSUM, F_PHI, F_QMASS = 9, 10, 11, 12, 13, 14
FIELD_NCOMP = {F_NUSGS1: 3, F_ALSGS1: 3, F_RHS1: 4, F_RK3O: 4, F_RK3OO: 4}

NAVG = 23          # field_avg arrays (21 without temperature)
AVG_NAMES = ["uavg", "vavg", "wavg", "uu", "uv", "uw", "vv", "vw", "ww", "pavg", "p2avg",
             "wxavg", "wyavg", "wzavg", "wxwx", "wxwy", "wxwz", "wywy", "wywz", "wzwz", "ssavg",
             "tavg", "t2avg"]

PH_SUBSTEPINIT, PH_SGS, PH_RHSNLHS, PH_DIVGS, PH_POISSON, PH_UCALC, PH_MEANPG, PH_ENERGY, PH_STEPINIT = range(9)


class Body(C.Structure):
    _fields_ = [("kind", i64), ("cx", f64), ("cy", f64), ("cz", f64), ("r", f64), ("p0", f64)]


_CONFIG_FIELDS = [
    ("re", f64), ("pr", f64), ("gr", f64), ("grdir", i64), ("tflu_i", f64), ("tsol_i", f64),
    ("ireset", i64), ("iread", i64), ("iavg", i64), ("ipzero", i64), ("eps_ptr", f64), ("udrv_i", f64),
    ("nend", i64), ("nprint", i64), ("npriavg", i64), ("npin", i64),
    ("tend", f64), ("ptb_tst", f64), ("avg_tst", f64),
    ("idtopt", i64), ("dt_size", f64), ("cflfac", f64),
    ("resid1", f64), ("nlev", i64), ("nbli", i64), ("ioldv", i64), ("mgitr", i64), ("imgsor", i64),
    ("wwsor", f64),
    ("iles", i64), ("insmdl", i64), ("itemdl", i64), ("idvmon", i64), ("csgsts", f64), ("csgshf", f64),
    ("filter", i64),
    ("ibmon", i64), ("masson", i64), ("imovingon", i64), ("ihtrans", i64), ("idecomp", i64),
    ("bc_ybtm", i64), ("bc_ytop", i64), ("bc_zbtm", i64), ("bc_ztop", i64),
    ("bc_t_ybtm", i64), ("bc_t_ytop", i64), ("val_t_ybtm", f64), ("val_t_ytop", f64),
    ("bc_t_zbtm", i64), ("bc_t_ztop", i64), ("val_t_zbtm", f64), ("val_t_ztop", f64),
    ("ich", i64), ("iconjg", i64),
    ("xprdic", i64), ("yprdic", i64), ("zprdic", i64), ("iintp", i64),
    ("poisson", i64), ("precision", i64), ("body", Body),
]


class Config(C.Structure):
    _fields_ = _CONFIG_FIELDS

    def as_dict(self) -> Dict[str, Any]:
        d = {}
        for name, typ in _CONFIG_FIELDS:
            v = getattr(self, name)
            if name == "body":
                v = {k: getattr(v, k) for k, _ in Body._fields_}
            d[name] = v
        return d


_GRID_PTRS_D = ["x", "y", "z"]
_GRID_PTRS_I = ["ipv", "jpv", "kpv", "imv", "jmv", "kmv", "fixil", "fixjl", "fixkl", "fixiu", "fixju", "fixku"]
_GRID_PTRS_D0 = ["c2cx", "c2cy", "c2cz", "c2cxi", "c2cyi", "c2czi", "f2fx", "f2fy", "f2fz",
                 "f2fxi", "f2fyi", "f2fzi", "xmp", "ymp", "zmp"]


class Grid(C.Structure):
    _fields_ = ([("n1", i64), ("n2", i64), ("n3", i64), ("n1m", i64), ("n2m", i64), ("n3m", i64),
                 ("xl", f64), ("yl", f64), ("zl", f64)]
                + [(n, PD) for n in _GRID_PTRS_D]
                + [(n, PI) for n in _GRID_PTRS_I]
                + [(n, PD) for n in _GRID_PTRS_D0])


class Ibm(C.Structure):
    _fields_ = [("nintp", i64 * 4), ("nbody", i64 * 4), ("fc", PI * 4), ("intpindx", PI * 4),
                ("geomfac", PD * 4), ("nzero", i64), ("inz", PI), ("jnz", PI), ("knz", PI),
                ("nwall_dvm", PI), ("cstar", PD), ("kstar", PD), ("omega", PI)]


class StepReport(C.Structure):
    _fields_ = [("ntime", i64), ("ihist", i64), ("m", i64), ("time", f64), ("dt", f64),
                ("cflmax", f64), ("dvmax", f64), ("qmmax", f64), ("pmi", f64 * 5), ("pmiavg", f64),
                ("qvol", f64 * 3), ("tvol", f64 * 3), ("csgsts", f64), ("csgshf", f64),
                ("nutavg", f64), ("nutmax", f64), ("alpavg", f64), ("alpmax", f64),
                ("cd", f64 * 3), ("heat_flux", f64 * 3), ("ubulk", f64),
                ("tbulk_fluid", f64), ("tbulk_solid", f64), ("poisson_iters", i64 * 3),
                ("phase_ms", f64 * 4), ("qflux", f64), ("poisson_unconverged", i64), ("heat_body", f64)]

    def as_dict(self) -> Dict[str, Any]:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if hasattr(v, "__len__"):
                v = list(v)
            out[name] = v
        return out


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(PD)


def _iptr(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(PI)


@dataclass
class Packed:
    """A ctypes struct plus the numpy arrays it points into."""
    struct: Any
    keep: List[np.ndarray] = field(default_factory=list)


def pack_grid(g) -> Packed:
    """g: a gridgen.GridMetrics (or anything with the same attributes)."""
    keep = []
    s = Grid()
    s.n1, s.n2, s.n3 = g.n1, g.n2, g.n3
    s.n1m, s.n2m, s.n3m = g.n1m, g.n2m, g.n3m
    s.xl, s.yl, s.zl = g.xl, g.yl, g.zl
    for n in _GRID_PTRS_D + _GRID_PTRS_D0:
        a = np.ascontiguousarray(getattr(g, n), dtype=np.float64)
        keep.append(a)
        setattr(s, n, _dptr(a))
    for n in _GRID_PTRS_I:
        a = np.ascontiguousarray(getattr(g, n), dtype=np.int64)
        keep.append(a)
        setattr(s, n, _iptr(a))
    return Packed(s, keep)


def pack_config(d: Dict[str, Any]) -> Config:
    c = Config()
    for name, _ in _CONFIG_FIELDS:
        if name == "body":
            b = d.get("body", {})
            for k, _t in Body._fields_:
                setattr(c.body, k, b.get(k, 0))
        else:
            setattr(c, name, d.get(name, 0))
    return c


def pack_ibm(t: Dict[str, Any], n1m: int, n2m: int, n3m: int) -> Packed:
    """t: dict with keys nintp[4], nbody[4], fc[l] (nbody,3), intpindx[l] (nintp,3),
    geomfac[l] (nintp,27), nzero, inz/jnz/knz, nwall (n3m,n2m,n1m) or None,
    cstar, kstar (6,n3m,n2m,n1m), omega — arrays in Fortran element order."""
    keep = []
    s = Ibm()
    for l in range(4):
        s.nintp[l] = int(t["nintp"][l])
        s.nbody[l] = int(t["nbody"][l])
        fc = np.ascontiguousarray(t["fc"][l], dtype=np.int64).reshape(-1)
        ix = np.ascontiguousarray(t["intpindx"][l], dtype=np.int64).reshape(-1)
        gf = np.ascontiguousarray(t["geomfac"][l], dtype=np.float64).reshape(-1)
        if fc.size == 0:
            fc = np.zeros(3, np.int64)
        if ix.size == 0:
            ix = np.zeros(3, np.int64)
        if gf.size == 0:
            gf = np.zeros(27, np.float64)
        keep += [fc, ix, gf]
        s.fc[l] = _iptr(fc)
        s.intpindx[l] = _iptr(ix)
        s.geomfac[l] = _dptr(gf)
    s.nzero = int(t.get("nzero", 0))
    for name in ("inz", "jnz", "knz"):
        a = np.ascontiguousarray(t.get(name, np.zeros(1, np.int64)), dtype=np.int64)
        if a.size == 0:
            a = np.zeros(1, np.int64)
        keep.append(a)
        setattr(s, name, _iptr(a))
    for name, dt in (("nwall_dvm", np.int64), ("cstar", np.float64), ("kstar", np.float64), ("omega", np.int64)):
        a = t.get(name)
        if a is None:
            setattr(s, name, None)
            continue
        a = np.ascontiguousarray(a, dtype=dt).reshape(-1)
        keep.append(a)
        setattr(s, name, _dptr(a) if dt == np.float64 else _iptr(a))
    return Packed(s, keep)


def declare_api(lib, prefix: str, case_type=C.c_void_p) -> None:
    """Attach argtypes/restype to the lesgpu_* style entry points of `lib`."""
    P = C.POINTER(case_type)
    sig = {
        "create": ([C.POINTER(Config), C.POINTER(Grid), P], C.c_int),
        "load_ibm": ([case_type, C.POINTER(Ibm)], C.c_int),
        "set_fields": ([case_type, PD, PD, PD, PD, PD, f64, f64, i64, i64], C.c_int),
        "start": ([case_type], C.c_int),
        "step": ([case_type, C.POINTER(StepReport)], C.c_int),
        "get_fields": ([case_type, PD, PD, PD, PD, PD], C.c_int),
        "get_array": ([case_type, i64, PD], C.c_int),
        "set_array": ([case_type, i64, PD], C.c_int),
        "run_phase": ([case_type, i64, i64], C.c_int),
        "get_report": ([case_type, C.POINTER(StepReport)], C.c_int),
        "get_averages": ([case_type, PD, PI, C.c_int], C.c_int),
        "destroy": ([case_type], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, prefix + name)
        fn.argtypes = args
        fn.restype = res
