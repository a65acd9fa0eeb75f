"""Python host driver over the lesgpu C ABI.

`Solver` drives one case through an ABI-compatible shared library: the
sequence solver.f90:28-80 (create, load pre-processing tables, load the
initial field, start) followed by one lesgpu_step per time step.  Arrays
cross the boundary as numpy float64 arrays of shape (n3+1, n2+1, n1+1) in C
order, which is the Fortran (0:n1,0:n2,0:n3) layout byte for byte.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import abi


class LesError(RuntimeError):
    def __init__(self, where: str, code: int, msg: str = ""):
        super().__init__(f"{where} failed: {abi.ERR_NAMES.get(code, code)} {msg}".strip())
        self.code = code


class Solver:
    def __init__(self, lib: C.CDLL, prefix: str, case, *, load_fields: bool = True):
        self.lib = lib
        self.prefix = prefix
        self.case = case
        abi.declare_api(lib, prefix)
        self._strerror = getattr(lib, prefix + "strerror", None)
        if self._strerror is not None:
            self._strerror.restype = C.c_char_p
            self._strerror.argtypes = [C.c_int]
        self.cfg = abi.pack_config(case.settings)
        self.grid = abi.pack_grid(case.grid)
        self.h = C.c_void_p()
        self._call("create", C.byref(self.cfg), C.byref(self.grid.struct), C.byref(self.h))
        g = case.grid
        self.shape = g.shape
        self.nt = int(np.prod(self.shape))
        if case.ibm is not None:
            self.ibm = abi.pack_ibm(case.ibm, g.n1m, g.n2m, g.n3m)
            self._call("load_ibm", self.h, C.byref(self.ibm.struct))
        if load_fields:
            self.set_fields(case.fields, case.time, case.dt, case.ihist, case.m)
            self._call("start", self.h)

    # ------------------------------------------------------------------
    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def _call(self, name, *args):
        rc = self._fn(name)(*args)
        if rc != 0:
            msg = self._strerror(rc).decode() if self._strerror is not None else ""
            raise LesError(self.prefix + name, rc, msg)
        return rc

    def set_fields(self, f: Dict[str, np.ndarray], time: float, dt: float, ihist: int, m: int):
        arrs = [np.ascontiguousarray(f[k], dtype=np.float64) for k in ("u", "v", "w", "p")]
        t = f.get("t")
        t = np.ascontiguousarray(t, dtype=np.float64) if t is not None else None
        for a in arrs:
            assert a.shape == self.shape
        ptr = lambda a: a.ctypes.data_as(abi.PD) if a is not None else None
        self._call("set_fields", self.h, *(ptr(a) for a in arrs), ptr(t), float(time), float(dt),
                   int(ihist), int(m))

    def start(self):
        self._call("start", self.h)

    def step(self) -> Dict:
        rep = abi.StepReport()
        self._call("step", self.h, C.byref(rep))
        return rep.as_dict()

    def report(self) -> Dict:
        rep = abi.StepReport()
        self._call("get_report", self.h, C.byref(rep))
        return rep.as_dict()

    def fields(self) -> Dict[str, np.ndarray]:
        out = {k: np.empty(self.shape) for k in ("u", "v", "w", "p", "t")}
        self._call("get_fields", self.h, *(out[k].ctypes.data_as(abi.PD) for k in ("u", "v", "w", "p", "t")))
        return out

    def get(self, field: int) -> np.ndarray:
        nc = abi.FIELD_NCOMP.get(field, 1)
        out = np.empty((nc,) + self.shape) if nc > 1 else np.empty(self.shape)
        self._call("get_array", self.h, int(field), out.ctypes.data_as(abi.PD))
        return out

    def set(self, field: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._call("set_array", self.h, int(field), a.ctypes.data_as(abi.PD))

    def averages(self, reset: bool = False):
        """field_avg sums as {name: (n3m, n2m, n1m) array} and the sample count."""
        g = self.case.grid
        na = abi.NAVG if self.case.settings.get("ihtrans", 0) == 1 else abi.NAVG - 2
        out = np.empty((na, g.n3m, g.n2m, g.n1m))
        n = C.c_int64()
        self._call("get_averages", self.h, out.ctypes.data_as(abi.PD), C.byref(n), int(reset))
        return {abi.AVG_NAMES[a]: out[a] for a in range(na)}, n.value

    def phase(self, ph: int, msub: int = 1):
        self._call("run_phase", self.h, int(ph), int(msub))

    def close(self):
        if self.h:
            self._fn("destroy")(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
