"""GB300 (sm_103a) implementation of LESwHT's per-time-step solver hot path.

The compute path is liblesgpu.so (hand-written CUDA, C ABI in
include/lesgpu.h).  This package builds and loads it and provides the Python
host driver (`solver.Solver`), the grid/case generators and the file formats.

There is no CPU fallback: `load_library()` raises if the CUDA library cannot
be built or loaded.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import abi
from .build import EXEC, SO, build

_LIB = None


def load_library(rebuild: bool = False) -> C.CDLL:
    """Load liblesgpu.so (building it first if its sources are newer)."""
    global _LIB
    if _LIB is not None and not rebuild:
        return _LIB
    path = build(force=rebuild)
    if not Path(path).exists():
        raise RuntimeError(f"liblesgpu.so missing at {path}; the CUDA path is mandatory")
    lib = C.CDLL(str(path))
    abi.declare_api(lib, "lesgpu_")
    lib.lesgpu_step_async.argtypes = [C.c_void_p, C.c_int64]
    lib.lesgpu_step_async.restype = C.c_int
    lib.lesgpu_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    lib.lesgpu_stream.restype = C.c_int
    lib.lesgpu_use_graph.argtypes = [C.c_void_p, C.c_int]
    lib.lesgpu_use_graph.restype = C.c_int
    lib.lesgpu_strerror.argtypes = [C.c_int]
    lib.lesgpu_strerror.restype = C.c_char_p
    lib.lesgpu_abi_version.restype = C.c_int
    lib.lesgpu_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
    lib.lesgpu_launch_count.restype = C.c_int
    lib.lesgpu_tuning.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.c_int64, C.POINTER(C.c_int64)]
    lib.lesgpu_tuning.restype = C.c_int
    lib.lesgpu_instrument.argtypes = [C.c_void_p, C.c_int64]
    lib.lesgpu_instrument.restype = C.c_int
    lib.lesgpu_instrument_read.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.lesgpu_instrument_read.restype = C.c_int
    lib.lesgpu_set_device.argtypes = [C.c_int64]
    lib.lesgpu_set_device.restype = C.c_int
    _LIB = lib
    return lib


def tuning(lib, handle) -> list:
    """The autotuner's choices for a started case: [(dir, ncomp, fp32, lanes)]."""
    buf = (C.c_int64 * 256)()
    n = C.c_int64()
    if lib.lesgpu_tuning(handle, buf, 64, C.byref(n)) != 0:
        raise RuntimeError("lesgpu_tuning failed")
    return [tuple(buf[4 * q:4 * q + 4]) for q in range(min(n.value, 64))]


def exec_path(rebuild: bool = False) -> Path:
    """The compiled case driver (lesgpu_exec), built with the library."""
    build(force=rebuild)
    if not EXEC.exists():
        raise RuntimeError(f"lesgpu_exec missing at {EXEC}")
    return EXEC


def gpu_solver(case, **kw):
    """A Solver over liblesgpu.so for `case` (a cases.Case)."""
    from .solver import Solver
    return Solver(load_library(), "lesgpu_", case, **kw)
