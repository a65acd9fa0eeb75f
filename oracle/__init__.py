"""ORACLE -- test infrastructure only.

CPU restatement (C11 + OpenMP) of the LESwHT per-time-step solver.  It is the
parity checker of the GPU library and the timed CPU baseline of bench.py;
nothing in the product package imports it.  Parity of this restatement with
the Fortran reference is unpinned by any reference output (the reference ships
no solver outputs and cannot be compiled here); see lesref_internal.h.

    import oracle
    lib = oracle.load()            # builds liblesref.so on first use
    s = leswht_gb300.solver.Solver(lib, "ref_", case)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SO = BUILD / "liblesref.so"
SOURCES = ["lesref_core.c", "lesref_mmtm.c", "lesref_sgs.c", "lesref_engy.c", "lesref_poiss.c"]
HEADERS = ["lesref_internal.h", "lesref.h", "../include/lesgpu.h"]


def _stale() -> bool:
    if not SO.exists():
        return True
    t = SO.stat().st_mtime
    return any((HERE / s).stat().st_mtime > t for s in SOURCES + HEADERS)


def build(force: bool = False) -> Path:
    """Compile liblesref.so with gcc (portable flags: runs on x86_64 and aarch64)."""
    if not force and not _stale():
        return SO
    BUILD.mkdir(exist_ok=True)
    tmp = SO.with_suffix(".so.tmp%d" % os.getpid())
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-Wall", "-Wno-unused-variable", "-Wno-unused-function",
           "-o", str(tmp)] + [str(HERE / s) for s in SOURCES] + ["-lm"]
    subprocess.run(cmd, check=True, cwd=HERE)
    os.replace(tmp, SO)
    return SO


_LIB = None


def load() -> C.CDLL:
    global _LIB
    if _LIB is None:
        build()
        _LIB = C.CDLL(str(SO))
        _LIB.ref_fft_1d.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
        _LIB.ref_fft_1d.restype = C.c_int
        _LIB.ref_thomas.argtypes = [C.c_int64] + [C.POINTER(C.c_double)] * 5 + [C.c_int]
        _LIB.ref_thomas.restype = C.c_int
    return _LIB
