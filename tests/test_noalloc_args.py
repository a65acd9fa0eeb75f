"""Argument checks of the allocation-free Poisson entry point.

lesgpu_poisson_ftft_noalloc serves callers that cannot allocate device
memory.  Its transforms assume a grid that is periodic and uniform in x and
z, and it reads every wall-normal table from host memory, so it must refuse
a grid that breaks either assumption, or lacks a table, before it touches
the GPU.  Each refusal here happens before any CUDA call, so these tests run
without a GPU.
"""
import ctypes as C

import numpy as np
import pytest

from leswht_gb300 import abi, cases


@pytest.fixture()
def fn(gpu_lib):
    f = gpu_lib.lesgpu_poisson_ftft_noalloc
    f.argtypes = [C.POINTER(abi.Grid), C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _call(fn, grid):
    # the device pointers are never dereferenced on these paths
    return fn(C.byref(grid.struct), C.c_void_p(256), C.c_void_p(512), None)


def test_rejects_null_buffers_and_grid(fn):
    grid = abi.pack_grid(cases.channel(16, 16, 8).grid)
    assert fn(None, C.c_void_p(256), C.c_void_p(512), None) == abi.ERR_ARG
    assert fn(C.byref(grid.struct), None, C.c_void_p(512), None) == abi.ERR_ARG
    assert fn(C.byref(grid.struct), C.c_void_p(256), None, None) == abi.ERR_ARG


@pytest.mark.parametrize("name", ["ipv", "kpv", "jpv", "fixjl", "fixju", "f2fxi", "f2fzi", "f2fyi", "c2cyi"])
def test_rejects_null_table(fn, name):
    grid = abi.pack_grid(cases.channel(16, 16, 8).grid)
    setattr(grid.struct, name, None)
    assert _call(fn, grid) == abi.ERR_ARG


def test_rejects_non_periodic_x(fn):
    # the open cylinder's x direction does not wrap: ipv(n1m) = n1m + 1
    g = cases.PRESETS["cylinder100"]().grid
    assert g.ipv[-1] != 1
    assert _call(fn, abi.pack_grid(g)) == abi.ERR_UNSUPPORTED


def test_rejects_non_periodic_z(fn):
    g = cases.channel(16, 16, 8).grid
    g.kpv = np.array(g.kpv, dtype=np.int64)
    g.kpv[-1] = g.n3m + 1
    assert _call(fn, abi.pack_grid(g)) == abi.ERR_UNSUPPORTED


@pytest.mark.parametrize("axis", ["f2fxi", "f2fzi"])
def test_rejects_stretched_periodic_direction(fn, axis):
    g = cases.channel(16, 16, 8).grid
    v = np.array(getattr(g, axis), dtype=np.float64)
    v[3] *= 1.01                      # one spacing 1 % off: not uniform
    setattr(g, axis, v)
    assert _call(fn, abi.pack_grid(g)) == abi.ERR_UNSUPPORTED


def test_accepts_six_decimal_spacing_noise(fn):
    # A uniform grid read back from its 6-decimal text may differ in the last
    # digit; that passes the uniformity check.  The grid is chosen too large
    # for the fixed scratch (512 x 256 x 64 needs about 100 MiB), so the call
    # then stops at the scratch-size check, still before any CUDA call.
    from leswht_gb300 import gridgen
    xs = [4.0 * np.pi * i / 512 for i in range(513)]
    ys = [-1.0 + 2.0 * j / 256 for j in range(257)]
    zs = [np.pi * k / 64 for k in range(65)]
    g, _, _ = gridgen.make_grid_lines(xs, ys, zs, xprdic=True, zprdic=True)
    v = np.array(g.f2fxi, dtype=np.float64)
    v[2] *= 1.0 + 4e-7
    g.f2fxi = v
    assert _call(fn, abi.pack_grid(g)) == abi.ERR_TOO_LARGE
