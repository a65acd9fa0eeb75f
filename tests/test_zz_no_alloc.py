"""The allocation-free Poisson entry point against the case-based solve.

lesgpu_poisson_ftft_noalloc serves callers that cannot call cudaMalloc (a
runtime with its own pre-sized device pool, a real-time loop that must stay
out of the driver's allocator, a plugin that must not bypass its host's
allocator): it keeps the solver's temporaries in a fixed device array and
works on buffers the caller already owns.  Two calls in a row, with
different right-hand sides, must each reproduce the case-based solve
(lesgpu_run_phase POISSON) within the Poisson parity tolerance; the second
call also shows that the shared array's leftover contents do not leak into a
new solve.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _interior(a, g):
    return a[1:g.n3m + 1, 1:g.n2m + 1, 1:g.n1m + 1]


def test_noalloc_poisson_matches_case_solve():
    torch = pytest.importorskip("torch")
    lib = leswht_gb300.load_library()
    fn = lib.lesgpu_poisson_ftft_noalloc
    fn.argtypes = [C.POINTER(abi.Grid), C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int

    case = cases.channel(32, 32, 16)
    g = case.grid
    solver = leswht_gb300.gpu_solver(case)
    grid = abi.pack_grid(g)
    rng = np.random.default_rng(20261203)
    for call in range(2):
        d = np.zeros(g.shape)
        d[1:g.n3m + 1, 1:g.n2m + 1, 1:g.n1m + 1] = rng.standard_normal((g.n3m, g.n2m, g.n1m))
        # the existing entry point
        solver.set(abi.F_DIVGSUM, d)
        solver.phase(abi.PH_POISSON)
        want = solver.get(abi.F_PHI)
        # the allocation-free one, on caller-owned device buffers
        dd = torch.from_numpy(d).cuda()
        phi = torch.full(g.shape, np.nan, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = fn(C.byref(grid.struct), C.c_void_p(dd.data_ptr()), C.c_void_p(phi.data_ptr()), C.c_void_p(stream))
        assert rc == 0, lib.lesgpu_strerror(rc)
        torch.cuda.synchronize()
        got = phi.cpu().numpy()
        a, b = _interior(got, g), _interior(want, g)
        assert np.all(np.isfinite(a))
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err <= TOL, (call, err)


def test_noalloc_rejects_grid_beyond_its_scratch():
    lib = leswht_gb300.load_library()
    fn = lib.lesgpu_poisson_ftft_noalloc
    fn.argtypes = [C.POINTER(abi.Grid), C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    case = cases.channel(16, 16, 8)
    grid = abi.pack_grid(case.grid)
    # claim a 2048 x 16 x 8 grid: refused on the size check, before any device work
    grid.struct.n1m, grid.struct.n1 = 2048, 2049
    rc = fn(C.byref(grid.struct), C.c_void_p(8), C.c_void_p(8), None)
    assert rc == abi.ERR_TOO_LARGE
    assert b"fixed scratch" in lib.lesgpu_strerror(rc)
