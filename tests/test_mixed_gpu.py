"""The mixed-precision form (FP32 stencils, SGS and x/z ADI sweeps, FP32
multigrid cycles; FP64 y sweeps, FFT Poisson, multigrid residual / defect
correction / coarsest level, projection, flow-rate and divergence) against the
FP64 form on the same case.

Stated error bounds (relative L2 of each field against the FP64 form): u, v,
w, t within 1e-5 after one step and 1e-4 after ten on the channel; the
pressure, which the projection builds from small differences of the FP32
right-hand sides, within 1e-3; divergence after projection below 1e-6 (the
Poisson solve and projection stay FP64).
"""
import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases

pytestmark = pytest.mark.gpu


def rel(a, b):
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def pair(builder):
    f64 = builder(abi.PREC_FP64)
    mix = builder(abi.PREC_MIXED)
    return leswht_gb300.gpu_solver(f64), leswht_gb300.gpu_solver(mix)


@pytest.mark.parametrize("nsteps,tol", [(1, 1e-5), (10, 1e-4)])
def test_channel_mixed_close_to_fp64(nsteps, tol):
    a, b = pair(lambda prec: cases.channel(32, 32, 16, precision=prec))
    for _ in range(nsteps):
        ra, rb = a.step(), b.step()
    fa, fb = a.fields(), b.fields()
    for k in ("u", "v", "w", "p", "t"):
        e = rel(fb[k], fa[k])
        assert e <= (1e-3 if k == "p" else tol), (k, e)
        assert e > 0.0 or k == "p", k            # the mixed path really differs
    assert rb["dvmax"] < 1e-6
    assert rb["csgsts"] == pytest.approx(ra["csgsts"], rel=1e-3)


def test_cylinder_mixed_close_to_fp64():
    a, b = pair(lambda prec: cases.cylinder(64, 48, 8, precision=prec))
    for _ in range(3):
        ra, rb = a.step(), b.step()
    fa, fb = a.fields(), b.fields()
    for k in ("u", "v", "w", "t"):
        assert rel(fb[k], fa[k]) <= 1e-4, k
    assert rb["dvmax"] < 1e-5
    assert rb["cd"][0] == pytest.approx(ra["cd"][0], rel=1e-3, abs=1e-6)


def test_mixed_is_deterministic():
    x = leswht_gb300.gpu_solver(cases.channel(32, 32, 16, precision=abi.PREC_MIXED))
    y = leswht_gb300.gpu_solver(cases.channel(32, 32, 16, precision=abi.PREC_MIXED))
    for _ in range(3):
        x.step(); y.step()
    fx, fy = x.fields(), y.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert np.array_equal(fx[k], fy[k]), k


@pytest.mark.parametrize("build", [
    lambda prec: cases.cylinder(64, 48, 8, precision=prec),                                   # poiss_z_ft
    lambda prec: cases.with_poisson(cases.channel(32, 32, 16, zwalls=True, precision=prec),   # poiss_x_ft
                                    abi.POISSON_X_FT, nlev=3),
])
def test_fp32_multigrid_meets_the_fp64_test(build):
    """The mixed form's multigrid cycles run in FP32 under an FP64 defect
    correction: on the same divergence and a tight RESID1 it stops on the same
    FP64 residual test, and phi matches the FP64 form's to 1e-8 relative."""
    ca, cb = build(abi.PREC_FP64), build(abi.PREC_MIXED)
    for c in (ca, cb):
        c.settings.update(resid1=1e-10, mgitr=2000)
    a, b = leswht_gb300.gpu_solver(ca), leswht_gb300.gpu_solver(cb)
    for s in (a, b):
        s.phase(abi.PH_STEPINIT)
        s.phase(abi.PH_SUBSTEPINIT, 1)
    a.phase(abi.PH_SGS, 1)
    a.phase(abi.PH_RHSNLHS, 1)
    a.phase(abi.PH_DIVGS, 1)
    b.set(abi.F_DIVGSUM, a.get(abi.F_DIVGSUM))
    for s in (a, b):
        s.phase(abi.PH_POISSON, 1)
    ia, ib = a.report()["poisson_iters"][0], b.report()["poisson_iters"][0]
    assert 1 <= ia < 2000 and 1 <= ib < 2000 and abs(ia - ib) <= max(2, ia // 5)
    assert rel(b.get(abi.F_PHI), a.get(abi.F_PHI)) <= 1e-8



def test_fp32_fft_with_fp64_correction_matches_fp64_transforms(monkeypatch):
    """poiss_ftft in the mixed form: FP32 transforms under the FP64 defect
    correction give the FP64 transforms' phi to 1e-10 relative, up to the
    constant (which the 7-point operator does not see)."""
    c = cases.channel(64, 32, 32, precision=abi.PREC_MIXED)
    solvers = []
    for forced in ("0", "1"):
        monkeypatch.setenv("LESGPU_FFT_MIXED", forced)
        s = leswht_gb300.gpu_solver(c)
        assert [w for d, nc, f32, w in leswht_gb300.tuning(s.lib, s.h) if d == 5] == [int(forced)]
        solvers.append(s)
    a, b = solvers
    for s in (a, b):
        s.phase(abi.PH_STEPINIT)
        s.phase(abi.PH_SUBSTEPINIT, 1)
    a.phase(abi.PH_SGS, 1)
    a.phase(abi.PH_RHSNLHS, 1)
    a.phase(abi.PH_DIVGS, 1)
    b.set(abi.F_DIVGSUM, a.get(abi.F_DIVGSUM))
    for s in (a, b):
        s.phase(abi.PH_POISSON, 1)
    g = c.grid
    sl = np.s_[1:g.n3m + 1, 1:g.n2m + 1, 1:g.n1m + 1]
    pa, pb = a.get(abi.F_PHI)[sl], b.get(abi.F_PHI)[sl]
    pa, pb = pa - pa.mean(), pb - pb.mean()
    assert rel(pb, pa) <= 1e-10
