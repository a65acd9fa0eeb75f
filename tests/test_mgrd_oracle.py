"""The oracle's poiss_mgrd (BiCGSTAB + MG3D) restatement, pinned without a
GPU: it solves the same discrete system as the oracle's direct FFT solver
(poiss_ftft) and its multigrid solver (poiss_z_ft), and it rejects the
configurations it does not reproduce."""
import numpy as np
import pytest

from leswht_gb300 import abi, cases, solver


def phi_after_divergence(lib, case):
    s = solver.Solver(lib, "ref_", case)
    for ph, m in ((abi.PH_STEPINIT, 1), (abi.PH_SUBSTEPINIT, 1), (abi.PH_SGS, 1), (abi.PH_RHSNLHS, 1),
                  (abi.PH_DIVGS, 1), (abi.PH_POISSON, 1)):
        s.phase(ph, m)
    return s.get(abi.F_PHI), s.report()["poisson_iters"][0]


@pytest.mark.parametrize("build, other, tol", [(lambda: cases.channel(16, 16, 8), abi.POISSON_FTFT, 1e-13),
                                               (lambda: cases.cylinder(32, 24, 4, nlev=2), abi.POISSON_Z_FT, 1e-10)])
def test_same_solution_as_the_other_solvers(oracle_lib, build, other, tol):
    ref = cases.with_poisson(build(), other)
    ref.settings.update(resid1=tol, mgitr=2000)
    m = cases.with_poisson(build(), abi.POISSON_MGRD)
    m.settings.update(resid1=tol)
    pr, _ = phi_after_divergence(oracle_lib, ref)
    pm, it = phi_after_divergence(oracle_lib, m)
    g = ref.grid
    sl = np.s_[1:g.n3m + 1, 1:g.n2m + 1, 1:g.n1m + 1]
    a = pr[sl] - pr[1, g.n2m, 1]
    b = pm[sl] - pm[1, g.n2m, 1]
    assert 1 <= it < m.settings["mgitr"]
    assert np.abs(a - b).max() <= 1e-8 * np.abs(a).max()


def test_residual_below_tolerance(oracle_lib):
    c = cases.with_poisson(cases.cylinder(32, 24, 4, nlev=2), abi.POISSON_MGRD)
    s = solver.Solver(oracle_lib, "ref_", c)
    for ph, m in ((abi.PH_STEPINIT, 1), (abi.PH_SUBSTEPINIT, 1), (abi.PH_SGS, 1), (abi.PH_RHSNLHS, 1), (abi.PH_DIVGS, 1)):
        s.phase(ph, m)
    b = s.get(abi.F_DIVGSUM)
    s.phase(abi.PH_POISSON, 1)
    assert s.report()["poisson_iters"][0] < c.settings["mgitr"]
    assert np.isfinite(s.get(abi.F_PHI)).all() and np.abs(b).max() > 0


@pytest.mark.parametrize("change, code", [(dict(nlev=4), abi.ERR_CONFIG),            # 8 cells in z: not divisible by 16
                                          (dict(yprdic=1, bc_ybtm=4, bc_ytop=4), abi.ERR_UNSUPPORTED)])
def test_rejected_configurations(oracle_lib, change, code):
    c = cases.with_poisson(cases.channel(16, 16, 8), abi.POISSON_MGRD)
    c.settings.update(change)
    with pytest.raises(solver.LesError) as e:
        solver.Solver(oracle_lib, "ref_", c)
    assert e.value.code == code
