"""The oracle's poiss_x_ft (FFT in x + z-semicoarsened multigrid per x mode)
restatement, pinned without a GPU: it solves the same discrete system as the
oracle's direct FFT solver (poiss_ftft) on a periodic channel and as its
BiCGSTAB + MG3D solver (poiss_mgrd) on a duct with walls in z, through the
multigrid modes and the zebra-SOR modes alike; the constant of the solution
is the one poiss_x_ft.f90:215-232 fixes; unsupported configurations are
rejected."""
import numpy as np
import pytest

from leswht_gb300 import abi, cases, solver


def phi_after_divergence(lib, case):
    s = solver.Solver(lib, "ref_", case)
    for ph, m in ((abi.PH_STEPINIT, 1), (abi.PH_SUBSTEPINIT, 1), (abi.PH_SGS, 1), (abi.PH_RHSNLHS, 1),
                  (abi.PH_DIVGS, 1), (abi.PH_POISSON, 1)):
        s.phase(ph, m)
    return s.get(abi.F_PHI), s.report()["poisson_iters"][0]


def _same_up_to_a_constant(pa, pb, g, rel):
    sl = np.s_[1:g.n3m + 1, 1:g.n2m + 1, 1:g.n1m + 1]
    a = pa[sl] - pa[1, g.n2m, 1]
    b = pb[sl] - pb[1, g.n2m, 1]
    assert np.abs(a - b).max() <= rel * np.abs(a).max()


@pytest.mark.parametrize("zwalls, other, imgsor", [(False, abi.POISSON_FTFT, 170),     # every mode by multigrid
                                                   (False, abi.POISSON_FTFT, 2),       # modes 3.. by zebra SOR
                                                   (True, abi.POISSON_MGRD, 170)])     # z walls: kpm/kmm not wrapped
def test_same_solution_as_the_other_solvers(oracle_lib, zwalls, other, imgsor):
    build = lambda: cases.channel(16, 16, 8, zwalls=zwalls)
    ref = cases.with_poisson(build(), other)
    ref.settings.update(resid1=1e-12, mgitr=3000)
    x = cases.with_poisson(build(), abi.POISSON_X_FT, nlev=2)
    x.settings.update(resid1=1e-12, mgitr=3000, imgsor=imgsor)
    pr, _ = phi_after_divergence(oracle_lib, ref)
    px, it = phi_after_divergence(oracle_lib, x)
    assert 1 <= it < 3000
    _same_up_to_a_constant(pr, px, x.grid, 1e-10)


def test_upper_wall_mean_is_zero(oracle_lib):
    """ICH = 1: the f2fx-weighted mean of phi(:, n2m, 1) is subtracted."""
    c = cases.with_poisson(cases.channel(16, 16, 8), abi.POISSON_X_FT, nlev=2)
    assert c.settings["ich"] == 1
    phi, _ = phi_after_divergence(oracle_lib, c)
    g = c.grid
    line = phi[1, g.n2m, 1:g.n1m + 1]
    assert abs((line * g.f2fx[1:g.n1m + 1]).sum()) <= 1e-13 * np.abs(line).sum() * g.f2fx[1:g.n1m + 1].max()


@pytest.mark.parametrize("build, change", [(lambda: cases.cylinder(32, 24, 4, nlev=2), {}),   # x not periodic
                                           (lambda: cases.channel(16, 16, 8), dict(nlev=4))])  # 8 z cells < 2^4
def test_rejected_configurations(oracle_lib, build, change):
    c = cases.with_poisson(build(), abi.POISSON_X_FT, nlev=2)
    c.settings.update(change)
    with pytest.raises(solver.LesError) as e:
        solver.Solver(oracle_lib, "ref_", c)
    assert e.value.code == abi.ERR_CONFIG
