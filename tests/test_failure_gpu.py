"""Failure paths, injected on the host (no GPU fault is involved).

* An iterative Poisson solve that reaches MGITR above its tolerance: the
  reference prints a warning and goes on (poiss_z_ft.f90:289,
  poiss_mgrd.f90:204); the library does the same, counts the solves in the
  step report (equal to the oracle's count), and with lesgpu_set_strict the
  step returns LESGPU_ERR_NOT_CONVERGED after completing.
* A non-finite value seeded into a host array before lesgpu_set_fields:
  the next step reports LESGPU_ERR_NAN.
"""
import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases, solver

pytestmark = pytest.mark.gpu


def _starved(case, mgitr=1):
    case.settings.update(mgitr=mgitr, resid1=1e-30)
    return case


@pytest.mark.parametrize("poisson", [abi.POISSON_Z_FT, abi.POISSON_MGRD])
def test_iteration_limit_is_reported(oracle_lib, poisson):
    case = cases.cylinder(64, 48, 8)
    if poisson == abi.POISSON_MGRD:
        case = cases.with_poisson(case, abi.POISSON_MGRD)
    case = _starved(case)
    g = leswht_gb300.gpu_solver(case)
    r = solver.Solver(oracle_lib, "ref_", case)
    rg, rr = g.step(), r.step()
    assert rg["poisson_unconverged"] > 0
    assert rg["poisson_unconverged"] == rr["poisson_unconverged"]
    assert rg["poisson_iters"] == rr["poisson_iters"]
    g.close(); r.close()


def test_converged_solves_report_zero(oracle_lib):
    case = cases.cylinder(64, 48, 8)
    g = leswht_gb300.gpu_solver(case)
    rg = g.step()
    assert rg["poisson_unconverged"] == 0 and max(rg["poisson_iters"]) > 0
    g.close()


def test_strict_mode_returns_not_converged():
    case = _starved(cases.cylinder(64, 48, 8))
    g = leswht_gb300.gpu_solver(case)
    assert g.lib.lesgpu_set_strict(g.h, 1) == 0
    with pytest.raises(solver.LesError) as e:
        g.step()
    assert e.value.code == abi.ERR_NOT_CONVERGED
    rep = g.report()                        # the step completed; its report is there
    assert rep["ntime"] == 1 and rep["poisson_unconverged"] > 0
    assert g.lib.lesgpu_set_strict(g.h, 0) == 0
    g.step()                                # back to the reference's behaviour: no error
    g.close()


def test_nan_in_host_field_is_reported():
    case = cases.channel(32, 32, 16)
    u = case.fields["u"].copy()
    u[5, 7, 9] = np.nan
    case.fields["u"] = u
    g = leswht_gb300.gpu_solver(case)
    with pytest.raises(solver.LesError) as e:
        g.step()
    assert e.value.code == abi.ERR_NAN
    g.close()
