"""GPU parity with conjugate heat transfer (ICONJG = 1): the cylinder
conducts heat, with c*, k* and the fluid mask omega from conjg_intp (solid
heat-capacity ratio 0.5, conductivity ratio 4), so rhs_t's face
conductivities, the energy ADI's c*/k* coefficients, the omega mask on the
convection terms and (constant flow rate) the c*-weighted temperature volume
all carry non-trivial values.  Tolerance: relative L2 <= 1e-10 per field
after one step."""
import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import cases, solver

pytestmark = pytest.mark.gpu


def rel(a, b):
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


@pytest.mark.parametrize("build", [lambda: cases.cylinder(64, 48, 8),          # open flow, ICH = 0
                                   lambda: cases.cylinder_array(48, 40, 8)])   # periodic row, ICH = 1
def test_one_step(oracle_lib, build):
    c = cases.with_conjugate(build(), 0.5, 4.0)
    om = np.asarray(c.ibm["omega"])
    assert c.settings["iconjg"] == 1 and 0 < int(om.sum()) < om.size
    g, r = leswht_gb300.gpu_solver(c), solver.Solver(oracle_lib, "ref_", c)
    rg, rr = g.step(), r.step()
    assert rg["poisson_iters"] == rr["poisson_iters"]
    fg, fr = g.fields(), r.fields()
    for k in ("u", "v", "w", "p", "t"):
        assert rel(fg[k], fr[k]) <= 1e-10, (k, rel(fg[k], fr[k]))
    assert rg["dvmax"] < 1e-5
