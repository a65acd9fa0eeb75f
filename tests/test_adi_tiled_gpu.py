"""The tiled FP32 tridiagonal sweep (lines staged in shared memory, one warp
per line) against the 32-lane warp-scan sweep it restructures: the same
chunks and recurrences, so the mixed form's velocity and pressure after a
few steps are bitwise equal whichever of the two runs the x and z sweeps --
on the periodic channel (periodic x and z lines) and on the open cylinder
(non-periodic x lines, periodic z lines).  The temperature sweep's
coefficients are formed as (1 + cre alpha) times the metric in the tiled
form and as the general conjugate expression with unit tables in the
warp-scan form, which the compiler may contract differently: t is held to
FP32 rounding (1e-6 relative)."""
import numpy as np
import pytest

import leswht_gb300
from leswht_gb300 import abi, cases

pytestmark = pytest.mark.gpu


def run(monkeypatch, case, form, steps=3):
    monkeypatch.setenv("LESGPU_ADI_FP32_FORM", str(form))
    s = leswht_gb300.gpu_solver(case)
    for _ in range(steps):
        s.step()
    f = s.fields()
    s.close()
    return f


@pytest.mark.parametrize("name", ["channel", "cylinder"])
def test_tiled_sweep_equals_warp_scan(monkeypatch, name):
    if name == "channel":
        case = cases.channel(32, 32, 16, precision=abi.PREC_MIXED)
    else:
        case = cases.cylinder(64, 48, 8, precision=abi.PREC_MIXED)
    a = run(monkeypatch, case, 32)
    b = run(monkeypatch, case, 128)
    for k in ("u", "v", "w", "p"):
        assert np.array_equal(a[k], b[k]), k
    d = np.linalg.norm(a["t"] - b["t"]) / np.linalg.norm(b["t"])
    assert d <= 1e-6, d
