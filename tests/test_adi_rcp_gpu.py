"""The pivot reciprocal of the FP64 tridiagonal sweeps: Newton-Raphson
iteration from an FP32 seed built from the bit pattern, within 2 ulp of the
correctly rounded 1/x over the pivots the sweeps meet, and the plain
division outside the seed's exponent window."""
import ctypes as C

import numpy as np
import pytest

import leswht_gb300

pytestmark = pytest.mark.gpu


def test_reciprocal_within_two_ulp():
    lib = leswht_gb300.load_library()
    fn = lib.lesgpu_check_rcp
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
    fn.restype = C.c_int
    rng = np.random.default_rng(5)
    mag = 10.0 ** rng.uniform(-29.5, 29.5, 200000)
    x = mag * rng.choice([-1.0, 1.0], mag.size)
    x = np.concatenate([x, [1.0, -1.0, 3.0, 0.1, 1.0 / 3.0, 1e-40, -1e40, 1e-300, 1e300, 2.0 ** -126, 2.0 ** 127]])
    # both sides of the seed's exponent window [-99, 99]
    edge = [2.0 ** -99, np.nextafter(2.0 ** -99, 0.0), 2.0 ** -100, np.nextafter(2.0 ** 100, 0.0), 2.0 ** 100,
            1.9999999999999998 * 2.0 ** 99, 1.0000000000000002 * 2.0 ** -99]
    x = np.concatenate([x, edge, [-e for e in edge]])
    x = np.ascontiguousarray(x, dtype=np.float64)
    r = np.empty_like(x)
    assert fn(x.ctypes.data, r.ctypes.data, x.size) == 0
    exact = 1.0 / x
    assert np.all(np.abs(r - exact) <= 2.0 * np.spacing(np.abs(exact)))
