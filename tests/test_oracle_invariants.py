"""Invariants that pin the CPU oracle where the reference ships no outputs:
FFT against numpy, tridiagonal residuals, the discrete divergence after the
direct (FFT) projection, periodic ghost consistency and determinism."""
import ctypes as C

import numpy as np
import pytest

from leswht_gb300 import abi, cases, solver

PD = C.POINTER(C.c_double)


@pytest.mark.parametrize("n", [2, 3, 5, 8, 12, 16, 30, 48, 64, 96, 128, 384])
def test_fft_matches_numpy(oracle_lib, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    buf = np.empty(2 * n)
    buf[0::2], buf[1::2] = x.real, x.imag
    out = np.empty(2 * n)
    assert oracle_lib.ref_fft_1d(n, buf.ctypes.data_as(PD), out.ctypes.data_as(PD), -1) == 0
    y = out[0::2] + 1j * out[1::2]
    ref = np.fft.fft(x)
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))
    assert oracle_lib.ref_fft_1d(n, out.ctypes.data_as(PD), buf.ctypes.data_as(PD), 1) == 0
    z = buf[0::2] + 1j * buf[1::2]
    assert np.max(np.abs(z - x)) <= 1e-14 * n


@pytest.mark.parametrize("periodic", [0, 1])
@pytest.mark.parametrize("n", [3, 17, 64, 257])
def test_thomas_residual(oracle_lib, n, periodic):
    rng = np.random.default_rng(n + 7 * periodic)
    a = -rng.random(n)
    c = -rng.random(n)
    b = 2.5 + rng.random(n)
    r = rng.standard_normal(n)
    x = np.empty(n)
    assert oracle_lib.ref_thomas(n, a.ctypes.data_as(PD), b.ctypes.data_as(PD), c.ctypes.data_as(PD),
                                 r.ctypes.data_as(PD), x.ctypes.data_as(PD), periodic) == 0
    res = b * x
    res[1:] += a[1:] * x[:-1]
    res[:-1] += c[:-1] * x[1:]
    if periodic:
        res[0] += a[0] * x[-1]
        res[-1] += c[-1] * x[0]
    assert np.max(np.abs(res - r)) <= 1e-13 * np.max(np.abs(r))


@pytest.fixture(scope="module")
def stepped(oracle_lib):
    c = cases.channel(16, 16, 8)
    s = solver.Solver(oracle_lib, "ref_", c)
    reps = [s.step() for _ in range(3)]
    return c, s, reps


def test_projection_is_divergence_free(stepped):
    c, s, reps = stepped
    for r in reps:
        assert r["dvmax"] < 1e-11           # poiss_ftft is a direct solve


def test_periodic_ghosts_consistent(stepped):
    c, s, _ = stepped
    g = c.grid
    f = s.fields()
    for k in ("u", "w", "t"):
        a = f[k]
        np.testing.assert_array_equal(a[1:g.n3m + 1, 1:g.n2m + 1, 0], a[1:g.n3m + 1, 1:g.n2m + 1, g.n1m])
        np.testing.assert_array_equal(a[1:g.n3m + 1, 1:g.n2m + 1, g.n1], a[1:g.n3m + 1, 1:g.n2m + 1, 1])
        np.testing.assert_array_equal(a[0, 1:g.n2m + 1, 1:g.n1m + 1], a[g.n3m, 1:g.n2m + 1, 1:g.n1m + 1])


def test_flow_rate_controller_tracks_target(stepped):
    _, _, reps = stepped
    assert abs(reps[-1]["ubulk"] - 1.0) < 1e-2
    assert reps[-1]["csgsts"] >= 0.0 and reps[-1]["csgshf"] >= 0.0


def test_oracle_repeatable(oracle_lib):
    """OpenMP reductions combine thread partials in arrival order (as the
    reference's do), so repeated runs agree to rounding, not bit for bit."""
    c = cases.channel(16, 16, 8)
    outs = []
    for _ in range(2):
        s = solver.Solver(oracle_lib, "ref_", c)
        s.step()
        outs.append(s.fields())
    for k in outs[0]:
        a, b = outs[0][k], outs[1][k]
        assert np.linalg.norm(a - b) <= 1e-11 * max(np.linalg.norm(a), 1e-300)


def test_poisson_residual(oracle_lib):
    """phi solves the discrete Poisson operator of poiss_ftft (x, z spectral
    second differences, y three-point) up to the pinned null mode."""
    c = cases.channel(16, 16, 8)
    s = solver.Solver(oracle_lib, "ref_", c)
    g = c.grid
    rng = np.random.default_rng(3)
    d = np.zeros(g.shape)
    inner = (slice(1, g.n3m + 1), slice(1, g.n2m + 1), slice(1, g.n1m + 1))
    d[inner] = rng.standard_normal((g.n3m, g.n2m, g.n1m))
    d[inner] -= np.sum(d[inner] * g.f2fy[1:g.n2m + 1][None, :, None]) / np.sum(
        np.ones_like(d[inner]) * g.f2fy[1:g.n2m + 1][None, :, None])
    s.set(abi.F_DIVGSUM, d)
    s.phase(abi.PH_POISSON)
    phi = s.get(abi.F_PHI)[inner]
    # apply the operator: x/z periodic second differences, y Neumann walls
    dx2 = g.f2fxi[1] ** 2
    dz2 = g.f2fzi[1] ** 2
    lap = (np.roll(phi, 1, 2) - 2 * phi + np.roll(phi, -1, 2)) * dx2
    lap += (np.roll(phi, 1, 0) - 2 * phi + np.roll(phi, -1, 0)) * dz2
    j = np.arange(1, g.n2m + 1)
    fy = g.f2fyi[j][None, :, None]
    up = np.zeros_like(phi); up[:, :-1, :] = (phi[:, 1:, :] - phi[:, :-1, :]) * g.c2cyi[j[:-1] + 1][None, :, None]
    dn = np.zeros_like(phi); dn[:, 1:, :] = (phi[:, 1:, :] - phi[:, :-1, :]) * g.c2cyi[j[1:]][None, :, None]
    lap += (up - dn) * fy
    res = lap - d[inner]
    scale = np.max(np.abs(d[inner]))
    # poiss_ftft pins the (k=1,i=1) mode: its last y equation is replaced and
    # phi(n2m) of that mode is reset to 0 after the shift
    # (poiss_ftft.f90:93-112), so the residual is a plane constant on the top
    # two rows and zero everywhere else
    pm = res.mean(axis=(0, 2), keepdims=True)
    assert np.max(np.abs(res - pm)) < 1e-11 * scale
    assert np.max(np.abs(pm[:, :-2, :])) < 1e-11 * scale
