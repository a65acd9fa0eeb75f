"""Statistics of a run: the quantities the mixed-precision form is judged by
against the FP64 form (mean and rms fields, drag, Strouhal and Nusselt
numbers).

The reference defines the time averages (field_avg, misc_hist.f90:287-527:
dt-weighted sums of u, v, w, u_i u_j, p, p^2, vorticity, S:S, T, T^2 at the
cell centres) and the drag history (draglift, slv_auxi.f90:666-840).  It
computes no Nusselt or Strouhal number; the definitions here are this
library's, applied identically to both forms:

* cylinder Nusselt number: the heat the thermal direct forcing adds to the
  fluid per unit time (step report `heat_body`, the thermal counterpart of
  draglift's force integral) over the body surface and the body-to-inflow
  temperature difference, in units of the conductive flux 1/(Re Pr):
  Nu = heat_body Re Pr / (pi D Lz dT);
* channel Nusselt number: twice the mean wall-normal temperature gradient at
  the walls (one-sided second order from the two first cell centres and the
  wall value) over the mixed-mean temperature's difference from the wall
  value, averaged over both walls;
* Strouhal number: the dominant frequency of the lift history times D / U,
  from a Hann-windowed, zero-padded periodogram of the history resampled to
  a uniform step, with parabolic interpolation of the peak.
"""
from __future__ import annotations

import math
from typing import Dict, Optional, Sequence

import numpy as np


def time_mean(times: Sequence[float], dts: Sequence[float], values: Sequence[float]) -> float:
    """dt-weighted mean of a per-step history."""
    d = np.asarray(dts, dtype=np.float64)
    v = np.asarray(values, dtype=np.float64)
    return float(np.sum(d * v) / np.sum(d))


def mean_and_rms(avg: Dict[str, np.ndarray], window: float) -> Dict[str, np.ndarray]:
    """Mean and rms fields from field_avg's dt-weighted sums over `window`
    time units: u, v, w, p (and t) means; u', v', w', p' (and t') rms."""
    out = {}
    for m in ("uavg", "vavg", "wavg", "pavg", "tavg"):
        if m in avg:
            out[m[0]] = avg[m] / window
    pairs = {"u": "uu", "v": "vv", "w": "ww"}
    for k, q in pairs.items():
        out[k + "_rms"] = np.sqrt(np.maximum(avg[q] / window - out[k] ** 2, 0.0))
    out["p_rms"] = np.sqrt(np.maximum(avg["p2avg"] / window - out["p"] ** 2, 0.0))
    if "t2avg" in avg:
        out["t_rms"] = np.sqrt(np.maximum(avg["t2avg"] / window - out["t"] ** 2, 0.0))
    return out


def plane_profile(a: np.ndarray) -> np.ndarray:
    """Mean over x and z of an (n3m, n2m, n1m) cell-centre array: a profile in y."""
    return a.mean(axis=(0, 2))


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    den = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (den if den > 0 else 1.0)


def channel_nusselt(tmean: np.ndarray, umean: np.ndarray, grid, t_wall: float = 0.0) -> float:
    """Nusselt number of a channel with isothermal walls at t_wall, from the
    mean temperature and streamwise velocity at the cell centres."""
    T = plane_profile(tmean)
    U = plane_profile(umean)
    ymp = np.asarray(grid.ymp, dtype=np.float64)
    y = np.asarray(grid.y, dtype=np.float64)
    f2fy = np.asarray(grid.f2fy, dtype=np.float64)
    n2m = grid.n2m
    wy = f2fy[1:n2m + 1]
    tm = float(np.sum(U * T * wy) / np.sum(U * wy))        # mixed-mean temperature

    def grad(t1, t2, d1, d2):       # derivative at the wall of the parabola through (0, t_wall), (d1, t1), (d2, t2)
        a1, a2 = t1 - t_wall, t2 - t_wall
        return (a1 * d2 * d2 - a2 * d1 * d1) / (d1 * d2 * (d2 - d1))

    yb, yt = y[0], y[n2m]
    g_b = grad(T[0], T[1], ymp[1] - yb, ymp[2] - yb)
    g_t = grad(T[n2m - 1], T[n2m - 2], yt - ymp[n2m], yt - ymp[n2m - 1])
    half = 0.5 * (yt - yb)
    return float(0.5 * (g_b + g_t) * 2.0 * half / (tm - t_wall))


def cylinder_nusselt(heat_body: float, re: float, pr: float, d: float, lz: float, dtemp: float) -> float:
    """Mean Nusselt number of a body of diameter d and span lz."""
    return float(heat_body * re * pr / (math.pi * d * lz * dtemp))


def strouhal(times: Sequence[float], lift: Sequence[float], d: float = 1.0, u: float = 1.0,
             min_periods: float = 2.0) -> Optional[float]:
    """Dominant frequency of the lift history times d / u, or None when the
    history holds fewer than `min_periods` periods of it (or no oscillation)."""
    t = np.asarray(times, dtype=np.float64)
    y = np.asarray(lift, dtype=np.float64)
    if t.size < 16 or not np.all(np.diff(t) > 0):
        return None
    n = int(2 ** math.ceil(math.log2(t.size)))
    tu = np.linspace(t[0], t[-1], n)
    yu = np.interp(tu, t, y)
    yu = yu - yu.mean()
    if not np.any(yu):
        return None
    pad = 16                                  # zero padding: the peak to a sixteenth of a bin
    spec = np.abs(np.fft.rfft(yu * np.hanning(n), pad * n)) ** 2
    spec[:pad] = 0.0
    k = int(np.argmax(spec))
    if k < 1 or k >= spec.size - 1:
        return None
    a, b, c = spec[k - 1], spec[k], spec[k + 1]
    den = a - 2 * b + c
    kk = k + (0.5 * (a - c) / den if den != 0 else 0.0)
    span = (tu[-1] - tu[0]) * n / (n - 1)     # the sampled record's length
    f = kk / (pad * span)
    if f * span < min_periods:
        return None
    return float(f * d / u)
