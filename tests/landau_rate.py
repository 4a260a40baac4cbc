"""Frequency and damping rate of linear Landau damping from a series of the
electric energy: the peaks of log sqrt(EE) (parabolic interpolation around
each sampled maximum) give the frequency from their spacing (|E| peaks twice
per period) and the rate from a least-squares line through them.

Linear theory for k = 0.5 and a unit Maxwellian: omega = 1.4156,
gamma = -0.1533 (the known answer the Landau-Poisson literature quotes for
this case)."""
from __future__ import annotations

import numpy as np

OMEGA_K05 = 1.4156
GAMMA_K05 = -0.1533


def rate(ts, ee, t_max):
    """(omega, gamma, peaks) from times ts and electric energies ee, using the
    peaks at t <= t_max."""
    ts = np.asarray(ts, dtype=float)
    y = 0.5 * np.log(np.asarray(ee, dtype=float))
    h = ts[1] - ts[0]
    peaks = []
    for i in range(1, len(y) - 1):
        if y[i] > y[i - 1] and y[i] >= y[i + 1]:
            den = y[i - 1] - 2 * y[i] + y[i + 1]
            d = 0.5 * (y[i - 1] - y[i + 1]) / den if den != 0 else 0.0
            peaks.append((ts[i] + d * h, y[i] - 0.25 * (y[i - 1] - y[i + 1]) * d))
    sel = [p for p in peaks if p[0] <= t_max]
    tp = np.array([p[0] for p in sel])
    yp = np.array([p[1] for p in sel])
    omega = np.pi / np.mean(np.diff(tp))
    gamma = np.polyfit(tp, yp, 1)[0]
    return float(omega), float(gamma), sel
