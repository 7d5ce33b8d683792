"""Shear-wave splitting of SKS seismograms by the eigenvalue method of Silver &
Chan (1991, J. Geophys. Res. 96, 16429-16454).

The reference measures splitting with an external program (an_split, named in
applications/test/cal_split.pl:7, not part of the tree); this module restates
the published method so that the FP32-compensated and FP64 seismograms of one
run can be compared by the same code.

For a trial fast axis phi (degrees from the radial axis x toward the
transverse axis y) and delay dt, the horizontal components are rotated into
fast and slow, the slow component is advanced by dt, and the smaller
eigenvalue lambda2 of their 2x2 covariance over the analysis window is taken;
the (phi, dt) minimising lambda2 is the splitting estimate.  The covariances
of all trial pairs follow from windowed cross-correlations of x and y at the
trial lags, so the grid search costs a few array operations.
"""
from __future__ import annotations

import numpy as np


def _lagged_sums(x: np.ndarray, y: np.ndarray, i0: int, i1: int, kmax: int) -> dict:
    """S_ab(k) = sum_{t in [i0,i1)} a(t) b(t+k) and T_ab(k) = sum a(t+k) b(t+k), k = 0..kmax."""
    n = i1 - i0
    xw, yw = x[i0:i1], y[i0:i1]
    out = {k: np.empty(kmax + 1) for k in ("Sxx", "Sxy", "Syx", "Syy", "Txx", "Txy", "Tyy")}
    for k in range(kmax + 1):
        xs, ys = x[i0 + k:i1 + k], y[i0 + k:i1 + k]
        if len(xs) < n:  # past the end of the record: zeros
            xs = np.pad(xs, (0, n - len(xs)))
            ys = np.pad(ys, (0, n - len(ys)))
        out["Sxx"][k] = xw @ xs
        out["Sxy"][k] = xw @ ys
        out["Syx"][k] = yw @ xs
        out["Syy"][k] = yw @ ys
        out["Txx"][k] = xs @ xs
        out["Txy"][k] = xs @ ys
        out["Tyy"][k] = ys @ ys
    return out


def eigen_grid(x: np.ndarray, y: np.ndarray, dt: float, window: tuple[int, int], max_delay: float = 3.0,
               dphi: float = 0.25):
    """The trial grid: fast axes (rad, [nphi]) and lambda2, lambda1 ([nphi][ndelay])."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    i0, i1 = int(window[0]), int(window[1])
    if not (0 <= i0 < i1 <= len(x)):
        raise ValueError("window outside the record")
    kmax = int(round(max_delay / dt))
    S = _lagged_sums(x, y, i0, i1, kmax)
    phi = np.deg2rad(np.arange(-90.0, 90.0, dphi))[:, None]
    c, s = np.cos(phi), np.sin(phi)
    c11 = c * c * S["Sxx"][0] + 2 * c * s * S["Sxy"][0] + s * s * S["Syy"][0]          # fast, unshifted
    c22 = s * s * S["Txx"][None, :] - 2 * c * s * S["Txy"][None, :] + c * c * S["Tyy"][None, :]
    c12 = (-c * s * S["Sxx"][None, :] + c * c * S["Sxy"][None, :] - s * s * S["Syx"][None, :]
           + c * s * S["Syy"][None, :])
    c11 = np.broadcast_to(c11, c22.shape)
    half = 0.5 * (c11 + c22)
    rad = np.sqrt(np.maximum(0.25 * (c11 - c22) ** 2 + c12 ** 2, 0.0))
    return phi[:, 0], half - rad, half + rad


def splitting(x: np.ndarray, y: np.ndarray, dt: float, window: tuple[int, int], max_delay: float = 3.0,
              dphi: float = 0.25) -> dict:
    """Silver-Chan estimate from the radial (x) and transverse (y) components.

    window: sample range [i0, i1) holding the SKS phase.  Returns phi (deg, in
    [-90, 90)), delay (s), the minimum lambda2 / lambda1 and the grids' steps."""
    phi, lam2, lam1 = eigen_grid(x, y, dt, window, max_delay, dphi)
    phi = phi[:, None]
    j = np.unravel_index(int(np.argmin(lam2)), lam2.shape)
    return {"phi_deg": float(np.rad2deg(phi[j[0], 0])), "delay_s": float(j[1] * dt),
            "lambda_ratio": float(lam2[j] / lam1[j]) if lam1[j] > 0 else float("nan"),
            "dphi_deg": dphi, "ddelay_s": dt}


def apply_splitting(x: np.ndarray, y: np.ndarray, phi_deg: float, delay_s: float, dt: float):
    """Split a horizontal wave: rotate into fast/slow at phi, delay the slow
    component by delay_s (linear interpolation), rotate back."""
    p = np.deg2rad(phi_deg)
    c, s = np.cos(p), np.sin(p)
    f = c * x + s * y
    sl = -s * x + c * y
    t = np.arange(len(x)) * dt
    sl = np.interp(t - delay_s, t, sl, left=0.0, right=0.0)
    return c * f - s * sl, s * f + c * sl


def sks_window(x: np.ndarray, dt: float, half_width: float) -> tuple[int, int]:
    """Analysis window centred on the radial component's largest amplitude."""
    i = int(np.argmax(np.abs(x)))
    h = int(round(half_width / dt))
    return max(0, i - h), min(len(x), i + h)
