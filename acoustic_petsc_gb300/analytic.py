"""Analytic receiver signals of the acoustic source programs, the comparison the reference
draws in 2d/weno4/line_source/results/green.py (the receiver's p.dat against the Green's
function convolved with the source wavelet), written here for both dimensions.

Both programs solve u_tt = c^2 lap u + S(t) delta(x - x_s) with the wavelet of source.c,
S(t) = -2 (t - t0) f0^2 exp(-f0^2 (t - t0)^2), t0 = 4 / f0, put into one cell as S / h^dim.

* 3D (3d/weno4/point_source): G = delta(t - r/c) / (4 pi c^2 r), so
  u(r, t) = S(t - r/c) / (4 pi c^2 r).
* 2D (2d/weno4/line_source): G = H(t - r/c) / (2 pi c^2 sqrt(t^2 - r^2/c^2)) (green.py's
  kernel).  With s = t - tau - r/c = w^2 the convolution integral loses its inverse-square-
  root singularity: u = 1/(pi c^2) int_0^sqrt(t - r/c) S(t - r/c - w^2) / sqrt(w^2 + 2 r/c) dw,
  evaluated by Gauss-Legendre quadrature (green.py instead sums the sampled kernel).
"""
from __future__ import annotations

import numpy as np


def source_wavelet(t, f0):
    """Source(t) of source.c (3d/weno4/point_source: f0 = 100; 2d/weno4/line_source: 65)"""
    t = np.asarray(t, dtype=np.float64)
    t0 = 4.0 / f0
    return -2.0 * (t - t0) * f0 * f0 * np.exp(-1.0 * f0 * f0 * (t - t0) * (t - t0))


def point_source_receiver_3d(t, r, c, f0):
    """u at distance r > 0 from the 3D point source at times t (source switched on at t = 0)"""
    t = np.asarray(t, dtype=np.float64)
    return source_wavelet(t - r / c, f0) / (4.0 * np.pi * c * c * r)


def line_source_receiver_2d(t, r, c, f0, order=400):
    """u at distance r > 0 from the 2D line source at times t"""
    t = np.atleast_1d(np.asarray(t, dtype=np.float64))
    xg, wg = np.polynomial.legendre.leggauss(order)
    out = np.zeros_like(t)
    for q, tq in enumerate(t):
        a = tq - r / c
        if a <= 0.0:
            continue
        half = 0.5 * np.sqrt(a)
        w = half * (xg + 1.0)
        out[q] = (half * wg * source_wavelet(a - w * w, f0) / np.sqrt(w * w + 2.0 * r / c)).sum() / (np.pi * c * c)
    return out


def relative_l2_misfit(u, u_ref):
    """||u - u_ref|| / ||u_ref|| over the samples"""
    u = np.asarray(u, dtype=np.float64)
    u_ref = np.asarray(u_ref, dtype=np.float64)
    return float(np.sqrt(((u - u_ref) ** 2).sum() / (u_ref**2).sum()))
