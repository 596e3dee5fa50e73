"""Seeded synthetic inputs of the benchmark configurations (host side).

The reference ships no datasets; each configuration is generated from its
description with fixed seeds, identically for the GPU path and the CPU oracle.
"""
from __future__ import annotations

import math

import numpy as np

# 5-point Gauss rule on [-1/2, 1/2] (3d/weno4/Navier-Stokes-3D/hype.h:76-78)
X_GP5 = np.array([0.0, -0.2692346550528416, 0.2692346550528416, -0.4530899229693320, 0.4530899229693320])
W_GP5 = np.array([0.28444444444444444, 0.23931433524968326, 0.23931433524968326, 0.11846344252809456,
                  0.11846344252809456])


def _avg1d(n: int, h: float, x0: float, centre: float, sigma: float) -> np.ndarray:
    """Cell averages of exp(-(x-c)^2/(2 sigma^2)) by the 5-point rule at the correct
    points x_c + x_gp h (the 2D form of 2d/HyPE-2D/initialize_solution.c:58-63)."""
    xc = x0 + (np.arange(n) + 0.5) * h
    pts = xc[:, None] + X_GP5[None, :] * h
    return (np.exp(-((pts - centre) ** 2) / (2.0 * sigma * sigma)) * W_GP5[None, :]).sum(axis=1)


def euler_pulse(n: int = 256, gamma: float = 1.4, amp: float = 1e-3, sigma: float = 0.04) -> np.ndarray:
    """3D Euler acoustic pulse on [0,1]^3, periodic: rho = 1 + dp, u = 0, p = 1/gamma + dp,
    dp = amp exp(-r^2/(2 sigma^2)) about the centre.  AoS [k][j][i][5] cell averages
    (the Gaussian is separable, so the tensor 5^3 rule factorises exactly)."""
    h = 1.0 / n
    g = _avg1d(n, h, 0.0, 0.5, sigma)
    dp = amp * (g[:, None, None] * g[None, :, None] * g[None, None, :])
    U = np.zeros((n, n, n, 5))
    U[..., 0] = 1.0 + dp
    U[..., 4] = (1.0 / gamma + dp) / (gamma - 1.0)
    return U


def taylor_green(n: int = 256, gamma: float = 1.4) -> np.ndarray:
    """The Taylor-Green vortex of 3d/weno4/Navier-Stokes-3D/initial_condition.c:9-31 on
    [-pi, pi]^3 (rho 1, u = sin x cos y cos z, v = -cos x sin y cos z, w = 0,
    p = 100/gamma + (cos 2z + 2)(cos 2x + cos 2y - 2)/16) at the cell centres, AoS
    [k][j][i][5]."""
    h = 2.0 * math.pi / n
    x = -math.pi + (np.arange(n) + 0.5) * h
    sx, cx, c2 = np.sin(x), np.cos(x), np.cos(2.0 * x)
    U = np.empty((n, n, n, 5))
    U[..., 0] = 1.0
    U[..., 1] = sx[None, None, :] * cx[None, :, None] * cx[:, None, None]
    U[..., 2] = -cx[None, None, :] * sx[None, :, None] * cx[:, None, None]
    U[..., 3] = 0.0
    p = 100.0 / gamma + (1.0 / 16.0) * (c2[:, None, None] + 2.0) * (c2[None, None, :] + c2[None, :, None] - 2.0)
    U[..., 4] = p / (gamma - 1.0) + 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2)
    return U


def euler_blast(n: int = 512, gamma: float = 1.4, seed: int = 2024, p_ratio: float = 10.0, rho_ratio: float = 8.0,
                r0: float = 0.1, pert: float = 1e-3) -> np.ndarray:
    """Spherical blast on [0,1]^3 (cell-centre values): inside r < r0 p = 10 p0, rho = 8 rho0;
    rho0 = 1, p0 = 1/gamma; p carries a seeded uniform relative perturbation of +-pert."""
    h = 1.0 / n
    x = (np.arange(n) + 0.5) * h - 0.5
    rng = np.random.default_rng(seed)
    U = np.zeros((n, n, n, 5))
    for k in range(n):  # plane by plane keeps the temporaries small at 512^3
        r2 = x[None, :] ** 2 + x[:, None] ** 2 + x[k] ** 2
        inside = r2 < r0 * r0
        rho = np.where(inside, rho_ratio, 1.0)
        p = np.where(inside, p_ratio / gamma, 1.0 / gamma) * (1.0 + pert * rng.uniform(-1.0, 1.0, size=(n, n)))
        U[k, :, :, 0] = rho
        U[k, :, :, 4] = p / (gamma - 1.0)
    return U


def ctcs_gaussian(n: int = 512, sigma: float = 0.05, c: float = 1.0, cfl: float = 0.5):
    """2D CTCS start: nodes x_i = -1 + i h on [-1,1]^2, h = 2/n, p0 = exp(-r^2/(2 sigma^2)),
    zero initial p_t: p1 = p0 + 1/2 (c dt)^2 lap_h p0 with zero exterior.
    Returns (p0, p1, h, dt, alpha)."""
    h = 2.0 / n
    dt = cfl * h / c
    x = -1.0 + np.arange(n) * h
    X, Y = np.meshgrid(x, x)
    p0 = np.exp(-(X * X + Y * Y) / (2.0 * sigma * sigma))
    pad = np.zeros((n + 2, n + 2))
    pad[1:-1, 1:-1] = p0
    lap = (pad[2:, 1:-1] + pad[:-2, 1:-1] + pad[1:-1, 2:] + pad[1:-1, :-2] - 4.0 * p0) / (h * h)
    p1 = p0 + 0.5 * (c * dt) ** 2 * lap
    return p0, p1, h, dt, c * dt / h


def monopole_batch(ninst: int = 256, seed: int = 7, nmin: int = 64, nmax: int = 1024, c: float = 1.0,
                   cfl: float = 0.5):
    """Batched-acoustics instances: sides log-uniform in [nmin, nmax], source centre
    U[-0.8,0.8]^2, sigma U[0.02,0.1], points per wavelength U[8,32] -> f = c/(ppw h)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(ninst):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        h = 2.0 / n
        xs, ys = rng.uniform(-0.8, 0.8, size=2)
        sigma = rng.uniform(0.02, 0.1)
        ppw = rng.uniform(8.0, 32.0)
        out.append(dict(nx=n, ny=n, xmin=-1.0, ymin=-1.0, h=h, c0=c, dt=cfl * h / c, xs=float(xs), ys=float(ys),
                        sigma=float(sigma), freq=c / (ppw * h)))
    return out


def _prim2cons_mp(model: int, eos, V: np.ndarray) -> np.ndarray:
    """vectorised conserved state of the 2D multiphase models (same formulas as the library)"""
    g1, p1, g2, p2 = eos
    Q = np.empty_like(V)
    if model == 0:  # DI4: V = rho, u, v, p, phi
        phi = V[..., 4]
        g = 1.0 + (g1 - 1.0) * (g2 - 1.0) / ((1.0 - phi) * (g1 - 1.0) + phi * (g2 - 1.0))
        pinf = ((g - 1.0) / g) * (g1 * p1 * phi / (g1 - 1.0) + g2 * p2 * (1.0 - phi) / (g2 - 1.0))
        Q[..., 0] = V[..., 0]
        Q[..., 1] = V[..., 0] * V[..., 1]
        Q[..., 2] = V[..., 0] * V[..., 2]
        Q[..., 3] = 0.5 * V[..., 0] * (V[..., 1] ** 2 + V[..., 2] ** 2) + (V[..., 3] + g * pinf) / (g - 1.0)
        Q[..., 4] = phi
        return Q
    a1 = V[..., 5]
    a2 = 1.0 - a1
    g = 1.0 + ((g1 - 1.0) * (g2 - 1.0)) / ((g2 - 1.0) * a1 + (g1 - 1.0) * a2)
    pi = ((g - 1.0) / g) * (g1 * p1 * a1 / (g1 - 1.0) + g2 * p2 * a2 / (g2 - 1.0))
    rho = a1 * V[..., 0] + a2 * V[..., 1]
    Q[..., 0] = a1 * V[..., 0]
    Q[..., 1] = a2 * V[..., 1]
    Q[..., 2] = rho * V[..., 2]
    Q[..., 3] = rho * V[..., 3]
    Q[..., 4] = (V[..., 4] + g * pi) / (g - 1.0) + 0.5 * rho * (V[..., 2] ** 2 + V[..., 3] ** 2)
    Q[..., 5] = a1
    return Q


# water (phase 1) and air (phase 2) as stiffened gases, SI units
KAPILA_EOS = (4.4, 6.0e8, 1.4, 0.0)


def kapila_bubble(n: int = 1024, model: int = 1, smear: float = 2.0, eps: float = 1e-6):
    """Shock-driven air-bubble collapse on [0,1]^2 m: air bubble r = 0.1 at the centre
    (air fraction 1-eps inside, eps outside, tanh-smoothed over `smear` cells), water
    1000 kg/m^3 at 1e5 Pa, air 1 kg/m^3, pressure 1e8 Pa for x < 0.2 (same smoothing).
    Phase 1 = water (gamma 4.4, p_inf 6e8 Pa), phase 2 = air (1.4, 0).  Cell-centre
    values; AoS [j][i][nv] (model 1: Kapila five-equation, model 0: diffuse interface)."""
    h = 1.0 / n
    x = (np.arange(n) + 0.5) * h
    X, Y = np.meshgrid(x, x)
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2)
    t_b = 0.5 * (1.0 + np.tanh((r - 0.1) / (smear * h)))  # 0 inside the bubble, 1 outside
    a_water = eps + (1.0 - 2.0 * eps) * t_b
    t_p = 0.5 * (1.0 - np.tanh((X - 0.2) / (smear * h)))  # 1 for x < 0.2
    p = 1.0e5 + (1.0e8 - 1.0e5) * t_p
    if model == 1:
        V = np.zeros((n, n, 6))
        V[..., 0] = 1000.0
        V[..., 1] = 1.0
        V[..., 4] = p
        V[..., 5] = a_water
    else:
        V = np.zeros((n, n, 5))
        V[..., 0] = a_water * 1000.0 + (1.0 - a_water) * 1.0
        V[..., 3] = p
        V[..., 4] = a_water
    return _prim2cons_mp(model, KAPILA_EOS, V), h


MP3D_EOS = (1.4, 0.0, 1.6, 0.0)  # 3d/weno4/Viscous-Multiphase-Fourth-Order/hype.h:39-42


def mp3d_prim2cons(V: np.ndarray, eos=MP3D_EOS) -> np.ndarray:
    """PDEPrim2Cons of the 3D multiphase program (pde.c:27-45), vectorised"""
    g1, p1, g2, p2 = eos
    phi = V[..., 5]
    g = 1.0 + (g1 - 1.0) * (g2 - 1.0) / ((1.0 - phi) * (g1 - 1.0) + phi * (g2 - 1.0))
    pinf = ((g - 1.0) / g) * (g1 * p1 * phi / (g1 - 1.0) + g2 * p2 * (1.0 - phi) / (g2 - 1.0))
    Q = np.empty_like(V)
    Q[..., 0] = V[..., 0]
    Q[..., 1:4] = V[..., 0:1] * V[..., 1:4]
    Q[..., 4] = 0.5 * V[..., 0] * (V[..., 1] ** 2 + V[..., 2] ** 2 + V[..., 3] ** 2) + (V[..., 4] + g * pinf) / (g - 1.0)
    Q[..., 5] = phi
    return Q


def mp3d_layers(nx: int, ny: int, nz: int, eos=MP3D_EOS, width: float = 0.02) -> np.ndarray:
    """the layered set-up of 3d/weno4/Viscous-Multiphase-Fourth-Order/initial_condition.c on
    z in [-1/2, 1/2]: a shocked layer (rho 1.3765, w 0.3948, p 1.57) below z = -0.25, the same
    phase at rest, a light-gas layer (rho 0.138, phi 0) for |z| < 0.1, the phase at rest above;
    the interfaces smoothed over `width`; AoS [k][j][i][6]"""
    z = -0.5 + (np.arange(nz) + 0.5) / nz
    s = lambda a: 0.5 * (1.0 + np.tanh(a / width))
    w_shock = 1.0 - s(z + 0.25)
    w_gas = s(z + 0.1) * (1.0 - s(z - 0.1))
    V = np.zeros((nz, ny, nx, 6))
    V[..., 0] = (1.0 + 0.3765 * w_shock - 0.862 * w_gas)[:, None, None]
    V[..., 3] = (0.3948 * w_shock)[:, None, None]
    V[..., 4] = (1.0 + 0.57 * w_shock)[:, None, None]
    V[..., 5] = (1.0 - w_gas)[:, None, None]
    return mp3d_prim2cons(V, eos)


def kapila_drop(n: int, seed: int = 5, width: float = 0.02) -> np.ndarray:
    """a circular drop of phase 1 (radius 0.25, density 1) in phase 2 (density 0.125) on [0,1]^2
    with seeded 1 % velocity noise, pressure 1, both phases gamma 1.4 (the EOS compiled into
    2d/HyPE-2D); volume fraction in [1e-3, 1 - 1e-3]; Kapila conservative variables
    (a1 rho1, a2 rho2, rho u, rho v, E, a1), AoS [j][i][6]"""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    r = np.sqrt((x[None, :] - 0.5) ** 2 + (x[:, None] - 0.5) ** 2)
    a1 = 1e-3 + (1 - 2e-3) * 0.5 * (1 - np.tanh((r - 0.25) / width))
    u, v = 0.01 * rng.standard_normal((n, n)), 0.01 * rng.standard_normal((n, n))
    rho = a1 * 1.0 + (1 - a1) * 0.125
    Q = np.empty((n, n, 6))
    Q[..., 0] = a1 * 1.0
    Q[..., 1] = (1 - a1) * 0.125
    Q[..., 2] = rho * u
    Q[..., 3] = rho * v
    Q[..., 4] = 1.0 / 0.4 + 0.5 * rho * (u * u + v * v)
    Q[..., 5] = a1
    return Q

