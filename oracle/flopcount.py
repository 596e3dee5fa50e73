"""Algorithmic operation count of the reference's 3D Euler CWENO4 + Rusanov RHS and SSPRK(4,3)
stage (TEST INFRASTRUCTURE ONLY): a counting scalar type run through a transcription of the
reference's own expression trees, line for line, so that every add, multiply, divide, square
root, pow and comparison the reference program performs for one cell and one RK stage is
tallied exactly.

Transcribed (same expressions, same operation order; the CWENO4 coefficients are checked against
the C restatement, which the tests pin bit for bit to the reference compiled in place):
  weno()               3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:38-259
  evaluate_polynomial  3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:12-21
  PDEConsFlux          3d/weno4/Navier-Stokes-3D/pde.c:40-88 (general normal: the reference
                       multiplies by every component of n, zeros included)
  PDELLFRiemannSolver  3d/weno4/Navier-Stokes-3D/pde.c:164-187
  Gauss-point sum      3d/weno4/Navier-Stokes-3D/rhs_function.c:310-312 (Euler: no viscous term)
  divergence           3d/weno4/Navier-Stokes-3D/rhs_function.c:419-433
  SSP stage            SSPRK(4,3): u1 = u + dt/2 L, u2 = u1 + dt/2 L, u3 = 2/3 u + 1/3 u2 + dt/6 L,
                       u4 = u3 + dt/2 L (PETSc TSSSP RKS3, 4 stages; dt/2, dt/6 formed once per step)
Per cell and stage: 5 weno() calls, 5 x 24 trace evaluations, 3 faces x 4 Gauss points of
LLF (each face solved once; one low face of each direction per cell), the flux sums, the
divergence and the stage combination.  The reference also reconstructs the first ghost layer
(6 n^2 extra cells of n^3) and, in the Navier-Stokes program it belongs to, the gradient
traces; neither is counted (the first is a boundary effect, the second is viscous work).

Usage: python oracle/flopcount.py   (prints one JSON object)
"""
from __future__ import annotations

import collections
import json
import math

COUNT = collections.Counter()


class F:
    """a float that tallies every arithmetic operation applied to it"""
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = float(v.v if isinstance(v, F) else v)

    @staticmethod
    def _v(o):
        return o.v if isinstance(o, F) else float(o)

    def _op(self, o, kind, fn, rev=False):
        COUNT[kind] += 1
        a, b = self.v, F._v(o)
        return F(fn(b, a) if rev else fn(a, b))

    def __add__(self, o): return self._op(o, "add", lambda a, b: a + b)
    def __radd__(self, o): return self._op(o, "add", lambda a, b: a + b, True)
    def __sub__(self, o): return self._op(o, "add", lambda a, b: a - b)
    def __rsub__(self, o): return self._op(o, "add", lambda a, b: a - b, True)
    def __mul__(self, o): return self._op(o, "mul", lambda a, b: a * b)
    def __rmul__(self, o): return self._op(o, "mul", lambda a, b: a * b, True)
    def __truediv__(self, o): return self._op(o, "div", lambda a, b: a / b)
    def __rtruediv__(self, o): return self._op(o, "div", lambda a, b: a / b, True)

    def __neg__(self):
        COUNT["neg"] += 1
        return F(-self.v)

    def __lt__(self, o):
        COUNT["cmp"] += 1
        return self.v < F._v(o)

    def __gt__(self, o):
        COUNT["cmp"] += 1
        return self.v > F._v(o)


def fpow(a, b):
    COUNT["pow"] += 1
    return F(math.pow(F._v(a), F._v(b)))


def fsqrt(a):
    COUNT["sqrt"] += 1
    return F(math.sqrt(F._v(a)))


def fabs_(a):
    COUNT["abs"] += 1
    return F(abs(F._v(a)))


def fmax(a, b):  # PetscMax(a, b) = a < b ? b : a
    return b if a < b else a


r1_6, r1_12, r3_20, r1_120 = 1.0 / 6.0, 1.0 / 12.0, 3.0 / 20.0, 1.0 / 120.0
r13_3, r7_6, r61_48 = 13.0 / 3.0, 7.0 / 6.0, 61.0 / 48.0
small_num = 1.0e-12


def weno(U_x, U_y, U_z, U_xy, U_yz, U_zx, U_xyz):
    """reconstruction.c:38-259, line for line (the constants of the linear weights are
    formed from gammaHi / gammaLo as there, outside the cell's data)"""
    gammaHi = gammaLo = 0.85
    p = 4.0
    gamma_R4 = gammaHi
    gamma_R3 = [(1.0 - gammaHi) * gammaLo] + [r1_6 * (1 - gammaHi) * (1 - gammaLo)] * 6
    u_0 = U_xy[0]
    u_ip1, u_jp1, u_kp1 = U_x[3], U_y[3], U_z[3]
    u_im1, u_jm1, u_km1 = U_x[1], U_y[1], U_z[1]
    u_ip2, u_jp2, u_kp2 = U_x[4], U_y[4], U_z[4]
    u_im2, u_jm2, u_km2 = U_x[0], U_y[0], U_z[0]
    u_ip1jp1, u_jp1kp1, u_kp1ip1 = U_xy[1], U_yz[1], U_zx[1]
    u_ip1jm1, u_jp1km1, u_kp1im1 = U_xy[2], U_yz[2], U_zx[2]
    u_im1jp1, u_jm1kp1, u_km1ip1 = U_xy[3], U_yz[3], U_zx[3]
    u_im1jm1, u_jm1km1, u_km1im1 = U_xy[4], U_yz[4], U_zx[4]
    (u_ip1jp1kp1, u_im1jp1kp1, u_ip1jm1kp1, u_ip1jp1km1, u_im1jm1kp1, u_im1jp1km1, u_ip1jm1km1,
     u_im1jm1km1) = U_xyz
    # fourth-order stencil (:90-108)
    u_xR4 = r1_120 * (11.0 * u_im2 - 82.0 * u_im1 + 82.0 * u_ip1 - 11.0 * u_ip2)
    u_yR4 = r1_120 * (11.0 * u_jm2 - 82.0 * u_jm1 + 82.0 * u_jp1 - 11.0 * u_jp2)
    u_zR4 = r1_120 * (11.0 * u_km2 - 82.0 * u_km1 + 82.0 * u_kp1 - 11.0 * u_kp2)
    u_xxR4 = 0.5 * (u_im1 - 2.0 * u_0 + u_ip1)
    u_yyR4 = 0.5 * (u_jm1 - 2.0 * u_0 + u_jp1)
    u_zzR4 = 0.5 * (u_km1 - 2.0 * u_0 + u_kp1)
    u_xyR4 = 0.25 * (u_im1jm1 - u_im1jp1 - u_ip1jm1 + u_ip1jp1)
    u_yzR4 = 0.25 * (u_jm1km1 - u_jm1kp1 - u_jp1km1 + u_jp1kp1)
    u_xzR4 = 0.25 * (u_km1im1 - u_km1ip1 - u_kp1im1 + u_kp1ip1)
    u_xxxR4 = r1_12 * (-u_im2 + 2.0 * (u_im1 - u_ip1) + u_ip2)
    u_yyyR4 = r1_12 * (-u_jm2 + 2.0 * (u_jm1 - u_jp1) + u_jp2)
    u_zzzR4 = r1_12 * (-u_km2 + 2.0 * (u_km1 - u_kp1) + u_kp2)
    u_xxyR4 = 0.25 * (-u_im1jm1 + u_im1jp1 - u_ip1jm1 + u_ip1jp1) + 0.5 * (u_jm1 - u_jp1)
    u_xyyR4 = 0.5 * (u_im1 - u_ip1) + 0.25 * (u_ip1jp1 - u_im1jm1 - u_im1jp1 + u_ip1jm1)
    u_yyzR4 = 0.25 * (-u_jm1km1 + u_jm1kp1 - u_jp1km1 + u_jp1kp1) + 0.5 * (u_km1 - u_kp1)
    u_yzzR4 = 0.5 * (u_jm1 - u_jp1) + 0.25 * (u_jp1kp1 - u_jm1km1 - u_jm1kp1 + u_jp1km1)
    u_xxzR4 = 0.25 * (-u_km1im1 + u_kp1im1 - u_km1ip1 + u_kp1ip1) + 0.5 * (u_km1 - u_kp1)
    u_xzzR4 = 0.5 * (u_im1 - u_ip1) + 0.25 * (u_kp1ip1 - u_km1im1 - u_kp1im1 + u_km1ip1)
    u_xyzR4 = 0.125 * (u_ip1jp1kp1 - u_im1jp1kp1 - u_ip1jm1kp1 - u_ip1jp1km1 + u_im1jm1kp1 + u_im1jp1km1 +
                       u_ip1jm1km1 - u_im1jm1km1)
    # (:110-116)
    IS_R4 = (u_xR4 * u_xR4 + u_yR4 * u_yR4 + u_zR4 * u_zR4 +
             r13_3 * (u_xxR4 * u_xxR4 + u_yyR4 * u_yyR4 + u_zzR4 * u_zzR4) +
             r7_6 * (u_xyR4 * u_xyR4 + u_yzR4 * u_yzR4 + u_xzR4 * u_xzR4) +
             0.2 * (u_xR4 * u_xxxR4 + u_yR4 * u_yyyR4 + u_zR4 * u_zzzR4) +
             4.7 * (u_xxyR4 * u_xxyR4 + u_xxzR4 * u_xxzR4 + u_xyyR4 * u_xyyR4 + u_xzzR4 * u_xzzR4 +
                    u_yyzR4 * u_yyzR4 + u_yzzR4 * u_yzzR4) +
             39.06 * (u_xxxR4 * u_xxxR4 + u_yyyR4 * u_yyyR4 + u_zzzR4 * u_zzzR4) +
             r61_48 * u_xyzR4 * u_xyzR4)
    w_R4 = gamma_R4 / fpow((IS_R4 + small_num), p)
    total = w_R4
    ux, uy, uz, uxx, uyy, uzz, uxy, uyz, uxz = ([None] * 7 for _ in range(9))
    # centred third-order stencil (:123-131)
    ux[0] = 0.5 * (u_ip1 - u_im1)
    uy[0] = 0.5 * (u_jp1 - u_jm1)
    uz[0] = 0.5 * (u_kp1 - u_km1)
    uxx[0] = 0.5 * (u_im1 - 2.0 * u_0 + u_ip1)
    uyy[0] = 0.5 * (u_jm1 - 2.0 * u_0 + u_jp1)
    uzz[0] = 0.5 * (u_km1 - 2.0 * u_0 + u_kp1)
    uxy[0] = 0.25 * (u_ip1jp1 - u_ip1jm1 - u_im1jp1 + u_im1jm1)
    uyz[0] = 0.25 * (u_jp1kp1 - u_jp1km1 - u_jm1kp1 + u_jm1km1)
    uxz[0] = 0.25 * (u_kp1ip1 - u_kp1im1 - u_km1ip1 + u_km1im1)
    # +x (:135-143)
    ux[1] = -1.5 * u_0 + 2.0 * u_ip1 - 0.5 * u_ip2
    uy[1] = 0.5 * (u_jp1 - u_jm1)
    uz[1] = 0.5 * (u_kp1 - u_km1)
    uxx[1] = 0.5 * (u_0 - 2.0 * u_ip1 + u_ip2)
    uyy[1] = 0.5 * (u_jm1 - 2.0 * u_0 + u_jp1)
    uzz[1] = 0.5 * (u_km1 - 2.0 * u_0 + u_kp1)
    uxy[1] = 0.5 * (u_ip1jp1 - u_ip1jm1) - uy[1]
    uyz[1] = 0.25 * (u_jp1kp1 - u_jp1km1 - u_jm1kp1 + u_jm1km1)
    uxz[1] = 0.5 * (u_kp1ip1 - u_km1ip1) - uz[1]
    # -x (:147-155)
    ux[2] = -2.0 * u_im1 + 0.5 * u_im2 + 1.5 * u_0
    uy[2] = 0.5 * (u_jp1 - u_jm1)
    uz[2] = 0.5 * (u_kp1 - u_km1)
    uxx[2] = 0.5 * (u_im2 - 2.0 * u_im1 + u_0)
    uyy[2] = 0.5 * (u_jm1 - 2.0 * u_0 + u_jp1)
    uzz[2] = 0.5 * (u_km1 - 2.0 * u_0 + u_kp1)
    uxy[2] = 0.5 * (u_im1jm1 - u_im1jp1) + uy[2]
    uyz[2] = 0.25 * (u_jp1kp1 - u_jp1km1 - u_jm1kp1 + u_jm1km1)
    uxz[2] = 0.5 * (u_km1im1 - u_kp1im1) + uz[2]
    # +y (:159-167)
    ux[3] = 0.5 * (u_ip1 - u_im1)
    uy[3] = -1.5 * u_0 + 2.0 * u_jp1 - 0.5 * u_jp2
    uz[3] = 0.5 * (u_kp1 - u_km1)
    uxx[3] = 0.5 * (u_im1 - 2.0 * u_0 + u_ip1)
    uyy[3] = 0.5 * (u_0 - 2.0 * u_jp1 + u_jp2)
    uzz[3] = 0.5 * (u_km1 - 2.0 * u_0 + u_kp1)
    uxy[3] = 0.5 * (u_ip1jp1 - u_im1jp1) - ux[3]
    uyz[3] = 0.5 * (u_jp1kp1 - u_jp1km1) - uz[3]
    uxz[3] = 0.25 * (u_kp1ip1 - u_kp1im1 - u_km1ip1 + u_km1im1)
    # -y (:171-179)
    ux[4] = 0.5 * (u_ip1 - u_im1)
    uy[4] = -2.0 * u_jm1 + 0.5 * u_jm2 + 1.5 * u_0
    uz[4] = 0.5 * (u_kp1 - u_km1)
    uxx[4] = 0.5 * (u_im1 - 2.0 * u_0 + u_ip1)
    uyy[4] = 0.5 * (u_jm2 - 2.0 * u_jm1 + u_0)
    uzz[4] = 0.5 * (u_km1 - 2.0 * u_0 + u_kp1)
    uxy[4] = 0.5 * (u_im1jm1 - u_ip1jm1) + ux[4]
    uyz[4] = 0.5 * (u_jm1km1 - u_jm1kp1) + uz[4]
    uxz[4] = 0.25 * (u_kp1ip1 - u_kp1im1 - u_km1ip1 + u_km1im1)
    # +z (:183-191)
    ux[5] = 0.5 * (u_ip1 - u_im1)
    uy[5] = 0.5 * (u_jp1 - u_jm1)
    uz[5] = -1.5 * u_0 + 2.0 * u_kp1 - 0.5 * u_kp2
    uxx[5] = 0.5 * (u_im1 - 2.0 * u_0 + u_ip1)
    uyy[5] = 0.5 * (u_jm1 - 2.0 * u_0 + u_jp1)
    uzz[5] = 0.5 * (u_0 - 2.0 * u_kp1 + u_kp2)
    uxy[5] = 0.25 * (u_ip1jp1 - u_ip1jm1 - u_im1jp1 + u_im1jm1)
    uyz[5] = 0.5 * (u_jp1kp1 - u_jm1kp1) - uy[5]
    uxz[5] = 0.5 * (u_kp1ip1 - u_kp1im1) - ux[5]
    # -z (:195-203)
    ux[6] = 0.5 * (u_ip1 - u_im1)
    uy[6] = 0.5 * (u_jp1 - u_jm1)
    uz[6] = -2.0 * u_km1 + 0.5 * u_km2 + 1.5 * u_0
    uxx[6] = 0.5 * (u_im1 - 2.0 * u_0 + u_ip1)
    uyy[6] = 0.5 * (u_jm1 - 2.0 * u_0 + u_jp1)
    uzz[6] = 0.5 * (u_km2 - 2.0 * u_km1 + u_0)
    uxy[6] = 0.25 * (u_ip1jp1 - u_ip1jm1 - u_im1jp1 + u_im1jm1)
    uyz[6] = 0.5 * (u_jm1km1 - u_jp1km1) + uy[6]
    uxz[6] = 0.5 * (u_km1im1 - u_km1ip1) + ux[6]
    # (:205-215)
    w_R3 = [None] * 7
    for i in range(7):
        IS = ((ux[i] * ux[i] + uy[i] * uy[i] + uz[i] * uz[i]) +
              r13_3 * (uxx[i] * uxx[i] + uyy[i] * uyy[i] + uzz[i] * uzz[i]) +
              r7_6 * (uxy[i] * uxy[i] + uyz[i] * uyz[i] + uxz[i] * uxz[i]))
        w_R3[i] = gamma_R3[i] / fpow((IS + small_num), p)
        total = total + w_R3[i]
    w_R4 = w_R4 / total
    for i in range(7):
        w_R3[i] = w_R3[i] / total
    # (:220-234): linear and nonlinear sums, starting from 0.0 as there
    names = ("x", "y", "z", "xx", "yy", "zz", "xy", "yz", "xz")
    lin = {q: F(0.0) for q in names}
    nl = dict(lin)
    comp = {"x": ux, "y": uy, "z": uz, "xx": uxx, "yy": uyy, "zz": uzz, "xy": uxy, "yz": uyz, "xz": uxz}
    for i in range(7):
        for q in names:
            lin[q] = lin[q] + gamma_R3[i] * comp[q][i]
            nl[q] = nl[q] + w_R3[i] * comp[q][i]
    wt_ratio = w_R4 / gamma_R4
    R4 = {"x": u_xR4, "y": u_yR4, "z": u_zR4, "xx": u_xxR4, "yy": u_yyR4, "zz": u_zzR4, "xy": u_xyR4,
          "yz": u_yzR4, "xz": u_xzR4}
    coeffs = [u_0] + [wt_ratio * (R4[q] - lin[q]) + nl[q] for q in names]
    coeffs += [wt_ratio * c for c in (u_xxxR4, u_yyyR4, u_zzzR4, u_xxyR4, u_xyyR4, u_yyzR4, u_yzzR4, u_xxzR4,
                                      u_xzzR4, u_xyzR4)]
    return coeffs


def evaluate_polynomial(x, y, z, c):
    """reconstruction.c:12-21 (x, y, z are the face Gauss-point constants)"""
    return (c[0] + c[1] * x + c[2] * y + c[3] * z +
            c[4] * (x * x - r1_12) + c[5] * (y * y - r1_12) + c[6] * (z * z - r1_12) +
            c[7] * x * y + c[8] * y * z + c[9] * z * x +
            c[10] * x * (x * x - r3_20) + c[11] * y * (y * y - r3_20) + c[12] * z * (z * z - r3_20) +
            c[13] * (x * x - r1_12) * y + c[14] * x * (y * y - r1_12) +
            c[15] * (y * y - r1_12) * z + c[16] * y * (z * z - r1_12) +
            c[17] * (x * x - r1_12) * z + c[18] * x * (z * z - r1_12) + c[19] * x * y * z)


GAMMA = 1.4


def pde_cons_flux(Q, nx, ny, nz):
    """pde.c:40-88 (the admissibility tests count as two comparisons)"""
    rho = Q[0]
    r1_rho = 1.0 / rho
    u = r1_rho * Q[1]
    v = r1_rho * Q[2]
    w = r1_rho * Q[3]
    E = Q[4]
    p = (GAMMA - 1.0) * (E - 0.5 * rho * (u * u + v * v + w * w))
    _ = rho < 1.0e-14
    _ = p < 1.0e-12
    Fl = [nx * rho * u + ny * rho * v + nz * rho * w,
          nx * (rho * u * u + p) + ny * rho * u * v + nz * rho * u * w,
          nx * rho * u * v + ny * (rho * v * v + p) + nz * rho * v * w,
          nx * rho * u * w + ny * rho * v * w + nz * (rho * w * w + p),
          (E + p) * (nx * u + ny * v + nz * w)]
    a = fsqrt(r1_rho * GAMMA * p)
    s_max = fabs_(u * nx + v * ny + w * nz) + a
    return s_max, Fl


def llf(QL, QR, nx, ny, nz):
    """pde.c:164-187"""
    sl, FL = pde_cons_flux(QL, nx, ny, nz)
    sr, FR = pde_cons_flux(QR, nx, ny, nz)
    s_max = fmax(sl, sr)
    return s_max, [0.5 * (FR[c] + FL[c] - s_max * (QR[c] - QL[c])) for c in range(5)]


GP = 0.5 / math.sqrt(3.0)
X_GP = [-GP, -GP, GP, GP]
Y_GP = [-GP, GP, -GP, GP]
W_GP = [0.25] * 4


def count_cell_stage(seed: int = 1):
    """tallies of one cell-stage by part; also the stencils and coefficients for the check"""
    import random

    rnd = random.Random(seed)

    def stencil(base):
        Ux = [F(base + 0.01 * rnd.random()) for _ in range(5)]
        Uy = [F(base + 0.01 * rnd.random()) for _ in range(5)]
        Uz = [F(base + 0.01 * rnd.random()) for _ in range(5)]
        c0 = F(base + 0.01 * rnd.random())
        Ux[2] = Uy[2] = Uz[2] = c0
        Uxy = [c0] + [F(base + 0.01 * rnd.random()) for _ in range(4)]
        Uyz = [c0] + [F(base + 0.01 * rnd.random()) for _ in range(4)]
        Uzx = [c0] + [F(base + 0.01 * rnd.random()) for _ in range(4)]
        Uxyz = [F(base + 0.01 * rnd.random()) for _ in range(8)]
        return Ux, Uy, Uz, Uxy, Uyz, Uzx, Uxyz

    parts = {}
    # 1. reconstruction: weno() per variable, then its 24 face traces (rhs_function.c:185-274)
    COUNT.clear()
    bases = [1.0, 0.1, 0.1, 0.1, 2.5]
    coefs, args = [], []
    for c in range(5):
        a = stencil(bases[c])
        args.append([[x.v for x in arr] for arr in a])
        coefs.append(weno(*a))
    parts["weno"] = dict(COUNT)
    COUNT.clear()
    traces = [[None] * 24 for _ in range(5)]
    for c in range(5):
        for f in range(4):
            for face, (x, y, z) in enumerate(((-0.5, X_GP[f], Y_GP[f]), (0.5, X_GP[f], Y_GP[f]),
                                              (X_GP[f], -0.5, Y_GP[f]), (X_GP[f], 0.5, Y_GP[f]),
                                              (X_GP[f], Y_GP[f], -0.5), (X_GP[f], Y_GP[f], 0.5))):
                traces[c][4 * face + f] = evaluate_polynomial(x, y, z, coefs[c])
    parts["traces"] = dict(COUNT)
    # 2. the three low faces of the cell, 4 Gauss points each: LLF and the weighted sum
    #    (rhs_function.c:276-417); the smax comparison (s_c > s_max_c) once per Gauss point
    COUNT.clear()
    smax = F(0.0)
    for d, n in enumerate(((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0))):
        flux = [F(0.0)] * 5
        for f in range(4):
            QL = [traces[c][4 * (2 * d + 1) + f] for c in range(5)]
            QR = [traces[c][4 * (2 * d) + f] for c in range(5)]
            s, fl = llf(QL, QR, *n)
            if s > smax:
                smax = s
            flux = [flux[c] + W_GP[f] * fl[c] for c in range(5)]
    parts["faces"] = dict(COUNT)
    # 3. divergence (rhs_function.c:419-433) and the SSP combination of the four stages
    COUNT.clear()
    r1_h = 256.0
    Fh = [F(0.1 * (q + 1)) for q in range(6)]
    for c in range(5):
        _ = (-r1_h * (Fh[1] - Fh[0]) - r1_h * (Fh[3] - Fh[2]) - r1_h * (Fh[5] - Fh[4]))
    parts["divergence"] = dict(COUNT)
    COUNT.clear()
    u, w, L, half_dt, dt6 = F(1.0), F(1.1), F(0.01), F(1e-4), F(3e-5)
    for c in range(5):
        _ = u + half_dt * L                              # stage 1
        _ = w + half_dt * L                              # stage 2
        _ = (2.0 / 3.0) * u + (1.0 / 3.0) * w + dt6 * L  # stage 3
        _ = w + half_dt * L                              # stage 4
    parts["stage_combination_4_stages"] = dict(COUNT)
    return parts, args, coefs


def main():
    parts, args, coefs = count_cell_stage()
    kinds = ("add", "mul", "div", "sqrt", "pow", "abs", "cmp", "neg")
    per_stage = collections.Counter()
    for name, cnt in parts.items():
        scale = 0.25 if name == "stage_combination_4_stages" else 1.0
        for k, v in cnt.items():
            per_stage[k] += v * scale
    flops = per_stage["add"] + per_stage["mul"] + per_stage["div"] + per_stage["sqrt"] + per_stage["pow"]
    out = {"per_cell_stage": {k: per_stage.get(k, 0) for k in kinds},
           "flops_per_cell_stage": flops,
           "convention": "add/sub, mul, div, sqrt and pow count one flop each; abs, comparisons and negations "
                         "are tallied but not counted as flops",
           "parts": parts}
    # the transcription against the C restatement (pinned bit for bit to the reference)
    try:
        import ctypes as C
        import os
        import sys

        sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
        from oracle import pyoracle as O

        O.build(None)
        D = C.POINTER(C.c_double)
        fn = O.lib().orc_cweno4_ref_args
        fn.argtypes = [D] * 8
        worst = 0.0
        for c in range(5):
            arrs = [(C.c_double * len(a))(*a) for a in args[c]]
            outc = (C.c_double * 20)()
            fn(*[C.cast(a, D) for a in arrs], C.cast(outc, D))
            worst = max(worst, max(abs(outc[q] - coefs[c][q].v) for q in range(20)))
        out["transcription_vs_restatement_max_abs_diff"] = worst
    except Exception as ex:  # pragma: no cover - report only
        out["transcription_check"] = f"not run: {ex}"
    return out


if __name__ == "__main__":
    print(json.dumps(main(), indent=1))
