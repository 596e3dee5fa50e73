"""Regenerate the golden fixtures of tests/golden/ (run where the reference
tree is available; the GPU machine has none, so the fixtures are committed).

* point_source_p.dat    -- the reference's checked-in receiver trace
                           3d/ctcs/point_source/results/p.dat (251 samples)
* accuracy_tables.json  -- the reference's published accuracy numbers
                           (2d/weno4/standing_wave/results/Error.dat,
                            3d/weno4/plane_wave/results/main.tex:39-42)
* ref_euler_*.npz       -- inputs and outputs of the reference's own RHSFunction
                           (3d/weno4/Navier-Stokes-3D/rhs_function.c with the
                           CWENO4 weno() of Viscous-Multiphase-Fourth-Order,
                           viscous flux zero) compiled through oracle/petsc_shim,
                           and of 3 SSP RKS3/4-stage steps of the same; the
                           *_hllc / *_rothllc cases switch its Riemann solver to
                           the reference's PDEHLLCRiemannSolver / PDErotHLLCRiemannSolver
* ref_euler_*_weno3.npz -- the same for the third-order WENO Euler program
                           3d/weno3/Euler (its rhs_function.c, reconstruction.c,
                           pde.c), stepped with its monitor disabled (fixed dt)
* ref_acoustic_*.npz    -- the acoustic FV RHS of 3d/weno4/plane_wave (R4 face
                           gradients, central flux) and 3 SSP RKS3 steps of it, under
                           periodic, adiabatic and mixed walls
* ref_ns3d_*.npz        -- the viscous RHS of 3d/weno4/Navier-Stokes-3D as shipped (R4
                           values and gradients, Rusanov + averaged PDEViscFlux,
                           mu 0.01, Pr 1, Cv 2.5) and 3 steps of it with the
                           program's own dt (viscous speed included)
* ns3d_tgv_ke.csv       -- the reference's checked-in kinetic energy / dissipation
                           history of its 32^3 Taylor-Green run
                           (3d/weno4/Navier-Stokes-3D/ke.csv: t, KE, dissipation every
                           10 steps)
* ref_sw2d_*.npz        -- the 2D acoustic FV RHS of 2d/weno4/standing_wave and 3 steps of
                           it with SSP RK104 and with RKS3/4 stages, under periodic,
                           adiabatic and mixed walls
* ref_mp3d_*.npz        -- the 3D primitive-variable multiphase RHS of
                           3d/weno4/Viscous-Multiphase-Fourth-Order (RHSFunctionPrimitive:
                           primitive CWENO4, 33-node PAD fallback, rotated HLLC, phi term,
                           viscous speed in dt) and 3 SSP RKS3/4 steps of it; "sharp"
                           trips the fallback
* ref_h2d_*.npz         -- the path-conservative RHS of 2d/HyPE-2D with its Kapila model
                           (order N = 1 and 3, Rusanov + Roe-path fluctuation, volume
                           term, node admissibility) and 3 steps of its stepper for N;
                           "sharp" states trip the first-order fallback
* ref_ctcs2d.npz        -- the reference's CTCS() (2d/ctcs/plane_wave/wave.c)
                           on a zero-exterior grid
* ref_bubble_*.npz      -- the reference's 2D diffuse-interface RHSFunction
                           (2d/weno4/bubble) and RK104 steps of it; "sharp" trips the
                           admissibility fallback
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as O  # noqa: E402

REF = os.environ.get("HYPE_REF_DIR", "/root/reference")


def euler_case(n, seed, bc, amp=0.2, sig=0.15, vel=0.05):
    """seeded smooth state with a pulse and random momentum (cell-centre values)"""
    h = 1.0 / n
    x = (np.arange(n) + 0.5) * h
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2
    dp = amp * np.exp(-r2 / (2 * sig**2))
    rng = np.random.default_rng(seed)
    U = np.zeros((n, n, n, 5))
    U[..., 0] = 1.0 + dp
    U[..., 1:4] = vel * rng.standard_normal((n, n, n, 3))
    p = 1.0 / 1.4 + dp
    U[..., 4] = p / 0.4 + 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2) / U[..., 0]
    return U


CASES = [("periodic", 8, 11, (0, 0, 0, 0, 0, 0)), ("walls", 8, 12, (1, 1, 2, 2, 1, 2)),
         ("mixed", 9, 13, (2, 2, 0, 0, 1, 1))]


def ns3d_fixtures():
    """the Navier-Stokes-3D fixtures (viscous RHS, 3 steps, the Taylor-Green history)"""
    for name, n, seed, bc in CASES:
        cfg = O.euler_cfg(n, 1.0 / n, cfl=0.4, bc=bc, recon=1, mu=0.01)
        U = euler_case(n, seed + 200, bc, vel=0.1)
        R, dt, rc = O.ref_euler_rhs(cfg, U)
        assert rc == 0
        U3, t3, dt3, rc3 = O.ref_euler_run(cfg, U, 3)
        assert rc3 == 0
        np.savez_compressed(os.path.join(HERE, f"ref_ns3d_{name}.npz"), U=U, RHS=R, dt=dt, U3=U3, t3=t3, dt3=dt3,
                            bc=np.array(bc), n=n, cfl=0.4, flux=0, recon=1, mu=0.01, prandtl=1.0, cv=2.5)
    with open(os.path.join(REF, "3d/weno4/Navier-Stokes-3D/ke.csv")) as f, \
            open(os.path.join(HERE, "ns3d_tgv_ke.csv"), "w") as g:
        g.write(f.read())


def sw2d_fixtures():
    """the 2d/weno4/standing_wave fixtures (RHS, 3 RK104 steps, 3 RKS3/4 steps)"""
    for name, bc, seed in (("periodic", (0,) * 4, 41), ("adiabatic", (4,) * 4, 42), ("mixed", (4, 4, 0, 0), 43)):
        nx, ny, h = 9, 7, 0.3
        cfg = O.sw2d_cfg(nx, ny, h, -0.2, 0.1, bc)
        U = np.random.default_rng(seed).standard_normal((ny, nx, 2))
        R = O.ref_sw2d_rhs(cfg, U)
        U104, t104 = O.ref_sw2d_run(cfg, U, 3, 0.01, stepper=1)
        U43, t43 = O.ref_sw2d_run(cfg, U, 3, 0.01, stepper=0)
        np.savez_compressed(os.path.join(HERE, f"ref_sw2d_{name}.npz"), U=U, RHS=R, U104=U104, t104=t104, U43=U43,
                            t43=t43, dt=0.01, h=h, xmin=-0.2, ymin=0.1, nx=nx, ny=ny, bc=np.array(bc))


def mp3d_state(cfg, n, seed, sharp=False):
    """a gas bubble (phi = 0) in the other phase with random velocities and pressure"""
    nx, ny, nz = n
    rng = np.random.default_rng(seed)
    h = cfg.h
    z, y, x = ((np.arange(m) + 0.5) * h for m in (nz, ny, nx))
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    r = np.sqrt((X - 0.5 * nx * h) ** 2 + (Y - 0.5 * ny * h) ** 2 + (Z - 0.5 * nz * h) ** 2)
    w = 0.02 if sharp else 0.15
    phi = 0.5 * (1 + np.tanh((r - 0.25 * nz * h) / (w * nz * h)))
    V = np.zeros((nz, ny, nx, 6))
    V[..., 0] = 0.138 + (1.0 - 0.138) * phi + 0.01 * rng.random((nz, ny, nx))
    V[..., 1:4] = 0.05 * rng.standard_normal((nz, ny, nx, 3))
    V[..., 4] = 1.0 + 0.1 * rng.random((nz, ny, nx))
    V[..., 5] = phi
    return O.mp3d_prim2cons(cfg, V)


def mp3d_fixtures():
    """the Viscous-Multiphase-Fourth-Order fixtures (RHS + dt, 3 steps)"""
    n = (7, 6, 8)
    for name, bc, seed, sharp in (("transmissive", (2,) * 6, 51, False), ("periodic", (0,) * 6, 52, False),
                                  ("walls", (1, 1, 2, 2, 1, 1), 53, False), ("sharp", (2,) * 6, 54, True)):
        cfg = O.mp3d_cfg(n, 1.0 / 8, cfl=0.9, bc=bc)
        U = mp3d_state(cfg, n, seed, sharp)
        R, dt, rc = O.ref_mp3d_rhs(cfg, U)
        assert rc == 0
        U3, t3, dt3, rc3 = O.ref_mp3d_run(cfg, U, 3)
        assert rc3 == 0
        np.savez_compressed(os.path.join(HERE, f"ref_mp3d_{name}.npz"), U=U, RHS=R, dt=dt, U3=U3, t3=t3, dt3=dt3,
                            n=np.array(n), h=1.0 / 8, cfl=0.9, bc=np.array(bc), eos=np.array(O.MP3D_EOS),
                            mu=np.array(O.MP3D_MU))


def h2d_fixtures():
    """the 2d/HyPE-2D Kapila fixtures (RHS + dt, 3 steps) for N = 1 and N = 3"""
    for N in (1, 3):
        for name, bc, seed, sharp in (("mixed", (2, 2, 0, 0), 71, False), ("sharp", (0, 0, 2, 2), 72, True)):
            nx, ny, h = 9, 8, 1.0 / 9
            cfg = O.h2d_cfg(N, nx, ny, h, cfl=0.9, bc=bc)
            U = O.kp5_state(nx, ny, seed + N, sharp)
            R, dt, rc = O.ref_h2d_rhs(cfg, U)
            assert rc == 0
            U3, t3, dt3, rc3 = O.ref_h2d_run(cfg, U, 3)
            assert rc3 == 0
            np.savez_compressed(os.path.join(HERE, f"ref_h2d_n{N}_{name}.npz"), U=U, RHS=R, dt=dt, U3=U3, t3=t3,
                                N=N, nx=nx, ny=ny, h=h, cfl=0.9, bc=np.array(bc), eos=np.array(O.H2D_EOS))


def source_fixtures():
    """3d/weno4/point_source and 2d/weno4/line_source: the RHS at a time t of a random state
    and a run from rest (the program's initial condition) with the receiver's p.dat lines"""
    rng = np.random.default_rng(81)
    for name, bc in (("periodic", (0,) * 6), ("mixed", (4, 4, 0, 0, 4, 4))):
        n, h, dt, src, rec = 16, 0.5, 0.0005, (8, 8, 8), (11, 10, 9)
        cfg = O.acoustic_cfg(n, h, bc=bc, c=O.PSRC3D_C)
        U = 1e-3 * rng.standard_normal((n, n, n, 2))
        R, line = O.ref_psrc3d_rhs(cfg, src, rec, 0.037, U)
        Un, tn, pdat = O.ref_psrc3d_run(cfg, src, rec, np.zeros_like(U), 24, dt, initial_rhs=True)
        np.savez_compressed(os.path.join(HERE, f"ref_psrc3d_{name}.npz"), U=U, RHS=R, t_rhs=0.037, line=line, Un=Un,
                            tn=tn, pdat=pdat, steps=24, dt=dt, h=h, n=n, bc=np.array(bc), src=np.array(src),
                            rec=np.array(rec), c=O.PSRC3D_C, f0=O.PSRC3D_F0)
    for name, bc, stepper in (("periodic", (0,) * 4, 1), ("mixed", (4, 4, 0, 0), 0)):
        n, h, dt, src, rec = 48, 1.0, 0.001, (24, 24), (30, 28)
        cfg = O.sw2d_cfg(n, n, h, bc=bc, c=O.LSRC2D_C)
        U = 1e-3 * rng.standard_normal((n, n, 2))
        R, line = O.ref_lsrc2d_rhs(cfg, src, rec, 0.05, U)
        Un, tn, pdat = O.ref_lsrc2d_run(cfg, src, rec, np.zeros_like(U), 30, dt, stepper=stepper)
        np.savez_compressed(os.path.join(HERE, f"ref_lsrc2d_{name}.npz"), U=U, RHS=R, t_rhs=0.05, line=line, Un=Un,
                            tn=tn, pdat=pdat, steps=30, dt=dt, h=h, n=n, bc=np.array(bc), src=np.array(src),
                            rec=np.array(rec), c=O.LSRC2D_C, f0=O.LSRC2D_F0, stepper=stepper)


def main():
    O.build(REF)
    src = os.path.join(REF, "3d/ctcs/point_source/results/p.dat")
    with open(src) as f, open(os.path.join(HERE, "point_source_p.dat"), "w") as g:
        g.write(f.read())
    tables = {"standing_wave_2d_Error_dat": [], "plane_wave_3d_main_tex": []}
    with open(os.path.join(REF, "2d/weno4/standing_wave/results/Error.dat")) as f:
        for line in f:
            if line.strip():
                tables["standing_wave_2d_Error_dat"].append([float(v) for v in line.split()])
    tables["plane_wave_3d_main_tex"] = [[16, 7.23e-03, 6.48e-04], [32, 5.06e-04, 4.54e-05], [64, 3.15e-05, 2.82e-06],
                                        [128, 1.94e-06, 1.74e-07]]
    with open(os.path.join(HERE, "accuracy_tables.json"), "w") as f:
        json.dump(tables, f, indent=1)
    for flux, tag in ((0, ""), (1, "_hllc"), (2, "_rothllc")):
        for name, n, seed, bc in CASES:
            if flux and name == "mixed":
                continue
            cfg = O.euler_cfg(n, 1.0 / n, cfl=0.4, bc=bc, flux=flux)
            U = euler_case(n, seed, bc, vel=0.05 if flux == 0 else 0.2)
            R, dt, rc = O.ref_euler_rhs(cfg, U)
            assert rc == 0
            U3, t3, dt3, rc3 = O.ref_euler_run(cfg, U, 3)
            assert rc3 == 0
            np.savez_compressed(os.path.join(HERE, f"ref_euler_{name}{tag}.npz"), U=U, RHS=R, dt=dt, U3=U3, t3=t3,
                                dt3=dt3, bc=np.array(bc), n=n, cfl=0.4, flux=flux)
    for name, n, seed, bc in CASES:  # 3d/weno3/Euler: WENO3, Rusanov, dt fixed by the first RHS call
        cfg = O.euler_cfg(n, 1.0 / n, cfl=0.4, bc=bc, recon=3)
        U = euler_case(n, seed + 100, bc, vel=0.1)
        R, dt, rc = O.ref_euler_rhs(cfg, U)
        assert rc == 0
        U3, t3, dt3, rc3 = O.ref_euler_run(cfg, U, 3, dt_mode=1)
        assert rc3 == 0
        np.savez_compressed(os.path.join(HERE, f"ref_euler_{name}_weno3.npz"), U=U, RHS=R, dt=dt, U3=U3, t3=t3,
                            dt3=dt3, bc=np.array(bc), n=n, cfl=0.4, flux=0, recon=3, dt_mode=1)
    for name, bc, seed in (("periodic", (0,) * 6, 31), ("adiabatic", (4,) * 6, 32), ("mixed", (4, 4, 0, 0, 4, 4), 33)):
        shape = (7, 6, 5)
        cfg = O.acoustic_cfg(shape, 0.3, bc=bc)
        U = np.random.default_rng(seed).standard_normal((shape[2], shape[1], shape[0], 2))
        R = O.ref_acoustic_rhs(cfg, U)
        U3, t3 = O.ref_acoustic_run(cfg, U, 3, 0.01)
        np.savez_compressed(os.path.join(HERE, f"ref_acoustic_{name}.npz"), U=U, RHS=R, U3=U3, t3=t3, dt=0.01, h=0.3,
                            shape=np.array(shape), bc=np.array(bc))
    ns3d_fixtures()
    sw2d_fixtures()
    mp3d_fixtures()
    h2d_fixtures()
    source_fixtures()
    n = 32
    x = -1 + np.arange(n) * (2.0 / n)
    Xg, Yg = np.meshgrid(x, x)
    p0 = np.exp(-(Xg**2 + Yg**2) / (2 * 0.2**2))
    a, b, rc = O.ref_ctcs2d_run(p0, 0.999 * p0, 2.0 / n, 1.0, 0.5 * 2.0 / n, 1, 25)
    assert rc == 0
    np.savez_compressed(os.path.join(HERE, "ref_ctcs2d.npz"), p0=p0, p1=0.999 * p0, h=2.0 / n, dt=0.5 * 2.0 / n,
                        steps=25, p_old=a, p=b)
    # 2D diffuse-interface RHS of 2d/weno4/bubble (its compiled-in EOS), smooth and sharp interfaces
    for name, smear, nst in (("smooth", 2.0, 3), ("sharp", 0.05, 2)):
        nx, ny, h = 22, 18, 1.0 / 22
        cfg = O.mp2d_cfg(nx, ny, h, -0.5, -0.45, cfl=0.9, bc=(1, 2, 0, 0) if name == "sharp" else (1, 2, 2, 2))
        U = bubble_state(nx, ny, h, -0.5, -0.45, smear=smear, seed=7)
        R, dt, rc = O.ref_bubble_rhs(cfg, U)
        assert rc == 0
        U3, t3, dt3, rc3 = O.ref_bubble_run(cfg, U, nst)
        assert rc3 == 0
        np.savez_compressed(os.path.join(HERE, f"ref_bubble_{name}.npz"), U=U, RHS=R, dt=dt, U3=U3, t3=t3, dt3=dt3,
                            bc=np.array(list(cfg.bc)), nx=nx, ny=ny, h=h, xmin=-0.5, ymin=-0.45, cfl=0.9, steps=nst)
    print("golden fixtures written to", HERE)


def bubble_state(nx, ny, h, xmin, ymin, R0=0.3, smear=2.0, seed=None):
    """bubble_collapse-like primitive field (2d/weno4/bubble/initial_condition.c:173-202
    shape, smaller radius), with seeded velocities, as conserved variables"""
    x = xmin + (np.arange(nx) + 0.5) * h
    y = ymin + (np.arange(ny) + 0.5) * h
    X, Y = np.meshgrid(x, y)
    th = np.tanh((np.sqrt(X**2 + Y**2) - R0) / (smear * h))
    V = np.zeros((ny, nx, 5))
    V[..., 0] = 0.5 * ((1e-2 + 1.0) + (1.0 - 1e-2) * th)
    V[..., 3] = 0.5 * ((1.0 + 100.0) + (100.0 - 1.0) * th)
    V[..., 4] = 0.5 * ((0.0 + 1.0) + (1.0 - 0.0) * th)
    if seed is not None:
        rng = np.random.default_rng(seed)
        V[..., 1:3] = 0.1 * rng.standard_normal((ny, nx, 2))
    return O.mp_prim2cons(0, O.BUBBLE_EOS, V)


if __name__ == "__main__":
    main()
