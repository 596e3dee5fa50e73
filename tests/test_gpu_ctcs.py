"""CTCS leapfrog on the GPU: bit-identical to the CPU checker (which is
bit-identical to the reference's own C), and the 3D point-source receiver trace
reproduces the reference's checked-in p.dat."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_drop_in_single_update_bitwise(hype, oracle):
    rng = np.random.default_rng(1)
    p0, p1 = rng.random((33, 47)), rng.random((33, 47))
    for bc in (0, 3):
        out = hype.CTCS(p0, p1, 0.41, bc)
        _, ref = oracle.ctcs2d_plane(p0, p1, 0.41, bc, 1)
        assert np.array_equal(out, ref)


def test_golden_reference_ctcs2d(hype):
    z = np.load(os.path.join(GOLDEN, "ref_ctcs2d.npz"))
    lf = hype.Leapfrog(z["p0"].shape, dx=float(z["h"]), dt=float(z["dt"]), c0=1.0, form=0, bc=3)
    lf.set(z["p0"], z["p1"])
    lf.UpdatePressure(int(z["steps"]))
    a, b = lf.get()
    assert np.array_equal(a, z["p_old"]) and np.array_equal(b, z["p"])


@pytest.mark.parametrize("bc", [0, 3])
def test_plane_form_chunks_and_remainder_bitwise(hype, oracle, bc):
    from acoustic_petsc_gb300 import workloads

    p0, p1, h, dt, alpha = workloads.ctcs_gaussian(96)
    lf = hype.Leapfrog(p0.shape, dx=h, dt=dt, c0=1.0, form=0, bc=bc)
    lf.set(p0, p1)
    lf.UpdatePressure(77)  # two captured 30-step chunks + 17 direct launches
    lf.UpdatePressure(31)
    a, b = lf.get()
    ao, bo = oracle.ctcs2d_plane(p0, p1, alpha, bc, 108)
    assert np.array_equal(a, ao) and np.array_equal(b, bo)


def test_config1_512_1000_steps_bitwise(hype, oracle):
    """2D CTCS 512^2 on [-1,1]^2, c=1, CFL 0.5, zero-Dirichlet, Gaussian, 1000 steps."""
    from acoustic_petsc_gb300 import workloads

    p0, p1, h, dt, alpha = workloads.ctcs_gaussian(512)
    lf = hype.Leapfrog(p0.shape, dx=h, dt=dt, c0=1.0, form=0, bc=3)
    lf.set(p0, p1)
    lf.UpdatePressure(1000)
    a, b = lf.get()
    ao, bo = oracle.ctcs2d_plane(p0, p1, alpha, 3, 1000)
    assert np.array_equal(b, bo) and np.array_equal(a, ao)


def test_point_source_3d_reproduces_p_dat(hype, oracle):
    z = np.zeros((100, 100, 100))
    lf = hype.Leapfrog(z.shape, dx=0.5, dt=0.0005, c0=250.0, form=1, order=4, bc=0, f0=100.0, src=(50, 50, 50),
                       rec=(57, 57, 57))
    lf.set(z, z)
    rec = lf.UpdatePressure(251)
    text = "".join("%e\t%e\n" % (it * 0.0005, rec[it]) for it in range(251))
    with open(os.path.join(GOLDEN, "point_source_p.dat")) as f:
        assert text == f.read()
    cfg = oracle.CtcsCfg()
    cfg.dim, cfg.nx, cfg.ny, cfg.nz, cfg.order, cfg.bc = 3, 100, 100, 100, 4, 0
    cfg.dx = cfg.dy = cfg.dz = 0.5
    cfg.dt, cfg.c0, cfg.f0 = 0.0005, 250.0, 100.0
    cfg.src_i = cfg.src_j = cfg.src_k = 50
    cfg.rec_i = cfg.rec_j = cfg.rec_k = 57
    a, b, r = oracle.ctcs_pointsrc(cfg, z, z, 251, receiver=True)
    ga, gb = lf.get()
    assert np.array_equal(gb, b) and np.array_equal(ga, a) and np.array_equal(rec, r)


@pytest.mark.parametrize("order,bc", [(2, 3), (4, 0), (4, 3)])
def test_point_source_2d_bitwise(hype, oracle, order, bc):
    n = 70
    z = np.zeros((n, n))
    lf = hype.Leapfrog(z.shape, dx=1.0, dt=0.001, c0=300.0, form=1, order=order, bc=bc, f0=65.0, src=(30, 41),
                       rec=(50, 20))
    lf.set(z, z)
    rec = lf.UpdatePressure(95)
    cfg = oracle.CtcsCfg()
    cfg.dim, cfg.nx, cfg.ny, cfg.nz, cfg.order, cfg.bc = 2, n, n, 1, order, bc
    cfg.dx = cfg.dy = cfg.dz = 1.0
    cfg.dt, cfg.c0, cfg.f0 = 0.001, 300.0, 65.0
    cfg.src_i, cfg.src_j, cfg.src_k = 30, 41, 0
    cfg.rec_i, cfg.rec_j, cfg.rec_k = 50, 20, 0
    a, b, r = oracle.ctcs_pointsrc(cfg, z, z, 95, receiver=True)
    ga, gb = lf.get()
    assert np.array_equal(gb, b) and np.array_equal(rec, r)


def test_line_source_2d_program_matches_greens_function(hype):
    """2d/ctcs/line_source's program (500^2 nodes of h = 1, 4th-order stencil, c0 = 580,
    dt = 1e-3, 502 steps, periodic, source (250,250), receiver (330,330)) against its
    results/green.py comparison, the 2D Green's function convolved with the wavelet: 1.5 %
    relative L2 misfit with the CPU checker (second order in time), bound 3 %"""
    from acoustic_petsc_gb300 import analytic

    n = 500
    z = np.zeros((n, n))
    lf = hype.Leapfrog(z.shape, dx=1.0, dt=0.001, c0=580.0, form=1, order=4, bc=0, f0=65.0, src=(250, 250),
                       rec=(330, 330))
    lf.set(z, z)
    rec = lf.UpdatePressure(502)
    t = np.arange(502) * 0.001
    misfit = analytic.relative_l2_misfit(rec, analytic.line_source_receiver_2d(t, 80 * np.sqrt(2.0), 580.0, 65.0))
    print(f"CTCS line source 500^2: receiver misfit {misfit:.3e}")
    assert misfit < 0.03
