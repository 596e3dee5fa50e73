"""The analytic receiver signals the source programs are compared with (the kernel of
2d/weno4/line_source/results/green.py): the quadrature of the 2D convolution against a
brute-force sum of the sampled kernel, and the 3D signal's delay and amplitude."""
import numpy as np

from acoustic_petsc_gb300 import analytic


def test_line_source_quadrature_matches_sampled_convolution():
    c, f0, r = 580.0, 65.0, 80 * np.sqrt(2.0)
    t = np.linspace(0.0, 0.5, 26)
    u = analytic.line_source_receiver_2d(t, r, c, f0)
    # green.py's discrete convolution, with a 1e-6 s sampling and the kernel averaged over
    # each sample interval (its integrable singularity at t = r/c otherwise dominates)
    dt = 1e-6
    tau = np.arange(0.0, 0.5 + dt, dt)
    src = analytic.source_wavelet(tau, f0)
    a = np.maximum(tau - r / c, 0.0)
    b = np.maximum(tau + dt - r / c, 0.0)
    # int of 1/sqrt(s (s + 2r/c)) ds = 2 asinh(sqrt(s c / (2 r)))
    Gint = (2 * np.arcsinh(np.sqrt(b * c / (2 * r))) - 2 * np.arcsinh(np.sqrt(a * c / (2 * r)))) / (2 * np.pi * c * c)
    m = 1 << int(np.ceil(np.log2(2 * len(tau))))
    conv = np.fft.irfft(np.fft.rfft(src, m) * np.fft.rfft(Gint, m), m)[: len(tau)]
    ref = np.interp(t, tau, conv)
    assert analytic.relative_l2_misfit(u, ref) < 1e-3


def test_point_source_signal_delay_and_amplitude():
    c, f0, r = 250.0, 100.0, 6.0
    t = np.linspace(0.0, 0.2, 20001)
    u = analytic.point_source_receiver_3d(t, r, c, f0)
    s = analytic.source_wavelet(t, f0)
    shift = int(round((r / c) / (t[1] - t[0])))
    assert np.allclose(u[shift:], s[: len(t) - shift] / (4 * np.pi * c * c * r), rtol=0, atol=1e-9 * np.abs(u).max())
    assert abs(np.abs(u).max() - np.abs(s).max() / (4 * np.pi * c * c * r)) <= 1e-6 * np.abs(u).max()


def test_reference_ctcs_point_source_trace_matches_analytic_signal():
    """the reference's own receiver trace of 3d/ctcs/point_source (results/p.dat, the same
    source, receiver and grid as 3d/weno4/point_source: h = 0.5, c = 250, f0 = 100, 7 cells
    apart on the diagonal) against S(t - r/c) / (4 pi c^2 r): 0.27 % relative L2"""
    import os

    from conftest import GOLDEN

    d = np.loadtxt(os.path.join(GOLDEN, "point_source_p.dat"))
    ua = analytic.point_source_receiver_3d(d[:, 0], 7 * np.sqrt(3.0) * 0.5, 250.0, 100.0)
    assert analytic.relative_l2_misfit(d[:, 1], ua) < 5e-3
