"""The allocation-free RHS entry point (hype_euler_rhs_noalloc).

It exists for callers that cannot let the library allocate device memory (a
host that owns all device memory through its own pool and passes pre-allocated
device vectors, or a latency-critical loop that cannot afford cudaMalloc's
implicit synchronisation).  It must give what the context-based entry point
hype_euler_rhs_device gives on the same device inputs, call after call, even
though every call reuses the same fixed scratch array.  This file is collected
last so that a failure here never hides the other tests' results.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 RHS parity tolerance used throughout the GPU tests


def _state(shape, seed):
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    U = np.zeros((nz, ny, nx, 5))
    U[..., 0] = 1.0 + 0.2 * rng.random((nz, ny, nx))
    U[..., 1:4] = 0.1 * rng.standard_normal((nz, ny, nx, 3))
    U[..., 4] = (1 / 1.4 + 0.1 * rng.random((nz, ny, nx))) / 0.4 + 0.5 * (U[..., 1:4] ** 2).sum(-1) / U[..., 0]
    return U


def _params(hype, shape, bc, **kw):
    nx, ny, nz = shape
    ctx = hype.AppCtx(N_x=nx, N_y=ny, N_z=nz, h=1.0 / nx, CFL=0.4, boundaries=bc, **kw)
    return ctx, ctx.params()


def _soa(torch, U):
    return torch.from_numpy(np.ascontiguousarray(U.transpose(3, 0, 1, 2))).reshape(-1).to("cuda")


def _existing(hype, torch, ctx, dU):
    """RHS through the context-based entry point (the reference result here)."""
    s = hype.EulerSolver(ctx)
    out = torch.empty_like(dU)
    dt = C.c_double()
    rc = hype.lib().hype_euler_rhs_device(s._h, 0.0, C.c_void_p(dU.data_ptr()), C.c_void_p(out.data_ptr()),
                                          C.byref(dt))
    assert rc == 0
    s.close()
    return out.cpu().numpy(), dt.value


def _noalloc(hype, torch, params, dU, stream=None, want_dt=True):
    out = torch.full_like(dU, float("nan"))
    dt = C.c_double()
    handle = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = hype.lib().hype_euler_rhs_noalloc(C.byref(params), C.c_void_p(dU.data_ptr()), C.c_void_p(out.data_ptr()),
                                           C.byref(dt) if want_dt else None, handle)
    assert rc == 0, hype._lib.errstr(rc)
    if stream is not None:
        stream.synchronize()
    else:
        torch.cuda.synchronize()
    return out.cpu().numpy(), dt.value


def test_noalloc_matches_existing_entry_on_two_calls_in_a_row(hype):
    torch = pytest.importorskip("torch")
    cases = [((16, 16, 16), (0,) * 6, 21), ((13, 9, 11), (1, 1, 2, 2, 1, 2), 22)]
    for shape, bc, seed in cases:  # two consecutive calls with different grids share the scratch
        ctx, params = _params(hype, shape, bc)
        dU = _soa(torch, _state(shape, seed))
        got, dt_got = _noalloc(hype, torch, params, dU)
        want, dt_want = _existing(hype, torch, ctx, dU)
        assert np.abs(got - want).max() <= TOL * np.abs(want).max()
        assert abs(dt_got - dt_want) <= TOL * dt_want
    # and the same grid twice in a row: the second call must not see the first call's leftovers
    ctx, params = _params(hype, (16, 16, 16), (0,) * 6)
    dU = _soa(torch, _state((16, 16, 16), 23))
    a, _ = _noalloc(hype, torch, params, dU)
    b, _ = _noalloc(hype, torch, params, dU)
    want, _ = _existing(hype, torch, ctx, dU)
    assert np.abs(a - want).max() <= TOL * np.abs(want).max()
    assert np.abs(b - want).max() <= TOL * np.abs(want).max()


def test_noalloc_rejects_grids_beyond_the_fixed_scratch(hype):
    torch = pytest.importorskip("torch")
    assert hype.lib().hype_euler_noalloc_max_ext() == 18 ** 3
    ctx, params = _params(hype, (17, 16, 16), (0,) * 6)
    dU = torch.zeros(5 * 17 * 16 * 16, dtype=torch.float64, device="cuda")
    out = torch.zeros_like(dU)
    rc = hype.lib().hype_euler_rhs_noalloc(C.byref(params), C.c_void_p(dU.data_ptr()), C.c_void_p(out.data_ptr()),
                                           None, None)
    assert rc == hype._lib.HYPE_ERR_ARG


# precision (FP64, FP32) x flux (Rusanov, HLLC, rotated HLLC) x reconstruction (CWENO4, R4, WENO3)
OPTIONS = [(prec, flux, recon) for prec in (0, 1) for flux in (0, 1, 2) for recon in (0, 1, 3)]


@pytest.mark.parametrize("prec,flux,recon", OPTIONS)
def test_noalloc_options_match_existing_entry(hype, prec, flux, recon):
    """every option the entry point accepts gives the context path's result, FP32 traces and
    fluxes included (their layout inside the fixed array differs from the FP64 one); odd grid,
    mixed boundaries"""
    torch = pytest.importorskip("torch")
    shape, bc = (13, 9, 11), (1, 1, 2, 2, 0, 0)
    ctx, params = _params(hype, shape, bc, precision=prec, flux=flux, recon=recon)
    dU = _soa(torch, _state(shape, 31 + flux + 3 * recon))
    got, dt_got = _noalloc(hype, torch, params, dU)
    want, dt_want = _existing(hype, torch, ctx, dU)
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    assert abs(dt_got - dt_want) <= TOL * dt_want


def test_noalloc_against_the_oracle(hype, oracle):
    """the odd 13x9x11 grid with mixed boundaries directly against the CPU checker's RHS"""
    torch = pytest.importorskip("torch")
    shape, bc = (13, 9, 11), (1, 1, 2, 2, 1, 2)
    U = _state(shape, 22)
    _, params = _params(hype, shape, bc)
    got, dt_got = _noalloc(hype, torch, params, _soa(torch, U))
    Ro, smax, rc, _ = oracle.euler_rhs(oracle.euler_cfg(shape, 1.0 / shape[0], cfl=0.4, bc=bc), U)
    assert rc == 0
    want = np.ascontiguousarray(Ro.transpose(3, 0, 1, 2)).reshape(-1)
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    assert abs(dt_got - 0.4 / shape[0] / (3.0 * smax)) <= TOL * dt_got


def test_noalloc_on_a_stream_without_dt(hype):
    """a caller's stream and dt_out = NULL (the call returns without waiting): the result,
    read after that stream is synchronised, equals the context path's"""
    torch = pytest.importorskip("torch")
    shape, bc = (12, 10, 14), (0, 0, 1, 1, 2, 2)
    ctx, params = _params(hype, shape, bc)
    dU = _soa(torch, _state(shape, 41))
    st = torch.cuda.Stream()
    got, _ = _noalloc(hype, torch, params, dU, stream=st, want_dt=False)
    want, _ = _existing(hype, torch, ctx, dU)
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_positivity_fallback(hype, prec):
    """positivity = 1: a state whose high-order traces break the density floor next to a
    near-vacuum cell falls back to first order there, as the context path does"""
    torch = pytest.importorskip("torch")
    shape, bc = (14, 12, 10), (2, 2, 2, 2, 2, 2)
    U = _state(shape, 51)
    U[5, 6, 7, 0] = 1e-9
    U[5, 6, 7, 1:4] = 0.0
    U[5, 6, 7, 4] = 1e-6
    ctx, params = _params(hype, shape, bc, precision=prec, positivity=1)
    dU = _soa(torch, U)
    got, dt_got = _noalloc(hype, torch, params, dU)
    want, dt_want = _existing(hype, torch, ctx, dU)
    assert np.isfinite(got).all()
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    assert abs(dt_got - dt_want) <= TOL * dt_want
