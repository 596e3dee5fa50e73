"""The C ABI library: it loads without a GPU, exports every entry point that
include/hype_gpu.h declares, and validates arguments before touching CUDA."""
import ctypes as C
import os
import re

from conftest import ROOT


def _declared():
    with open(os.path.join(ROOT, "include", "hype_gpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"\b(hype_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(hype):
    L = hype.lib()
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(hype._lib.SYMBOLS)


def test_version_and_strerror(hype):
    L = hype.lib()
    assert b"sm_103a" in L.hype_version()
    assert L.hype_strerror(2).startswith(b"inadmissible")


def test_invalid_arguments_rejected_without_gpu(hype):
    L = hype.lib()
    H = hype._lib
    p = H.EulerParams()
    p.nx = p.ny = p.nz = 2  # too small
    p.h, p.cfl, p.gamma = 0.1, 0.4, 1.4
    h = C.c_void_p()
    assert L.hype_euler_create(C.byref(p), C.byref(h)) == H.HYPE_ERR_ARG
    p.nx = p.ny = p.nz = 8
    p.bc[0] = H.BC_PERIODIC
    p.bc[1] = H.BC_REFLECTIVE  # periodic must be paired
    assert L.hype_euler_create(C.byref(p), C.byref(h)) == H.HYPE_ERR_ARG
    c = H.CtcsParams()
    c.dim = 4
    assert L.hype_ctcs_create(C.byref(c), C.byref(h)) == H.HYPE_ERR_ARG
    m = (H.MonoInstance * 1)()
    m[0].nx = 2
    assert L.hype_batch_create(1, m, C.byref(h)) == H.HYPE_ERR_ARG
    assert L.hype_euler_step(None, 1, None, None, None) == H.HYPE_ERR_ARG
    # the learned gate's per-step option and flag readback, 3D and 2D
    buf = (C.c_ubyte * 8)()
    assert L.hype_euler_set_gate_per_step(None, 1) == H.HYPE_ERR_ARG
    assert L.hype_euler_gate_flags(None, buf, 0) == H.HYPE_ERR_ARG
    assert L.hype_mp2d_set_gate_per_step(None, 1) == H.HYPE_ERR_ARG
    assert L.hype_mp2d_gate_flags(None, buf, 1) == H.HYPE_ERR_ARG


def test_library_is_in_tree(hype):
    path = hype._lib.library_path()
    assert os.path.commonpath([path, ROOT]) == ROOT and os.path.exists(path)
