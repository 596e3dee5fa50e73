"""ctypes binding of ``libhype_gb300.so`` (the C ABI of ``include/hype_gpu.h``).

There is no CPU fallback: when the library is missing or cannot be loaded,
``lib()`` raises.  Structures mirror the header field by field.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

_L = None

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
F = C.POINTER(C.c_float)

HYPE_OK, HYPE_ERR_ARG, HYPE_ERR_STATE, HYPE_ERR_CUDA, HYPE_ERR_NOMEM, HYPE_ERR_UNSUPPORTED = range(6)
BC_PERIODIC, BC_REFLECTIVE, BC_TRANSMISSIVE, BC_ZERO, BC_ADIABATIC = range(5)
RECON_CWENO4, RECON_LINEAR4, RECON_LEARNED, RECON_WENO3 = 0, 1, 2, 3
PREC_FP64, PREC_FP32, PREC_DF64 = 0, 1, 2
DT_MONITOR, DT_FROZEN, DT_FIXED = 0, 1, 2
FLUX_RUSANOV, FLUX_HLLC, FLUX_ROTHLLC = 0, 1, 2
MP_DI4, MP_KAPILA5 = 0, 1
STEP_SSPRK43, STEP_SSPRK104 = 0, 1
STAGE_AUTO, STAGE_UNFUSED = 0, 1

# every entry point the header declares (checked by the CPU test suite)
SYMBOLS = [
    "hype_euler_create", "hype_euler_destroy", "hype_euler_rhs", "hype_euler_rhs_device", "hype_euler_upload",
    "hype_euler_download", "hype_euler_state_device", "hype_euler_step", "hype_euler_sync",
    "hype_ctcs2d_update", "hype_ctcs_create", "hype_ctcs_destroy", "hype_ctcs_set", "hype_ctcs_get",
    "hype_ctcs_step", "hype_ctcs_level_device", "hype_ctcs_sync",
    "hype_batch_create", "hype_batch_destroy", "hype_batch_set_tile", "hype_batch_get_tile", "hype_batch_set",
    "hype_batch_get",
    "hype_batch_step", "hype_batch_sync", "hype_batch_set_classes", "hype_batch_get_classes",
    "hype_batch_instance_times",
    "hype_strerror", "hype_last_error", "hype_launch_count", "hype_version",
    "hype_euler_stream", "hype_euler_profile", "hype_euler_profile_read", "hype_set_device", "hype_device_count",
    "hype_euler_rhs_noalloc", "hype_euler_noalloc_max_ext", "hype_euler_set_stage_kernel",
    "hype_mp2d_create", "hype_mp2d_destroy", "hype_mp2d_rhs", "hype_mp2d_upload", "hype_mp2d_download",
    "hype_mp2d_step", "hype_mp2d_sync", "hype_mp2d_stream", "hype_mp2d_set_mlp", "hype_mp2d_set_recon",
    "hype_mp2d_indicator_stats", "hype_mp2d_set_gate_per_step", "hype_mp2d_gate_flags", "hype_mp2d_sample_features",
    "hype_euler_get_params", "hype_mp2d_get_params",
    "hype_write_petsc_vec", "hype_read_petsc_vec", "hype_write_vtk", "hype_euler_write_restart",
    "hype_euler_read_restart", "hype_euler_write_vtk", "hype_mp2d_write_restart", "hype_mp2d_read_restart",
    "hype_mp2d_write_vtk", "hype_acoustic_create", "hype_acoustic_destroy", "hype_acoustic_upload",
    "hype_acoustic_download", "hype_acoustic_rhs", "hype_acoustic_step", "hype_acoustic_sync", "hype_acoustic_stream",
    "hype_acoustic_rhs_t", "hype_acoustic_set_point_source", "hype_acoustic_trace", "hype_acoustic2d_rhs_t",
    "hype_acoustic2d_set_point_source", "hype_acoustic2d_trace",
    "hype_euler_set_mlp", "hype_euler_set_recon", "hype_euler_indicator_stats", "hype_euler_set_gate_per_step",
    "hype_euler_gate_flags", "hype_euler_sample_features",
    "hype_mlp_nparam", "hype_mlp_score", "hype_mlp_grad", "hype_mlp_train", "hype_euler_shadow_step",
    "hype_euler_monitor", "hype_acoustic2d_create", "hype_acoustic2d_destroy", "hype_acoustic2d_upload",
    "hype_acoustic2d_download", "hype_acoustic2d_rhs", "hype_acoustic2d_step", "hype_acoustic2d_sync",
    "hype_acoustic2d_stream", "hype_mp3d_create", "hype_mp3d_destroy", "hype_mp3d_get_params", "hype_mp3d_rhs",
    "hype_mp3d_upload", "hype_mp3d_download", "hype_mp3d_step", "hype_mp3d_sync", "hype_mp3d_stream",
    "hype_pc2d_create", "hype_pc2d_destroy", "hype_pc2d_get_params", "hype_pc2d_rhs", "hype_pc2d_upload",
    "hype_pc2d_download", "hype_pc2d_step", "hype_pc2d_sync", "hype_pc2d_stream",
]


class HypeError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        msg = f"{where}: {errstr(code)}"
        if detail:
            msg += f" [{detail}]"
        super().__init__(msg)


class EulerParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("x_min", C.c_double), ("y_min", C.c_double), ("z_min", C.c_double), ("h", C.c_double),
                ("cfl", C.c_double), ("gamma", C.c_double), ("bc", C.c_int * 6),
                ("recon", C.c_int), ("precision", C.c_int), ("dt_mode", C.c_int), ("flux", C.c_int),
                ("positivity", C.c_int), ("mu", C.c_double), ("prandtl", C.c_double), ("cv", C.c_double)]


class Mp2dParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("x_min", C.c_double), ("y_min", C.c_double), ("h", C.c_double),
                ("cfl", C.c_double), ("bc", C.c_int * 4), ("model", C.c_int), ("g1", C.c_double), ("p1", C.c_double),
                ("g2", C.c_double), ("p2", C.c_double), ("stepper", C.c_int), ("precision", C.c_int),
                ("dt_mode", C.c_int), ("recon", C.c_int)]


class AcousticParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("x_min", C.c_double), ("y_min", C.c_double),
                ("z_min", C.c_double), ("h", C.c_double), ("c", C.c_double), ("dt", C.c_double), ("bc", C.c_int * 6),
                ("recon", C.c_int), ("precision", C.c_int)]


class Status(C.Structure):
    _fields_ = [("bad_cell", C.c_longlong), ("smax", C.c_double), ("rhs_evals", C.c_longlong)]


class Pc2dParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("x_min", C.c_double), ("y_min", C.c_double), ("h", C.c_double),
                ("cfl", C.c_double), ("bc", C.c_int * 4), ("order", C.c_int), ("g1", C.c_double), ("p1", C.c_double),
                ("g2", C.c_double), ("p2", C.c_double)]


class Mp3dParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("x_min", C.c_double), ("y_min", C.c_double),
                ("z_min", C.c_double), ("h", C.c_double), ("cfl", C.c_double), ("bc", C.c_int * 6),
                ("g1", C.c_double), ("p1", C.c_double), ("g2", C.c_double), ("p2", C.c_double), ("mu1", C.c_double),
                ("mu2", C.c_double), ("dt_mode", C.c_int)]


class Acoustic2dParams(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("x_min", C.c_double), ("y_min", C.c_double), ("h", C.c_double),
                ("c", C.c_double), ("dt", C.c_double), ("bc", C.c_int * 4), ("stepper", C.c_int)]


class CtcsParams(C.Structure):
    _fields_ = [("dim", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("form", C.c_int), ("order", C.c_int), ("bc", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double), ("dt", C.c_double),
                ("c0", C.c_double), ("f0", C.c_double), ("src", C.c_int * 3), ("rec", C.c_int * 3)]


class MonoInstance(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("xmin", C.c_double), ("ymin", C.c_double),
                ("h", C.c_double), ("c0", C.c_double), ("dt", C.c_double), ("xs", C.c_double),
                ("ys", C.c_double), ("sigma", C.c_double), ("freq", C.c_double)]


def library_path() -> str:
    return _build.LIB


def lib():
    """Load the library (building it first if only the sources exist)."""
    global _L
    if _L is not None:
        return _L
    path = _build.LIB
    if not os.path.exists(path):
        _build.build()
    L = C.CDLL(path)
    V = C.c_void_p
    P = C.POINTER
    sig = {
        "hype_euler_create": ([P(EulerParams), P(V)], C.c_int),
        "hype_euler_destroy": ([V], None),
        "hype_euler_rhs": ([V, C.c_double, D, D, D], C.c_int),
        "hype_euler_set_stage_kernel": ([V, C.c_int], C.c_int),
        "hype_euler_rhs_device": ([V, C.c_double, V, V, D], C.c_int),
        "hype_euler_upload": ([V, D], C.c_int),
        "hype_euler_download": ([V, D], C.c_int),
        "hype_euler_state_device": ([V], C.c_void_p),
        "hype_euler_step": ([V, C.c_int, D, D, P(Status)], C.c_int),
        "hype_euler_sync": ([V], C.c_int),
        "hype_ctcs2d_update": ([C.c_int, C.c_int, C.c_double, C.c_int, D, D, D], C.c_int),
        "hype_ctcs_create": ([P(CtcsParams), P(V)], C.c_int),
        "hype_ctcs_destroy": ([V], None),
        "hype_ctcs_set": ([V, D, D], C.c_int),
        "hype_ctcs_get": ([V, D, D], C.c_int),
        "hype_ctcs_step": ([V, C.c_int, C.c_int, D], C.c_int),
        "hype_ctcs_level_device": ([V, C.c_int], C.c_void_p),
        "hype_ctcs_sync": ([V], C.c_int),
        "hype_batch_create": ([C.c_int, P(MonoInstance), P(V)], C.c_int),
        "hype_batch_destroy": ([V], None),
        "hype_batch_set_tile": ([V, C.c_int, C.c_int], C.c_int),
        "hype_batch_get_tile": ([V, I, I], C.c_int),
        "hype_batch_set": ([V, C.c_int, D, D], C.c_int),
        "hype_batch_get": ([V, C.c_int, D, D], C.c_int),
        "hype_batch_step": ([V, C.c_int, C.c_int], C.c_int),
        "hype_batch_set_classes": ([V, C.c_int], C.c_int),
        "hype_batch_get_classes": ([V, I, I], C.c_int),
        "hype_batch_instance_times": ([V, D], C.c_int),
        "hype_batch_sync": ([V], C.c_int),
        "hype_strerror": ([C.c_int], C.c_char_p),
        "hype_last_error": ([], C.c_char_p),
        "hype_launch_count": ([], C.c_longlong),
        "hype_version": ([], C.c_char_p),
        "hype_euler_stream": ([V], C.c_void_p),
        "hype_euler_monitor": ([V, D, D], C.c_int),
        "hype_euler_profile": ([V, C.c_int], C.c_int),
        "hype_euler_profile_read": ([V, D, P(C.c_longlong)], C.c_int),
        "hype_set_device": ([C.c_int], C.c_int),
        "hype_device_count": ([P(C.c_int)], C.c_int),
        "hype_euler_rhs_noalloc": ([P(EulerParams), V, V, D, V], C.c_int),
        "hype_euler_noalloc_max_ext": ([], C.c_longlong),
        "hype_mp2d_create": ([P(Mp2dParams), P(V)], C.c_int),
        "hype_mp2d_destroy": ([V], None),
        "hype_mp2d_rhs": ([V, C.c_double, D, D, D], C.c_int),
        "hype_mp2d_upload": ([V, D], C.c_int),
        "hype_mp2d_download": ([V, D], C.c_int),
        "hype_mp2d_step": ([V, C.c_int, D, D, P(C.c_longlong)], C.c_int),
        "hype_mp2d_sync": ([V], C.c_int),
        "hype_mp2d_stream": ([V], C.c_void_p),
        "hype_mp2d_set_mlp": ([V, F, C.c_float], C.c_int),
        "hype_mp2d_set_recon": ([V, C.c_int], C.c_int),
        "hype_mp2d_indicator_stats": ([V, P(C.c_longlong), C.c_int], C.c_int),
        "hype_mp2d_set_gate_per_step": ([V, C.c_int], C.c_int),
        "hype_mp2d_gate_flags": ([V, C.c_void_p, C.c_int], C.c_int),
        "hype_mp2d_sample_features": ([V, C.c_longlong, F, F, P(C.c_longlong)], C.c_int),
        "hype_euler_get_params": ([V, P(EulerParams)], C.c_int),
        "hype_mp2d_get_params": ([V, P(Mp2dParams)], C.c_int),
        "hype_write_petsc_vec": ([C.c_char_p, D, C.c_longlong, C.c_int], C.c_int),
        "hype_read_petsc_vec": ([C.c_char_p, D, C.c_longlong], C.c_int),
        "hype_write_vtk": ([C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                            C.c_double, C.c_int, P(C.c_char_p), D], C.c_int),
        "hype_euler_write_restart": ([V, C.c_char_p], C.c_int),
        "hype_euler_read_restart": ([V, C.c_char_p], C.c_int),
        "hype_euler_write_vtk": ([V, C.c_char_p], C.c_int),
        "hype_mp2d_write_restart": ([V, C.c_char_p], C.c_int),
        "hype_mp2d_read_restart": ([V, C.c_char_p], C.c_int),
        "hype_mp2d_write_vtk": ([V, C.c_char_p], C.c_int),
        "hype_acoustic_create": ([P(AcousticParams), P(V)], C.c_int),
        "hype_acoustic_destroy": ([V], None),
        "hype_acoustic_upload": ([V, D], C.c_int),
        "hype_acoustic_download": ([V, D], C.c_int),
        "hype_acoustic_rhs": ([V, D, D], C.c_int),
        "hype_acoustic_step": ([V, C.c_int, C.c_double, D, I], C.c_int),
        "hype_acoustic_sync": ([V], C.c_int),
        "hype_acoustic_stream": ([V], C.c_void_p),
        "hype_acoustic_rhs_t": ([V, C.c_double, D, D], C.c_int),
        "hype_acoustic_set_point_source": ([V, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                            C.c_int], C.c_int),
        "hype_acoustic_trace": ([V, D, D, C.c_int, P(C.c_longlong)], C.c_int),
        "hype_acoustic2d_create": ([P(Acoustic2dParams), P(V)], C.c_int),
        "hype_acoustic2d_destroy": ([V], None),
        "hype_acoustic2d_upload": ([V, D], C.c_int),
        "hype_acoustic2d_download": ([V, D], C.c_int),
        "hype_acoustic2d_rhs": ([V, D, D], C.c_int),
        "hype_acoustic2d_step": ([V, C.c_int, C.c_double, D, I], C.c_int),
        "hype_acoustic2d_sync": ([V], C.c_int),
        "hype_acoustic2d_stream": ([V], C.c_void_p),
        "hype_acoustic2d_rhs_t": ([V, C.c_double, D, D], C.c_int),
        "hype_acoustic2d_set_point_source": ([V, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int], C.c_int),
        "hype_acoustic2d_trace": ([V, D, D, C.c_int, P(C.c_longlong)], C.c_int),
        "hype_mp3d_create": ([P(Mp3dParams), P(V)], C.c_int),
        "hype_mp3d_destroy": ([V], None),
        "hype_mp3d_get_params": ([V, P(Mp3dParams)], C.c_int),
        "hype_mp3d_rhs": ([V, C.c_double, D, D, D], C.c_int),
        "hype_mp3d_upload": ([V, D], C.c_int),
        "hype_mp3d_download": ([V, D], C.c_int),
        "hype_mp3d_step": ([V, C.c_int, D, D, P(C.c_longlong)], C.c_int),
        "hype_mp3d_sync": ([V], C.c_int),
        "hype_mp3d_stream": ([V], C.c_void_p),
        "hype_pc2d_create": ([P(Pc2dParams), P(V)], C.c_int),
        "hype_pc2d_destroy": ([V], None),
        "hype_pc2d_get_params": ([V, P(Pc2dParams)], C.c_int),
        "hype_pc2d_rhs": ([V, C.c_double, D, D, D], C.c_int),
        "hype_pc2d_upload": ([V, D], C.c_int),
        "hype_pc2d_download": ([V, D], C.c_int),
        "hype_pc2d_step": ([V, C.c_int, D, D, P(C.c_longlong)], C.c_int),
        "hype_pc2d_sync": ([V], C.c_int),
        "hype_pc2d_stream": ([V], C.c_void_p),
        "hype_euler_set_mlp": ([V, F, C.c_float], C.c_int),
        "hype_euler_set_recon": ([V, C.c_int], C.c_int),
        "hype_euler_indicator_stats": ([V, P(C.c_longlong), P(C.c_longlong), C.c_int], C.c_int),
        "hype_euler_set_gate_per_step": ([V, C.c_int], C.c_int),
        "hype_euler_gate_flags": ([V, C.c_void_p, C.c_int], C.c_int),
        "hype_euler_sample_features": ([V, C.c_longlong, F, F, P(C.c_longlong)], C.c_int),
        "hype_euler_shadow_step": ([V, D, D, D], C.c_int),
        "hype_mlp_nparam": ([], C.c_int),
        "hype_mlp_score": ([F, C.c_int, F, F], C.c_int),
        "hype_mlp_grad": ([F, F, C.c_int, F, C.c_float, F, D], C.c_int),
        "hype_mlp_train": ([F, F, C.c_int, F, C.c_int, C.c_int, C.c_float, C.c_float, C.c_uint, D], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _L = L
    return L


_P = None


def probes():
    """The test and measurement library (libhype_probes.so: the FMA issue ceiling and the
    double-float primitive probe), kept out of the public C ABI; loaded after lib()."""
    global _P
    if _P is not None:
        return _P
    lib()
    if not os.path.exists(_build.PROBE_LIB):
        _build.build()
    P = C.CDLL(_build.PROBE_LIB)
    P.hype_probe_fma_peak.argtypes, P.hype_probe_fma_peak.restype = [C.c_int, D], C.c_int
    P.hype_df64_probe.argtypes, P.hype_df64_probe.restype = [D, D, C.c_longlong, D], C.c_int
    _P = P
    return P


def errstr(code: int) -> str:
    try:
        return lib().hype_strerror(code).decode()
    except Exception:  # pragma: no cover - message only
        return f"status {code}"


def check(code: int, where: str) -> None:
    if code != HYPE_OK:
        detail = lib().hype_last_error().decode() if code in (HYPE_ERR_CUDA, HYPE_ERR_ARG) else ""
        raise HypeError(code, where, detail)


def launches() -> int:
    return int(lib().hype_launch_count())
