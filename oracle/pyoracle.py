"""ctypes bindings of the CPU checker (TEST INFRASTRUCTURE ONLY).

Importable by tests/, the smoke check and bench.py's CPU-baseline leg.  It
binds two things:

* ``liboracle.so`` -- the C restatement in ``hype_oracle.c`` (always built by
  ``build()``);
* ``_ref/*`` -- the reference's own C sources compiled in place through the
  PETSc shim (only where the reference tree is present when ``build()`` runs).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_ref_euler = None
_ref_ctcs2d = None

D = C.POINTER(C.c_double)


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


# where this recipe looks for the reference tree when HYPE_REF_DIR is not set (the
# container that builds the checker); the GPU machine has no reference tree
_REF_DEFAULT = "/root/reference"


def ref_dir() -> str | None:
    """The reference tree the checker compiles in place: HYPE_REF_DIR, else the recipe's
    default location; None where neither exists (then only the restatement is built)."""
    d = os.environ.get("HYPE_REF_DIR") or _REF_DEFAULT
    return d if os.path.isdir(d) else None


def build(ref: str | None = None, quiet: bool = True) -> None:
    """make the restatement; also the reference checker when the tree exists."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE, "liboracle"], check=True, stdout=out)
    ref_dir = ref or globals()["ref_dir"]()
    if ref_dir and os.path.isdir(ref_dir):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], check=True, stdout=out)


class EulerCfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("xmin", C.c_double), ("ymin", C.c_double), ("zmin", C.c_double),
                ("h", C.c_double), ("cfl", C.c_double), ("gamma", C.c_double),
                ("bc", C.c_int * 6), ("recon", C.c_int), ("nthreads", C.c_int), ("flux", C.c_int),
                ("positivity", C.c_int), ("mu", C.c_double), ("prandtl", C.c_double), ("cv", C.c_double)]


class CtcsCfg(C.Structure):
    _fields_ = [("dim", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("order", C.c_int), ("bc", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("dt", C.c_double), ("c0", C.c_double), ("f0", C.c_double),
                ("src_i", C.c_int), ("src_j", C.c_int), ("src_k", C.c_int),
                ("rec_i", C.c_int), ("rec_j", C.c_int), ("rec_k", C.c_int),
                ("it0", C.c_int)]


class MonoCfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int),
                ("xmin", C.c_double), ("ymin", C.c_double), ("h", C.c_double),
                ("c0", C.c_double), ("dt", C.c_double), ("xs", C.c_double), ("ys", C.c_double),
                ("sigma", C.c_double), ("freq", C.c_double), ("it0", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_euler_rhs.argtypes = [C.POINTER(EulerCfg), D, D, D, C.POINTER(C.c_long)]
        L.orc_acoustic_rhs.argtypes = [C.POINTER(AcousticCfg), D, D]
        L.orc_euler_last_smax_visc.argtypes = []
        L.orc_euler_last_smax_visc.restype = C.c_double
        L.orc_tgv_ic.argtypes = [C.POINTER(EulerCfg), D]
        L.orc_tgv_ic.restype = None
        L.orc_kinetic_energy.argtypes = [C.POINTER(EulerCfg), D]
        L.orc_kinetic_energy.restype = C.c_double
        L.orc_dissipation.argtypes = [C.POINTER(EulerCfg), D]
        L.orc_dissipation.restype = C.c_double
        L.orc_acoustic_run.argtypes = [C.POINTER(AcousticCfg), C.c_int, C.c_double, C.c_double, D, D,
                                       C.POINTER(C.c_int)]
        L.orc_acoustic_plane_wave_ic.argtypes = [C.POINTER(AcousticCfg), D]
        L.orc_acoustic_plane_wave_ic.restype = None
        L.orc_acoustic_plane_wave_errors.argtypes = [C.POINTER(AcousticCfg), D, C.c_double, D, D]
        L.orc_acoustic_plane_wave_errors.restype = None
        L.orc_euler_run.argtypes = [C.POINTER(EulerCfg), C.c_int, C.c_int, D, D, D, C.POINTER(C.c_long)]
        L.orc_mp3d_rhs.argtypes = [C.POINTER(Mp3dCfg), D, D, D, D, D]
        L.orc_mp3d_run.argtypes = [C.POINTER(Mp3dCfg), C.c_int, C.c_int, D, D, D]
        L.orc_mp3d_fallbacks.argtypes = [C.c_int]
        L.orc_mp3d_fallbacks.restype = C.c_long
        L.orc_mp3d_prim2cons.argtypes = [C.POINTER(Mp3dCfg), D, D]
        L.orc_mp3d_prim2cons.restype = None
        L.orc_mp3d_cons2prim.argtypes = [C.POINTER(Mp3dCfg), D, D]
        L.orc_mp3d_cons2prim.restype = None
        L.orc_h2d_rhs.argtypes = [C.POINTER(H2dCfg), D, D, D]
        L.orc_h2d_run.argtypes = [C.POINTER(H2dCfg), C.c_int, D, D, D]
        L.orc_sw2d_rhs.argtypes = [C.POINTER(Sw2dCfg), D, D]
        L.orc_sw2d_run.argtypes = [C.POINTER(Sw2dCfg), C.c_int, C.c_int, C.c_double, C.c_double, D, D,
                                   C.POINTER(C.c_int)]
        L.orc_sw2d_ic.argtypes = [C.POINTER(Sw2dCfg), D]
        L.orc_sw2d_ic.restype = None
        L.orc_sw2d_errors.argtypes = [C.POINTER(Sw2dCfg), D, C.c_double, D, D]
        L.orc_sw2d_errors.restype = None
        L.orc_ctcs2d_plane.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, D, D, D]
        L.orc_ctcs_pointsrc.argtypes = [C.POINTER(CtcsCfg), D, C.c_int, D, D, D, D]
        L.orc_ctcs_monopole.argtypes = [C.POINTER(MonoCfg), C.c_int, D, D, D]
        L.orc_cweno4_ref_args.argtypes = [D] * 8
        L.orc_eval_poly3.argtypes = [C.c_double, C.c_double, C.c_double, D]
        L.orc_eval_poly3.restype = C.c_double
        L.orc_rusanov.argtypes = [D, D, C.c_int, C.c_double, D, C.POINTER(C.c_int)]
        L.orc_rusanov.restype = C.c_double
        L.orc_threads.restype = C.c_int
        L.orc_set_point_source.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                           C.c_int]
        L.orc_set_point_source.restype = None
        L.orc_set_trace_buffer.argtypes = [D, D, C.c_int]
        L.orc_set_trace_buffer.restype = None
        L.orc_trace_count.restype = C.c_int
        L.orc_acoustic_rhs_at.argtypes = [C.POINTER(AcousticCfg), C.c_double, D, D]
        L.orc_sw2d_rhs_at.argtypes = [C.POINTER(Sw2dCfg), C.c_double, D, D]
        L.orc_positivity_fallbacks.argtypes = [C.c_int]
        L.orc_positivity_fallbacks.restype = C.c_long
        _lib = L
    return _lib


def threads() -> int:
    return lib().orc_threads()


def euler_cfg(n, h, cfl=0.4, gamma=1.4, bc=(0,) * 6, origin=(0.0, 0.0, 0.0), recon=0, nthreads=0, flux=0, mu=0.0,
              prandtl=1.0, cv=2.5,
              positivity=0):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    c = EulerCfg()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.xmin, c.ymin, c.zmin = origin
    c.h, c.cfl, c.gamma = h, cfl, gamma
    for q in range(6):
        c.bc[q] = bc[q]
    c.recon, c.nthreads, c.flux, c.positivity = recon, nthreads, flux, positivity
    c.mu, c.prandtl, c.cv = mu, prandtl, cv
    return c


def euler_rhs(cfg: EulerCfg, U: np.ndarray):
    """RHS of an AoS [k][j][i][5] state. Returns (rhs, s_max, status, bad)."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    smax = C.c_double(0.0)
    bad = C.c_long(-1)
    rc = lib().orc_euler_rhs(C.byref(cfg), _dp(U), _dp(R), C.byref(smax), C.byref(bad))
    return R, smax.value, rc, bad.value


def last_smax_visc() -> float:
    return lib().orc_euler_last_smax_visc()


def tgv_ic(cfg: EulerCfg) -> np.ndarray:
    U = np.zeros((cfg.nz, cfg.ny, cfg.nx, 5))
    lib().orc_tgv_ic(C.byref(cfg), _dp(U))
    return U


def kinetic_energy(cfg: EulerCfg, U) -> float:
    return lib().orc_kinetic_energy(C.byref(cfg), _dp(np.ascontiguousarray(U, dtype=np.float64)))


def dissipation(cfg: EulerCfg, U) -> float:
    return lib().orc_dissipation(C.byref(cfg), _dp(np.ascontiguousarray(U, dtype=np.float64)))


def euler_run(cfg: EulerCfg, U: np.ndarray, nsteps: int, dt_mode: int = 0, dt: float = 0.0):
    """nsteps of SSPRK(4,3). Returns (U_new, t, dt_next, status)."""
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    d = C.c_double(dt)
    bad = C.c_long(-1)
    rc = lib().orc_euler_run(C.byref(cfg), nsteps, dt_mode, _dp(U), C.byref(t), C.byref(d), C.byref(bad))
    return U, t.value, d.value, rc


def ctcs2d_plane(p_old, p, alpha, bc, nsteps):
    ny, nx = p.shape
    a = np.array(p_old, dtype=np.float64, order="C", copy=True)
    b = np.array(p, dtype=np.float64, order="C", copy=True)
    s = np.zeros_like(b)
    lib().orc_ctcs2d_plane(nx, ny, alpha, bc, nsteps, _dp(a), _dp(b), _dp(s))
    return a, b


def ctcs_pointsrc(cfg: CtcsCfg, p_old, p, nsteps, c=None, receiver=False):
    a = np.array(p_old, dtype=np.float64, order="C", copy=True)
    b = np.array(p, dtype=np.float64, order="C", copy=True)
    s = np.zeros_like(b)
    rec = np.zeros(nsteps) if receiver else None
    cp = _dp(np.ascontiguousarray(c, dtype=np.float64)) if c is not None else None
    lib().orc_ctcs_pointsrc(C.byref(cfg), cp, nsteps, _dp(a), _dp(b), _dp(s), _dp(rec) if receiver else None)
    return a, b, rec


def ctcs_monopole(cfg: MonoCfg, p_old, p, nsteps):
    a = np.array(p_old, dtype=np.float64, order="C", copy=True)
    b = np.array(p, dtype=np.float64, order="C", copy=True)
    s = np.zeros_like(b)
    lib().orc_ctcs_monopole(C.byref(cfg), nsteps, _dp(a), _dp(b), _dp(s))
    return a, b


# ---------------------------------------------------------------- reference
def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libref_euler.so"))


_REF_FLUX_LIB = {0: "libref_euler.so", 1: "libref_euler_hllc.so", 2: "libref_euler_rothllc.so"}
_ref_euler_libs = {}


def _ref_euler_fns(cfg):
    """(rhs, run) entry points of the reference program for cfg: the CWENO4 Euler RHS
    with its Riemann solver (cfg.flux), or the WENO3 Euler program (cfg.recon == 3)."""
    if cfg.recon == 3:
        if cfg.flux != 0:
            raise ValueError("the WENO3 reference program has the Rusanov flux only")
        key, name, pre = "w3", "libref_euler_w3.so", "ref_euler_w3_"
    elif cfg.mu > 0.0:
        if cfg.recon != 1 or cfg.flux != 0 or cfg.mu != 0.01 or cfg.prandtl != 1.0 or cfg.cv != 2.5:
            raise ValueError("the Navier-Stokes-3D reference program reconstructs with R4, has the Rusanov flux and "
                             "mu 0.01, Pr 1, Cv 2.5")
        key, name, pre = "ns3d", "libref_ns3d.so", "ref_ns3d_"
    else:
        key, name, pre = cfg.flux, _REF_FLUX_LIB[cfg.flux], "ref_euler_"
    if key not in _ref_euler_libs:
        L = C.CDLL(os.path.join(HERE, "_ref", name))
        IP = C.POINTER(C.c_int)
        rhs, run = getattr(L, pre + "rhs"), getattr(L, pre + "run")
        rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, IP, D, D, D]
        run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, IP,
                        C.c_int, C.c_int, D, D, D]
        _ref_euler_libs[key] = (rhs, run)
    return _ref_euler_libs[key]


def ref_euler_rhs(cfg: EulerCfg, U):
    rhs, _ = _ref_euler_fns(cfg)
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    dt = C.c_double(0.0)
    bc = (C.c_int * 6)(*cfg.bc)
    rc = rhs(cfg.nx, cfg.ny, cfg.nz, cfg.xmin, cfg.ymin, cfg.zmin, cfg.h, cfg.cfl, bc, _dp(U), _dp(R), C.byref(dt))
    return R, dt.value, rc


def ref_euler_run(cfg: EulerCfg, U, nsteps, dt_mode=0, dt=0.0):
    _, run = _ref_euler_fns(cfg)
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    d = C.c_double(dt)
    bc = (C.c_int * 6)(*cfg.bc)
    rc = run(cfg.nx, cfg.ny, cfg.nz, cfg.xmin, cfg.ymin, cfg.zmin, cfg.h, cfg.cfl, bc, nsteps, dt_mode, _dp(U),
             C.byref(t), C.byref(d))
    return U, t.value, d.value, rc


# ---------------------------------------------------------------- acoustic FV (plane_wave)
class AcousticCfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("xmin", C.c_double), ("ymin", C.c_double),
                ("zmin", C.c_double), ("h", C.c_double), ("c", C.c_double), ("bc", C.c_int * 6), ("recon", C.c_int),
                ("nthreads", C.c_int)]


def acoustic_cfg(n, h, bc=(0,) * 6, recon=1, c=1.0, nthreads=0):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    g = AcousticCfg()
    g.nx, g.ny, g.nz, g.h, g.c = nx, ny, nz, h, c
    for q in range(6):
        g.bc[q] = bc[q]
    g.recon, g.nthreads = recon, nthreads
    return g


def acoustic_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    lib().orc_acoustic_rhs(C.byref(cfg), _dp(U), _dp(R))
    return R


def acoustic_run(cfg, U, nsteps, dt, t_final=0.0):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    n = C.c_int(0)
    lib().orc_acoustic_run(C.byref(cfg), int(nsteps), float(dt), float(t_final), _dp(U), C.byref(t), C.byref(n))
    return U, t.value, n.value


def plane_wave_ic(cfg):
    U = np.zeros((cfg.nz, cfg.ny, cfg.nx, 2))
    lib().orc_acoustic_plane_wave_ic(C.byref(cfg), _dp(U))
    return U


def plane_wave_errors(cfg, U, t):
    U = np.ascontiguousarray(U, dtype=np.float64)
    l2, li = C.c_double(), C.c_double()
    lib().orc_acoustic_plane_wave_errors(C.byref(cfg), _dp(U), float(t), C.byref(l2), C.byref(li))
    return l2.value, li.value


_ref_acoustic = None


def _ref_acoustic_lib():
    global _ref_acoustic
    if _ref_acoustic is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_acoustic.so"))
        IP = C.POINTER(C.c_int)
        L.ref_acoustic_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, IP, D, D]
        L.ref_acoustic_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, IP, C.c_int, C.c_double, C.c_double, D, D]
        _ref_acoustic = L
    return _ref_acoustic


def ref_acoustic_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    bc = (C.c_int * 6)(*cfg.bc)
    _ref_acoustic_lib().ref_acoustic_rhs(cfg.nx, cfg.ny, cfg.nz, cfg.h, bc, _dp(U), _dp(R))
    return R


def ref_acoustic_run(cfg, U, nsteps, dt, t_final=0.0):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    bc = (C.c_int * 6)(*cfg.bc)
    _ref_acoustic_lib().ref_acoustic_run(cfg.nx, cfg.ny, cfg.nz, cfg.h, bc, int(nsteps), float(dt), float(t_final),
                                         _dp(U), C.byref(t))
    return U, t.value


# ---------------------------------------------------------------- 3D primitive multiphase
class Mp3dCfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("h", C.c_double), ("cfl", C.c_double),
                ("bc", C.c_int * 6), ("g1", C.c_double), ("p1", C.c_double), ("g2", C.c_double), ("p2", C.c_double),
                ("mu1", C.c_double), ("mu2", C.c_double), ("nthreads", C.c_int)]


# the constants compiled into 3d/weno4/Viscous-Multiphase-Fourth-Order (hype.h:37-42)
MP3D_EOS = (1.4, 0.0, 1.6, 0.0)
MP3D_MU = (1.4, 1.6)


def mp3d_cfg(n, h, cfl=0.9, bc=(2,) * 6, eos=MP3D_EOS, mu=MP3D_MU, nthreads=0):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    c = Mp3dCfg()
    c.nx, c.ny, c.nz, c.h, c.cfl = nx, ny, nz, h, cfl
    for q in range(6):
        c.bc[q] = bc[q]
    c.g1, c.p1, c.g2, c.p2 = eos
    c.mu1, c.mu2 = mu
    c.nthreads = nthreads
    return c


def mp3d_rhs(cfg, U):
    """(RHS, dt, s_max_c, s_max_v, status)"""
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    dt, sc, sv = C.c_double(), C.c_double(), C.c_double()
    rc = lib().orc_mp3d_rhs(C.byref(cfg), _dp(U), _dp(R), C.byref(dt), C.byref(sc), C.byref(sv))
    return R, dt.value, sc.value, sv.value, rc


def mp3d_run(cfg, U, nsteps, dt_mode=0, dt=0.0):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    d = C.c_double(dt)
    rc = lib().orc_mp3d_run(C.byref(cfg), int(nsteps), int(dt_mode), _dp(U), C.byref(t), C.byref(d))
    return U, t.value, d.value, rc


def mp3d_prim2cons(cfg, V):
    V = np.ascontiguousarray(V, dtype=np.float64)
    Q = np.empty_like(V)
    for idx in np.ndindex(V.shape[:-1]):
        lib().orc_mp3d_prim2cons(C.byref(cfg), _dp(np.ascontiguousarray(V[idx])), _dp(Q[idx]))
    return Q


_ref_mp3d = None


def _ref_mp3d_lib():
    global _ref_mp3d
    if _ref_mp3d is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_mp3d.so"))
        IP = C.POINTER(C.c_int)
        L.ref_mp3d_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, IP, D, D, D]
        L.ref_mp3d_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, IP, C.c_int, C.c_int, D, D, D]
        _ref_mp3d = L
    return _ref_mp3d


def ref_mp3d_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    dt = C.c_double()
    bc = (C.c_int * 6)(*cfg.bc)
    rc = _ref_mp3d_lib().ref_mp3d_rhs(cfg.nx, cfg.ny, cfg.nz, cfg.h, cfg.cfl, bc, _dp(U), _dp(R), C.byref(dt))
    return R, dt.value, rc


def ref_mp3d_run(cfg, U, nsteps, dt_mode=0):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t, dt = C.c_double(), C.c_double()
    bc = (C.c_int * 6)(*cfg.bc)
    rc = _ref_mp3d_lib().ref_mp3d_run(cfg.nx, cfg.ny, cfg.nz, cfg.h, cfg.cfl, bc, int(nsteps), int(dt_mode), _dp(U),
                                      C.byref(t), C.byref(dt))
    return U, t.value, dt.value, rc


# ---------------------------------------------------------------- 2D path-conservative (HyPE-2D)
class H2dCfg(C.Structure):
    _fields_ = [("N", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("h", C.c_double), ("cfl", C.c_double),
                ("bc", C.c_int * 4), ("g1", C.c_double), ("p1", C.c_double), ("g2", C.c_double), ("p2", C.c_double),
                ("nthreads", C.c_int)]


# GAMMA_1, PI_1, GAMMA_2, PI_2 compiled into 2d/HyPE-2D (hype.h:41-44)
H2D_EOS = (1.4, 0.0, 1.4, 0.0)


def h2d_cfg(N, nx, ny, h, cfl=0.9, bc=(2,) * 4, eos=H2D_EOS, nthreads=0):
    c = H2dCfg()
    c.N, c.nx, c.ny, c.h, c.cfl = N, nx, ny, h, cfl
    for q in range(4):
        c.bc[q] = bc[q]
    c.g1, c.p1, c.g2, c.p2 = eos
    c.nthreads = nthreads
    return c


def h2d_rhs(cfg, U):
    """(RHS, dt, status)"""
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    dt = C.c_double()
    rc = lib().orc_h2d_rhs(C.byref(cfg), _dp(U), _dp(R), C.byref(dt))
    return R, dt.value, rc


def h2d_run(cfg, U, nsteps):
    """nsteps with the program's stepper for N and the dt of the first RHS: (U, t, dt, status)"""
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t, dt = C.c_double(), C.c_double()
    rc = lib().orc_h2d_run(C.byref(cfg), int(nsteps), _dp(U), C.byref(t), C.byref(dt))
    return U, t.value, dt.value, rc


_ref_h2d = None


def _ref_h2d_lib():
    global _ref_h2d
    if _ref_h2d is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_hype2d_kp5.so"))
        IP = C.POINTER(C.c_int)
        L.ref_hype2d_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, IP, D,
                                     D, D]
        L.ref_hype2d_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, IP,
                                     C.c_int, D, D, D]
        _ref_h2d = L
    return _ref_h2d


def ref_h2d_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    dt = C.c_double()
    bc = (C.c_int * 4)(*cfg.bc)
    rc = _ref_h2d_lib().ref_hype2d_rhs(cfg.N, cfg.nx, cfg.ny, 0.0, 0.0, cfg.h, cfg.cfl, bc, _dp(U), _dp(R),
                                       C.byref(dt))
    return R, dt.value, rc


def ref_h2d_run(cfg, U, nsteps):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t, dt = C.c_double(), C.c_double()
    bc = (C.c_int * 4)(*cfg.bc)
    rc = _ref_h2d_lib().ref_hype2d_run(cfg.N, cfg.nx, cfg.ny, 0.0, 0.0, cfg.h, cfg.cfl, bc, int(nsteps), _dp(U),
                                       C.byref(t), C.byref(dt))
    return U, t.value, dt.value, rc


def kp5_state(nx, ny, seed, sharp=False):
    """a seeded Kapila state Q = (a1 rho1, a2 rho2, rho u, rho v, E, a1) with EOS (1.4, 0, 1.4, 0):
    a circular region of phase 1 in phase 2, random velocities and pressures"""
    rng = np.random.default_rng(seed)
    y, x = (np.arange(ny) + 0.5) / ny, (np.arange(nx) + 0.5) / nx
    Y, X = np.meshgrid(y, x, indexing="ij")
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2)
    w = 0.01 if sharp else 0.08
    a1 = 1e-3 + (1 - 2e-3) * 0.5 * (1 - np.tanh((r - 0.25) / w))
    r1, r2 = 1.0 + 0.1 * rng.random((ny, nx)), 0.125 + 0.01 * rng.random((ny, nx))
    u, v = 0.1 * rng.standard_normal((ny, nx)), 0.1 * rng.standard_normal((ny, nx))
    p = 1.0 + 0.1 * rng.random((ny, nx))
    rho = a1 * r1 + (1 - a1) * r2
    Q = np.stack([a1 * r1, (1 - a1) * r2, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v), a1], -1)
    return Q


# ---------------------------------------------------------------- 2D acoustic FV (standing_wave)
class Sw2dCfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("xmin", C.c_double), ("ymin", C.c_double), ("xmax", C.c_double),
                ("ymax", C.c_double), ("h", C.c_double), ("c", C.c_double), ("bc", C.c_int * 4)]


def sw2d_cfg(nx, ny, h, xmin=0.0, ymin=0.0, bc=(4,) * 4, c=1.0, xmax=None, ymax=None):
    g = Sw2dCfg()
    g.nx, g.ny, g.h, g.c = nx, ny, h, c
    g.xmin, g.ymin = xmin, ymin
    g.xmax = xmin + nx * h if xmax is None else xmax
    g.ymax = ymin + ny * h if ymax is None else ymax
    for q in range(4):
        g.bc[q] = bc[q]
    return g


def standing_wave_cfg(N):
    """the 2d/weno4/standing_wave program's set-up (hype.c:30-50): [-1,1]^2, adiabatic walls"""
    return sw2d_cfg(N, N, (1.0 - -1.0) / N, -1.0, -1.0, (4,) * 4, 1.0, 1.0, 1.0)


def sw2d_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    lib().orc_sw2d_rhs(C.byref(cfg), _dp(U), _dp(R))
    return R


def sw2d_run(cfg, U, nsteps, dt, t_final=0.0, stepper=1):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    n = C.c_int(0)
    lib().orc_sw2d_run(C.byref(cfg), int(stepper), int(nsteps), float(dt), float(t_final), _dp(U), C.byref(t),
                       C.byref(n))
    return U, t.value, n.value


def sw2d_ic(cfg):
    U = np.zeros((cfg.ny, cfg.nx, 2))
    lib().orc_sw2d_ic(C.byref(cfg), _dp(U))
    return U


def sw2d_errors(cfg, U, t):
    U = np.ascontiguousarray(U, dtype=np.float64)
    l2, li = C.c_double(), C.c_double()
    lib().orc_sw2d_errors(C.byref(cfg), _dp(U), float(t), C.byref(l2), C.byref(li))
    return l2.value, li.value


_ref_sw2d = None


def _ref_sw2d_lib():
    global _ref_sw2d
    if _ref_sw2d is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_sw2d.so"))
        IP = C.POINTER(C.c_int)
        L.ref_sw2d_rhs.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, IP, D, D]
        L.ref_sw2d_run.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, IP, C.c_int, C.c_int,
                                   C.c_double, C.c_double, D, D]
        L.ref_sw2d_program.argtypes = [C.c_int, D, D, D, D]
        _ref_sw2d = L
    return _ref_sw2d


def ref_sw2d_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    bc = (C.c_int * 4)(*cfg.bc)
    _ref_sw2d_lib().ref_sw2d_rhs(cfg.nx, cfg.ny, cfg.xmin, cfg.ymin, cfg.h, bc, _dp(U), _dp(R))
    return R


def ref_sw2d_run(cfg, U, nsteps, dt, t_final=0.0, stepper=1):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    bc = (C.c_int * 4)(*cfg.bc)
    _ref_sw2d_lib().ref_sw2d_run(cfg.nx, cfg.ny, cfg.xmin, cfg.ymin, cfg.h, bc, int(stepper), int(nsteps), float(dt),
                                 float(t_final), _dp(U), C.byref(t))
    return U, t.value


def ref_sw2d_program(N):
    """the whole standing-wave program at N x N: (l2, linf, U0, U_final)"""
    U0 = np.zeros((N, N, 2))
    U1 = np.zeros((N, N, 2))
    l2, li = C.c_double(), C.c_double()
    _ref_sw2d_lib().ref_sw2d_program(int(N), C.byref(l2), C.byref(li), _dp(U0), _dp(U1))
    return l2.value, li.value, U0, U1


# ---------------------------------------------------------------- point / line source
class _Source:
    """the point source and receiver of 3d/weno4/point_source / 2d/weno4/line_source set
    on the restatement for the duration of a with-block; ``trace()`` then gives the (t, u)
    the receiver recorded at each RHS evaluation (at most ``capacity``) and the count"""

    def __init__(self, src, f0, rec, capacity):
        self.src = tuple(src) + (0,) * (3 - len(src)) if src is not None else None
        self.rec = tuple(rec) + (0,) * (3 - len(rec)) if rec is not None else None
        self.f0, self.capacity = f0, int(capacity)
        self._t = np.zeros(max(self.capacity, 1))
        self._u = np.zeros(max(self.capacity, 1))

    def __enter__(self):
        sx, sy, sz = self.src if self.src else (0, 0, 0)
        rx, ry, rz = self.rec if self.rec else (0, 0, 0)
        lib().orc_set_point_source(int(self.src is not None), sx, sy, sz, float(self.f0), int(self.rec is not None),
                                   rx, ry, rz)
        lib().orc_set_trace_buffer(_dp(self._t), _dp(self._u), self.capacity)
        return self

    def __exit__(self, *exc):
        lib().orc_set_point_source(0, 0, 0, 0, 1.0, 0, 0, 0, 0)
        self.count = lib().orc_trace_count()
        lib().orc_set_trace_buffer(None, None, 0)
        return False

    def trace(self):
        m = min(self.count, self.capacity)
        return self._t[:m].copy(), self._u[:m].copy(), self.count


def point_source(src, f0, rec, capacity=100000):
    return _Source(src, f0, rec, capacity)


def acoustic_rhs_at(cfg, t, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    lib().orc_acoustic_rhs_at(C.byref(cfg), float(t), _dp(U), _dp(R))
    return R


def sw2d_rhs_at(cfg, t, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    lib().orc_sw2d_rhs_at(C.byref(cfg), float(t), _dp(U), _dp(R))
    return R


# the programs' compiled-in constants: wave_speed (hype.h:39 / :38) and Source's f0
# (source.c:13 / :14)
PSRC3D_C, PSRC3D_F0 = 250.0, 100.0
LSRC2D_C, LSRC2D_F0 = 580.0, 65.0

_ref_psrc = None
_ref_lsrc = None


def _read_pdat(d):
    path = os.path.join(d, "results", "p.dat")
    if not os.path.exists(path):
        return np.zeros((0, 2))
    return np.loadtxt(path, ndmin=2)


def _ref_psrc_lib():
    global _ref_psrc
    if _ref_psrc is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_psrc3d.so"))
        IP = C.POINTER(C.c_int)
        L.ref_psrc3d_rhs.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, IP, IP, IP, C.c_double, D, D, C.c_char_p]
        L.ref_psrc3d_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, IP, IP, IP, C.c_int, C.c_int, C.c_double,
                                     C.c_double, D, D, C.c_char_p]
        _ref_psrc = L
    return _ref_psrc


def _ref_lsrc_lib():
    global _ref_lsrc
    if _ref_lsrc is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_lsrc2d.so"))
        IP = C.POINTER(C.c_int)
        L.ref_lsrc2d_rhs.argtypes = [C.c_int, C.c_int, C.c_double, IP, IP, IP, C.c_double, D, D, C.c_char_p]
        L.ref_lsrc2d_run.argtypes = [C.c_int, C.c_int, C.c_double, IP, IP, IP, C.c_int, C.c_int, C.c_double,
                                     C.c_double, D, D, C.c_char_p]
        _ref_lsrc = L
    return _ref_lsrc


def ref_psrc3d_rhs(cfg, src, rec, t, U):
    """the RHS of 3d/weno4/point_source at time t and its receiver line (results/p.dat)"""
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "results"))
        rc = _ref_psrc_lib().ref_psrc3d_rhs(cfg.nx, cfg.ny, cfg.nz, cfg.h, (C.c_int * 6)(*cfg.bc), (C.c_int * 3)(*src),
                                            (C.c_int * 3)(*rec), float(t), _dp(U), _dp(R), d.encode())
        assert rc == 0
        return R, _read_pdat(d)


def ref_psrc3d_run(cfg, src, rec, U, nsteps, dt, t_final=0.0, initial_rhs=False):
    """TSSolve of 3d/weno4/point_source from U (t = 0): (U, t, receiver lines (t, u))"""
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "results"))
        rc = _ref_psrc_lib().ref_psrc3d_run(cfg.nx, cfg.ny, cfg.nz, cfg.h, (C.c_int * 6)(*cfg.bc), (C.c_int * 3)(*src),
                                            (C.c_int * 3)(*rec), int(initial_rhs), int(nsteps), float(dt),
                                            float(t_final), _dp(U), C.byref(t), d.encode())
        assert rc == 0
        return U, t.value, _read_pdat(d)


def ref_lsrc2d_rhs(cfg, src, rec, t, U):
    """the RHS of 2d/weno4/line_source at time t and its receiver line"""
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "results"))
        rc = _ref_lsrc_lib().ref_lsrc2d_rhs(cfg.nx, cfg.ny, cfg.h, (C.c_int * 4)(*cfg.bc), (C.c_int * 2)(*src),
                                            (C.c_int * 2)(*rec), float(t), _dp(U), _dp(R), d.encode())
        assert rc == 0
        return R, _read_pdat(d)


def ref_lsrc2d_run(cfg, src, rec, U, nsteps, dt, t_final=0.0, stepper=1):
    """TSSolve of 2d/weno4/line_source from U (t = 0): (U, t, receiver lines (t, u))"""
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "results"))
        rc = _ref_lsrc_lib().ref_lsrc2d_run(cfg.nx, cfg.ny, cfg.h, (C.c_int * 4)(*cfg.bc), (C.c_int * 2)(*src),
                                            (C.c_int * 2)(*rec), int(stepper), int(nsteps), float(dt), float(t_final),
                                            _dp(U), C.byref(t), d.encode())
        assert rc == 0
        return U, t.value, _read_pdat(d)


def ref_ctcs2d_run(p_old, p, h, c0, dt, zero_bc, nsteps):
    global _ref_ctcs2d
    if _ref_ctcs2d is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_ctcs2d.so"))
        L.ref_ctcs2d_run.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, D, D]
        _ref_ctcs2d = L
    ny, nx = p.shape
    a = np.array(p_old, dtype=np.float64, order="C", copy=True)
    b = np.array(p, dtype=np.float64, order="C", copy=True)
    rc = _ref_ctcs2d.ref_ctcs2d_run(nx, ny, h, c0, dt, int(zero_bc), nsteps, _dp(a), _dp(b))
    return a, b, rc


def ref_point_source_trace() -> np.ndarray:
    """Run the reference's 3d/ctcs/point_source program (compiled through the
    shim) in a scratch directory and return its receiver file as text."""
    exe = os.path.join(HERE, "_ref", "ref_point_source")
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "results"))
        subprocess.run([exe], cwd=d, check=True, stdout=subprocess.DEVNULL)
        with open(os.path.join(d, "results", "p.dat")) as f:
            return f.read()


# ---------------------------------------------------------------- 2D multiphase
class Mp2dCfg(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("xmin", C.c_double), ("ymin", C.c_double), ("h", C.c_double),
                ("cfl", C.c_double), ("bc", C.c_int * 4), ("model", C.c_int), ("g1", C.c_double), ("p1", C.c_double),
                ("g2", C.c_double), ("p2", C.c_double), ("nthreads", C.c_int)]


# the reference bubble code's compiled-in EOS (2d/weno4/bubble/hype.h: g1, p1, g2, p2)
BUBBLE_EOS = (4.4, 6000.0, 1.4, 0.0)


def mp2d_cfg(nx, ny, h, xmin=0.0, ymin=0.0, cfl=0.9, bc=(2, 2, 2, 2), model=0, eos=BUBBLE_EOS, nthreads=0):
    c = Mp2dCfg()
    c.nx, c.ny, c.xmin, c.ymin, c.h, c.cfl = nx, ny, xmin, ymin, h, cfl
    for q in range(4):
        c.bc[q] = bc[q]
    c.model = model
    c.g1, c.p1, c.g2, c.p2 = eos
    c.nthreads = nthreads
    return c


def _mp_lib():
    L = lib()
    if not getattr(L, "_mp_bound", False):
        L.orc_mp2d_rhs.argtypes = [C.POINTER(Mp2dCfg), D, D, D, C.POINTER(C.c_long), C.POINTER(C.c_long)]
        L.orc_mp2d_run.argtypes = [C.POINTER(Mp2dCfg), C.c_int, C.c_int, C.c_int, D, D, D, C.POINTER(C.c_long)]
        L.orc_mp_prim2cons.argtypes = [C.c_int, D, D, D]
        L.orc_mp_cons2prim.argtypes = [C.c_int, D, D, D]
        L._mp_bound = True
    return L


def mp2d_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    smax = C.c_double()
    bad = C.c_long(-1)
    fb = C.c_long(0)
    rc = _mp_lib().orc_mp2d_rhs(C.byref(cfg), _dp(U), _dp(R), C.byref(smax), C.byref(bad), C.byref(fb))
    return R, smax.value, rc, fb.value


def mp2d_run(cfg, U, nsteps, stepper=0, dt_mode=0, dt=0.0):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t = C.c_double(0.0)
    d = C.c_double(dt)
    bad = C.c_long(-1)
    rc = _mp_lib().orc_mp2d_run(C.byref(cfg), nsteps, stepper, dt_mode, _dp(U), C.byref(t), C.byref(d), C.byref(bad))
    return U, t.value, d.value, rc


def mp_prim2cons(model, eos, V):
    """vectorised over the leading axes"""
    V = np.ascontiguousarray(V, dtype=np.float64)
    nv = V.shape[-1]
    Q = np.empty_like(V)
    e = np.array(eos, dtype=np.float64)
    L = _mp_lib()
    Vf, Qf = V.reshape(-1, nv), Q.reshape(-1, nv)
    for q in range(Vf.shape[0]):
        L.orc_mp_prim2cons(model, _dp(e), Vf[q].ctypes.data_as(D), Qf[q].ctypes.data_as(D))
    return Q


_ref_bub = None


def _ref_bubble_lib():
    global _ref_bub
    if _ref_bub is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libref_bubble.so"))
        IP = C.POINTER(C.c_int)
        L.ref_bubble_rhs.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, IP, D, D, D]
        L.ref_bubble_run.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, IP, C.c_int, D, D,
                                     D]
        _ref_bub = L
    return _ref_bub


def ref_bubble_rhs(cfg, U):
    U = np.ascontiguousarray(U, dtype=np.float64)
    R = np.zeros_like(U)
    dt = C.c_double()
    bc = (C.c_int * 4)(*cfg.bc)
    rc = _ref_bubble_lib().ref_bubble_rhs(cfg.nx, cfg.ny, cfg.xmin, cfg.ymin, cfg.h, cfg.cfl, bc, _dp(U), _dp(R),
                                          C.byref(dt))
    return R, dt.value, rc


def ref_bubble_run(cfg, U, nsteps):
    U = np.array(U, dtype=np.float64, order="C", copy=True)
    t, d = C.c_double(), C.c_double()
    bc = (C.c_int * 4)(*cfg.bc)
    rc = _ref_bubble_lib().ref_bubble_run(cfg.nx, cfg.ny, cfg.xmin, cfg.ymin, cfg.h, cfg.cfl, bc, nsteps, _dp(U),
                                          C.byref(t), C.byref(d))
    return U, t.value, d.value, rc
