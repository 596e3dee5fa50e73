"""GB300 (sm_103a) implementation of HyPE's finite-volume RHS, SSP-RK stepper
and CTCS leapfrog acoustics behind a C ABI (include/hype_gpu.h).

The compute path is ``lib/libhype_gb300.so`` built from ``csrc/*.cu``; this
package only binds it (``_lib``) and mirrors the reference's operator interface
(``hype``).  There is no CPU fallback.
"""
from . import _build, _lib
from ._lib import HypeError, lib, launches
from .hype import (AcousticFV2D, AcousticFV3D, AppCtx, BatchLeapfrog, CTCS, EulerSolver, Leapfrog, Monopole, Multiphase2D, Multiphase3D, PathConservative2D, read_petsc_vec,
                   write_petsc_vec, write_vtk)

__all__ = ["AcousticFV2D", "AcousticFV3D", "AppCtx", "BatchLeapfrog", "CTCS", "EulerSolver", "HypeError", "Leapfrog", "Monopole", "Multiphase2D", "Multiphase3D", "PathConservative2D", "lib", "launches",
           "build", "read_petsc_vec", "write_petsc_vec", "write_vtk"]


def build(verbose: bool = False) -> str:
    return _build.build(verbose=verbose)
