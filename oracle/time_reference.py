"""Per-core rate of the reference's own CPU code for the 3D Euler path against the C
restatement (TEST INFRASTRUCTURE ONLY; needs the reference tree, so it runs where the
checker is built from it, not on a machine without that tree).

Both are timed on one core over the same seeded sample (the Gaussian-pulse workload at
n^3, periodic, CFL 0.4, one SSPRK(4,3) step = 4 RHS evaluations):
  * reference CWENO4: the Navier-Stokes-3D RHSFunction (rhs_function.c:12-443) with the CWENO4
    weno() of Viscous-Multiphase-Fourth-Order and a zero viscous flux, the SSP RKS3 stepping of
    the shim (what the oracle pins bit for bit);
  * reference WENO3: the whole 3d/weno3/Euler RHS program;
  * restatement: oracle/hype_oracle.c with the same options, one thread and all threads.
Usage: python oracle/time_reference.py [n]   (prints one JSON object)
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from acoustic_petsc_gb300 import workloads  # noqa: E402
from oracle import pyoracle as O  # noqa: E402


def _rate(fn, cells, reps=1):
    fn()  # warm (allocations, page faults)
    t0 = time.perf_counter()
    for _ in range(reps):
        fn()
    return cells * reps / (time.perf_counter() - t0)


def main(n: int = 32) -> dict:
    O.build(O.ref_dir())
    if not O.ref_available():
        raise SystemExit("the reference tree is not present: nothing to time")
    U = workloads.euler_pulse(n)
    out = {"sample": f"{n}^3 Gaussian pulse, periodic, CFL 0.4, 1 SSPRK(4,3) step (4 RHS evaluations)",
           "cpu": platform.processor() or platform.machine(), "host_threads": os.cpu_count()}
    for recon, tag in ((0, "cweno4"), (3, "weno3")):
        c1 = O.euler_cfg(n, 1.0 / n, cfl=0.4, recon=recon, nthreads=1)
        ca = O.euler_cfg(n, 1.0 / n, cfl=0.4, recon=recon, nthreads=os.cpu_count() or 1)
        ref = _rate(lambda: O.ref_euler_run(c1, U, 1), n**3)
        port1 = _rate(lambda: O.euler_run(c1, U, 1), n**3, reps=3)
        portn = _rate(lambda: O.euler_run(ca, U, 1), n**3, reps=3)
        out[tag] = {"reference_1core": ref, "restatement_1thread": port1, "restatement_all_threads": portn,
                    "threads": O.threads(), "restatement_over_reference_per_core": port1 / ref,
                    "unit": "cell-updates/s"}
    return out


if __name__ == "__main__":
    print(json.dumps(main(int(sys.argv[1]) if len(sys.argv) > 1 else 32)))
