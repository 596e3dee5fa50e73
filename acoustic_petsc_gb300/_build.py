"""Build recipe of the sm_103a shared library (no cmake, no torch extension).

Every ``csrc/*.cu`` is compiled by ``nvcc`` in parallel and linked into
``acoustic_petsc_gb300/lib/libhype_gb300.so`` (in-tree, git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libhype_gb300.so")
# test and measurement support (the FMA issue ceiling, the double-float primitive probe): a
# library of its own, kept out of the public C ABI
PROBES = os.path.join(CSRC, "probes")
PROBE_LIB = os.path.join(LIBDIR, "libhype_probes.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# per-file extra flags: the CTCS, 2D multiphase, 2D acoustic and path-conservative kernels keep the reference's
# rounding (no FMA contraction): results bit-identical to the CPU restatement
EXTRA = {"ctcs.cu": ["-fmad=false"], "mphase2d.cu": ["-fmad=false"], "acoustic2d.cu": ["-fmad=false"],
         "pc2d.cu": ["-fmad=false"]}


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhype_gb300.so")


def sources() -> list[str]:
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def build(verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(PKG, "..", "include", "hype_gpu.h")]
    deps += [os.path.join(PROBES, f) for f in os.listdir(PROBES)]
    newest_dep = max(os.path.getmtime(d) for d in deps)
    if (all(os.path.exists(x) and os.path.getmtime(x) >= newest_dep for x in (LIB, PROBE_LIB))
            and not os.environ.get("HYPE_FORCE_BUILD")):
        return LIB
    procs = []
    objs = []
    probe_objs = []
    units = [(f, os.path.join(CSRC, f)) for f in sources()]
    units += [(f, os.path.join(PROBES, f)) for f in sorted(os.listdir(PROBES)) if f.endswith(".cu")]
    for f, src in units:
        obj = os.path.join(OBJDIR, f.replace(".cu", ".o"))
        (probe_objs if os.path.dirname(src) == PROBES else objs).append(obj)
        # host code never contracts a*b+c into an FMA (g++ does by default on aarch64): the
        # host-side tables (source wavelet, Gaussian factors) must round like the reference
        cmd = [cc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "-Xptxas", "-warn-spills",
               "-I", CSRC, *EXTRA.get(f, []), "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((f, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for f, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(f"{f}:\n{out.decode(errors='replace')}")
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], check=True)
    os.replace(tmp, LIB)
    tmp = PROBE_LIB + ".tmp"
    subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *probe_objs, "-L", LIBDIR, "-lhype_gb300", "-lcudart",
                    "-Xlinker", "-rpath,$ORIGIN"], check=True)
    os.replace(tmp, PROBE_LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
