"""Build the in-tree CUDA library ``pythonmhd_gb300/libpythonmhd_gb300.so`` for sm_103a.

The translation units are compiled in parallel with nvcc and linked into one
shared library with a plain C ABI (``include/pythonmhd_gb300.h``):

* ``csrc/kernels_exact.cu``  -- the step kernels with ``-fmad=false``
* ``csrc/kernels_fast.cu``   -- the same kernels with FMA contraction
* ``csrc/kernels_checked.cu`` -- the exact kernels with every global index checked
* ``csrc/capi.cu``           -- handles, copies and the CUDA-graph evolve loop
* ``csrc/kernels3d_exact.cu`` / ``csrc/kernels3d_fast.cu`` -- the 3D hydro step kernels
* ``csrc/capi3d.cu``         -- the 3D handle and its evolve loop
* ``csrc/noalloc.cu``        -- the CFL timestep for callers that cannot allocate
* ``csrc/validate.cu``       -- the initial-state check (the reference's validatePrimVars)
* ``csrc/icgen.cu``          -- initial states on the GPU (turbulence field algebra, Orszag-Tang)
* ``csrc/adjoint.cu``        -- the reverse-mode adjoint of the MHD step; its pointwise
  stage functions (``csrc/adjoint_gen.cuh``) are generated from ``adjoint/stages.py``
  first, its stage kernels are in ``csrc/adjoint_kernels.cuh``
* ``csrc/adjoint_branch.cu`` -- the adjoint's branch-recording / -replaying forward sweep
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpythonmhd_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

UNITS = [
    ("kernels_exact.cu", ["-fmad=false"]),
    ("kernels_fast.cu", ["-fmad=true"]),
    ("kernels_checked.cu", ["-fmad=false"]),
    ("capi.cu", []),
    ("kernels3d_exact.cu", ["-fmad=false"]),
    ("kernels3d_fast.cu", ["-fmad=true"]),
    ("capi3d.cu", []),
    ("noalloc.cu", ["-fmad=false"]),
    ("validate.cu", ["-fmad=false"]),
    ("icgen.cu", ["-fmad=false", "--extended-lambda"]),
    ("adjoint.cu", []),
    ("adjoint_branch.cu", []),
]
ADJ_GEN = os.path.join(CSRC, "adjoint_gen.cuh")
ADJ_PY = os.path.join(PKG, "adjoint")


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pythonmhd_gb300")


def _sources():
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    srcs += [os.path.join(ADJ_PY, f) for f in os.listdir(ADJ_PY) if f.endswith(".py")]
    srcs.append(os.path.join(ROOT, "include", "pythonmhd_gb300.h"))
    srcs.append(os.path.abspath(__file__))
    return srcs


def generate_adjoint() -> str:
    """Write ``csrc/adjoint_gen.cuh`` from the adjoint stage definitions (only if it changed)."""
    from .adjoint import codegen
    return codegen.write(ADJ_GEN)


def is_stale() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(ADJ_GEN):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library if it is missing or older than its sources."""
    if not force and not is_stale():
        return LIB
    generate_adjoint()
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    common = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    # extra nvcc flags for tuning builds (e.g. -DMHD_MIN_BLOCKS=3)
    common += os.environ.get("PYTHONMHD_GB300_NVCC_FLAGS", "").split()
    procs = []
    objs = []
    for src, extra in UNITS:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        cmd = common + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(" ".join(cmd) + "\n" + out.decode(errors="replace"))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    link = [nvcc, ARCH, "-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
