"""Generate ``csrc/adjoint_gen.cuh``: forward and reverse device functions of
every pointwise stage of the MHD cycle (``stages.py``), for the GPU adjoint.

    python -m pythonmhd_gb300.adjoint.codegen [out_path]
"""
from __future__ import annotations

import os
import sys

from . import dsl, stages

# name, function, inputs, params, keyword arguments
STAGES = [
    ("plm0", stages.plm_cell, 22, 2, dict(axis=0)),
    ("plm1", stages.plm_cell, 22, 2, dict(axis=1)),
    ("pslope0", stages.ppm_slope, 22, 1, dict(axis=0)),
    ("pslope1", stages.ppm_slope, 22, 1, dict(axis=1)),
    ("ppmi0", stages.ppm_iface, 42, 1, dict(axis=0)),
    ("ppmi1", stages.ppm_iface, 42, 1, dict(axis=1)),
    ("ppmt0", stages.ppm_trace, 21 + stages.EIG_BASE, 2, dict(axis=0)),
    ("ppmt1", stages.ppm_trace, 21 + stages.EIG_BASE, 2, dict(axis=1)),
    ("face0", stages.face_state, 10, 4, dict(sb=4)),
    ("face1", stages.face_state, 10, 4, dict(sb=5)),
    ("roe1_0", stages.roe1, 15, 2, dict(axis=0, efix=False)),
    ("roe1_1", stages.roe1, 15, 2, dict(axis=1, efix=False)),
    ("roe2_0", stages.roe2, 29, 2, dict(axis=0, efix=False)),
    ("roe2_1", stages.roe2, 29, 2, dict(axis=1, efix=False)),
    ("roe1_0_efix", stages.roe1, 15, 2, dict(axis=0, efix=True)),
    ("roe1_1_efix", stages.roe1, 15, 2, dict(axis=1, efix=True)),
    ("roe2_0_efix", stages.roe2, 29, 2, dict(axis=0, efix=True)),
    ("roe2_1_efix", stages.roe2, 29, 2, dict(axis=1, efix=True)),
    ("ez", stages.cell_ez, 4, 0, {}),
    ("emf", stages.emf_corner, 12, 0, {}),
    ("ctu0", stages.ctu_side, 29, 6, dict(axis=0)),
    ("ctu1", stages.ctu_side, 29, 6, dict(axis=1)),
    ("half", stages.half_ez, 19, 2, {}),
    ("final", stages.final_cell, 43, 3, {}),
    ("fhx", stages.face_half_x, 3, 1, {}),
    ("fhy", stages.face_half_y, 3, 1, {}),
]

# Stages whose forward statements divide and take square roots on the integer pipes
# (mhdk::ddiv / mhdk::sqrt); the others use the FP64 instructions.  Both give the IEEE
# bits.  Measured per kernel: the integer-pipe forms make the small CT, half-step and
# update stages faster, but the taped reconstruction and Roe kernels, which sit at
# the 255-register cap, 16-30% slower.
INTEGER_PIPE_DIVSQRT = {"ez", "emf", "ctu0", "ctu1", "half", "final", "fhx", "fhy", "face0", "face1"}

HEADER = """// GENERATED by pythonmhd_gb300/adjoint/codegen.py from adjoint/stages.py -- do not edit.
// Forward (<stage>_fwd), branch-recording / branch-replaying forward (<stage>_fwdb)
// and reverse-mode (<stage>_rev) device functions of the pointwise stages of one
// MHD CTU+CT cycle.
#pragma once
"""


def generate() -> str:
    parts = [HEADER]
    for name, fn, nin, npar, kw in STAGES:
        t = dsl.trace(f"g_{name}", fn, nin, npar, **kw)
        parts.append(f"// ---- {name}: {nin} inputs, {npar} params, {len(t.outputs)} outputs\n")
        if name in INTEGER_PIPE_DIVSQRT:
            parts.append("#undef DSL_FDIV\n#undef DSL_FSQRT\n#define DSL_FDIV mhdk::ddiv\n#define DSL_FSQRT mhdk::sqrt\n")
        else:
            parts.append("#undef DSL_FDIV\n#undef DSL_FSQRT\n#define DSL_FDIV __ddiv_rn\n#define DSL_FSQRT __dsqrt_rn\n")
        parts.append(f"constexpr int g_{name}_NI = {nin}, g_{name}_NP = {max(npar, 1)}, g_{name}_NO = {len(t.outputs)}, "
                     f"g_{name}_NT = {dsl.tape_words(t)}, g_{name}_NB = {dsl.branch_words(t)};\n")
        parts.append(dsl.emit_cuda(t))
    return "\n".join(parts)


def write(path):
    src = generate()
    old = None
    if os.path.exists(path):
        with open(path) as f:
            old = f.read()
    if old != src:
        with open(path, "w") as f:
            f.write(src)
    return path


if __name__ == "__main__":
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    print(write(sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "csrc", "adjoint_gen.cuh")))
