"""Shared pieces of the CPU oracle for the 2D unsplit Godunov step.

TEST INFRASTRUCTURE ONLY. The oracle is a NumPy restatement of the reference
algorithm (PythonMHD, ``Source/*``), written so that every floating-point
operation happens in the same order as in the reference. Its only users are
``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``; the
product path (``pythonmhd_gb300``) never imports it.

Conventions used throughout the oracle:

* A "sweep vector" is a (7, ...) array in the reference's sweep ordering.
  x-sweep: [rho, vx, vy, vz, By, Bz, p]   (or [rho, mx, my, mz, By, Bz, E])
  y-sweep: [rho, vx, vy, vz, Bz, Bx, p]   (Source/EvolveFunctions_MHD.py:415-438)
* A ``Frame`` names the normal and the two transverse velocity slots of a sweep.
  The reference's y-direction routines are its x-direction routines with the
  slots relabelled (normal = vy, t1 = vz, t2 = vx), including the order of every
  sum, so one generic routine per formula reproduces both bit for bit.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# Source/PythonMHD_Constants.py:7-8 (FOUR_THIRDS is truncated on purpose)
SMALL_VALUE = 0.000000000001
FOUR_THIRDS = 1.333333333333333
# Source/PythonMHD_Constants.py:11-12
OUTFLOW = 0
PERIODIC = 1


@dataclass(frozen=True)
class Frame:
    n: int
    t1: int
    t2: int
    # order in which the reference accumulates a row of L times a 7-vector
    # (Source/RiemannSolvers_MHD_Roe_HelperModule.py:505-512 for x,
    #  :1015-1022 for y; the PPM projections use the same order)
    @property
    def proj_order(self):
        return (0, self.n, self.t1, self.t2, 6, 4, 5)


FRAME_X = Frame(1, 2, 3)
FRAME_Y = Frame(2, 3, 1)


def wrap_index(idx: np.ndarray, n: int, bc: int) -> np.ndarray:
    """Map ghost cell indices onto interior cells: clamp (outflow) or wrap (periodic)."""
    if bc == PERIODIC:
        return np.mod(idx, n)
    return np.clip(idx, 0, n - 1)


def take_x(a: np.ndarray, idx: np.ndarray) -> np.ndarray:
    return np.take(a, idx, axis=-1)


def take_y(a: np.ndarray, idx: np.ndarray) -> np.ndarray:
    return np.take(a, idx, axis=-2)


_floor_tally = {"hits": 0}


def reset_floor_tally() -> None:
    """Zero the running count of floored values (see ``apply_floors_inplace``)."""
    _floor_tally["hits"] = 0


def floor_tally() -> int:
    """Values raised by the floors since the last ``reset_floor_tally``."""
    return _floor_tally["hits"]


def apply_floors_inplace(v: np.ndarray, min_d: float, min_last: float) -> np.ndarray:
    """Density floor on slot 0 and pressure/energy floor on the last slot.

    Follows Source/PrimCons_HelperModule.py:499-554.  The reference counts the
    values it clamps for a warning text that it then discards; the oracle adds that
    count to a running tally (``floor_tally``) that tests compare with the GPU's
    floor-hit counter.  The clamps themselves are unchanged.
    """
    d = v[0]
    low = d < min_d
    d[low] = min_d
    last = v[v.shape[0] - 1]
    low_last = last < min_last
    last[low_last] = min_last
    _floor_tally["hits"] += int(np.count_nonzero(low)) + int(np.count_nonzero(low_last))
    return v


def np_sign_one(x: np.ndarray) -> np.ndarray:
    """sign(x) with sign(0) -> 1 (Source/RiemannSolvers_MHD_Roe_HelperModule.py:286-287)."""
    s = np.sign(x)
    s[s == 0] = 1
    return s
