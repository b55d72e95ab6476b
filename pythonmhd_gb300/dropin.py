"""Install the GPU evolve functions into a PythonMHD checkout.

The reference driver picks its evolve function from module attributes at run
time (Source/Simulation.py:312-324: ``evolveMHD.evolve_2D_mhd`` /
``evolveHydro.evolve_2D_hydro``, and the 1D ones) and calls it at
Source/Simulation.py:349-377.
Assigning those attributes swaps in the GPU step; initialization files and the
``Simulation`` driver stay unchanged:

    import pythonmhd_gb300.dropin as dropin
    dropin.install()                    # before Simulation(...).run()

``Source`` must be importable (PythonMHD's directory on ``sys.path``).
"""
from __future__ import annotations

import functools
import importlib

from . import evolve

TARGETS = (
    ("Source.EvolveFunctions_MHD", "evolve_2D_mhd", evolve.evolve_2D_mhd),
    ("Source.EvolveFunctions_Hydro", "evolve_2D_hydro", evolve.evolve_2D_hydro),
    ("Source.EvolveFunctions_MHD", "evolve_1D_mhd", evolve.evolve_1D_mhd),
    ("Source.EvolveFunctions_Hydro", "evolve_1D_hydro", evolve.evolve_1D_hydro),
    ("Source.EvolveFunctions_Hydro", "evolve_3D_hydro", evolve.evolve_3D_hydro),
    ("Source.EvolveFunctions_MHD", "evolve_3D_mhd", evolve.evolve_3D_mhd),
)

_saved: dict = {}


def install(arith: str | None = None):
    """Replace the reference's 1D, 2D and 3D evolve functions; returns the patched modules.

    ``arith`` ("exact" or "fast") overrides PYTHONMHD_GB300_ARITH for these calls.
    """
    mods = []
    for modname, attr, fn in TARGETS:
        m = importlib.import_module(modname)
        key = (modname, attr)
        if key not in _saved:
            _saved[key] = getattr(m, attr)
        new = functools.partial(fn, arith=arith) if arith else fn
        setattr(m, attr, new)
        mods.append(m)
    return mods


def uninstall():
    """Put the reference's own functions back."""
    for (modname, attr), orig in list(_saved.items()):
        m = importlib.import_module(modname)
        setattr(m, attr, orig)
        del _saved[(modname, attr)]
