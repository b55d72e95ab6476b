"""How strongly the reference algorithm's own output reacts to rounding-level changes
of its input, per golden case.

The reference branches on exact ties and signs: the corner EMF takes one of three
formulas by the sign of the face mass flux, including exactly zero
(Source/CornerEMF_HelperModule.py:496-525), and the Roe eigenvector normalisation
switches on cf^2 - a^2 <= 0 and a^2 - cs^2 <= 0 (Source/RiemannSolvers_MHD_Roe_
HelperModule.py:258-283), which are rounding-level coin flips when the transverse
field vanishes.  On states that sit on such a tie -- a symmetric Orszag-Tang face
with exactly zero mass flux, a 1D state with B_t == 0 -- the reference's result
depends on the last bit of intermediate values.  ``sensitivity`` measures that:
it perturbs every prim and cons input value by one unit in the last place (seeded
random signs, three draws) and returns the largest one-cycle change of the
oracle's output (the oracle reproduces the reference bit for bit), relative per
field.  Any arithmetic that is not bit-identical to the reference -- FMA
contraction, a different summation order -- can only be expected to match it to
this level on such a state.
"""
import numpy as np

from tests.golden_io import load
from tests.gpu_util import field_rel_err


def _ulp_perturb(a, rng):
    a = np.asarray(a, dtype=np.float64)
    up = rng.choice([True, False], size=a.shape)
    return np.where(a == 0.0, a, np.nextafter(a, np.where(up, np.inf, -np.inf)))


def sensitivity(path, draws=3, seed=0):
    from oracle import hydro2d, mhd2d
    p, i, _ = load(path)
    mhd = "fbx" in i
    if not p["t_start"] < p["t_end"]:
        return 0.0
    rng = np.random.default_rng(seed)
    tail = (p["t_start"], p["t_end"], p["start_cycle"], p["start_cycle"] + 1, p["gamma"], p["cfl"], p["min_d"],
            p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])

    def run(prim, cons):
        if mhd:
            return mhd2d.evolve(prim, cons, i["fbx"], i["fby"], p["dx"], p["dy"], p["bcx"], p["bcy"], *tail)[:4]
        return hydro2d.evolve(prim, cons, p["dx"], p["dy"], p["bcx"], p["bcy"], *tail)[:2]

    base = run(i["prim"], i["cons"])
    worst = 0.0
    for _ in range(draws):
        out = run(_ulp_perturb(i["prim"], rng), _ulp_perturb(i["cons"], rng))
        worst = max(worst, max(field_rel_err(a, b) for a, b in zip(out, base)))
    return worst
