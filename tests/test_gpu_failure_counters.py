"""Failure detection without a GPU fault: floor-hit counters, the non-finite flag,
the initial-state check and the batched work-list check.

* ``mhd2d_stats``' floor-hit count equals the number of values the reference's own
  floor routine raised on every 2D and 1D golden case (the count it builds for a
  warning it discards, Source/PrimCons_HelperModule.py:499-554), exactly.
* A NaN planted in the upload sets the non-finite flag; a fresh upload clears it.
* ``mhd2d_validate`` restates the reference's validatePrimVars
  (Source/SimulationGrid_HelperModule.py:282-410): a negative density planted in
  the upload is found before any cycle runs, and ``check_state`` raises the
  reference's RuntimeError.
* A corrupt batched work list (a tile out of range, a tile repeated, a tile
  missing) is rejected on the host before launch; a valid reordering of the list
  gives bitwise the same result.
"""
import json
import os

import numpy as np
import pytest

from pythonmhd_gb300 import _lib
from pythonmhd_gb300 import initial_conditions as ic
from pythonmhd_gb300.solver import Batch2D, Grid1D, Grid2D
from tests.golden_io import GOLDEN_DIR, case_id, golden_files, load

pytestmark = pytest.mark.gpu
ARG = 1


def _reference_counts():
    with open(os.path.join(GOLDEN_DIR, "floor_counts.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("arith", ["exact", "fast"])
@pytest.mark.parametrize("path", golden_files("mhd") + golden_files("hydro") + golden_files("mhd1d")
                         + golden_files("hydro1d"), ids=case_id)
def test_floor_hits_equal_the_reference_count(path, arith):
    """Counts of the reference's own floor routine on each case (tests/golden/floor_counts.json,
    which the oracle's tally reproduces on the CPU)."""
    name = case_id(path)
    mhd = name.startswith("mhd")
    p, i, _ = load(path)
    recon = 2 if p["order"] == 2 else 0
    kw = dict(mhd=mhd, recon=recon, entropy_fix=p["efix"], eps=p["eps"], min_d=p["min_d"], min_p=p["min_p"],
              min_e=p["min_e"], arith=arith)
    if "1d" in name.split("_")[0]:
        g = Grid1D(i["prim"].shape[-1], p["dx"], p["bcx"], p["gamma"], **kw)
        g.upload(i["prim"], i["cons"])
    else:
        ny, nx = i["prim"].shape[1:]
        g = Grid2D(ny, nx, p["dx"], p["dy"], p["bcx"], p["bcy"], p["gamma"], **kw)
        g.upload(i["prim"], i["cons"], i.get("fbx"), i.get("fby"))
    try:
        if p["t_start"] < p["t_end"]:
            g.advance(p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["cfl"])
        st = g.stats()
        assert st["floor_hits"] == _reference_counts()[name]
        assert not st["nan"]
    finally:
        g.close()


def test_nan_flag_and_fresh_upload():
    prim, cons, fbx, fby, dx, dy = ic.orszag_tang(24, 20)
    g = Grid2D(20, 24, dx, dy, 1, 1, 5.0 / 3.0, mhd=True, recon=2, arith="exact")
    try:
        bad_p, bad_c = prim.copy(), cons.copy()
        bad_p[7, 3, 4] = np.nan
        bad_c[7, 3, 4] = np.nan
        g.upload(bad_p, bad_c, fbx, fby)
        assert g.validate()["nonfinite"] == 1
        with pytest.raises(_lib.MhdError):
            g.advance(0.0, 1.0, 0, 3, 0.4)
        assert g.stats()["nan"]
        g.upload(prim, cons, fbx, fby)
        assert g.stats() == {"floor_hits": 0, "nan": False}
        g.advance(0.0, 1.0, 0, 3, 0.4)
        assert g.stats() == {"floor_hits": 0, "nan": False}
    finally:
        g.close()


def test_validate_finds_a_negative_density_before_any_cycle():
    prim, cons, fbx, fby, dx, dy = ic.orszag_tang(24, 20)
    g = Grid2D(20, 24, dx, dy, 1, 1, 5.0 / 3.0, mhd=True, recon=2, arith="exact")
    try:
        g.upload(prim, cons, fbx, fby)
        assert all(v == 0 for v in g.validate().values())
        g.check_state()
        bad = prim.copy()
        bad[0, 7, 9] = -0.5
        bad[0, 2, 2] = 1e-14           # below the 1e-12 floor, not negative
        g.upload(bad, cons, fbx, fby)
        c = g.validate()
        # the reference's energy of each cell, in its order of operations
        e = 0.5 * bad[0] * (bad[1] * bad[1] + bad[2] * bad[2] + bad[3] * bad[3])
        e += bad[7] / (5.0 / 3.0 - 1.0)
        e += 0.5 * (bad[4] * bad[4] + bad[5] * bad[5] + bad[6] * bad[6])
        assert c == {"nonfinite": 0, "density_negative": 1, "density_low": 2, "pressure_negative": 0,
                     "pressure_low": 0, "energy_negative": int(np.sum(e < 0)), "energy_low": int(np.sum(e < 1e-12))}
        with pytest.raises(RuntimeError, match="negative density"):
            g.check_state()
    finally:
        g.close()


def _batch(insts, recon=1):
    b = Batch2D(insts, mhd=True, recon=recon, arith="exact")
    for k, inst in enumerate(insts):
        b.upload(k, inst["prim"], inst["cons"], inst["fbx"], inst["fby"])
    return b


def test_corrupt_work_lists_are_rejected_and_a_reordered_list_is_exact():
    insts = ic.orszag_tang_batch(count=3, seed=8, sizes=(16, 24, 40))
    b = _batch(insts)
    try:
        for space in range(6):
            t = b.get_tiles(space)
            n = len(t)
            assert n > 0
            for bad in (np.vstack([t, t[:1]]),                        # a tile twice
                        t[1:],                                        # a tile missing
                        np.vstack([t[:-1], t[:1]])):                  # one missing, one repeated
                with pytest.raises(_lib.MhdError) as e:
                    b.set_tiles(space, bad)
                assert e.value.status == ARG
            for col, val in ((0, 3), (0, -1), (1, 10 ** 6), (2, 7), (3, 1)):   # out of range / misaligned
                bad = t.copy()
                bad[n // 2, col] = val
                with pytest.raises(_lib.MhdError) as e:
                    b.set_tiles(space, bad)
                assert e.value.status == ARG
            assert np.array_equal(b.get_tiles(space), t)              # the installed list stays
        b.advance(0.0, 1.0, 0, 4, 0.4)
        want = [b.download(k) for k in range(3)]
    finally:
        b.close()
    b = _batch(insts)
    try:
        for space in range(6):
            b.set_tiles(space, b.get_tiles(space)[::-1])              # largest index first
        b.advance(0.0, 1.0, 0, 4, 0.4)
        for k in range(3):
            for a, w in zip(b.download(k), want[k]):
                assert np.array_equal(a, w)
        hits, nan = b.stats()
        assert not nan.any() and (hits == 0).all()
    finally:
        b.close()
