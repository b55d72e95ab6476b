"""The CPU oracle reproduces the reference's own outputs bit for bit.

The fixtures were produced by running the reference PythonMHD step
(Source/EvolveFunctions_MHD.py:393, Source/EvolveFunctions_Hydro.py:350) with
tests/golden/make_golden.py; this pins the oracle before anything is checked
against it.
"""
import numpy as np
import pytest

from oracle import hydro2d, mhd2d
from tests.golden_io import HYDRO_KEYS, MHD_KEYS, case_id, golden_files, load


@pytest.mark.parametrize("path", golden_files("mhd"), ids=case_id)
def test_oracle_mhd_matches_reference_bitwise(path):
    p, i, o = load(path)
    res = mhd2d.evolve(i["prim"], i["cons"], i["fbx"], i["fby"], p["dx"], p["dy"], p["bcx"], p["bcy"],
                       p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"],
                       p["cfl"], p["min_d"], p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])
    for k, v in zip(MHD_KEYS, res):
        assert np.array_equal(np.asarray(v), o[k]), k


@pytest.mark.parametrize("path", golden_files("hydro"), ids=case_id)
def test_oracle_hydro_matches_reference_bitwise(path):
    p, i, o = load(path)
    res = hydro2d.evolve(i["prim"], i["cons"], p["dx"], p["dy"], p["bcx"], p["bcy"],
                         p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"],
                         p["cfl"], p["min_d"], p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])
    for k, v in zip(HYDRO_KEYS, res):
        assert np.array_equal(np.asarray(v), o[k]), k


def test_golden_set_is_complete():
    assert len(golden_files("mhd")) >= 18
    assert len(golden_files("hydro")) >= 8


@pytest.mark.parametrize("path", golden_files("mhd1d") + golden_files("hydro1d"), ids=case_id)
def test_oracle_1d_matches_reference_bitwise(path):
    """The 1D restatement (oracle/evolve1d.py) against evolve_1D_mhd / evolve_1D_hydro
    (Source/EvolveFunctions_MHD.py:195, Source/EvolveFunctions_Hydro.py:232)."""
    from oracle import evolve1d
    p, i, o = load(path)
    fn = evolve1d.evolve_mhd if case_id(path).startswith("mhd1d") else evolve1d.evolve_hydro
    res = fn(i["prim"], i["cons"], p["dx"], p["bcx"], p["t_start"], p["t_end"], p["start_cycle"],
             p["max_cycles"], p["gamma"], p["cfl"], p["min_d"], p["min_p"], p["min_e"], p["order"], p["efix"],
             p["eps"])
    for k, v in zip(HYDRO_KEYS, res):
        assert np.array_equal(np.asarray(v), o[k]), k


def test_golden_1d_set_is_complete():
    assert len(golden_files("mhd1d")) >= 8
    assert len(golden_files("hydro1d")) >= 7


@pytest.mark.parametrize("path", golden_files("hydro3d"), ids=case_id)
def test_oracle_3d_hydro_matches_reference_bitwise(path):
    """The 3D restatement (oracle/hydro3d.py) against evolve_3D_hydro
    (Source/EvolveFunctions_Hydro.py:559)."""
    from oracle import hydro3d
    p, i, o = load(path)
    res = hydro3d.evolve(i["prim"], i["cons"], p["dx"], p["dy"], p["dz"], p["bcx"], p["bcy"], p["bcz"],
                         p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"], p["cfl"],
                         p["min_d"], p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])
    for k, v in zip(HYDRO_KEYS, res):
        assert np.array_equal(np.asarray(v), o[k]), k


def test_golden_3d_set_is_complete():
    assert len(golden_files("hydro3d")) >= 16


def test_3d_floor_cases_apply_floors():
    """The floor fixtures move when the floors are lowered: the floors act there."""
    from oracle import hydro3d
    for name in ("floors_ppm", "floors_order0"):
        p, i, o = load([f for f in golden_files("hydro3d") if case_id(f).endswith(name)][0])
        res = hydro3d.evolve(i["prim"], i["cons"], p["dx"], p["dy"], p["dz"], p["bcx"], p["bcy"], p["bcz"],
                             p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"], p["cfl"],
                             1e-12, 1e-12, 1e-12, p["order"], p["efix"], p["eps"])
        assert not np.array_equal(res[1], o["cons"])


MHD3D_KEYS = ("prim", "cons", "fbx", "fby", "fbz", "t", "cycle", "sl_prim", "sl_cons", "sl_fbx", "sl_fby", "sl_fbz",
              "sl_t")


@pytest.mark.parametrize("path", golden_files("mhd3d"), ids=case_id)
def test_oracle_3d_mhd_matches_reference_bitwise(path):
    """The 3D MHD restatement (oracle/mhd3d.py) against evolve_3D_mhd
    (Source/EvolveFunctions_MHD.py:750).  The reference's x predictor computes its y
    terms in np.longdouble (80-bit on the x86 host that made these fixtures), and so
    does the oracle; on a host whose long double differs the last bits can too."""
    import platform

    from oracle import mhd3d
    p, i, o = load(path)
    res = mhd3d.evolve(i["prim"], i["cons"], i["fbx"], i["fby"], i["fbz"], p["dx"], p["dy"], p["dz"], p["bcx"],
                       p["bcy"], p["bcz"], p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"],
                       p["cfl"], p["min_d"], p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])
    exact = platform.machine() in ("x86_64", "AMD64")
    for k, v in zip(MHD3D_KEYS, res):
        v = np.asarray(v)
        if exact:
            assert np.array_equal(v, o[k]), k
        else:
            assert np.allclose(v, o[k], rtol=1e-12, atol=1e-12 * max(1.0, float(np.max(np.abs(o[k]))))), k


def test_golden_3d_mhd_set_is_complete():
    assert len(golden_files("mhd3d")) >= 15


def test_ot128_full_run_oracle_pinned_to_reference():
    """The oracle's 407-cycle PPM Orszag-Tang run (128², t 0 -> 0.5) has the same
    final-state digest as the reference's own run (tests/golden/make_ot128_digests.py)."""
    import json
    from tests.golden import make_ot128_digests as ot
    with open(ot.OUT) as f:
        d = json.load(f)
    assert d["reference_ppm"] == d["oracle_ppm"]
    assert d["reference_ppm"]["cycle"] > 300 and d["oracle_plm"]["t"] == 0.5


def test_long_run_digests_cover_every_run():
    """tests/golden/long_run_digests.json holds a digest of the reference's own run for
    every run of tests/golden/make_long_run_digests.py (the generator checks the
    oracle's runs against them)."""
    import json
    from tests.golden import make_long_run_digests as lr
    with open(lr.OUT) as f:
        d = json.load(f)
    assert set(d) == set(lr.RUNS)
    assert all(len(v["sha256"]) == 64 and v["cycle"] > 10 for v in d.values())


def _field_rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    if a.ndim == 4:
        return max(float(np.max(np.abs(a[i] - b[i]))) / max(float(np.max(np.abs(b[i]))), 1e-300)
                   for i in range(a.shape[0]))
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-300)


def test_oracle_3d_mhd_40_cycles_vs_reference():
    """40 cycles of the reference's evolve_3D_mhd (tests/golden/make_mhd3d_long.py):
    the oracle with the reference's long-double predictor terms equals it bit for bit
    on an x86 host; its FP64-predictor form (the CUDA step's) stays within 1e-12."""
    import platform

    from oracle import mhd3d
    from tests.golden import make_mhd3d_long as m
    prim, cons, fbx, fby, fbz, dx, dy, dz = m.initial_state()
    o = np.load(m.OUT)
    exact = platform.machine() in ("x86_64", "AMD64")
    r = mhd3d.evolve(prim, cons, fbx, fby, fbz, dx, dy, dz, 1, 1, 1, *m.ARGS, long_double=True)
    for k, v in zip(m.KEYS, r[:7]):
        if exact:
            assert np.array_equal(np.asarray(v), o[k]), k
        else:
            assert _field_rel(v, o[k]) <= 1e-12, k
    r = mhd3d.evolve(prim, cons, fbx, fby, fbz, dx, dy, dz, 1, 1, 1, *m.ARGS, long_double=False)
    assert int(r[6]) == int(o["cycle"]) == m.CYCLES
    for k, v in zip(m.KEYS[:5], r[:5]):
        assert _field_rel(v, o[k]) <= 1e-12, k


def _floor_counts():
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "floor_counts.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("path", golden_files("mhd") + golden_files("hydro") + golden_files("mhd1d")
                         + golden_files("hydro1d"), ids=case_id)
def test_oracle_floor_tally_matches_reference_counts(path):
    """The oracle's floor tally equals the number of values the reference's own floor
    routine raised on the same case (tests/golden/make_floor_counts.py wraps
    Source/PrimCons_HelperModule.py:499-554 to count them)."""
    from oracle import common, evolve1d
    name = case_id(path)
    p, i, _ = load(path)
    common.reset_floor_tally()
    tail = (p["t_start"], p["t_end"], p["start_cycle"], p["max_cycles"], p["gamma"], p["cfl"], p["min_d"],
            p["min_p"], p["min_e"], p["order"], p["efix"], p["eps"])
    if name.startswith("mhd1d"):
        evolve1d.evolve_mhd(i["prim"], i["cons"], p["dx"], p["bcx"], *tail)
    elif name.startswith("hydro1d"):
        evolve1d.evolve_hydro(i["prim"], i["cons"], p["dx"], p["bcx"], *tail)
    elif name.startswith("mhd"):
        mhd2d.evolve(i["prim"], i["cons"], i["fbx"], i["fby"], p["dx"], p["dy"], p["bcx"], p["bcy"], *tail)
    else:
        hydro2d.evolve(i["prim"], i["cons"], p["dx"], p["dy"], p["bcx"], p["bcy"], *tail)
    assert common.floor_tally() == _floor_counts()[name]


def test_floor_counts_cover_the_floor_cases():
    c = _floor_counts()
    assert c["mhd_floors"] > 0 and c["hydro_floors"] > 0 and c["mhd1d_floors"] > 0


def _driver_digests():
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "driver_digests.json")) as f:
        return json.load(f)


def run_driver_case(case, run_fn):
    """Run one of the reference driver's recorded workloads with ``run_fn(state, w, save_prec,
    plot_prec)`` -> (t, cycle, stops [(t, cycle, kinds, state)], final_state) and compare
    every stop and the end with the reference's digests."""
    from pythonmhd_gb300 import driver
    from tests.golden import make_driver_digests as mdd
    want = _driver_digests()[case]
    w = want["workload"]
    state, dx, dy, bcx, bcy = mdd.initial_state(case)
    state = tuple(a for a in state if a is not None)
    assert mdd.digest(*state) == want["initial_sha256"]
    sp = driver.time_precision(w["save_dt"], w["t_lim"]) if w["save_dt"] > 0 else 0
    pp = driver.time_precision(w["plot_dt"], w["t_lim"]) if w["plot_dt"] > 0 else 0
    t, cyc, stops, final = run_fn(state, w, sp, pp)
    got = [{"t": float(s[0]), "cycle": int(s[1]), "kinds": int(s[2]), "sha256": mdd.digest(*s[3])} for s in stops]
    assert got == want["stops"]
    assert {"t": float(t), "cycle": int(cyc), "sha256": mdd.digest(*final)} == want["final"]


@pytest.mark.parametrize("case", sorted(_driver_digests()))
def test_oracle_driver_matches_the_reference_driver(case):
    """oracle/driver.py against the reference's own Simulation.run() (Source/Simulation.py:
    277-434, run headless by tests/golden/make_driver_digests.py): every stop's time, cycle,
    kind and state, and the final state, bit for bit."""
    from oracle import driver as odriver

    def run(state, w, sp, pp):
        fb = state[2:] if len(state) == 4 else (None, None)
        return odriver.run(state[0], state[1], fb[0], fb[1], w["dx"], w["dy"], w["bcx"], w["bcy"], w["t_lim"],
                           w["max_cycles"], w["gamma"], w["cfl"], 1e-12, 1e-12, 1e-12, w["order"], False, 0.5,
                           save_dt=w["save_dt"], save_prec=sp, plot_dt=w["plot_dt"], plot_prec=pp)

    run_driver_case(case, run)


def test_reference_is_tie_sensitive_only_on_the_known_cases():
    """The reference's own one-cycle output moves by more than 1e-12 under one-ulp input
    changes only on the two golden states that sit on exact ties of its branches
    (tests/conditioning.py); everywhere else it is well conditioned to 1e-13."""
    from tests.conditioning import sensitivity
    s = {case_id(f): sensitivity(f) for f in golden_files("mhd") + golden_files("hydro")}
    assert {k for k, v in s.items() if v > 1e-12} == {"mhd_ot_order0", "mhd_zero_btran"}
    assert s["mhd_zero_btran"] > 1e-7 and s["mhd_ot_order0"] > 1e-12
    assert all(v <= 1e-12 for k, v in s.items() if k not in ("mhd_ot_order0", "mhd_zero_btran"))
