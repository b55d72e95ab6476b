"""The drop-in installs into the module attributes the reference driver reads
(Source/Simulation.py:312-324) and can be undone.  A stand-in ``Source`` package
is used so the test needs neither the reference nor a GPU."""
import sys
import types

from pythonmhd_gb300 import dropin, evolve


def _fake_source(monkeypatch):
    pkg = types.ModuleType("Source")
    pkg.__path__ = []
    mhd = types.ModuleType("Source.EvolveFunctions_MHD")
    hyd = types.ModuleType("Source.EvolveFunctions_Hydro")
    mhd.evolve_2D_mhd = lambda *a, **k: "reference-mhd"
    hyd.evolve_2D_hydro = lambda *a, **k: "reference-hydro"
    mhd.evolve_1D_mhd = lambda *a, **k: "reference-mhd-1d"
    hyd.evolve_1D_hydro = lambda *a, **k: "reference-hydro-1d"
    hyd.evolve_3D_hydro = lambda *a, **k: "reference-hydro-3d"
    mhd.evolve_3D_mhd = lambda *a, **k: "reference-mhd-3d"
    monkeypatch.setitem(sys.modules, "Source", pkg)
    monkeypatch.setitem(sys.modules, "Source.EvolveFunctions_MHD", mhd)
    monkeypatch.setitem(sys.modules, "Source.EvolveFunctions_Hydro", hyd)
    return mhd, hyd


def test_install_and_uninstall(monkeypatch):
    mhd, hyd = _fake_source(monkeypatch)
    orig_m, orig_h = mhd.evolve_2D_mhd, hyd.evolve_2D_hydro
    dropin.install()
    assert mhd.evolve_2D_mhd is evolve.evolve_2D_mhd
    assert hyd.evolve_2D_hydro is evolve.evolve_2D_hydro
    assert mhd.evolve_1D_mhd is evolve.evolve_1D_mhd
    assert hyd.evolve_1D_hydro is evolve.evolve_1D_hydro
    assert hyd.evolve_3D_hydro is evolve.evolve_3D_hydro
    assert mhd.evolve_3D_mhd is evolve.evolve_3D_mhd
    dropin.uninstall()
    assert mhd.evolve_2D_mhd is orig_m and hyd.evolve_2D_hydro is orig_h
    assert mhd.evolve_1D_mhd() == "reference-mhd-1d"
    assert hyd.evolve_3D_hydro() == "reference-hydro-3d"


def test_install_with_arith_binds_the_mode(monkeypatch):
    mhd, hyd = _fake_source(monkeypatch)
    dropin.install(arith="fast")
    assert mhd.evolve_2D_mhd.keywords == {"arith": "fast"}
    assert mhd.evolve_2D_mhd.func is evolve.evolve_2D_mhd
    dropin.uninstall()


def test_evolve_keeps_reference_signature():
    import inspect
    ref = ["simulationGrid", "tStart", "tEnd", "startCycle", "maxCycles", "gamma", "cfl", "minDens",
           "minPres", "minEnergy", "reconstructOrder", "entropyFix", "epsilon"]
    for fn in (evolve.evolve_2D_mhd, evolve.evolve_2D_hydro, evolve.evolve_1D_mhd, evolve.evolve_1D_hydro,
               evolve.evolve_3D_hydro):
        params = list(inspect.signature(fn).parameters)
        assert params[:len(ref)] == ref
        sig = inspect.signature(fn).parameters
        assert sig["reconstructOrder"].default == 0
        assert sig["entropyFix"].default is False
        assert sig["epsilon"].default == 0.5
    # the reference's evolve_3D_mhd turns its entropy fix on by default
    params = list(inspect.signature(evolve.evolve_3D_mhd).parameters)
    assert params[:len(ref)] == ref
    assert inspect.signature(evolve.evolve_3D_mhd).parameters["entropyFix"].default is True
