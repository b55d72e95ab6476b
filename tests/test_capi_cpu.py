"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, and
exports every entry point that include/pythonmhd_gb300.h declares.  No compute
call is made here (there is no GPU in this environment)."""
import ctypes
import os
import re

import pytest

from pythonmhd_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "pythonmhd_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mhd(?:1d|2d|3d|b)?_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("mhd2d_create", "mhd2d_upload", "mhd2d_advance", "mhd2d_download", "mhd2d_destroy",
              "mhd2d_strerror", "mhd1d_create", "mhdb_create", "mhd3d_create", "mhd3d_advance"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_the_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_strerror_names_every_status(lib):
    for code in range(0, 9):
        assert lib.mhd2d_strerror(code).decode() not in ("", "unknown status")
    assert lib.mhd2d_strerror(99).decode() == "unknown status"


def test_create_rejects_bad_arguments_before_touching_the_device(lib):
    h = ctypes.c_void_p()
    bad = [
        (1, 16, 0.1, 0.1, 1, 1),     # ny < 2
        (16, 1, 0.1, 0.1, 1, 1),     # nx < 2
        (16, 16, 0.0, 0.1, 1, 1),    # dx <= 0
        (16, 16, 0.1, 0.1, 2, 1),    # bad BC code
    ]
    for ny, nx, dx, dy, bx, by in bad:
        rc = lib.mhd2d_create(ny, nx, dx, dy, bx, by, 1.4, 1, 2, 0, 0.5, 1e-12, 1e-12, 1e-12, 0, ctypes.byref(h))
        assert rc == 1 and not h.value
    rc = lib.mhd2d_create(16, 16, 0.1, 0.1, 1, 1, 1.4, 1, 3, 0, 0.5, 1e-12, 1e-12, 1e-12, 0, ctypes.byref(h))
    assert rc == 1  # recon must be 0 (first order), 1 (PLM) or 2 (PPM)
    assert lib.mhd2d_upload(None, None, None, None, None) == 1
    lib.mhd2d_destroy(None)


def test_null_handle_calls_fail_cleanly(lib):
    t = ctypes.c_double()
    c = ctypes.c_longlong()
    assert lib.mhd2d_advance(None, 0.0, 1.0, 0, 1, 0.4, ctypes.byref(t), ctypes.byref(c), ctypes.byref(t)) == 1
    assert lib.mhd2d_download(None, 0, None, None, None, None) == 1


def test_adjoint_entry_points_reject_bad_arguments(lib):
    h = ctypes.c_void_p()
    # the adjoint covers first order (0), PLM (1) and PPM (2)
    rc = lib.mhd2d_adj_create(16, 16, 0.1, 0.1, 1, 1, 1.4, 3, 0, 0.5, 1e-12, 1e-12, 1e-12, ctypes.byref(h))
    assert rc == 1 and not h.value
    rc = lib.mhd2d_adj_create(1, 16, 0.1, 0.1, 1, 1, 1.4, 1, 0, 0.5, 1e-12, 1e-12, 1e-12, ctypes.byref(h))
    assert rc == 1 and not h.value
    assert lib.mhd2d_adj_cycle(None, 0.1, None, None) == 1
    assert lib.mhd2d_adj_backward(None, None, None) == 1
    assert lib.mhd2d_adj_forward(None, None, 1, 0.4, None, 0, None, None) == 1
    lib.mhd2d_adj_destroy(None)


def test_arithmetic_hooks_reject_bad_arguments_before_touching_the_device(lib):
    # mhd_softfp: op 0..4 (add, subtract, multiply, divide, sqrt), n >= 0, pointers for n > 0
    assert lib.mhd_softfp(5, None, None, None, 1) == 1
    assert lib.mhd_softfp(-1, None, None, None, 1) == 1
    assert lib.mhd_softfp(0, None, None, None, -1) == 1
    assert lib.mhd_softfp(3, None, None, None, 4) == 1
    assert lib.mhd_softfp(2, None, None, None, 0) == 0   # nothing to do: no launch
    assert lib.mhd_quotient6(None, None, -1) == 1
    assert lib.mhd_quotient6(None, None, 0) == 0


def test_adjoint_codegen_places_the_integer_pipe_division_per_stage():
    """The generated forward statements divide and take square roots on the integer pipes
    only in the stages listed in ``codegen.INTEGER_PIPE_DIVSQRT`` (the small CT, half-step
    and update stages, where that measured faster); the taped reconstruction and Roe
    stages keep the FP64 instructions."""
    from pythonmhd_gb300.adjoint import codegen
    src = codegen.generate()
    blocks = re.split(r"\n// ---- (\w+): ", src)[1:]
    seen = {}
    for name, body in zip(blocks[0::2], blocks[1::2]):
        m = re.search(r"#define DSL_FDIV (\S+)\n#define DSL_FSQRT (\S+)", body)
        assert m, name
        seen[name] = m.groups()
    assert set(seen) == {n for n, *_ in codegen.STAGES}
    for name, (div, sq) in seen.items():
        if name in codegen.INTEGER_PIPE_DIVSQRT:
            assert (div, sq) == ("mhdk::ddiv", "mhdk::sqrt"), name
        else:
            assert (div, sq) == ("__ddiv_rn", "__dsqrt_rn"), name
    assert {"roe1_0", "plm0", "pslope0", "ppmt0"}.isdisjoint(codegen.INTEGER_PIPE_DIVSQRT)


def test_driver_time_precision_follows_the_reference_rule():
    from pythonmhd_gb300 import driver
    assert driver.time_precision(0.01, 0.5) == 2
    assert driver.time_precision(0.1, 1.0) == 1
    assert driver.time_precision(0.0075, 0.03) == 4
    assert driver.time_precision(0.25, 0.125) == 3
    assert driver.time_precision(1.0 / 3.0, 1.0) == 10
    h = ctypes.c_void_p()
    assert lib_run_rejects_null(h)


def lib_run_rejects_null(h):
    from pythonmhd_gb300 import _lib
    lib = _lib.load()
    t = ctypes.c_double()
    c = ctypes.c_longlong()
    return lib.mhd2d_run(None, 1.0, 10, 0.4, -1.0, 0, -1.0, 0, None, None, ctypes.byref(t), ctypes.byref(c),
                         ctypes.byref(c)) == 1


def test_3d_entry_points_reject_bad_arguments(lib):
    h = ctypes.c_void_p()
    ok = [8, 8, 8, 0.1, 0.1, 0.1, 1, 1, 1, 1.4, 0, 2, 0, 0.5, 1e-12, 1e-12, 1e-12, 0]
    bad = {0: 1, 2: 1, 5: 0.0, 8: 2, 10: 2, 11: 3, 17: 2}   # ny < 2, nz < 2, dz <= 0, BC, physics, recon, arith
    for i, v in bad.items():
        args = list(ok)
        args[i] = v
        assert lib.mhd3d_create(*args, ctypes.byref(h)) == 1 and not h.value, i
    big = list(ok)
    big[0] = big[1] = big[2] = 2000   # (n+2)^3 above the 32-bit work-item range
    assert lib.mhd3d_create(*big, ctypes.byref(h)) == 6 and not h.value
    t = ctypes.c_double()
    c = ctypes.c_longlong()
    assert lib.mhd3d_advance(None, 0.0, 1.0, 0, 1, 0.4, ctypes.byref(t), ctypes.byref(c), ctypes.byref(t)) == 1
    assert lib.mhd3d_upload(None, None, None, None, None, None) == 1
    assert lib.mhd3d_download(None, 0, None, None, None, None, None) == 1
    lib.mhd3d_destroy(None)


def test_save_mat_writes_the_reference_layout_with_face_b(tmp_path):
    """driver.save_mat: the reference's .mat keys (Source/FileSaver.py:212-231) plus the
    face-centred B a restart needs, faceBz included for a 3D grid."""
    import numpy as np
    import scipy.io
    from pythonmhd_gb300 import driver
    rng = np.random.default_rng(3)
    prim, cons = rng.random((8, 3, 4, 2)), rng.random((8, 3, 4, 2))
    fbx, fby, fbz = rng.random((3, 5, 2)), rng.random((4, 4, 2)), rng.random((3, 4, 3))
    driver.save_mat(str(tmp_path / "s.mat"), prim, cons, fbx, fby, fbz)
    d = scipy.io.loadmat(str(tmp_path / "s.mat"))
    # Source/PythonMHD_Constants.py:86-104: DENSITY "Density", VX "Vx", ..., BX "Bx", ...,
    # PRESSURE "Pressure", ENERGY "Energy"
    for k, i in (("Density", 0), ("Vx", 1), ("Vy", 2), ("Vz", 3), ("Bx", 4), ("By", 5), ("Bz", 6), ("Pressure", 7)):
        np.testing.assert_array_equal(d[k], prim[i])
    np.testing.assert_array_equal(d["Energy"], cons[7])
    for k, a in (("faceBx", fbx), ("faceBy", fby), ("faceBz", fbz)):
        np.testing.assert_array_equal(d[k], a)
    # hydro: no face arrays
    driver.save_mat(str(tmp_path / "h.mat"), prim[:5], cons[:5])
    h = scipy.io.loadmat(str(tmp_path / "h.mat"))
    np.testing.assert_array_equal(h["Pressure"], prim[4])
    np.testing.assert_array_equal(h["Energy"], cons[4])
    assert not any(k.startswith("face") for k in h)
    assert "faceBx" not in h
