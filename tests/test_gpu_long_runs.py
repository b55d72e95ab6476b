"""Long runs through the drop-in evolve functions, bit for bit against digests of the
reference's own runs (``tests/golden/make_long_run_digests.py``): Brio-Wu and Sod
shock tubes (800 cells), a 2D hydro blast (128²) and a 3D hydro blast (32³), all
PPM, each for hundreds of cycles or tens of cycles in 3D.  Equal SHA-256 digests of
the final prim and cons mean equal states after the whole run.
"""
import json

import pytest

from pythonmhd_gb300 import evolve
from tests.golden import make_long_run_digests as lr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(lr.RUNS))
def test_long_run_bitwise_vs_reference(name):
    with open(lr.OUT) as f:
        want = json.load(f)[name]
    run = lr.RUNS[name]()
    r = getattr(evolve, lr.evolve_name(run))(lr.grid_of(run), *lr.args_of(run), arith="exact")
    assert (float(r[2]), int(r[3])) == (want["t"], want["cycle"])
    assert lr.digest(r[0], r[1]) == want["sha256"]
