"""The integer-pipe FP64 arithmetic (``csrc/softfp.cuh``) on the host.

The step kernels compute their divisions and square roots with integer
Newton-Raphson and an exact remainder check, and the header's add, subtract and
multiply likewise in integers.  The same header compiles for the host; this test
builds ``softfp_check.cpp`` with g++ and compares every operation bit for bit with
the host's IEEE-754 arithmetic on nine operand generators (random bit patterns,
close magnitudes, every exponent difference, runs of equal bits, exact and near-tie
quotients and squares, the limits of each fast path), with the Newton seeds both as
given and perturbed by up to 2^-12 relative.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "pythonmhd_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path_factory.mktemp("softfp") / "softfp_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "softfp_check.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2])
def test_integer_pipe_arithmetic_equals_host_ieee(checker, seed):
    res = subprocess.run([checker, "300000", str(seed)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-3000:]
    assert res.stdout.strip().splitlines()[-1] == "mismatches 0"
