"""The integer-pipe binary64 arithmetic of sdem_gb300/csrc/fp64_int.cuh
(square root, division, comparisons, exact multiplication by -1/2, the grid
floor and the floor of a quotient) is bit-identical to IEEE
round-to-nearest-even: compiled for the host and compared with the host's own
double arithmetic on random and adversarial operand pairs (every exponent,
close exponents, exact squares and quotients, near-ties, overflow and
underflow edges, zeros, subnormals, infinities, NaN)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "fp64_int_check.cpp")


@pytest.fixture(scope="module")
def fpi_check(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("fpi") / "fp64_int_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, SRC], check=True)
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_integer_binary64_matches_ieee(fpi_check, seed):
    r = subprocess.run([fpi_check, str(seed), "400000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    assert r.stdout.startswith("ok ")
