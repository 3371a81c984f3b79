"""The kernels divide several numerators by one divisor as q' = fma(r, y, q)
with y = RN(1/b), q = RN(a*y), r = fma(-q, b, a) (Markstein's correction);
this must equal IEEE a/b bit for bit on the ranges the hot path sees.  Checked
here on the CPU with libm fma (correctly rounded), the same arithmetic the
device's __fma_rn performs."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("mk") / "libmk.so")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", out,
                    os.path.join(HERE, "csrc", "markstein_check.c"), "-lm"], check=True)
    L = ctypes.CDLL(out)
    L.markstein_mismatches.restype = ctypes.c_longlong
    L.markstein_mismatches.argtypes = [ctypes.c_longlong, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                       ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    return L


@pytest.mark.parametrize("lo,hi", [(-60, 60), (-200, 200), (-30, 10)])
def test_random_quotients(lib, lo, hi):
    assert lib.markstein_mismatches(3_000_000, 12345 + lo, lo, hi, None, 0) == 0


def test_type_masses_and_inertias(lib):
    from sdem_gb300 import beds
    _, t = beds.hertz_poly_tables(41)
    d = np.ascontiguousarray(np.concatenate([t.mass, t.inertia]))
    assert lib.markstein_mismatches(3_000_000, 99, -40, 10, d.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    len(d)) == 0
