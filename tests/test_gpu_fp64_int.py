"""On the GPU: the integer-pipe binary64 arithmetic the kernels use for
sqrt, division, comparisons, the binning's floor and the AB2 -1/2 factor gives
the same bits as the hardware instructions (__dsqrt_rn, __ddiv_rn, __dmul_rn,
the FP64 comparisons), with the device's own rsqrt/rcp approximation seeds."""
import pytest

from sdem_gb300.capi import selftest_fp64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2])
def test_integer_arithmetic_matches_hardware(gpu_lib, seed):
    assert selftest_fp64(20_000_000, seed) == 0
