"""sdem_counters_lagged: with step k+1 already enqueued, the counters read for
step k equal the counters a synchronous run reads after step k, step by step;
a state rewritten by an upload starts over; multi-step calls fall back to the
last step's counters."""
import pytest

from sdem_gb300 import beds
from sdem_gb300.capi import DEMSystem

pytestmark = pytest.mark.gpu

STEPS = 12


def synchronous_counters(case):
    s = DEMSystem(case)
    out = []
    for _ in range(STEPS):
        s.step(1)
        out.append(s.counters())
    s.close()
    return out


def lagged_counters(s):
    out = []
    s.step_async(1)
    for k in range(1, STEPS + 1):
        if k < STEPS:
            s.step_async(1)            # step k+1 runs while step k's counters are read
            out.append(s.counters_lagged())
        else:
            out.append(s.counters())
    return out


@pytest.mark.parametrize("periodic", [False, True])
def test_lagged_counters_equal_synchronous(gpu_lib, periodic):
    if periodic:
        case = beds.periodic_lattice_case(800, 41, (1, 0, 1))
    else:
        case = beds.lattice_cloud_case(800, seed=42, finite_walls=True)
    want = synchronous_counters(case)
    assert want[-1]["pp"] > 0
    s = DEMSystem(case)
    got = lagged_counters(s)
    for k, (g, w) in enumerate(zip(got, want), start=1):
        assert g["iter"] == k
        assert g == w, f"step {k}"
    # an upload of the initial state restarts the iteration count and the
    # lagged reads with it
    s.upload(case.particles)
    again = lagged_counters(s)
    for k, (g, w) in enumerate(zip(again, want), start=1):
        assert g == w, f"after re-upload, step {k}"
    s.close()


def test_lagged_counters_fallbacks(gpu_lib):
    case = beds.lattice_cloud_case(800, seed=7, finite_walls=False)
    s = DEMSystem(case)
    # fewer than two steps since the upload: the last step's counters
    s.step_async(1)
    assert s.counters_lagged()["iter"] == 1
    # two single steps in one call: the first of them
    s.step_async(2)
    assert s.counters_lagged()["iter"] == 2
    # a long call replays the two-step graph: only every second step carries
    # a completion event, so the read falls back to the last step
    s.step_async(6)
    c = s.counters_lagged()
    assert c["iter"] in (8, 9)
    assert s.counters()["iter"] == 9
    s.close()
