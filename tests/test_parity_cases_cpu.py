"""Every case of the GPU parity suite builds and steps through the oracle on
the CPU (so a GPU run never fails on case generation), with many contacts."""
import pytest

from oracle.oracle import OracleSystem
from tests.test_gpu_parity import CASES


@pytest.mark.parametrize("name", sorted(CASES))
def test_case_steps_in_oracle(name):
    case = CASES[name]()
    o = OracleSystem(case)
    o.step(2)
    c = o.counters()
    assert c["pp"] > 50 and c["nlocal"] == case.particles.n
