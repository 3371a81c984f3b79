"""The 4M bidisperse (1:3) Hertz hopper of the third configuration discharging.

4,000,000 spheres of 0.5 and 1.5 mm (70:30), friction 0.5, restitution 0.7,
dt 5e-7 s, in four 60-degree finite planes over a 10 mm square outlet with a
column above (0.26 m wide).  The GPU runs 12,000 steps (6 ms): spheres leave
through the outlet and are deleted (one rank, Prtcl_Comm.f90:1569-1840), no
row or container overflows (SDEM_E_CL_FULL) although a large sphere can touch
dozens of small ones -- the row capacity follows the size ratio
(capi.row_capacity_for: 59 contacts per sphere here; the reference itself has
no per-sphere cap, only its restart writer's 20, Prtcl_CL_and_CF.f90:641,648)
-- and the next step from that state and contact list matches the oracle:
counters and contact sets equal, history, forces and torques within 1e-12
(a spring relative to the sum of the normal force's elastic and damping
magnitudes where those nearly cancel: a spring of 7e-11 m at an approach of
0.18 m/s differed by 1.2e-12 of itself, tests/helpers.py:hertz_spring_scale).
"""
import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds
from sdem_gb300.capi import DEMSystem, row_capacity_for
from tests.helpers import assert_step_matches

pytestmark = pytest.mark.gpu


def test_hopper_4m_discharges_then_matches_oracle(gpu_lib):
    case = beds.hopper_case(4_000_000, 3, width=0.26, outlet=10.0e-3)
    assert row_capacity_for(case.tables.radius) == 59
    g = DEMSystem(case)
    n0 = case.particles.n
    left = []
    for _ in range(6):
        g.step(2000)                   # raises SdemError on any device error (SDEM_E_CL_FULL included)
        left.append(n0 - g.counters()["nlocal"])
    st, cl = g.state(), g.contacts()
    per = np.bincount(cl[0], minlength=st.n)
    print(f"hopper 4M: spheres deleted after 2000..12000 steps {left}; most contacts on one sphere {per.max()}")
    assert left[-1] > left[0] > 0 and all(b >= a for a, b in zip(left, left[1:]))
    o = OracleSystem(beds.Case(case.name, case.opts, case.tables, case.walls, st, contacts=cl))
    g.step(1)
    o.step(1)
    assert_step_matches(g, o, what="hopper after 12000 steps", pre=st, case=case)
    o.close()
    g.close()
