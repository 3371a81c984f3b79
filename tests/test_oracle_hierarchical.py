"""The oracle's hierarchical search (CS_Method 2, Prtcl_Hrchl_Munjiza.f90)
finds the same contacts as the one-level search (the reference's stated
property: the levels change the candidates, not the contact set), counts its
cross-level candidates separately, and the steps agree to rounding."""
import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds
from tests.helpers import keyed_contacts

CASES = {
    "hopper_two_levels": lambda: beds.hopper_case(1500, 51),
    "poly_three_levels": lambda: beds.lattice_cloud_case(800, 71, ntypes=9, d_lo=0.3e-3, d_hi=1.2e-3, nn=0.9e-3),
    "periodic_two_levels": lambda: beds.periodic_lattice_case(800, 31, (1, 1, 1), d_lo=0.4e-3, d_hi=1.2e-3, ntypes=5),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_same_contacts_as_one_level(name):
    c1 = CASES[name]()
    c2 = beds.scaled(c1, cs_method=2)
    o1, o2 = OracleSystem(c1), OracleSystem(c2)
    for k in range(6):
        o1.step(1)
        o2.step(1)
        k1 = keyed_contacts(o1, c1.opts.base_wall_id)
        k2 = keyed_contacts(o2, c1.opts.base_wall_id)
        assert set(k1) == set(k2), (name, k)
    a, b = o1.counters(), o2.counters()
    for key in ("pp", "ppg", "pw", "nlocal"):
        assert a[key] == b[key]
    assert b["cnsv_cross"] > 0 and a["cnsv_cross"] == 0
    F1, _ = o1.forces()
    F2, _ = o2.forces()
    assert np.abs(F1 - F2).max() <= 1e-12 * np.abs(F1).max()
