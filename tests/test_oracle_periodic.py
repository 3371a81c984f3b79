"""Periodic directions in the oracle (ghost images of PC_Comm_For_Cntct, the
FineSearch3 / ContactForce_PPG pair, periodic wrap in Comm_For_Exchange):
a bed in a periodic box gives the same contact set and forces as the same bed
with its images placed explicitly, and particles wrap instead of leaving."""
import numpy as np

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, props
from sdem_gb300.geometry import WallSet


def periodic_pair_case(periodic, shift_axis, gap=-2e-6, v=0.1):
    t = props.build_tables(2, [1e-3], [2500.0], [5e7], [0.3], (0.3, 0.3, 0.1, 0.8, 0.8), [5e7], [0.3],
                           (0.3, 0.3, 0.1, 0.8, 0.8))
    L = 0.008
    o = beds.Options(dt=1e-6, minpoint=(0, 0, 0), maxpoint=(L, L, L), gravity=(0.0, 0.0, 0.0), cf_type=2,
                     pi_method=2, pri_method=2, periodic=tuple(periodic))
    r = 0.5e-3
    a = np.array([L / 2, L / 2, L / 2])
    b = a.copy()
    a[shift_axis] = r + 0.5 * gap + 1e-5          # near the min face
    b[shift_axis] = L - r - 0.5 * gap + 1e-5      # near the max face: touches a's image
    vel = np.zeros((2, 3))
    vel[0, shift_axis] = -v
    vel[1, shift_axis] = v
    p = beds.new_particles(np.stack([a, b]), np.array([1, 1]), t.radius, vel, 2, 2)
    return beds.Case("pp", o, t, WallSet(), p)


def test_periodic_image_contact_is_found_and_symmetric():
    for axis in range(3):
        per = [0, 0, 0]
        per[axis] = 1
        s = OracleSystem(periodic_pair_case(per, axis))
        s.step(1)
        c = s.counters()
        assert c["ppg"] == 2 and c["pp"] == 0, (axis, c)   # each particle sees the other's image
        F, T = s.forces()
        # a head-on image contact: equal and opposite up to the rounding of the shift
        np.testing.assert_allclose(F[0], -F[1], rtol=1e-9, atol=1e-15)
        assert abs(F[0, axis]) > 1e-6 and F[0, axis] > 0   # pushed away from the boundary


def test_non_periodic_same_geometry_has_no_contact():
    s = OracleSystem(periodic_pair_case([0, 0, 0], 1))
    s.step(1)
    assert s.counters()["ppg"] == 0 and s.counters()["pp"] == 0


def test_periodic_wrap_keeps_particles():
    case = beds.lattice_cloud_case(300, seed=71, vmax=30.0)
    case = beds.scaled(case, periodic=(1, 1, 1))
    case.walls = WallSet()
    s = OracleSystem(case)
    s.step(30)
    st = s.state()
    assert st.n == 300
    lo, hi = np.array(case.opts.minpoint), np.array(case.opts.maxpoint)
    assert np.all(st.posR[:, :3] >= lo) and np.all(st.posR[:, :3] < hi)
    assert s.counters()["ppg"] > 0
