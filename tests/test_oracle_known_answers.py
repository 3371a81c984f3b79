"""Known-answer tests that pin the CPU oracle (the reference ships no tests or
golden vectors; these analytic cases pin the restated physics instead)."""
import math

import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, props
from sdem_gb300.geometry import WallSet, box_walls


def two_sphere_case(cf_type, v, e_n=0.9, mu=0.3, d=1e-3, dt=2e-8, pi=2, pri=1, E=None, walls=None, box=0.01):
    if cf_type == props.CFT_LSD:
        E = E or props.lsd_youngs_for_stiffness(1e4, 0.05, d, 2500.0, 0.3)
    else:
        E = E or 5e7
    c = (mu, mu, 0.0, e_n, e_n)
    t = props.build_tables(cf_type, [d], [2500.0], [E], [0.3], c, [E], [0.3], c)
    o = beds.Options(dt=dt, minpoint=(0, 0, 0), maxpoint=(box, box, box), gravity=(0.0, 0.0, 0.0),
                     cf_type=cf_type, pi_method=pi, pri_method=pri)
    mid = box / 2
    pos = np.array([[mid - 0.5005 * d, mid, mid], [mid + 0.5005 * d, mid, mid]])
    vel = np.array([[v, 0, 0], [-v, 0, 0]])
    p = beds.new_particles(pos, np.array([1, 1]), t.radius, vel, o.tsize, o.rsize)
    return beds.Case("two", o, t, walls or WallSet(), p)


def run_until_separated(sysm, max_steps=200000, chunk=200):
    touched = False
    for _ in range(max_steps // chunk):
        sysm.step(chunk)
        c = sysm.counters()["pp"]
        touched = touched or c > 0
        st = sysm.state()
        gap = st.posR[1, 0] - st.posR[0, 0] - 2 * st.posR[0, 3]
        if touched and c == 0 and gap > 0:
            return st
    raise AssertionError("spheres did not separate")


@pytest.mark.parametrize("v", [0.05, 0.2])
def test_lsd_head_on_restitution(v):
    # Linear spring-dashpot with stiffness and damping frozen at first touch:
    # the damping coefficient of Prtcl_Property.f90:237 gives restitution e_n.
    case = two_sphere_case(props.CFT_LSD, v, e_n=0.9)
    s = OracleSystem(case)
    st = run_until_separated(s, chunk=50)
    vout = st.linVel[1, 0, 0] - st.linVel[0, 0, 0]
    ratio = vout / (2 * v)
    assert abs(ratio - 0.9) < 0.01, ratio


def test_hertz_head_on_restitution():
    # Hertz damping of Prtcl_Property.f90:244 (an empirical fit): restitution
    # close to e_n for a head-on impact.
    case = two_sphere_case(props.CFT_NLIN, 0.2, e_n=0.8, dt=2e-8)
    s = OracleSystem(case)
    st = run_until_separated(s, chunk=200)
    ratio = (st.linVel[1, 0, 0] - st.linVel[0, 0, 0]) / 0.4
    assert abs(ratio - 0.8) < 0.05, ratio


def test_momentum_conserved_in_head_on():
    case = two_sphere_case(props.CFT_NLIN, 0.2, e_n=0.8, dt=2e-8)
    s = OracleSystem(case)
    s.step(400)
    F, T = s.forces()
    assert s.counters()["pp"] == 1
    np.testing.assert_array_equal(F[0], -F[1])


def test_ab2_free_fall_closed_form():
    # AB2 with constant acceleration: v_n = v0 + n a dt, x_n = x0 + n v0 dt + a dt^2 (n^2-1)/2
    t = props.build_tables(1, [1e-3], [2500.0], [1e7], [0.3], (0.3, 0.3, 0.1, 0.9, 0.9), [1e7], [0.3],
                           (0.3, 0.3, 0.1, 0.9, 0.9))
    o = beds.Options(dt=1e-4, minpoint=(0, 0, 0), maxpoint=(1, 1, 1), pi_method=2, pri_method=2)
    p = beds.new_particles(np.array([[0.5, 0.9, 0.5]]), np.array([1]), t.radius, np.array([[0.0, 0.1, 0.0]]), 2, 2)
    p.linAcc[:] = (0.0, -9.81, 0.0)  # AB history already holds the constant acceleration
    s = OracleSystem(beds.Case("fall", o, t, WallSet(), p))
    n = 100
    s.step(n)
    st = s.state()
    a, dt = -9.81, 1e-4
    assert st.linVel[0, 0, 1] == pytest.approx(0.1 + n * a * dt, rel=1e-12)
    assert st.posR[0, 1] == pytest.approx(0.9 + n * 0.1 * dt + a * dt * dt * (n * n - 1) / 2, rel=1e-12)


def test_ab2_rotation_quirk_reads_linear_velocity():
    # Prtcl_Integration.f90:64: with PRI_Method=2 the rotation starts from linVel(1).
    t = props.build_tables(1, [1e-3], [2500.0], [1e7], [0.3], (0.3, 0.3, 0.1, 0.9, 0.9), [1e7], [0.3],
                           (0.3, 0.3, 0.1, 0.9, 0.9))
    o = beds.Options(dt=1e-5, minpoint=(0, 0, 0), maxpoint=(1, 1, 1), pi_method=2, pri_method=2,
                     gravity=(0.0, 0.0, 0.0))
    p = beds.new_particles(np.array([[0.5, 0.5, 0.5]]), np.array([1]), t.radius, np.array([[0.3, 0.2, 0.1]]), 2, 2)
    s = OracleSystem(beds.Case("q", o, t, WallSet(), p))
    s.step(1)
    np.testing.assert_array_equal(s.state().rotVel[0, 0], [0.3, 0.2, 0.1])
    o2 = beds.Options(**{**o.__dict__, "quirk_ab2_rot": 0})
    s2 = OracleSystem(beds.Case("q", o2, t, WallSet(), p))
    s2.step(1)
    np.testing.assert_array_equal(s2.state().rotVel[0, 0], [0.0, 0.0, 0.0])


def test_wall_rebound():
    # sphere dropped onto an infinite floor (no gravity): rebound ratio ~ e_n
    e = 0.8
    t = props.build_tables(2, [1e-3], [2500.0], [5e7], [0.3], (0.3, 0.3, 0.0, e, e), [5e7], [0.3],
                           (0.3, 0.3, 0.0, e, e))
    o = beds.Options(dt=2e-8, minpoint=(0, 0, 0), maxpoint=(0.01, 0.01, 0.01), gravity=(0.0, 0.0, 0.0), cf_type=2,
                     pi_method=2, pri_method=1)
    p = beds.new_particles(np.array([[0.005, 0.000501, 0.005]]), np.array([1]), t.radius,
                           np.array([[0.0, -0.2, 0.0]]), 2, 1)
    w = box_walls((0, 0, 0), (0.01, 0.01, 0.01))
    s = OracleSystem(beds.Case("w", o, t, w, p))
    touched = False
    for _ in range(2000):
        s.step(100)
        c = s.counters()["pw"]
        touched = touched or c > 0
        if touched and c == 0:
            break
    v = s.state().linVel[0, 0, 1]
    assert abs(v / 0.2 - e) < 0.05, v


def test_coulomb_sliding_on_floor():
    # a sphere pressed on the floor (gravity) and sliding: |F_t| = mu_k |F_n| once slipping
    mu = 0.3
    t = props.build_tables(2, [1e-3], [2500.0], [5e7], [0.3], (mu, mu, 0.0, 0.8, 0.8), [5e7], [0.3],
                           (mu, mu, 0.0, 0.8, 0.8))
    o = beds.Options(dt=1e-7, minpoint=(0, 0, 0), maxpoint=(0.01, 0.01, 0.01), gravity=(0.0, -9.81, 0.0), cf_type=2,
                     pi_method=1, pri_method=1)
    r = t.radius[0]
    m = t.mass[0]
    K = t.bpw[2]
    delta = (m * 9.81 / K) ** (2.0 / 3.0)
    p = beds.new_particles(np.array([[0.005, r - delta, 0.005]]), np.array([1]), t.radius,
                           np.array([[0.1, 0.0, 0.0]]), 1, 1)
    w = box_walls((0, 0, 0), (0.01, 0.01, 0.01))
    s = OracleSystem(beds.Case("slide", o, t, w, p))
    s.step(3000)
    F, T = s.forces()
    ft = math.hypot(F[0, 0], F[0, 2])
    fn = abs(F[0, 1])
    assert s.counters()["pw"] == 1
    assert ft == pytest.approx(mu * fn, rel=1e-9)


def test_rebound_on_fixed_sphere():
    # a sphere dropped head-on onto a fixed sphere of its own type (no gravity).
    # The pair's damping comes from the two-particle table (effective mass m/2),
    # while the fixed sphere acts as an infinite mass, so the rebound ratio is
    # a little above e_n (damping ratio smaller by sqrt(2))
    e = 0.8
    t = props.build_tables(2, [1e-3], [2500.0], [5e7], [0.3], (0.3, 0.3, 0.0, e, e), [5e7], [0.3],
                           (0.3, 0.3, 0.0, e, e))
    o = beds.Options(dt=2e-8, minpoint=(0, 0, 0), maxpoint=(0.01, 0.01, 0.01), gravity=(0.0, 0.0, 0.0), cf_type=2,
                     pi_method=2, pri_method=1)
    p = beds.new_particles(np.array([[0.005, 0.006001, 0.005]]), np.array([1]), t.radius,
                           np.array([[0.0, -0.2, 0.0]]), 2, 1)
    fx = beds.FixedSpheres(id=np.array([2], np.int32), ptype=np.array([1], np.int32),
                           pos=np.array([[0.005, 0.005, 0.005]]))
    s = OracleSystem(beds.Case("f", o, t, WallSet(), p, fixed=fx))
    touched = False
    for _ in range(2000):
        s.step(100)
        c = s.counters()["ppfix"]
        touched = touched or c > 0
        if touched and c == 0:
            break
    assert touched
    v = s.state().linVel[0, 0]
    assert e < v[1] / 0.2 < e + 0.1, v
    assert abs(v[0]) < 1e-12 and abs(v[2]) < 1e-12


def test_hertz_static_normal_force():
    # two Hertz spheres at rest pressed by delta: no damping (no relative
    # velocity) and no spring history, so the force is K delta^1.5 with
    # K = 4/3 E* sqrt(R*), E* = E / (2 (1 - nu^2)), R* = r / 2 (equal spheres)
    E, nu, d, delta = 5e7, 0.3, 1e-3, 3e-6
    case = two_sphere_case(props.CFT_NLIN, 0.0, e_n=0.8, E=E)
    mid = 0.005
    case.particles.posR[0, 0] = mid - (d - delta) / 2
    case.particles.posR[1, 0] = mid + (d - delta) / 2
    s = OracleSystem(case)
    s.step(1)
    F, T = s.forces()
    assert s.counters()["pp"] == 1
    K = 4.0 / 3.0 * (E / (2.0 * (1.0 - nu * nu))) * math.sqrt(d / 4.0)
    want = K * delta ** 1.5
    assert F[0, 0] == pytest.approx(-want, rel=1e-10) and F[1, 0] == pytest.approx(want, rel=1e-10)
    assert np.abs(F[:, 1:]).max() == 0.0 and np.abs(T).max() == 0.0


def test_hertz_elastic_impact_peak_overlap():
    # restitution 1 (no damping): a head-on impact reaches the Hertz maximum
    # overlap (15 m* v^2 / (16 E* sqrt(R*)))^(2/5) and leaves at the speed it came
    E, nu, d, v = 5e7, 0.3, 1e-3, 0.2
    case = two_sphere_case(props.CFT_NLIN, v, e_n=1.0, mu=0.0, E=E, dt=1e-8)
    s = OracleSystem(case)
    m = 2500.0 * math.pi / 6.0 * d ** 3
    Es = E / (2.0 * (1.0 - nu * nu))
    want = (15.0 * (m / 2.0) * (2.0 * v) ** 2 / (16.0 * Es * math.sqrt(d / 4.0))) ** 0.4
    peak, touched = 0.0, False
    for _ in range(4000):
        s.step(5)
        st = s.state()
        ov = d - (st.posR[1, 0] - st.posR[0, 0])
        peak = max(peak, ov)
        touched = touched or ov > 0
        if touched and ov < 0:
            break
    assert peak == pytest.approx(want, rel=2e-3), (peak, want)
    st = s.state()
    assert (st.linVel[1, 0, 0] - st.linVel[0, 0, 0]) / (2 * v) == pytest.approx(1.0, abs=2e-3)


def test_lsd_static_normal_force():
    # linear spring-dashpot at rest: VelRel_Init = max(|v_rn|, 0.01) = 0.01, so
    # the stiffness is Kn 0.01^0.4 and the force Kn 0.01^0.4 delta
    d, delta = 1e-3, 2e-6
    case = two_sphere_case(props.CFT_LSD, 0.0, e_n=0.9)
    mid = 0.005
    case.particles.posR[0, 0] = mid - (d - delta) / 2
    case.particles.posR[1, 0] = mid + (d - delta) / 2
    s = OracleSystem(case)
    s.step(1)
    F, _ = s.forces()
    kn = abs(case.tables.bpp.reshape(1, 1, props.BP_SIZE)[0, 0, 2])
    want = kn * 0.01 ** 0.4 * delta
    assert F[0, 0] == pytest.approx(-want, rel=1e-10) and F[1, 0] == pytest.approx(want, rel=1e-10)


def test_hertz_wall_static_force():
    # a sphere at rest pressed into an infinite floor by delta: the wall's
    # radius is infinite, so R* = r, and E* = 1 / ((1-nu^2)/E + (1-nu_w^2)/E_w)
    E, nu, d, delta = 5e7, 0.3, 1e-3, 4e-6
    walls = box_walls((0.0, 0.0, 0.0), (0.01, 0.01, 0.01))
    case = two_sphere_case(props.CFT_NLIN, 0.0, e_n=0.8, E=E, walls=walls)
    p = case.particles.take(np.array([0]))
    p.posR[0, :3] = (0.005, d / 2 - delta, 0.005)
    s = OracleSystem(beds.Case("wall", case.opts, case.tables, walls, p))
    s.step(1)
    F, T = s.forces()
    assert s.counters()["pw"] == 1
    Es = 1.0 / (2.0 * (1.0 - nu * nu) / E)
    want = 4.0 / 3.0 * Es * math.sqrt(d / 2.0) * delta ** 1.5
    assert F[0, 1] == pytest.approx(want, rel=1e-10)
    assert abs(F[0, 0]) == 0.0 and abs(F[0, 2]) == 0.0 and np.abs(T).max() == 0.0


def test_rolling_resistance_torque_on_a_spinning_sphere():
    # a sphere pressed into the floor and spinning about the floor's normal:
    # the contact point does not slide (omega is parallel to n), so the only
    # torque is the rolling resistance -mu_r |f_n| R* w_hat (CT_Model 1,
    # Prtcl_ContactForce_inc.f90), with R* = r against a wall
    E, nu, d, delta, mur, w = 5e7, 0.3, 1e-3, 4e-6, 0.1, 30.0
    c = (0.3, 0.3, mur, 0.8, 0.8)
    t = props.build_tables(props.CFT_NLIN, [d], [2500.0], [E], [nu], c, [E], [nu], c)
    o = beds.Options(dt=1e-8, minpoint=(0, 0, 0), maxpoint=(0.01, 0.01, 0.01), gravity=(0.0, 0.0, 0.0),
                     cf_type=props.CFT_NLIN, pi_method=2, pri_method=2)
    walls = box_walls((0.0, 0.0, 0.0), (0.01, 0.01, 0.01))
    p = beds.new_particles(np.array([[0.005, d / 2 - delta, 0.005]]), np.array([1]), t.radius,
                           np.zeros((1, 3)), o.tsize, o.rsize)
    p.rotVel[:, :, 1] = w
    s = OracleSystem(beds.Case("spin", o, t, walls, p))
    s.step(1)
    F, T = s.forces()
    Es = 1.0 / (2.0 * (1.0 - nu * nu) / E)
    fn = 4.0 / 3.0 * Es * math.sqrt(d / 2.0) * delta ** 1.5
    assert F[0, 1] == pytest.approx(fn, rel=1e-10) and abs(F[0, 0]) == 0.0 and abs(F[0, 2]) == 0.0
    assert T[0, 1] == pytest.approx(-mur * fn * d / 2.0, rel=1e-10)
    assert abs(T[0, 0]) == 0.0 and abs(T[0, 2]) == 0.0


@pytest.mark.parametrize("cf", [props.CFT_NLIN, props.CFT_LSD])
def test_pair_forces_cancel_in_a_cloud(cf):
    # without walls and gravity every force is a pair force, added to one
    # sphere and subtracted from the other: the forces of a dense moving
    # cloud sum to zero up to the rounding of each sphere's own sum
    import dataclasses
    case = beds.lattice_cloud_case(800, seed=41, cf_type=cf, ntypes=5)
    opts = dataclasses.replace(case.opts, gravity=(0.0, 0.0, 0.0))
    s = OracleSystem(beds.Case("cloud", opts, case.tables, WallSet(), case.particles))
    for _ in range(3):
        s.step(1)
        F, _ = s.forces()
        assert s.counters()["pp"] > 50 and s.counters()["pw"] == 0
        total = np.array([math.fsum(F[:, k]) for k in range(3)])
        assert np.abs(total).max() <= 1e-13 * np.abs(F).sum(), total


def test_moving_floor_drags_a_resting_sphere():
    # a floor moving along x at v (the wall's translational velocity,
    # G_add_PlaneWall's t_vel): the first step's spring is the relative
    # tangential displacement -v dt, so the sphere feels Kt sqrt(delta) v dt
    # along +x (Kt = 16/3 G* sqrt(R*) of the wall pair) besides the normal load
    E, nu, d, delta, v, dt = 5e7, 0.3, 1e-3, 4e-6, 0.05, 1e-7
    walls = box_walls((0.0, 0.0, 0.0), (0.01, 0.01, 0.01))
    walls.walls[0][16:19] = (v, 0.0, 0.0)                    # the floor (y = 0) moves along x
    case = two_sphere_case(props.CFT_NLIN, 0.0, e_n=0.8, mu=0.5, E=E, walls=walls, dt=dt)
    p = case.particles.take(np.array([0]))
    p.posR[0, :3] = (0.005, d / 2 - delta, 0.005)
    s = OracleSystem(beds.Case("conveyor", case.opts, case.tables, walls, p))
    s.step(1)
    F, _ = s.forces()
    G = E / (2.0 * (1.0 + nu))
    Gs = 1.0 / (2.0 * (2.0 - nu) / G)
    kt = 16.0 / 3.0 * Gs * math.sqrt(d / 2.0)
    assert F[0, 0] == pytest.approx(kt * math.sqrt(delta) * v * dt, rel=1e-10)
    assert F[0, 1] > 0.0 and abs(F[0, 2]) == 0.0


def test_forward_euler_free_fall_closed_form():
    # FE (PI_Method 1): x_{k+1} = x_k + v_k dt, v_{k+1} = v_k + a dt, so
    # v_n = v0 + n a dt and x_n = x0 + n v0 dt + a dt^2 n (n - 1) / 2
    t = props.build_tables(1, [1e-3], [2500.0], [1e7], [0.3], (0.3, 0.3, 0.1, 0.9, 0.9), [1e7], [0.3],
                           (0.3, 0.3, 0.1, 0.9, 0.9))
    o = beds.Options(dt=1e-4, minpoint=(0, 0, 0), maxpoint=(1, 1, 1), pi_method=1, pri_method=1)
    p = beds.new_particles(np.array([[0.5, 0.9, 0.5]]), np.array([1]), t.radius, np.array([[0.0, 0.1, 0.0]]),
                           o.tsize, o.rsize)
    s = OracleSystem(beds.Case("fall_fe", o, t, WallSet(), p))
    n = 100
    s.step(n)
    st = s.state()
    a, dt = -9.81, 1e-4
    assert st.linVel[0, 0, 1] == pytest.approx(0.1 + n * a * dt, rel=1e-12)
    assert st.posR[0, 1] == pytest.approx(0.9 + n * 0.1 * dt + a * dt * dt * n * (n - 1) / 2, rel=1e-12)
    assert st.linAcc[0, 0, 1] == pytest.approx(a, rel=1e-15)
