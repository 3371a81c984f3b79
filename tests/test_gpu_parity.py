"""Parity of the GB300 path (through the C ABI) with the CPU oracle.

Bars: contact sets (particle-particle and particle-wall) equal; contact
history, forces and torques within 1e-12 relative; counters equal.  The GPU
sums every particle's contacts in the reference's scatter order, so the only
floating-point difference left is ovrlp**1.5 / ovrlp**0.25 (sqrt forms vs
libm pow, ~1 ulp) and pow(V, 0.4/0.2) (CUDA vs libm).
"""
import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, props
from sdem_gb300.capi import DEMSystem, SdemError
from tests.helpers import assert_same_contact_sets, compare_history, force_scale, keyed_contacts

pytestmark = pytest.mark.gpu

RTOL = 1e-12   # forces, torques and contact history (the parity bar)


def cloud(**kw):
    base = dict(n=800, seed=11, ntypes=7)
    base.update(kw)
    return beds.lattice_cloud_case(**base)


def moving_floor(case, v=(0.2, 0.0, 0.05)):
    """The case with its floor (the first box wall) moving tangentially at v,
    the wall's translational velocity of G_add_PlaneWall."""
    import dataclasses
    from sdem_gb300.geometry import WallSet
    ws = WallSet(walls=[w.copy() for w in case.walls.walls], flags=[f.copy() for f in case.walls.flags])
    assert ws.walls[0][13] == 1.0     # the floor's normal is +y
    ws.walls[0][16:19] = v
    return dataclasses.replace(case, walls=ws)


CASES = {
    "hertz_ab2": lambda: cloud(),
    "lsd_ab2": lambda: cloud(seed=12, cf_type=props.CFT_LSD, ntypes=3),
    "hertz_finite_walls": lambda: cloud(seed=13, finite_walls=True),
    "hertz_ab3": lambda: cloud(seed=14, pi=3, pri=3),
    "lsd_fe": lambda: cloud(seed=15, cf_type=props.CFT_LSD, pi=1, pri=1),
    "hertz_ct2_noquirk": lambda: beds.scaled(cloud(seed=16), ct_model=2, quirk_ab2_rot=0),
    "mono_one_type": lambda: cloud(seed=17, ntypes=1, nn=0.995e-3),
    # a floor moving tangentially (the wall velocity in the force law and in
    # the near-wall refresh)
    "hertz_moving_floor": lambda: moving_floor(cloud(seed=18)),
    # periodic images (PC_Comm_For_Cntct, FineSearch3, ContactForce_PPG)
    "periodic_xyz": lambda: beds.periodic_lattice_case(800, 31, (1, 1, 1)),
    "periodic_y": lambda: beds.periodic_lattice_case(800, 32, (0, 1, 0)),
    "periodic_xz": lambda: beds.periodic_lattice_case(800, 33, (1, 0, 1)),
    "periodic_x_lsd": lambda: beds.periodic_lattice_case(800, 34, (1, 0, 0), cf_type=props.CFT_LSD, ntypes=3),
    # a small hopper: bidisperse 1:3 spheres, eight finite walls (inclined and
    # vertical quads, their edges and corners), an outlet that deletes
    "hopper": lambda: beds.hopper_case(1500, 51),
    # fixed spheres (FineSearch1, ContactForce_PPFix): a rough floor and a few inside
    "fixed_floor": lambda: beds.fixed_floor_case(800, 61),
    "fixed_floor_lsd_fe": lambda: beds.fixed_floor_case(800, 62, cf_type=props.CFT_LSD, ntypes=3, pi=1, pri=1),
    # hierarchical search (CS_Method 2): two levels (the 1:3 hopper), three levels
    # (diameters 0.3-1.2 mm), two levels with periodic images
    "hrchl_hopper": lambda: beds.scaled(beds.hopper_case(1500, 52), cs_method=2),
    "hrchl_poly3": lambda: beds.scaled(cloud(seed=71, ntypes=9, d_lo=0.3e-3, d_hi=1.2e-3, nn=0.9e-3), cs_method=2),
    "hrchl_periodic": lambda: beds.scaled(beds.periodic_lattice_case(800, 72, (1, 0, 1), d_lo=0.4e-3, d_hi=1.2e-3,
                                                                     ntypes=5), cs_method=2),
}


def compare_step(g, o, case, what):
    cg, co = g.counters(), o.counters()
    for k in ("pp", "pw", "cnsv", "nlocal"):
        assert cg[k] == co[k], f"{what}: counter {k}: gpu {cg[k]} oracle {co[k]}"
    kg = keyed_contacts(g, case.opts.base_wall_id)
    ko = keyed_contacts(o, case.opts.base_wall_id)
    assert_same_contact_sets(kg, ko, what)
    compare_history(kg, ko, RTOL)
    sg, so = g.state(), o.state()
    np.testing.assert_array_equal(sg.id, so.id)
    Fg, Tg = g.forces()
    Fo, To = o.forces()
    fs = force_scale(Fo, 1e-6 * max(np.abs(Fo).max(), 1e-30))
    ts = force_scale(To, 1e-6 * max(np.abs(To).max(), 1e-30))
    assert np.all(np.abs(Fg - Fo).max(axis=1) <= RTOL * fs), f"{what}: force mismatch"
    assert np.all(np.abs(Tg - To).max(axis=1) <= RTOL * ts), f"{what}: torque mismatch"
    # the state after the step: positions differ only through those forces
    np.testing.assert_allclose(sg.posR, so.posR, rtol=1e-13, atol=1e-18)
    vs = np.abs(so.linVel).max() + 1e-30
    assert np.abs(sg.linVel - so.linVel).max() <= 1e-12 * vs
    ws = np.abs(so.rotVel).max() + 1e-30
    assert np.abs(sg.rotVel - so.rotVel).max() <= 1e-12 * ws


@pytest.mark.parametrize("name", sorted(CASES))
def test_one_step_from_identical_inputs(gpu_lib, name):
    case = CASES[name]()
    g, o = DEMSystem(case), OracleSystem(case)
    g.step(1)
    o.step(1)
    assert g.counters()["pp"] > 50, "case should have many contacts"
    compare_step(g, o, case, name)


@pytest.mark.parametrize("name", ["hertz_ab2", "lsd_ab2", "hertz_finite_walls", "periodic_xyz", "periodic_xz",
                                  "hopper", "fixed_floor", "hrchl_hopper", "hrchl_poly3", "hertz_moving_floor"])
def test_twenty_steps_resynchronised(gpu_lib, name):
    """A chain of single steps, each from the oracle's state and contact list
    (restart-file style), so chaos cannot hide or create a mismatch."""
    case = CASES[name]()
    o = OracleSystem(case)
    for k in range(20):
        st = o.state()
        c = beds.Case(case.name, case.opts, case.tables, case.walls, st, contacts=o.contacts(), fixed=case.fixed)
        g = DEMSystem(c)
        g.step(1)
        o.step(1)
        compare_step(g, o, case, f"{name} step {k}")
        g.close()


@pytest.mark.parametrize("name", ["hertz_ab2", "lsd_ab2", "periodic_xyz", "fixed_floor", "hrchl_poly3",
                                  "hrchl_periodic"])
def test_free_run_trajectory(gpu_lib, name):
    """50 free-running steps: contact sets stay identical and the state within
    a loose bound (differences start at ~1 ulp per step)."""
    case = CASES[name]()
    g, o = DEMSystem(case), OracleSystem(case)
    for k in range(50):
        g.step(1)
        o.step(1)
        kg = keyed_contacts(g, case.opts.base_wall_id)
        ko = keyed_contacts(o, case.opts.base_wall_id)
        assert_same_contact_sets(kg, ko, f"{name} free step {k}")
    np.testing.assert_allclose(g.state().posR, o.state().posR, rtol=1e-11, atol=1e-15)


def test_contact_history_upload(gpu_lib):
    """Contacts handed over as a restart file lists them (both sides of every
    pair) carry their spring history into the next step."""
    case = CASES["hertz_ab2"]()
    o = OracleSystem(case)
    o.step(3)
    st = o.state()
    cont = o.contacts()
    c = beds.Case(case.name, case.opts, case.tables, case.walls, st, contacts=cont)
    g = DEMSystem(c)
    kg0 = keyed_contacts(g, case.opts.base_wall_id)
    ko0 = keyed_contacts(o, case.opts.base_wall_id)
    assert_same_contact_sets(kg0, ko0, "after upload")
    compare_history(kg0, ko0, 0.0)
    o2 = OracleSystem(c)
    g.step(1)
    o2.step(1)
    compare_step(g, o2, case, "restart chain")


def test_upload_download_roundtrip(gpu_lib):
    case = CASES["hertz_ab3"]()
    g = DEMSystem(case)
    s = g.state()
    p = case.particles
    for a, b in ((s.id, p.id), (s.ptype, p.ptype), (s.posR, p.posR), (s.linVel, p.linVel), (s.linAcc, p.linAcc),
                 (s.theta, p.theta), (s.rotVel, p.rotVel), (s.rotAcc, p.rotAcc)):
        np.testing.assert_array_equal(a, b)


def test_out_of_domain_delete_order(gpu_lib):
    """Particles that leave the domain are deleted by swap-with-last in the
    reference's five passes; the surviving order must match."""
    case = cloud(seed=21, n=400)
    case.walls.walls = case.walls.walls[1:]   # no floor
    case.walls.flags = case.walls.flags[1:]
    p = case.particles
    rng = np.random.default_rng(5)
    low = np.argsort(p.posR[:, 1])[:60]
    p.linVel[low, :, 1] = -rng.uniform(200.0, 400.0, len(low))[:, None]   # these fall out within a few steps
    g, o = DEMSystem(case), OracleSystem(case)
    for k in range(8):
        g.step(1)
        o.step(1)
        np.testing.assert_array_equal(g.state().id, o.state().id)
        assert g.counters()["nlocal"] == o.counters()["nlocal"]
    assert g.counters()["nlocal"] < case.particles.n
    compare_step(g, o, case, "after deletes")


def test_deterministic(gpu_lib):
    case = CASES["hertz_ab2"]()
    a, b = DEMSystem(case), DEMSystem(case)
    a.step(10)
    b.step(10)
    np.testing.assert_array_equal(a.state().posR, b.state().posR)
    np.testing.assert_array_equal(a.forces()[0], b.forces()[0])


def test_grid_error(gpu_lib):
    case = cloud(seed=22, n=50)
    case.particles.posR[3, 0] = 5.0   # far outside the padded grid (and the domain)
    g = DEMSystem(case)
    with pytest.raises(SdemError) as e:
        g.step(1)
    assert e.value.code == 6


def test_upload_checks_ids_and_types(gpu_lib):
    case = cloud(seed=25, n=200)
    g = DEMSystem(case)
    for field, value, code in (("id", None, 4), ("id", 10**6, 4), ("ptype", 99, 1)):
        p = case.particles.copy()
        if field == "id" and value is None:
            p.id[7] = p.id[3]                      # duplicate id
        elif field == "id":
            p.id[7] = value                        # above max_gid
        else:
            p.ptype[7] = value
        with pytest.raises(SdemError) as e:
            g.upload(p)
        assert e.value.code == code, (field, value)
        assert "index 7" in str(e.value)
    g.upload(case.particles)                       # a valid set is accepted again
    g.step(1)
    assert g.counters()["nlocal"] == case.particles.n


def test_row_capacity_error(gpu_lib):
    case = beds.scaled(cloud(seed=23), max_contacts_per_particle=1)
    g = DEMSystem(case)
    with pytest.raises(SdemError) as e:
        g.step(1)
    assert e.value.code == 3


def test_hopper_outflow_matches_oracle(gpu_lib):
    """60 free-running steps of the hopper: the outlet deletes spheres in the
    reference's swap-with-last order, wall and pair contact sets stay equal."""
    case = CASES["hopper"]()
    g, o = DEMSystem(case), OracleSystem(case)
    for k in range(60):
        g.step(1)
        o.step(1)
        np.testing.assert_array_equal(g.state().id, o.state().id)
        assert g.counters() == o.counters(), f"hopper step {k}"
        kg = keyed_contacts(g, case.opts.base_wall_id)
        ko = keyed_contacts(o, case.opts.base_wall_id)
        assert_same_contact_sets(kg, ko, f"hopper step {k}")
    assert g.counters()["nlocal"] < case.particles.n
    assert g.counters()["pw"] > 20
    np.testing.assert_allclose(g.state().posR, o.state().posR, rtol=1e-11, atol=1e-15)


def test_fixed_sphere_arguments(gpu_lib):
    case = CASES["fixed_floor"]()
    g = DEMSystem(case)
    fx = case.fixed
    with pytest.raises(SdemError) as e:      # ids must lie above the moving ids
        g.set_fixed(beds.FixedSpheres(id=np.array([1], np.int32), ptype=fx.ptype[:1], pos=fx.pos[:1]))
    assert e.value.code == 4
    per = CASES["periodic_y"]()
    c = beds.Case(per.name, per.opts, per.tables, per.walls, per.particles, fixed=beds.FixedSpheres(
        id=np.array([10**6], np.int32), ptype=np.array([1], np.int32), pos=per.particles.posR[:1, :3] + 1e-3))
    with pytest.raises(SdemError) as e:      # no fixed spheres with periodic directions
        DEMSystem(c)
    assert e.value.code == 10


def test_unsupported_options_are_refused(gpu_lib):
    case = beds.scaled(CASES["fixed_floor"](), cs_method=2)   # no fixed spheres in the hierarchical search
    with pytest.raises(SdemError) as e:
        DEMSystem(case)
    assert e.value.code == 10


def test_periodic_wrap_matches_oracle(gpu_lib):
    """Fast spheres cross the periodic faces: the GPU wraps them in place
    (Comm_For_Exchange) with the same ids, positions and image contacts."""
    case = beds.periodic_lattice_case(800, 35, (1, 1, 1), vmax=25.0)
    g, o = DEMSystem(case), OracleSystem(case)
    for k in range(40):
        g.step(1)
        o.step(1)
        kg = keyed_contacts(g, case.opts.base_wall_id)
        ko = keyed_contacts(o, case.opts.base_wall_id)
        assert_same_contact_sets(kg, ko, f"wrap step {k}")
        assert g.counters() == o.counters()
    sg, so = g.state(), o.state()
    np.testing.assert_array_equal(sg.id, so.id)
    lo, hi = np.array(case.opts.minpoint), np.array(case.opts.maxpoint)
    assert np.all(sg.posR[:, :3] >= lo) and np.all(sg.posR[:, :3] < hi)
    moved = np.abs(sg.posR[:, :3] - case.particles.posR[:, :3]).max()
    assert moved > 0.5 * (hi - lo).min(), "some sphere should have wrapped"
    np.testing.assert_allclose(sg.posR, so.posR, rtol=1e-11, atol=1e-15)


def test_periodic_history_roundtrip(gpu_lib):
    """Image contacts are listed under their local sphere only and come back
    through sdem_upload_contacts with their spring history."""
    case = beds.periodic_lattice_case(800, 36, (1, 0, 1))
    o = OracleSystem(case)
    o.step(2)
    c = beds.Case(case.name, case.opts, case.tables, case.walls, o.state(), contacts=o.contacts(), fixed=case.fixed)
    g = DEMSystem(c)
    kg0 = keyed_contacts(g, case.opts.base_wall_id)
    ko0 = keyed_contacts(o, case.opts.base_wall_id)
    assert_same_contact_sets(kg0, ko0, "after upload")
    compare_history(kg0, ko0, 0.0)
    g.step(1)
    o.step(1)
    assert g.counters()["ppg"] > 0
    compare_step(g, o, case, "periodic restart chain")


def test_periodic_side_of_two_cells_is_refused(gpu_lib):
    case = beds.periodic_lattice_case(100, 37, (1, 0, 0))
    hi = list(case.opts.maxpoint)
    hi[0] = 2.4e-3   # about two search cells
    case = beds.scaled(case, maxpoint=tuple(hi))
    with pytest.raises(SdemError) as e:
        DEMSystem(case)
    assert e.value.code == 10


def test_graph_replay_equals_single_steps(gpu_lib):
    """sdem_step(h, n>=4) replays a captured two-step CUDA graph; the result is
    bit-identical to n single-step calls (odd counts and parity realignment too)."""
    case = CASES["hertz_finite_walls"]()
    a, b = DEMSystem(case), DEMSystem(case)
    a.step(1)
    a.step(9)      # parity realigned by one plain step, then graph replays
    a.step(5)
    for _ in range(15):
        b.step(1)
    sa, sb = a.state(), b.state()
    np.testing.assert_array_equal(sa.posR, sb.posR)
    np.testing.assert_array_equal(sa.rotVel, sb.rotVel)
    np.testing.assert_array_equal(a.forces()[1], b.forces()[1])
    assert a.counters() == b.counters()
    assert keyed_contacts(a, case.opts.base_wall_id) == keyed_contacts(b, case.opts.base_wall_id)
