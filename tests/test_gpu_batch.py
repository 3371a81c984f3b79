"""Batched form (sdem_batch_*): beds of different sizes, materials, walls,
periodicity and search methods advanced together give the states, forces,
contact lists and counters of the same beds stepped alone, bit for bit --
through two-step graph replays, an odd remainder, a member stepped alone in
between (new parity) and a member re-uploaded with another size (its graphs
invalidated)."""
import numpy as np
import pytest

from sdem_gb300 import beds, props
from sdem_gb300.capi import DEMBatch, DEMSystem
from tests.test_gpu_full_size import sorted_contacts

pytestmark = pytest.mark.gpu

FIELDS = ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc")


def cases():
    return [
        beds.lattice_cloud_case(800, seed=11, ntypes=7),
        beds.lattice_cloud_case(600, seed=12, cf_type=props.CFT_LSD, ntypes=3, finite_walls=True),
        beds.periodic_lattice_case(700, 31, (1, 0, 1)),
        beds.hopper_case(1500, 51),
        beds.scaled(beds.lattice_cloud_case(500, seed=71, ntypes=9, d_lo=0.3e-3, d_hi=1.2e-3, nn=0.9e-3),
                    cs_method=2),
        beds.fixed_floor_case(600, 61),
    ]


def same(a, b, what):
    sa, sb = a.state(), b.state()
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(sa, f), getattr(sb, f), err_msg=f"{what}: {f}")
    Fa, Ta = a.forces()
    Fb, Tb = b.forces()
    np.testing.assert_array_equal(Fa, Fb, err_msg=f"{what}: F")
    np.testing.assert_array_equal(Ta, Tb, err_msg=f"{what}: T")
    ka, ha = sorted_contacts(a)
    kb, hb = sorted_contacts(b)
    np.testing.assert_array_equal(ka, kb, err_msg=f"{what}: contacts")
    np.testing.assert_array_equal(ha, hb, err_msg=f"{what}: history")
    assert a.counters() == b.counters(), what


def test_batch_equals_members_stepped_alone(gpu_lib):
    cs = cases()
    alone = [DEMSystem(c) for c in cs]
    members = [DEMSystem(c) for c in cs]
    batch = DEMBatch(members)
    for a in alone:
        a.step(10)
    batch.step(10)                      # five two-step graph replays
    for k, (a, m) in enumerate(zip(alone, members)):
        same(a, m, f"bed {k} after 10")
    for a in alone:
        a.step(3)
    batch.step(3)                       # one replay and a plain step
    for k, (a, m) in enumerate(zip(alone, members)):
        same(a, m, f"bed {k} after 13")
    # a member stepped alone changes its parity; the batch recaptures
    alone[2].step(1)
    members[2].step(1)
    for a in alone:
        a.step(4)
    batch.step(4)
    for k, (a, m) in enumerate(zip(alone, members)):
        same(a, m, f"bed {k} after a lone step")
    # a member re-uploaded with another particle set: its graphs are dropped
    # and the batch graph is captured again
    small = beds.lattice_cloud_case(300, seed=99, ntypes=2)
    alone[0].upload(small.particles)
    members[0].upload(small.particles)
    for a in alone:
        a.step(6)
    batch.step(6)
    for k, (a, m) in enumerate(zip(alone, members)):
        same(a, m, f"bed {k} after a re-upload")
    batch.close()
    for s in alone + members:
        s.close()


def test_batch_reports_member_errors(gpu_lib):
    ok = DEMSystem(beds.lattice_cloud_case(400, seed=5, ntypes=3))
    case = beds.lattice_cloud_case(400, seed=6, ntypes=3)
    # rows of one contact: the dense cloud overflows them on the first step
    bad = DEMSystem(beds.scaled(case, max_contacts_per_particle=1))
    batch = DEMBatch([ok, bad])
    with pytest.raises(Exception) as e:
        batch.step(2)
    assert "member 1" in str(e.value)
    batch.close()
    ok.close()
    bad.close()


def test_batch_of_many_sandboxes_in_groups(gpu_lib):
    # more members than one group holds (64): two group graphs on two streams
    rng = np.random.default_rng(4)
    cs = [beds.sandbox_case(rng, i, n_lo=200, n_hi=800) for i in range(70)]
    alone = [DEMSystem(c) for c in cs]
    members = [DEMSystem(c) for c in cs]
    batch = DEMBatch(members)
    for a in alone:
        a.step(7)
    batch.step(7)
    for k, (a, m) in enumerate(zip(alone, members)):
        sa, sm = a.state(), m.state()
        for f in FIELDS:
            np.testing.assert_array_equal(getattr(sa, f), getattr(sm, f), err_msg=f"sandbox {k}: {f}")
        assert a.counters() == m.counters(), f"sandbox {k}"
    batch.close()
    for s in alone + members:
        s.close()
