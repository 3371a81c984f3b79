"""Asynchronous output (sdem_snapshot_begin / _end / _contacts): the frozen
state, forces and contact list equal a synchronous download of an identical
run at the same step, bit for bit, while the steps issued after the snapshot
run during its download."""
import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, restart
from sdem_gb300.beds import Particles
from sdem_gb300.capi import DEMSystem
from tests.helpers import keyed_contacts

pytestmark = pytest.mark.gpu


def empty_like(sysm):
    cap, ts, rs = sysm.cfg.n_capacity, sysm.cfg.tsize, sysm.cfg.rsize
    return Particles(np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros((cap, 4)),
                     np.zeros((cap, ts, 3)), np.zeros((cap, ts, 3)), np.zeros((cap, 3)), np.zeros((cap, rs, 3)),
                     np.zeros((cap, rs, 3)))


def same_state(a, b):
    for f in ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc"):
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


@pytest.mark.parametrize("periodic", [False, True])
def test_snapshot_equals_synchronous_download(gpu_lib, periodic):
    if periodic:
        case = beds.periodic_lattice_case(800, 41, (1, 0, 1))
    else:
        case = beds.lattice_cloud_case(800, seed=42, finite_walls=True)
    a, b = DEMSystem(case), DEMSystem(case)
    a.step(5)
    out = empty_like(a)
    cap = a.cfg.n_capacity
    F, T = np.zeros((cap, 3)), np.zeros((cap, 3))
    a.snapshot_begin(out, F, T, contacts=True)
    a.step_async(7)                      # runs while the snapshot downloads
    snap, Fs, Ts = a.snapshot_end()
    b.step(5)
    same_state(snap, b.state())
    Fb, Tb = b.forces()
    np.testing.assert_array_equal(Fs, Fb)
    np.testing.assert_array_equal(Ts, Tb)
    o, q, t, v = a.snapshot_contacts()
    o2, q2, t2, v2 = b.contacts()
    np.testing.assert_array_equal(o, o2)
    np.testing.assert_array_equal(q, q2)
    np.testing.assert_array_equal(t, t2)
    np.testing.assert_array_equal(v, v2)
    # the run after the snapshot is unaffected by it
    a.step(0)
    b.step(7)
    same_state(a.state(), b.state())


def test_snapshot_before_any_step_reports_uploaded_history(gpu_lib):
    case = beds.lattice_cloud_case(600, seed=43)
    o = OracleSystem(case)
    o.step(3)
    c = beds.Case(case.name, case.opts, case.tables, case.walls, o.state(), contacts=o.contacts(), fixed=case.fixed)
    g = DEMSystem(c)
    out = empty_like(g)
    g.snapshot_begin(out, contacts=True)
    snap, _, _ = g.snapshot_end()
    same_state(snap, o.state())
    assert keyed_snapshot(g, snap.id, case.opts.base_wall_id) == keyed_contacts(o, case.opts.base_wall_id)


def keyed_snapshot(g, ids, base_wall_id):
    o, q, t, v = g.snapshot_contacts()
    return {(int(ids[o[k]]), int(q[k])): (t[k, 0], t[k, 1], t[k, 2], v[k]) for k in range(len(o))}


def test_snapshot_feeds_the_restart_writer(gpu_lib, tmp_path):
    case = beds.lattice_cloud_case(600, seed=44)
    g = DEMSystem(case)
    g.step(4)
    out = empty_like(g)
    g.snapshot_begin(out, contacts=True)
    g.step_async(3)
    snap, _, _ = g.snapshot_end()
    path = str(tmp_path / "RestartForSnap0000000004")
    restart.write_restart(path, snap, g.snapshot_contacts(), case.opts.tsize, case.opts.rsize,
                          case.opts.base_wall_id)
    p2, c2 = restart.read_restart(path, case.opts.tsize, case.opts.rsize, case.tables.radius)
    np.testing.assert_array_equal(p2.id, snap.id)
    np.testing.assert_array_equal(p2.posR, snap.posR)
    # a handle restarted from the file continues like the uninterrupted run
    h = DEMSystem(beds.Case(case.name, case.opts, case.tables, case.walls, p2, contacts=c2))
    ref = DEMSystem(case)
    ref.step(4)
    h.step(2)
    ref.step(2)
    np.testing.assert_array_equal(h.state().posR, ref.state().posR)
