"""Restart files in the reference's layout: write/read round trip, and a
restart chain through a file gives the same next step as the unbroken run
(oracle on CPU; the GPU variant is in test_gpu_restart.py)."""
import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, restart
from tests.helpers import assert_same_contact_sets, keyed_contacts


def stepped_case():
    case = beds.lattice_cloud_case(300, seed=31)
    o = OracleSystem(case)
    o.step(4)
    return case, o


def test_roundtrip(tmp_path):
    case, o = stepped_case()
    st = o.state()
    cont = o.contacts()
    path = str(tmp_path / "RestartForX0000000004")
    restart.write_restart(path, st, cont, case.opts.tsize, case.opts.rsize)
    p2, c2 = restart.read_restart(path, case.opts.tsize, case.opts.rsize, case.tables.radius,
                                  case.opts.minpoint, case.opts.maxpoint)
    for f in ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc"):
        np.testing.assert_array_equal(getattr(p2, f), getattr(st, f))
    a = {(int(st.id[i]), int(q)): tuple(t) + (v,) for i, q, t, v in zip(*cont)}
    b = {(int(p2.id[i]), int(q)): tuple(t) + (v,) for i, q, t, v in zip(*c2)}
    assert a == b


def test_file_layout_sizes(tmp_path):
    case, o = stepped_case()
    st = o.state()
    cont = o.contacts()
    path = str(tmp_path / "r")
    restart.write_restart(path, st, cont, 2, 2)
    n, nct = st.n, len(cont[0])
    pp = sum(1 for q in cont[1] if q <= case.opts.base_wall_id) // 2
    pw = sum(1 for q in cont[1] if q > case.opts.base_wall_id)
    nreal3 = 2 * (1 + 2 + 2) - 1
    size = 8 + 24 * n + 12 * n + 24 * nreal3 * n + 4 * n + 8 * nct + 32 * (pp + pw)
    assert (tmp_path / "r").stat().st_size == size
    head = np.fromfile(path, dtype=np.int32, count=2)
    assert tuple(head) == (n, nct)


def test_restart_chain_through_file(tmp_path):
    case, o = stepped_case()
    path = str(tmp_path / "r")
    restart.write_restart(path, o.state(), o.contacts(), case.opts.tsize, case.opts.rsize)
    p2, c2 = restart.read_restart(path, case.opts.tsize, case.opts.rsize, case.tables.radius)
    o2 = OracleSystem(beds.Case(case.name, case.opts, case.tables, case.walls, p2, contacts=c2))
    o.step(1)
    o2.step(1)
    assert_same_contact_sets(keyed_contacts(o, case.opts.base_wall_id), keyed_contacts(o2, case.opts.base_wall_id))
    F1, _ = o.forces()
    F2, _ = o2.forces()
    # the near-wall list is rebuilt after a restart, which changes nothing: identical
    np.testing.assert_array_equal(F1, F2)


def test_ncv_limit(tmp_path):
    p = beds.lattice_cloud_case(30, seed=1).particles
    owner = np.zeros(21, np.int32)
    partner = np.arange(2, 23, dtype=np.int32)
    with pytest.raises(restart.RestartError):
        restart.write_restart(str(tmp_path / "x"), p, (owner, partner, np.zeros((21, 3)), np.zeros(21)), 2, 2)
