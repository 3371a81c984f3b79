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


def _records_by_loop(ids, owner, partner, tand, vrel, base_wall_id):
    """The record numbering stated listing by listing: a new record for each
    (ids, history) not seen before, in order of first listing."""
    index, recs, pairs = {}, [], []
    for k in range(len(owner)):
        g, q = int(ids[owner[k]]), int(partner[k])
        h = np.array([*tand[k], vrel[k]], np.float64).tobytes()
        key = (g, q) if q > base_wall_id else (min(g, q), max(g, q), h)
        if key not in index:
            index[key] = len(recs) + 1
            recs.append((*tand[k], vrel[k]))
        pairs.append((q, index[key]))
    return np.array(pairs, np.int32), np.array(recs, np.float64).reshape(-1, 4)


@pytest.mark.parametrize("mixed", [False, True])
def test_writer_numbers_records_as_the_listing_order(tmp_path, mixed):
    # the vectorised writer against the listing-by-listing statement: local
    # pairs (two listings, one record), wall contacts, mutual contacts with
    # periodic images (two listings under the same ids, two histories), and a
    # run of four listings under one pair of ids
    case, o = stepped_case()
    st = o.state()
    owner, partner, tand, vrel = (np.asarray(a) for a in o.contacts())
    if mixed:
        extra_o = np.array([0, 1, 0, 1], np.int32)
        extra_q = np.array([st.id[1], st.id[0], st.id[1], st.id[0]], np.int32)
        extra_t = np.array([[1e-7, 0, 0], [2e-7, 0, 0], [1e-7, 0, 0], [3e-7, 0, 0]])
        extra_v = np.array([0.1, 0.2, 0.1, 0.3])
        owner = np.concatenate([owner, extra_o])
        partner = np.concatenate([partner, extra_q])
        tand = np.concatenate([tand, extra_t])
        vrel = np.concatenate([vrel, extra_v])
    path = str(tmp_path / "r")
    restart.write_restart(path, st, (owner, partner, tand, vrel), case.opts.tsize, case.opts.rsize,
                          case.opts.base_wall_id)
    order = np.argsort(owner, kind="stable")
    want_pairs, want_recs = _records_by_loop(st.id, owner[order], partner[order], tand[order], vrel[order],
                                             case.opts.base_wall_id)
    raw = np.fromfile(path, dtype=np.uint8)
    n, nct = np.frombuffer(raw, np.int32, count=2)
    nreal3 = 2 * (1 + case.opts.tsize + case.opts.rsize) - 1
    off = 8 + 24 * n + 12 * n + 24 * nreal3 * n + 4 * n
    pairs = np.frombuffer(raw, np.int32, count=2 * nct, offset=off).reshape(-1, 2)
    recs = np.frombuffer(raw, np.float64, offset=off + 8 * nct).reshape(-1, 4)
    np.testing.assert_array_equal(pairs, want_pairs)
    np.testing.assert_array_equal(recs, want_recs)


def test_fixed_coords_file(tmp_path):
    # FixedSpheresCoord.dat in the reference's record layout: positions,
    # diameters and types round-trip, ids continue above the moving ones, and
    # the reader refuses what PIO_ReadFixedCoord aborts on
    case = beds.fixed_floor_case(300, 61)
    fx = case.fixed
    path = str(tmp_path / "FixedSpheresCoord.dat")
    restart.write_fixed_coords(path, fx.pos, fx.ptype, case.tables.radius)
    assert (tmp_path / "FixedSpheresCoord.dat").stat().st_size == 36 * fx.n
    got = restart.read_fixed_coords(path, fx.n, 1000, case.tables.radius, case.opts.minpoint, case.opts.maxpoint)
    np.testing.assert_array_equal(got.pos, fx.pos)
    np.testing.assert_array_equal(got.ptype, fx.ptype)
    np.testing.assert_array_equal(got.id, np.arange(1001, 1001 + fx.n))
    with pytest.raises(restart.RestartError, match="file byte wrong"):
        restart.read_fixed_coords(path, fx.n + 1, 1000, case.tables.radius, case.opts.minpoint, case.opts.maxpoint)
    bad = np.fromfile(path, dtype=restart.FIXED_RECORD)
    bad["diam"][0] *= 1.001
    bad.tofile(path)
    with pytest.raises(restart.RestartError, match="Diameter not coordinate"):
        restart.read_fixed_coords(path, fx.n, 1000, case.tables.radius, case.opts.minpoint, case.opts.maxpoint)
    restart.write_fixed_coords(path, fx.pos + np.array([1.0, 0.0, 0.0]), fx.ptype, case.tables.radius)
    with pytest.raises(restart.RestartError, match="numPrtclFix"):
        restart.read_fixed_coords(path, fx.n, 1000, case.tables.radius, case.opts.minpoint, case.opts.maxpoint)
