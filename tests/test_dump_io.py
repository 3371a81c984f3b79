"""The tracer output of marked particles in the reference's layout
(Prtcl_DumpPrtcl.f90): marks from yDump, 52-byte records of the marked
particles every call, the contact flag from the live contact list, a file
when the cache is full and at the end, and the reference's checks."""
import os

import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, dump


def test_tracer_records(tmp_path):
    case = beds.lattice_cloud_case(800, seed=31)
    p = case.particles.copy()
    y_dump = float(np.median(p.posR[:, 1]))
    p.usrmark[:] = dump.reset_marks(p, y_dump)
    marked = np.flatnonzero(p.usrmark == dump.DUMP_FLAG)
    assert 0 < len(marked) < p.n and np.all(p.posR[marked, 1] >= y_dump)
    o = OracleSystem(beds.Case(case.name, case.opts, case.tables, case.walls, p))
    d = dump.PrtclDump(str(tmp_path) + "/", m_size=10000, write_cache_freq=2)
    for it in range(1, 61):
        o.step(1)
        if d.due(it):
            st = o.state()
            d.write_cache(it, st, o.contacts())
            if it == 2:
                first_state, first_contacts = st, o.contacts()
    final = d.dump(60)
    files = sorted(os.listdir(tmp_path))
    # 30 calls of len(marked) records: a file, named by its step, each time
    # the cache of 10,000 fills during a call, the rest at the end
    per = len(marked)
    want, count = [], 0
    for it in range(2, 61, 2):
        if (count + per) // 10000 > count // 10000:
            want.append(f"rank00000_{it:010d}")
        count += per
    if count % 10000:
        want.append("rank00000_0000000060")
    assert files == sorted(want) and len(want) >= 2
    recs = np.concatenate([np.fromfile(os.path.join(tmp_path, f), dtype=dump.RECORD) for f in files])
    assert dump.RECORD.itemsize == 52 and len(recs) == 30 * per
    r = recs[:per]
    st = first_state
    np.testing.assert_array_equal(r["itime"], 2)
    np.testing.assert_array_equal(r["id"], st.id[marked])
    np.testing.assert_array_equal(r["ptype"], st.ptype[marked])
    np.testing.assert_array_equal(r["pos"], st.posR[marked, :3].astype(np.float32))
    np.testing.assert_array_equal(r["linvel"], st.linVel[marked, 0].astype(np.float32))
    np.testing.assert_array_equal(r["rotvel"], st.rotVel[marked, 0].astype(np.float32))
    in_contact = np.zeros(st.n, bool)
    in_contact[np.asarray(first_contacts[0])] = True
    np.testing.assert_array_equal(r["cntct"], in_contact[marked].astype(np.int32))
    assert 0 < r["cntct"].sum() < per
    assert final.endswith("rank00000_0000000060")


def test_tracer_checks(tmp_path):
    with pytest.raises(dump.DumpError, match="So small mDumpPrtclSize"):
        dump.PrtclDump(str(tmp_path), m_size=9999)
    off = dump.PrtclDump(str(tmp_path), m_size=10, enabled=False)
    assert not off.due(100000) and off.dump(1) is None
