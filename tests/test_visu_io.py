"""The particle visualisation output in the reference's layout
(Prtcl_IOAndVisu.f90:63-131, 1048-1263): binary blocks in the documented
order, an XDMF time series that is well-formed XML and whose Seek offsets
point at those blocks, and the reference's fixed-width number formats."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, visu


@pytest.mark.parametrize("once", [False, True])
def test_visu_files(tmp_path, once):
    case = beds.lattice_cloud_case(300, seed=31)
    o = OracleSystem(case)
    opt = visu.VisuOptions(saveXDMFOnce=once, save_UsrMark=True, save_LinAcc=True, save_Theta=True,
                           save_RotAcc=True, save_CntctForce=True, save_Torque=True)
    n = case.particles.n
    w = visu.VisuWriter(str(tmp_path), "Bed", ifirst=1, ilast=4, save_visu=2, options=opt, np_in_domain=n)
    assert w.times == [0, 2, 4]
    for t in w.times:
        if t:
            o.step(2)
        F, T = o.forces()
        w.dump(t, o.state(), F, T)
    w.close()
    root = ET.parse(os.path.join(tmp_path, "PartVisuForBed.xmf")).getroot()
    grids = root.find("Domain").find("Grid").findall("Grid")
    assert [g.get("Name") for g in grids] == ["T0000000000", "T0000000002", "T0000000004"]
    st = o.state()
    F, T = o.forces()
    raw = np.fromfile(os.path.join(tmp_path, "PartVisuForBed0000000004"), dtype=np.uint8)
    want = [st.posR[:, :3], st.id, 2 * st.posR[:, 3], st.ptype, st.usrmark, st.linVel[:, 0], st.linAcc[:, 0],
            st.theta, st.rotVel[:, 0], st.rotAcc[:, 0], F, T]
    items = [grids[2].find("Geometry").find("DataItem")] + [a.find("DataItem") for a in grids[2].findall("Attribute")]
    assert len(items) == len(want)
    for item, arr in zip(items, want):
        seek = int(item.get("Seek"))
        dims, npart = (int(x) for x in item.get("Dimensions").split())
        dtype = np.int32 if item.get("DataType") == "Int" else np.float64
        assert npart == n and int(item.get("Precision")) == np.dtype(dtype).itemsize
        got = np.frombuffer(raw, dtype=dtype, count=dims * n, offset=seek)
        np.testing.assert_array_equal(got, np.asarray(arr, dtype).reshape(-1))
        assert item.text.strip() == "PartVisuForBed0000000004"
    assert raw.size == seek + dims * n * np.dtype(dtype).itemsize
    text = open(os.path.join(tmp_path, "PartVisuForBed.xmf")).read()
    # fixed-width numbers: I6 field count, I9 times, I2/I9 dimensions, I15 offsets
    assert f'Dimensions="     3">' in text
    assert '            ' + "        0        2        4" + '            </DataItem>' in text
    assert (f'<DataItem Format="Binary" DataType="Float" Precision="8" Endian="Native" '
            f'Dimensions=" 3{n:9d}" Seek="{0:15d}">') in text
