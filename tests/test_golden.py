"""The oracle against the golden fixtures of tests/golden/ (restart chains in
the reference's restart-file layout, made by tests/golden/make_golden.py):
from each input file, one step and ten steps reproduce the stored states,
contact lists with spring history, and the first step's forces and torques.
This pins the oracle to the fixtures; with a Fortran build of the reference,
regenerated fixtures pin it to the reference itself."""
import os

import numpy as np
import pytest

from oracle.oracle import OracleSystem
from tests.golden_io import CHAIN, GOLDEN, GOLDEN_DIR, forces, keyed, load, start
from tests.golden.cases import file_name
from tests.helpers import assert_same_contact_sets, compare_history

FIELDS = ("posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc")


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_oracle_reproduces_golden_chain(name):
    case, pre = start(name)
    o = OracleSystem(case)
    done = 0
    for k in CHAIN:
        o.step(k - done)
        done = k
        want_p, want_c = load(name, pre + k, case)
        st = o.state()
        np.testing.assert_array_equal(st.id, want_p.id)
        np.testing.assert_array_equal(st.ptype, want_p.ptype)
        for f in FIELDS:
            np.testing.assert_allclose(getattr(st, f), getattr(want_p, f), rtol=1e-13, atol=0, err_msg=f)
        kg, kw = keyed(st, o.contacts()), keyed(want_p, want_c)
        assert_same_contact_sets(kg, kw, f"{name} +{k}")
        compare_history(kg, kw, 1e-13)
        if k == 1:
            F, T = o.forces()
            Fw, Tw = forces(name, pre + 1)
            np.testing.assert_allclose(F, Fw, rtol=1e-13, atol=1e-13 * np.abs(Fw).max())
            np.testing.assert_allclose(T, Tw, rtol=1e-13, atol=1e-13 * np.abs(Tw).max())


def test_golden_files_have_the_reference_layout():
    # byte count of the restart layout: header, positions, (id, type, mark),
    # the real3 block, contacts per particle, listed pairs, TanDel records
    name = "hertz_poly"
    case, pre = start(name)
    p, c = load(name, pre, case)
    import gzip
    with gzip.open(os.path.join(GOLDEN_DIR, file_name(name, pre)), "rb") as f:
        raw = f.read()
    n, nct = np.frombuffer(raw, np.int32, count=2)
    assert n == p.n and nct == len(c[0])
    nreal3 = 2 * (1 + case.opts.tsize + case.opts.rsize) - 1
    pw = sum(1 for q in c[1] if q > case.opts.base_wall_id)
    ntan = (nct - pw) // 2 + pw
    assert len(raw) == 8 + 24 * n + 12 * n + 24 * nreal3 * n + 4 * n + 8 * nct + 32 * ntan
    # every case exercises contacts with history, and the hopper its outlet
    for nm in GOLDEN:
        cs, pr = start(nm)
        assert len(cs.contacts[0]) > 100, nm
    hop, pr = start("hopper")
    out, _ = load("hopper", pr + 10, hop)
    assert out.n < hop.particles.n
