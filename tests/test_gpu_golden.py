"""The GPU path (through the C ABI) against the golden fixtures of
tests/golden/: from each input restart file, one step reproduces the stored
contact list exactly, its spring history and the forces and torques within
1e-12 relative, and the state; ten free steps keep the contact set and the
positions within the free-run bound."""
import numpy as np
import pytest

from sdem_gb300.capi import DEMSystem
from tests.golden_io import CHAIN, GOLDEN, forces, keyed, load, start
from tests.helpers import assert_same_contact_sets, compare_history, force_scale

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_gpu_reproduces_golden_chain(gpu_lib, name):
    case, pre = start(name)
    g = DEMSystem(case)
    done = 0
    for k in CHAIN:
        g.step(k - done)
        done = k
        want_p, want_c = load(name, pre + k, case)
        st = g.state()
        np.testing.assert_array_equal(st.id, want_p.id)
        kg, kw = keyed(st, g.contacts()), keyed(want_p, want_c)
        assert_same_contact_sets(kg, kw, f"{name} +{k}")
        if k == 1:
            compare_history(kg, kw, 1e-12)
            F, T = g.forces()
            Fw, Tw = forces(name, pre + 1)
            fs = force_scale(Fw, 1e-6 * max(np.abs(Fw).max(), 1e-30))
            ts = force_scale(Tw, 1e-6 * max(np.abs(Tw).max(), 1e-30))
            assert np.all(np.abs(F - Fw).max(axis=1) <= 1e-12 * fs), "force mismatch"
            assert np.all(np.abs(T - Tw).max(axis=1) <= 1e-12 * ts), "torque mismatch"
            np.testing.assert_allclose(st.posR, want_p.posR, rtol=1e-13, atol=1e-18)
        else:
            np.testing.assert_allclose(st.posR, want_p.posR, rtol=1e-11, atol=1e-15)
    g.close()
