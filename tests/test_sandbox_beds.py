"""The batched workload's sandboxes (sdem_gb300.beds.sandbox_case): seeded,
within the configuration's ranges, inside their boxes, and steppable by the
oracle."""
import numpy as np

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, props


def test_sandboxes_are_seeded_and_in_range():
    a = [beds.sandbox_case(np.random.default_rng(4), i, n_lo=200, n_hi=600) for i in range(1)]
    rng1, rng2 = np.random.default_rng(4), np.random.default_rng(4)
    c1 = [beds.sandbox_case(rng1, i, n_lo=200, n_hi=600) for i in range(6)]
    c2 = [beds.sandbox_case(rng2, i, n_lo=200, n_hi=600) for i in range(6)]
    assert a[0].particles.n == c1[0].particles.n
    models = set()
    for x, y in zip(c1, c2):
        np.testing.assert_array_equal(x.particles.posR, y.particles.posR)
        p = x.particles
        assert 200 <= p.n <= 600
        assert p.ptype.min() >= 1 and p.ptype.max() <= 5
        lo, hi = np.array(x.opts.minpoint), np.array(x.opts.maxpoint)
        assert np.all(p.posR[:, :3] - p.posR[:, 3:4] > lo) and np.all(p.posR[:, :3] + p.posR[:, 3:4] < hi)
        assert x.walls.n == 5
        assert x.opts.dt == 2.0e-6
        models.add(x.opts.cf_type)
        ext = hi - lo
        assert 0.3 < ext[0] / ext[1] < 3.0 and 0.3 < ext[2] / ext[1] < 3.0
    assert models <= {props.CFT_LSD, props.CFT_NLIN}


def test_sandbox_steps_in_the_oracle():
    case = beds.sandbox_case(np.random.default_rng(4), 0, n_lo=300, n_hi=300)
    o = OracleSystem(case)
    o.step(3)
    assert o.counters()["nlocal"] == 300
