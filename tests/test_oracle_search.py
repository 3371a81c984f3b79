"""The oracle's NBS-Munjiza search finds exactly the pairs a brute-force
all-pairs test finds (same FP64 expression), for polydisperse clouds."""
import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds


def brute_pairs(posR):
    n = len(posR)
    out = set()
    for i in range(n):
        dr = posR[i, 3] + posR[i + 1:, 3]
        dr2 = dr * dr
        dx = posR[i, 0] - posR[i + 1:, 0]
        dy = posR[i, 1] - posR[i + 1:, 1]
        dz = posR[i, 2] - posR[i + 1:, 2]
        d2 = dz * dz + (dy * dy + dx * dx)
        for j in np.nonzero(d2 <= dr2)[0]:
            out.add((i, i + 1 + int(j)))
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_search_equals_brute_force(seed):
    case = beds.random_cloud_case(600, seed=seed, box=(0.012, 0.012, 0.012), ntypes=7)
    o = OracleSystem(case)
    o.step(1)
    ids = case.particles.id
    got = set()
    oi, pid, _, _ = o.contacts()
    st = o.state()
    for a, b in zip(oi, pid):
        if b <= case.opts.base_wall_id:
            ga = int(st.id[a])
            got.add((min(ga, int(b)), max(ga, int(b))))
    want = {(int(ids[i]), int(ids[j])) for i, j in brute_pairs(case.particles.posR)}
    want = {(min(a, b), max(a, b)) for a, b in want}
    assert got == want
    assert o.counters()["pp"] == len(want)
