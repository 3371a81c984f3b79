"""Seeded random sequential placement (sdem_gb300/csrc/bedgen.c) of the
settled 1M configuration's bed: no two spheres overlap, every sphere lies in
its region, the same seed gives the same bed, and the region's height follows
from the solid fraction."""
import math

import numpy as np
from scipy.spatial import cKDTree

from sdem_gb300 import beds, build


def test_rsp_no_overlaps_inside_and_deterministic():
    build.build()
    rng = np.random.default_rng(3)
    r = rng.uniform(0.4e-3, 0.6e-3, 3000)
    lo, hi = (0.0, 0.0, 0.0), (0.02, 0.02, 0.02)
    p = beds.rsp_positions(r, lo, hi, seed=9)
    assert np.all(p - r[:, None] >= -1e-15) and np.all(p + r[:, None] <= np.array(hi) + 1e-15)
    pairs = cKDTree(p).query_pairs(2 * r.max(), output_type="ndarray")
    d = np.linalg.norm(p[pairs[:, 0]] - p[pairs[:, 1]], axis=1)
    assert np.all(d >= r[pairs[:, 0]] + r[pairs[:, 1]])
    np.testing.assert_array_equal(p, beds.rsp_positions(r, lo, hi, seed=9))
    assert not np.array_equal(p, beds.rsp_positions(r, lo, hi, seed=10))


def test_rsp_case_fill_height():
    case = beds.hertz_poly_rsp_case(20000, 12, box=(0.02, 0.6, 0.02), fill=0.25)
    r = case.particles.posR[:, 3]
    h = (4.0 / 3.0 * math.pi * r ** 3).sum() / 0.25 / (0.02 * 0.02)
    top = (case.particles.posR[:, 1] + r).max()
    assert top <= h + 1e-12 and top > 0.95 * h
    assert case.contacts is None and np.all(case.particles.linVel == 0.0)
