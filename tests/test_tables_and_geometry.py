"""Host-side restatements (material tables, plane walls) agree bit for bit with
the oracle's C restatement of the same reference routines."""
import numpy as np
import pytest

from oracle import oracle
from sdem_gb300 import props
from sdem_gb300.geometry import box_walls, plane_wall


@pytest.mark.parametrize("cf", [props.CFT_LSD, props.CFT_NLIN])
def test_binary_property_matches_oracle(cf):
    rng = np.random.default_rng(0)
    for _ in range(50):
        di, dj = rng.uniform(2e-4, 5e-3, 2)
        rho = rng.uniform(1000, 8000)
        Ei, Ej = 10 ** rng.uniform(6, 10, 2)
        pri, prj = rng.uniform(0.1, 0.45, 2)
        mus, muk, mur = rng.uniform(0.05, 0.9, 3)
        en, et = rng.uniform(0.1, 0.99, 2)
        a = props.pure_property(di, rho, Ei, pri)
        b = props.pure_property(dj, rho, Ej, prj)
        for iswall in (False, True):
            bb = props.wall_pure_property(Ej, prj) if iswall else b
            py = props.binary_property(cf, a, bb, mus, muk, mur, en, et, iswall)
            c = oracle.binary_prop(cf, a.radius, a.mass, a.youngs, a.poisson, bb.radius, bb.mass, bb.youngs,
                                   bb.poisson, mus, muk, mur, en, et, iswall)
            np.testing.assert_array_equal(py, c)


def test_pure_property_matches_oracle():
    for d in (0.5e-3, 0.8e-3, 1e-3, 1.2e-3, 1.5e-3, 3.3e-3):
        p = props.pure_property(d, 2500.0, 1e7, 0.3)
        r, m, i = oracle.pure_prop(d, 2500.0)
        assert (p.radius, p.mass, p.inertia) == (r, m, i)


def test_same_type_quirk_of_binary_table():
    # Prtcl_Property.f90:137-138: record (i, j) is built from type i twice
    t = props.build_tables(props.CFT_NLIN, [0.8e-3, 1.2e-3], [2500.0] * 2, [5e7] * 2, [0.3] * 2,
                           (0.4, 0.4, 0.1, 0.8, 0.8), [5e7], [0.3], (0.4, 0.4, 0.1, 0.8, 0.8))
    bpp = t.bpp.reshape(2, 2, 11)   # [j, i]
    np.testing.assert_array_equal(bpp[0, 0], bpp[1, 0])   # (i=0, j=0) == (i=0, j=1)
    assert bpp[0, 1][0] != bpp[0, 0][0]


def test_plane_wall_matches_oracle():
    rng = np.random.default_rng(1)
    for _ in range(20):
        o = rng.uniform(-1, 1, 3)
        u = rng.uniform(-1, 1, 3)
        v = np.cross(u, rng.uniform(-1, 1, 3))
        pts = [o, o + u, o + u + v, o + v]
        w, f = plane_wall(*pts, wall_id=10000001)
        c = oracle.make_wall(*pts)
        np.testing.assert_array_equal(w[:16], c[:16])
        np.testing.assert_array_equal(w[19:], c[19:])


def test_box_walls_point_inward():
    ws = box_walls((0, 0, 0), (1, 2, 3))
    w, f = ws.arrays()
    w = w.reshape(-1, 25)
    centre = np.array([0.5, 1.0, 1.5])
    for row in w:
        assert row[12:15] @ centre + row[15] > 0
    assert list(f.reshape(-1, 4)[:, 2]) == [10000001 + k for k in range(5)]
