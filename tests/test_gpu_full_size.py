"""The benchmark beds at their full sizes.

- the 1M-sphere polydisperse Hertz bed (41 types, five walls), the 4M-sphere
  bidisperse hopper (one-level and hierarchical search) and the 20k
  monodisperse LSD bed (after 5000 steps of settling, restarted from the
  GPU's state and contact list): one step from identical inputs against the oracle
  (contact sets equal; history, forces, torques within 1e-12 relative;
  counters equal), with vectorised comparisons;
- the 1M bed over 20 steps: the captured two-step graph and single steps
  with lagged counter reads give bit-identical states and counters (a
  size-independent determinism property of the whole pipeline: search,
  in-list slots, force, gather, integration, delete).
"""
import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds
from sdem_gb300.capi import DEMSystem
from tests.helpers import force_scale

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def sorted_contacts(system):
    """(keys, history) of the live contact list, keys = (listing id, partner
    or wall id) packed in 64 bits, sorted."""
    ids = system.state().id.astype(np.int64)
    o, q, t, v = system.contacts()
    key = (ids[o] << 32) | (np.asarray(q, np.int64) & 0xFFFFFFFF)
    order = np.argsort(key, kind="stable")
    hist = np.concatenate([np.asarray(t, float), np.asarray(v, float)[:, None]], axis=1)
    return key[order], hist[order]


def compare_one_step(case):
    g, o = DEMSystem(case), OracleSystem(case)
    g.step(1)
    o.step(1)
    cg, co = g.counters(), o.counters()
    for k in ("pp", "pw", "cnsv", "nlocal"):
        assert cg[k] == co[k], f"counter {k}: gpu {cg[k]} oracle {co[k]}"
    assert cg["pp"] + cg["pw"] > 0, "the bed should be in contact"
    kg, hg = sorted_contacts(g)
    ko, ho = sorted_contacts(o)
    assert len(np.unique(kg)) == len(kg), "a contact is listed twice"
    np.testing.assert_array_equal(kg, ko)
    sc = np.maximum(np.abs(hg[:, :3]).max(axis=1), np.abs(ho[:, :3]).max(axis=1))
    sc = np.maximum(sc, 1e-25)
    assert (np.abs(hg[:, :3] - ho[:, :3]).max(axis=1) <= RTOL * sc).all(), "tangential history"
    sv = np.maximum(np.maximum(np.abs(hg[:, 3]), np.abs(ho[:, 3])), 1e-300)
    assert (np.abs(hg[:, 3] - ho[:, 3]) <= RTOL * sv).all(), "VelRel_Init"
    Fg, Tg = g.forces()
    Fo, To = o.forces()
    fs = force_scale(Fo, 1e-6 * max(np.abs(Fo).max(), 1e-30))
    ts = force_scale(To, 1e-6 * max(np.abs(To).max(), 1e-30))
    assert np.all(np.abs(Fg - Fo).max(axis=1) <= RTOL * fs), "force mismatch"
    assert np.all(np.abs(Tg - To).max(axis=1) <= RTOL * ts), "torque mismatch"
    sg, so = g.state(), o.state()
    np.testing.assert_array_equal(sg.id, so.id)
    np.testing.assert_allclose(sg.posR, so.posR, rtol=1e-13, atol=1e-18)
    g.close()


def test_hertz_poly_1m_one_step_matches_oracle(gpu_lib):
    # a packed bed: ~1.5 particle-particle contacts per sphere
    compare_one_step(beds.hertz_poly_case(n=1_000_000, seed=2))


def test_lsd_mono_20k_one_step_matches_oracle(gpu_lib):
    # the lattice starts without contacts: 5000 GPU steps (10 ms) let the
    # spheres collide, then both codes step once from that state and its
    # contact list (restart style)
    case0 = beds.lsd_mono_case(n=20_000, seed=1)
    run = DEMSystem(case0)
    run.step(5000)
    case = beds.Case(case0.name, case0.opts, case0.tables, case0.walls, run.state(), contacts=run.contacts())
    run.close()
    compare_one_step(case)


@pytest.mark.parametrize("cs_method", [1, 2])
def test_hopper_4m_one_step_matches_oracle(gpu_lib, cs_method):
    # 4M bidisperse (1:3) Hertz spheres in a hopper of four inclined finite
    # quads over a 10 mm outlet, plus a vertical column; one-level search and
    # the hierarchical search (CS_Method 2)
    case = beds.hopper_case(4_000_000, 3, width=0.26, outlet=10.0e-3)
    if cs_method == 2:
        case = beds.scaled(case, cs_method=2)
    compare_one_step(case)


def test_hertz_poly_1m_graph_and_single_steps_bit_identical(gpu_lib):
    case = beds.hertz_poly_case(n=1_000_000, seed=2)
    a = DEMSystem(case)
    a.step(20)                       # two-step graph replays
    b = DEMSystem(case)
    seen = []
    b.step_async(1)
    for k in range(1, 21):
        if k < 20:
            b.step_async(1)
            seen.append(b.counters_lagged()["iter"])
        else:
            seen.append(b.counters()["iter"])
    assert seen == list(range(1, 21))
    assert a.counters() == b.counters()
    sa, sb = a.state(), b.state()
    for f in ("id", "ptype", "usrmark", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc"):
        np.testing.assert_array_equal(getattr(sa, f), getattr(sb, f), err_msg=f)
    Fa, Ta = a.forces()
    Fb, Tb = b.forces()
    np.testing.assert_array_equal(Fa, Fb)
    np.testing.assert_array_equal(Ta, Tb)
    ka, ha = sorted_contacts(a)
    kb, hb = sorted_contacts(b)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(ha, hb)
    a.close()
    b.close()
