"""The 1M polydisperse Hertz configuration on its settled bed.

The bed is the bench's: seeded random sequential placement (solid fraction
0.25) settled under gravity by the GPU path (sdem_gb300.settle), in the
configuration's material (E 5e7 Pa, restitution 0.8, friction 0.4, dt 1e-6 s,
AB2).

- Contact-set horizon over the first 1,000 steps (a resynchronised chain):
  the GPU runs free for 1,000 steps; before its steps 1, 10, 100, 250, 500
  and 1,000 the oracle takes the GPU's state and contact list (restart
  style) and both step once.  Counters and contact sets are equal, contact
  history, forces and torques within 1e-12 relative, positions within 1e-13.
  Contact discovery (Prtcl_NBS_Munjiza.f90:503-530) is checked bit for bit
  at every checkpoint; chaos cannot hide or create a mismatch.
- Free run: the GPU and the oracle step the same settled bed independently
  and their contact sets are compared after every step; the first step at
  which they differ is reported (trajectories agree to ~1 ulp per step and
  then diverge, Prtcl_Integration.f90:15-88).  At 1M spheres for 20 steps, at
  20,000 spheres of the same material (0.02 x 0.6 x 0.02 m box) for 1,000.
"""
import json

import numpy as np
import pytest

from oracle.oracle import OracleSystem
from sdem_gb300 import beds, settle
from sdem_gb300.capi import DEMSystem
from tests.helpers import assert_step_matches, sorted_contacts

pytestmark = pytest.mark.gpu

CHECKPOINTS = (1, 10, 100, 250, 500, 1000)


@pytest.fixture(scope="module")
def settled_1m(gpu_lib):
    return settle.settled_hertz_poly_case(n=1_000_000, seed=2)


@pytest.fixture(scope="module")
def settled_20k(gpu_lib):
    return settle.settled_hertz_poly_case(n=20_000, seed=12, box=(0.02, 0.6, 0.02))


def test_settled_bed_is_settled(settled_1m):
    """At rest on its contacts: about two particle-particle contacts per
    sphere (a frictional random packing), slow spheres, a bed ~0.1 m high."""
    case = settled_1m
    with DEMSystem(case) as g:
        g.step(1)
        c = g.counters()
        st = g.state()
    v = np.linalg.norm(st.linVel[:, 0, :], axis=1)
    log = json.loads(case.note)["settling"]
    print(f"settled 1M bed: {c['pp'] / st.n:.3f} pp contacts per sphere, {c['pw']} wall contacts, "
          f"v mean {v.mean():.2e} m/s, median {np.median(v):.2e} m/s, max {v.max():.2e} m/s, "
          f"height {log[-1]['height']:.4f} m")
    assert c["pp"] > 1.5 * st.n
    assert v.mean() < 0.01 and np.median(v) < 0.01
    assert 0.08 < log[-1]["height"] < 0.12


def test_contact_sets_over_1000_steps_resynchronised(settled_1m):
    case = settled_1m
    g = DEMSystem(case)
    done = 0
    seen = []
    for k in CHECKPOINTS:
        g.step(k - 1 - done)           # the GPU's free run up to step k-1
        st, cl = g.state(), g.contacts()
        o = OracleSystem(beds.Case(case.name, case.opts, case.tables, case.walls, st, contacts=cl))
        g.step(1)                      # step k of the free run ...
        o.step(1)                      # ... and the oracle's step from the same inputs
        done = k
        seen.append((k, assert_step_matches(g, o, what=f"step {k}", pre=st, case=case)))
        o.close()
    g.close()
    print("resynchronised checkpoints:", seen)


def free_run(case, steps):
    g, o = DEMSystem(case), OracleSystem(case)
    first = None
    for k in range(1, steps + 1):
        g.step(1)
        o.step(1)
        kg, _ = sorted_contacts(g)
        ko, _ = sorted_contacts(o)
        if not np.array_equal(kg, ko):
            first = k
            break
    dx = float(np.abs(g.state().posR - o.state().posR).max())
    g.close()
    o.close()
    return first, dx


def test_free_run_1m_20_steps(settled_1m):
    first, dx = free_run(settled_1m, 20)
    print(f"free run, 1M settled bed: first step with different contact sets: {first or 'none in 20'}; "
          f"max position difference {dx:.3e} m")
    assert first is None, f"contact sets differ at free-run step {first}"


def test_free_run_20k_1000_steps(settled_20k):
    first, dx = free_run(settled_20k, 1000)
    print(f"free run, 20k settled bed: first step with different contact sets: {first or 'none in 1000'}; "
          f"max position difference {dx:.3e} m")
    assert first is None or first > 50, f"contact sets differ already at free-run step {first}"
