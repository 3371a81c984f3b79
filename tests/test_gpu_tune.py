"""The autotuner's knobs leave results unchanged, and the tuner picks one of
its candidates: a handle stepped with every launch shape, and a batch with
several group sizes, give bit-identical states, forces, contact lists and
counters."""
import numpy as np
import pytest

from sdem_gb300 import beds, tune
from sdem_gb300.capi import DEMBatch, DEMSystem
from tests.helpers import sorted_contacts

pytestmark = pytest.mark.gpu


def snapshot(s):
    st = s.state()
    F, T = s.forces()
    k, h = sorted_contacts(s)
    return st, F, T, k, h, s.counters()


def assert_identical(a, b):
    sa, Fa, Ta, ka, ha, ca = a
    sb, Fb, Tb, kb, hb, cb = b
    for f in ("id", "posR", "linVel", "linAcc", "theta", "rotVel", "rotAcc"):
        np.testing.assert_array_equal(getattr(sa, f), getattr(sb, f), err_msg=f)
    np.testing.assert_array_equal(Fa, Fb)
    np.testing.assert_array_equal(Ta, Tb)
    np.testing.assert_array_equal(ka, kb)
    np.testing.assert_array_equal(ha, hb)
    assert ca == cb


def test_launch_shapes_bit_identical(gpu_lib):
    case = beds.hertz_poly_case(n=200_000, seed=5)
    ref = None
    for chunks, fb, fp in ((2, 3, -1), (1, 2, -1), (3, 4, 30), (4, 8, -1), (2, 3, 20)):
        with DEMSystem(case) as s:
            s.set_launch(chunks, fb, fp)
            assert s.get_launch() == (chunks, fb, max(fp, 0))
            s.step(7)
            s.set_launch(1 if chunks > 1 else 2, 0, 0)   # a change between steps recaptures the graphs
            s.step(5)
            snap = snapshot(s)
        if ref is None:
            ref = snap
        else:
            assert_identical(ref, snap)


def test_batch_group_sizes_bit_identical(gpu_lib):
    rng = np.random.default_rng(44)
    cases = [beds.sandbox_case(rng, i, n_lo=2000, n_hi=6000) for i in range(7)]
    results = []
    for gs in (0, 2, 3):
        members = [DEMSystem(c) for c in cases]
        b = DEMBatch(members, group_size=gs)
        b.step(6)
        results.append([snapshot(m) for m in members])
        b.close()
        for m in members:
            m.close()
    for other in results[1:]:
        for a, b in zip(results[0], other):
            assert_identical(a, b)


def test_tuner_returns_a_candidate(gpu_lib, tmp_path, monkeypatch):
    monkeypatch.setattr(tune, "CACHE_DIR", str(tmp_path))
    case = beds.lattice_cloud_case(3000, seed=9)
    choice = tune.tune_handle(case, steps=3)
    assert choice["pipeline_chunks"] in tune.CHUNKS and choice["force_blocks_per_sm"] in tune.FORCE_BLOCKS
    n_cands = len(tune.FORCE_BLOCKS) * (1 + (len(tune.CHUNKS) - 1) * len(tune.FIRST_CHUNK))
    assert choice["cs_ratio"] == case.opts.cs_ratio and len(choice["tried"]) == n_cands
    assert tune.tune_handle(case, steps=3) == choice        # cached
    with DEMSystem(case) as s:
        tune.apply(s, choice)
        assert s.get_launch() == (choice["pipeline_chunks"], choice["force_blocks_per_sm"],
                                  max(choice["first_chunk_percent"], 0))
