"""The autotuner's host logic without a GPU: the choice is the fastest
measured candidate (ties keep the first), size classes separate beds that
must be tuned apart, and choices are cached by class."""
from sdem_gb300 import beds, tune


def test_best_of_picks_the_fastest_first_on_ties():
    times = {"a": 3.0, "b": 1.0, "c": 1.0, "d": 2.0}
    best, seen = tune.best_of(list(times), times.__getitem__)
    assert best == "b" and seen == times


def test_size_classes():
    a = beds.lattice_cloud_case(800, seed=1)
    b = beds.lattice_cloud_case(900, seed=2)
    c = beds.scaled(a, cs_method=2)
    d = beds.lattice_cloud_case(3200, seed=3)
    assert tune.size_class(a) == tune.size_class(b)
    assert tune.size_class(a) != tune.size_class(c) and tune.size_class(a) != tune.size_class(d)


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setattr(tune, "CACHE_DIR", str(tmp_path))
    tune._store("handle", {"k": {"pipeline_chunks": 3}})
    assert tune._load("handle") == {"k": {"pipeline_chunks": 3}}
    assert tune._load("batch") == {}


def test_handle_candidates_and_choice(tmp_path, monkeypatch):
    # tune_handle over a stand-in handle: every (chunks, force blocks, first
    # chunk share) candidate is timed once, the first chunk's share only with
    # more than one chunk, and the fastest shape is chosen and cached
    from sdem_gb300 import capi
    monkeypatch.setattr(tune, "CACHE_DIR", str(tmp_path))
    seen = []

    class FakeSystem:
        def __init__(self, case):
            self.shape = None

        def __enter__(self):
            return self

        def __exit__(self, *exc):
            return False

        def set_launch(self, c, f, p):
            self.shape = (c, f, p)
            seen.append(self.shape)

    monkeypatch.setattr(capi, "DEMSystem", FakeSystem)
    fastest = (3, 2, 25)
    timer = lambda h, steps: 1.0 if h.shape == fastest else 2.0 + 0.01 * len(seen)
    case = beds.lattice_cloud_case(800, seed=1)
    choice = tune.tune_handle(case, steps=3, timer=timer)
    assert (choice["pipeline_chunks"], choice["force_blocks_per_sm"], choice["first_chunk_percent"]) == fastest
    assert all(p == -1 for c, f, p in seen if c == 1)
    assert len(seen) == len(set(seen)) == len(tune.FORCE_BLOCKS) * (1 + (len(tune.CHUNKS) - 1) * len(tune.FIRST_CHUNK))
    seen.clear()
    assert tune.tune_handle(case, steps=3, timer=timer) == choice and not seen   # cached by size class
