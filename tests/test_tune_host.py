"""The autotuner's host logic without a GPU: the choice is the fastest
measured candidate (ties keep the first), size classes separate beds that
must be tuned apart, and choices are cached by class."""
import numpy as np

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
