"""Cache behaviour of the autotuner (sucemfem/autotune.py) with fake trial
timings, on the CPU: the fastest candidate wins, a cached choice is reused
without new trials (also by a new tuner object, i.e. across processes),
keys separate devices, kinds and size classes, and a disabled tuner makes
no trials."""
import json

from sucemfem import autotune


def _fake(times):
    calls = []

    def measure(c):
        calls.append(c)
        return times[c]
    return measure, calls


def test_fastest_candidate_is_chosen_and_cached(tmp_path):
    path = str(tmp_path / "cache.json")
    t = autotune.Autotuner(path=path, device="devA")
    measure, calls = _fake({2: 3.0, 4: 1.0, 8: 2.0})
    assert t.choose("serve_slots", "k", [2, 4, 8], measure, repeats=2) == 4
    assert len(calls) == 6 and t.trials == 6
    # second ask: from the cache, no trials
    measure2, calls2 = _fake({2: 0.1, 4: 9.0, 8: 9.0})
    assert t.choose("serve_slots", "k", [2, 4, 8], measure2) == 4
    assert calls2 == []
    # a new tuner on the same file (another process) sees the choice
    t2 = autotune.Autotuner(path=path, device="devA")
    assert t2.lookup("serve_slots", "k") == 4
    assert t2.choose("serve_slots", "k", [2, 4, 8], measure2) == 4 and calls2 == []
    d = json.load(open(path))
    assert d["devA|serve_slots|k"]["choice"] == 4


def test_keys_separate_device_kind_and_size(tmp_path):
    path = str(tmp_path / "cache.json")
    a = autotune.Autotuner(path=path, device="devA")
    b = autotune.Autotuner(path=path, device="devB")
    m1, _ = _fake({(256, 64): 2.0, (512, 64): 1.0})
    m2, _ = _fake({(256, 64): 1.0, (512, 64): 2.0})
    assert a.choose("lu_plan", "small", [(256, 64), (512, 64)], m1) == (512, 64)
    assert b.choose("lu_plan", "small", [(256, 64), (512, 64)], m2) == (256, 64)
    assert a.choose("lu_plan", "large", [(256, 64), (512, 64)], m2) == (256, 64)
    assert a.lookup("lu_plan", "small") == (512, 64)   # tuples survive the JSON round trip
    assert a.lookup("serve_slots", "small") is None


def test_disabled_tuner_makes_no_trials(tmp_path):
    t = autotune.Autotuner(path=str(tmp_path / "c.json"), device="d", enabled=False)
    m, calls = _fake({1: 1.0, 2: 0.5})
    assert t.choose("x", "k", [1, 2], m) == 1 and calls == []


def test_size_classes():
    a = autotune.size_class(316120, 13419440, "c64")
    assert a == autotune.size_class(320000, 13500000, "c64")
    assert a != autotune.size_class(600000, 13419440, "c64")
    assert a != autotune.size_class(316120, 13419440, "f32")
