"""The autotuner's cache (rascil_gb300/tuning.py) on CPU: rule-based
defaults for untuned shapes, recorded choices served from memory and from
the JSON file in a fresh process state, forget, a corrupt or foreign file
ignored, and concurrent records kept whole."""
import json
import threading

import pytest


@pytest.fixture
def tuning(tmp_path, monkeypatch):
    from rascil_gb300 import tuning as t
    monkeypatch.setenv("RASCIL_GB300_TUNING", str(tmp_path / "tuning.json"))
    monkeypatch.setattr(t, "_mem", {})
    monkeypatch.setattr(t, "_loaded", [False])
    return t


def _fresh(t):
    t._mem.clear()
    t._loaded[0] = False


def test_defaults_then_recorded_choice(tuning):
    key = tuning.shape_key(8192, 8192, 1e-5, 4, "fp32", 1e-5, True, 16744448, 16)
    assert tuning.choose(key, 8192, 8192, 16744448, 16) == {"sigma": 0.0, "tile": 0, "slab": 0}
    tuning.record(key, {"sigma": 1.75, "tile": 16, "slab": 2}, {"a": 1.0})
    assert tuning.choose(key, 8192, 8192, 1, 1) == {"sigma": 1.75, "tile": 16, "slab": 2}
    # served from the file after the in-memory state is gone
    _fresh(tuning)
    assert tuning.choose(key, 8192, 8192, 1, 1) == {"sigma": 1.75, "tile": 16, "slab": 2}
    data = json.load(open(tuning.cache_path()))
    assert data["version"] == 1 and data["entries"][key]["timings"] == {"a": 1.0}
    tuning.forget(key)
    _fresh(tuning)
    assert tuning.choose(key, 8192, 8192, 1, 1)["sigma"] == 0.0


def test_shape_key_separates_what_changes_the_choice(tuning):
    base = (2048, 2048, 1e-4, 1, "fp32", 1e-5, True, 1000, 8)
    keys = {tuning.shape_key(*base)}
    for i, v in ((0, 4096), (3, 4), (4, "fp64"), (5, 1e-12), (6, False), (7, 2000), (8, 16)):
        alt = list(base)
        alt[i] = v
        keys.add(tuning.shape_key(*alt))
    assert len(keys) == 8


@pytest.mark.parametrize("content", ["{not json", json.dumps({"version": 99, "entries": {
    "k": {"sigma": 1.5, "tile": 16, "slab": 2}}}), json.dumps({"version": 1, "entries": {
    "k": "garbage"}})])
def test_corrupt_or_foreign_cache_files_are_ignored(tuning, content):
    with open(tuning.cache_path(), "w") as f:
        f.write(content)
    assert tuning.choose("k", 256, 256, 1, 1) == {"sigma": 0.0, "tile": 0, "slab": 0}


def test_concurrent_records_are_all_kept(tuning):
    def rec(i):
        tuning.record("key%d" % i, {"sigma": 2.0, "tile": 16 + i % 2 * 16, "slab": 2}, {})

    threads = [threading.Thread(target=rec, args=(i,)) for i in range(16)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    _fresh(tuning)
    for i in range(16):
        assert tuning.choose("key%d" % i, 1, 1, 1, 1)["tile"] == 16 + i % 2 * 16
