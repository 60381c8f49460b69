"""Autotuner cache logic (CPU only)."""
import json


def test_choose_record_and_reload(tmp_path, monkeypatch):
    from rascil_gb300 import tuning
    path = tmp_path / "tuning.json"
    monkeypatch.setenv("RASCIL_GB300_TUNING", str(path))
    monkeypatch.setattr(tuning, "_mem", {})
    monkeypatch.setattr(tuning, "_loaded", [False])
    key = tuning.shape_key(512, 512, 5e-4, 1, "fp64", 1e-12, True, 129024, 1)
    assert tuning.choose(key, 512, 512, 129024, 1) == tuning.default_params(512, 512, 129024, 1)
    tuning.record(key, {"sigma": 1.5, "tile": 16, "slab": 2}, {"a": 1.0})
    data = json.loads(path.read_text())
    assert data["version"] == 1 and data["entries"][key]["sigma"] == 1.5
    # a fresh process reads the file back
    monkeypatch.setattr(tuning, "_mem", {})
    monkeypatch.setattr(tuning, "_loaded", [False])
    assert tuning.choose(key, 512, 512, 129024, 1) == {"sigma": 1.5, "tile": 16, "slab": 2}
    tuning.forget(key)
    assert tuning.choose(key, 512, 512, 129024, 1)["sigma"] == 0.0


def test_corrupt_cache_is_ignored(tmp_path, monkeypatch):
    from rascil_gb300 import tuning
    path = tmp_path / "tuning.json"
    path.write_text("{not json")
    monkeypatch.setenv("RASCIL_GB300_TUNING", str(path))
    monkeypatch.setattr(tuning, "_mem", {})
    monkeypatch.setattr(tuning, "_loaded", [False])
    key = tuning.shape_key(64, 64, 1e-3, 1, "fp32", 1e-5, True, 10, 1)
    assert tuning.choose(key, 64, 64, 10, 1)["sigma"] == 0.0
