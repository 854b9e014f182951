"""The schedule autotuner's cache logic, without a GPU: the first request for a key measures every
candidate and records the fastest in the JSON cache; later requests (also from a fresh process, i.e.
a cold in-memory cache) read the file and measure nothing."""
import json

import pytest

from cola_gb300 import tuning


def test_tuner_measures_once_then_reads_the_cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("COLA_GB300_TUNE_CACHE", str(path))
    monkeypatch.setattr(tuning, "_mem", None)
    calls = []

    def measure(s):
        calls.append(s)
        return {"onchip": 3e-6, "cluster8": 2e-6, "cluster16": None, "grid": 9e-6, "block": None}[s]
    assert tuning.choose("k1", measure) == "cluster8"
    assert calls == list(tuning.CANDIDATES)
    rec = json.loads(path.read_text())["k1"]
    assert rec["schedule"] == "cluster8" and set(rec["us_per_step_system"]) == {"onchip", "cluster8", "grid"}

    def boom(s):
        raise AssertionError("measured although the key is cached")
    assert tuning.choose("k1", boom) == "cluster8"
    monkeypatch.setattr(tuning, "_mem", None)  # a fresh process reads the file
    assert tuning.choose("k1", boom) == "cluster8"
    # another key is tuned separately and both stay in the file
    assert tuning.choose("k2", lambda s: {"grid": 1e-6}.get(s)) == "grid"
    assert set(json.loads(path.read_text())) == {"k1", "k2"}


def test_tuner_refuses_when_nothing_applies(tmp_path, monkeypatch):
    monkeypatch.setenv("COLA_GB300_TUNE_CACHE", str(tmp_path / "t.json"))
    monkeypatch.setattr(tuning, "_mem", None)
    with pytest.raises(RuntimeError, match="no schedule applies"):
        tuning.choose("k", lambda s: None)
