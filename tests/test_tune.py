"""Autotuner host logic: the on-disk cache and the switches (no GPU needed)."""
from __future__ import annotations

import json


def test_cache_round_trip(tmp_path, monkeypatch):
    from eigenfns_gb300 import tune
    path = tmp_path / "sub" / "tune.json"
    monkeypatch.setenv("EIGENFNS_GB300_TUNE_CACHE", str(path))
    assert tune.cache_path() == path and tune._load_cache() == {}
    tune._store("gpu|v|op|G=32|m=8", {"passes": 3, "subbatch_bytes": 1})
    tune._store("gpu|v|gram|8x8|K=1", {"kernel": 1, "units": 2})
    data = json.loads(path.read_text())
    assert data["gpu|v|op|G=32|m=8"]["passes"] == 3 and data["gpu|v|gram|8x8|K=1"]["units"] == 2
    path.write_text("not json")
    assert tune._load_cache() == {}


def test_switches_and_shapes(monkeypatch):
    from eigenfns_gb300 import tune
    monkeypatch.delenv("EF_AUTOTUNE", raising=False)
    assert not tune.enabled() and tune.enabled(True) and not tune.enabled(False)
    monkeypatch.setenv("EF_AUTOTUNE", "1")
    assert tune.enabled()
    assert tune.lobpcg_gram_shapes(32) == [(32, 32), (64, 32), (32, 64), (32, 96)]
    assert all(k in (1, 2) and 0 <= u <= 16 for k, u in tune.GRAM_CANDIDATES)


def test_stored_pipeline_is_applied_without_timing(tmp_path, monkeypatch):
    """apply_cached configures an operator from a stored choice of its grid edge and
    block size, and leaves it alone when there is none."""
    from eigenfns_gb300 import tune
    monkeypatch.setenv("EIGENFNS_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(tune, "_prefix", lambda device: "gpu|v")

    class Op:
        grid_size, device = 48, "cpu"

        def __init__(self):
            self.calls = []

        def configure(self, passes, subbatch_bytes):
            self.calls.append((passes, subbatch_bytes))

    tune._store("gpu|v|op|G=48|m=16", {"passes": 3, "subbatch_bytes": 12345, "ms": 1.0})
    op = Op()
    assert tune.apply_cached(op, 16) and op.calls == [(3, 12345)]
    assert not tune.apply_cached(op, 32) and op.calls == [(3, 12345)]
    assert not tune.apply_cached(object(), 16)
