"""Autotuner cache of the batched renderer: keys by GPU name and workload
class, reuse without re-timing, atomic rewrite, tolerance of a damaged file
(host logic only; the timing itself runs in the GPU batch tests)."""
from __future__ import annotations

import json

from zillumgl_gb300.scene import autotune_cache_key, cached_autotune


def test_key_rounds_the_workload_class():
    a = autotune_cache_key("GB300", [(1000, 128 * 128, 4), (500000, 1024 * 1024, 64)])
    b = autotune_cache_key("GB300", [(1100, 128 * 128, 4), (480000, 1000 * 1040, 64)])
    c = autotune_cache_key("B200", [(1000, 128 * 128, 4), (500000, 1024 * 1024, 64)])
    d = autotune_cache_key("GB300", [(1000, 128 * 128, 4)] * 64)
    assert a == b and a != c and a != d
    assert a.startswith("GB300|requests 2^1|")


def test_cache_reuses_and_stores(tmp_path):
    path = tmp_path / "tune.json"
    calls, applied = [], []
    cfg = {"block_size": 128, "queue_capacity": 32, "regen_threshold": 16, "schedule": 1, "scratch_mib": 0}

    def tune():
        calls.append(1)
        return dict(cfg)

    assert cached_autotune(path, "k1", tune, applied.append) == cfg
    assert len(calls) == 1 and applied == []
    assert json.loads(path.read_text()) == {"k1": cfg}
    # same key: no timing, the stored configuration is applied
    assert cached_autotune(path, "k1", tune, applied.append) == cfg
    assert len(calls) == 1 and applied == [cfg]
    # another key: timed and added beside the first
    other = dict(cfg, schedule=2)
    assert cached_autotune(path, "k2", lambda: dict(other), applied.append) == other
    assert set(json.loads(path.read_text())) == {"k1", "k2"}
    assert not list(tmp_path.glob("*.tmp*"))


def test_damaged_cache_counts_as_empty(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    cfg = {"block_size": 64, "queue_capacity": 8, "regen_threshold": 1, "schedule": 2, "scratch_mib": 0}
    assert cached_autotune(path, "k", lambda: dict(cfg), lambda c: None) == cfg
    assert json.loads(path.read_text()) == {"k": cfg}
