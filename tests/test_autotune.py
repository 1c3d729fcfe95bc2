"""Host logic of the batched-trace autotuner: cache keys, candidate choice
and the JSON cache (no GPU: the timer is a stand-in)."""
import json

import pytest

from rtgpu import autotune as A


def test_keys_bucket_similar_batches():
    k1 = A.size_bucket(256, 9_600_000, 256, 256)
    k2 = A.size_bucket(256, 9_000_000, 256, 256)
    k3 = A.size_bucket(256, 20_000_000, 256, 256)
    assert k1 == k2 != k3
    assert A.size_bucket(128, 9_600_000, 256, 256) != k1
    assert A.gpu_key("NVIDIA GB300", (10, 3), 152) == "NVIDIA GB300:sm103:152sm"
    assert "|" not in A.gpu_key("a|b", (10, 3), 1)


def test_candidates_are_valid_shapes():
    c = A.candidates()
    assert len(c) == len(A.THREADS) * len(A.GRABS) * len(A.ORDERS)
    assert all(x["threads"] in (64, 128, 256) and 1 <= x["grab"] <= 16 and x["order"] in (0, 1) for x in c)


def test_pick_fastest_and_ties_keep_first():
    a, b, c = ({"threads": t, "blocks_per_sm": 0, "grab": 1, "order": 0} for t in (64, 128, 256))
    assert A.pick([(a, 3.0), (b, 1.0), (c, 2.0)])["threads"] == 128
    assert A.pick([(a, 1.0), (b, 1.0)])["threads"] == 64
    with pytest.raises(ValueError):
        A.pick([])


def test_tune_measures_once_then_uses_cache(tmp_path):
    path = tmp_path / "t.json"
    calls = []

    def timer(cfg):
        calls.append(cfg)
        return 10.0 - cfg["grab"] + (0.5 if cfg["order"] else 0.0) + cfg["threads"] / 1000.0

    best = A.tune("gpu|bucket", timer, A.TuneCache(path))
    assert best["grab"] == 8 and best["order"] == 0 and best["threads"] == 64
    n = len(calls)
    assert n == len(A.candidates())
    again = A.tune("gpu|bucket", timer, A.TuneCache(path))  # a fresh cache object reads the file
    assert len(calls) == n and again == best
    forced = A.tune("gpu|bucket", timer, A.TuneCache(path), force=True)
    assert len(calls) == 2 * n and forced["grab"] == 8
    data = json.loads(path.read_text())
    assert data["gpu|bucket"]["grab"] == 8


def test_damaged_or_invalid_cache_is_ignored(tmp_path):
    path = tmp_path / "t.json"
    path.write_text("{not json")
    assert A.TuneCache(path).entries == {}
    path.write_text(json.dumps({"k": {"threads": 96, "grab": 1, "order": 0}, "j": [1, 2]}))
    assert A.TuneCache(path).entries == {}


def test_cache_path_from_environment(monkeypatch, tmp_path):
    monkeypatch.setenv("RTGPU_TUNE_CACHE", str(tmp_path / "x.json"))
    assert A.default_cache_path() == tmp_path / "x.json"
