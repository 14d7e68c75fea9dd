"""Autotuner host logic (no GPU): cache keys, persistence, selection."""
from miscellaneous_gb300 import autotune


def test_cache_key_buckets_points_by_power_of_two():
    a = autotune.cache_key(512, 512, 2.0, 6, 1 << 20, "GB300")
    b = autotune.cache_key(512, 512, 2.0, 6, (1 << 21) - 1, "GB300")
    c = autotune.cache_key(512, 512, 2.0, 6, 1 << 21, "GB300")
    assert a == b != c
    assert autotune.cache_key(512, 512, 2.0, 6, 0, "x").startswith("512x512|s2|K6|M2^0|")


def test_store_and_load_roundtrip(tmp_path):
    path = str(tmp_path / "sub" / "tune.json")
    assert autotune.load_cache(path) == {}
    autotune.store("k1", {"chunk": 128, "gather_variant": 2}, 0.25, path)
    autotune.store("k2", {"chunk": 256, "gather_variant": 1}, 0.5, path)
    data = autotune.load_cache(path)
    assert data["k1"]["tuning"] == {"chunk": 128, "gather_variant": 2} and data["k2"]["ms"] == 0.5


def test_corrupt_cache_is_ignored(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text("{not json")
    assert autotune.load_cache(str(p)) == {}


def test_pick_takes_fastest_and_keeps_order_on_ties():
    res = [({"a": 1}, 2.0), ({"a": 2}, 1.0), ({"a": 3}, 1.0)]
    assert autotune.pick(res) == ({"a": 2}, 1.0)
