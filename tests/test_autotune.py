"""Host logic of the tile-shape autotuner: the margin rule that keeps the
default height on a near tie, and the JSON cache of choices."""
import json

from imex_sflow2d_dev_gb300 import autotune as A


def test_default_height_kept_on_a_near_tie():
    assert A.choose([8, 16, 4], {8: 100.0, 16: 101.9, 4: 99.0}) == 8
    assert A.choose([8, 16, 4], {8: 100.0, 16: 102.1, 4: 99.0}) == 16
    # a later height must beat the best so far, not only the default
    assert A.choose([8, 16, 4], {8: 100.0, 16: 110.0, 4: 111.0}) == 16
    assert A.choose([8, 16, 4], {8: 100.0, 16: 110.0, 4: 113.0}) == 4
    assert A.choose([8], {8: 1.0}) == 8
    assert A.choose([8, 16], {8: 100.0, 16: 100.5}, margin=0.0) == 16


def test_tune_cache_round_trip(tmp_path):
    path = str(tmp_path / "tune.json")
    c = A.TuneCache(path)
    k = A.TuneCache.key("ensemble", 1, 2, 300 * 300, device="GB300")
    assert c.get(k) is None
    c.put(k, 16, {8: 1.0, 16: 1.1})
    d = A.TuneCache(path)
    assert d.get(k) == 16
    with open(path) as f:
        data = json.load(f)
    assert data[k]["score"] == {"8": 1.0, "16": 1.1}
    # the key separates precision, class count and size class
    assert A.TuneCache.key("ensemble", 2, 2, 300 * 300) != A.TuneCache.key("ensemble", 1, 2, 300 * 300)
    assert A.TuneCache.key("ensemble", 1, 3, 300 * 300) != A.TuneCache.key("ensemble", 1, 2, 300 * 300)
