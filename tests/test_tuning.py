"""The autotuner's cache layer and configuration table (CPU): file format,
keys, device matching, the setter calls, and the library's variant table."""
import json

from conftest import PKG  # noqa: F401  (puts the package on the path)


def test_cache_round_trip_and_keys(tmp_path):
    from bsfit import tuning as T
    p = tmp_path / "tune.json"
    c = T.load_cache(p)  # missing file: empty cache
    assert c == {"format": T.FORMAT, "devices": {}}
    choice = {"variant": 1, "warps_per_block": 4, "min_blocks": 5, "ms": 2.5, "candidates": {}}
    T.record(c, "NVIDIA GB300", 6, 13, choice)
    T.record(c, "NVIDIA GB300", 7, 15, dict(choice, variant=2, min_blocks=5))
    T.record(c, "other GPU", 6, 13, dict(choice, variant=0))
    T.save_cache(p, c)
    raw = json.loads(p.read_text())
    assert raw["format"] == "bsfit-tune-1"
    assert set(raw["devices"]["NVIDIA GB300"]) == {"6:13", "7:15"}
    assert "candidates" not in raw["devices"]["NVIDIA GB300"]["6:13"]
    c2 = T.load_cache(p)
    assert T.lookup(c2, "NVIDIA GB300", 7, 15)["variant"] == 2
    assert T.lookup(c2, "NVIDIA GB300", 8, 17) is None
    assert T.lookup(c2, "other GPU", 6, 13)["variant"] == 0


def test_apply_cache_sets_this_device_only(tmp_path):
    from bsfit import tuning as T
    c = T.empty_cache()
    T.record(c, "dev A", 6, 11, {"variant": 2, "warps_per_block": 2, "min_blocks": 4, "ms": 1.0})
    T.record(c, "dev A", 8, 17, {"variant": 1, "warps_per_block": 1, "min_blocks": 2, "ms": 9.0})
    T.record(c, "dev B", 6, 13, {"variant": 1, "warps_per_block": 4, "min_blocks": 5, "ms": 1.0})
    c["devices"]["dev A"]["bad key"] = {"variant": 0}
    calls = []
    n = T.apply_cache(c, "dev A", setter=lambda *a: calls.append(a))
    assert n == 2 and sorted(calls) == [(6, 11, 2, 2), (8, 17, 1, 1)]
    p = tmp_path / "t.json"
    T.save_cache(p, c)
    calls.clear()
    assert T.apply_cache(str(p), "dev B", setter=lambda *a: calls.append(a)) == 1
    assert calls == [(6, 13, 1, 4)]
    assert T.apply_cache(str(p), "dev C", setter=lambda *a: calls.append(a)) == 0


def test_corrupt_or_foreign_cache_is_empty(tmp_path):
    from bsfit import tuning as T
    p = tmp_path / "t.json"
    p.write_text("{not json")
    assert T.load_cache(p)["devices"] == {}
    p.write_text(json.dumps({"format": "something else", "devices": {"x": {}}}))
    assert T.load_cache(p)["devices"] == {}


def test_variant_table():
    """Variant 0 is each fit type's default register budget (6 resident
    4-warp blocks for 3D, 4 for 4D, 3 for 5D); the others are alternatives
    (fit type 8's variants 2 and 3 stage the 5D gathers through shared memory;
    fit type 6's variants 3 to 7 fit two ROIs per warp: 3 to 5 one per
    half-warp, 6 and 7 both in paired operations on all lanes)."""
    from bsfit import tuning as T
    assert [T.num_variants(f) for f in (5, 6, 7, 8)] == [0, 8, 3, 4]
    assert [T.min_blocks(6, v) for v in range(8)] == [6, 5, 4, 6, 5, 4, 4, 3]
    assert [T.rois_per_warp(6, v) for v in range(8)] == [1, 1, 1, 2, 2, 2, 2, 2]
    assert [T.rois_per_warp(f, 0) for f in (7, 8)] == [1, 1] and T.rois_per_warp(6, 8) == 0
    assert [T.min_blocks(7, v) for v in range(3)] == [4, 3, 5]
    assert [T.min_blocks(8, v) for v in range(4)] == [3, 2, 2, 1]
    assert T.min_blocks(8, 4) == 0 and T.min_blocks(6, -1) == 0
