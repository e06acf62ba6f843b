"""Tile-shape table of the autotuner: workload signature and JSON round trip
(host logic only; the timing itself is in test_gpu_tiles.py)."""
import json

from libgpw_gb300 import autotune, tasks as T


def test_signature_stable_and_discriminating():
    wl = T.config(1, npairs=200)
    k1 = autotune.signature(wl.levels, wl.tasks)
    assert k1 == autotune.signature(wl.levels, wl.tasks.copy())
    wl2 = T.config(2, npairs=200)
    assert autotune.signature(wl2.levels, wl2.tasks) != k1
    assert k1.count("|") == 3 and "64x64x64" in k1


def test_table_round_trip(tmp_path):
    p = str(tmp_path / "t.json")
    assert autotune.load_table(p) == {}
    autotune.save_table({"k": {"tile_z": [8]}}, p)
    assert json.load(open(p)) == {"k": {"tile_z": [8]}}
    assert autotune.load_table(p)["k"]["tile_z"] == [8]


def test_shipped_table_is_valid():
    tab = autotune.load_table(autotune.DEFAULT_TABLE)
    for key, ent in tab.items():
        assert all(tz in (0, 4, 8) for tz in ent["tile_z"]), key


def test_shipped_table_covers_benchmark_workloads():
    """The table shipped with the package applies to the five benchmark
    workloads (a change of the signature would silently drop the tuned shapes)."""
    tab = autotune.load_table(autotune.DEFAULT_TABLE)
    for c in (1, 2, 3, 4, 5):
        wl = T.config(c)
        key = autotune.signature(wl.levels, wl.tasks)
        assert key in tab, (c, key)
        assert len(tab[key]["tile_z"]) == len(wl.levels)
