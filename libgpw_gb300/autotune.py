"""Tile-shape autotuner of the mixed-precision path, with a JSON table.

The tiled kernels cut every orthorhombic grid level into tiles of 32 x (128/tz)
x tz points; tz (4 or 8) trades the number of tiles a cube touches against
the per-tile work of a pair.  On general-cell levels tz = 0 (no tiles: the
float-float kernel, one CTA per pair) is a third candidate.  ``gpw_taskset_autotune`` times one collocate +
integrate per candidate and level on the device.  This module keys the result
by a workload signature (grid levels and the task set's size, angular momentum
and exponent spread) and keeps it in a JSON table, so a task set of the same
kind reuses the shapes without timing again.

Table file: ``$GPW_TILE_TABLE`` if set, else ``tile_table.json`` beside this
module (shipped with the shapes measured for the benchmark workloads).
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_TABLE = os.path.join(HERE, "tile_table.json")


def table_path() -> str:
    return os.environ.get("GPW_TILE_TABLE", DEFAULT_TABLE)


def load_table(path: str | None = None) -> dict:
    path = path or table_path()
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def save_table(table: dict, path: str | None = None) -> None:
    path = path or table_path()
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
        f.write("\n")
    os.replace(tmp, path)


def signature(levels, tasks) -> str:
    """Key of a workload: per level the grid size and x spacing; the pair count
    (power of two), the largest la/lb and the decade range of zeta_a + zeta_b."""
    parts = []
    for lv in levels:
        lv = np.asarray(lv).reshape(())
        ng = "x".join(str(int(v)) for v in lv["npts"])
        h = float(np.asarray(lv["dh"]).reshape(3, 3)[0, 0])
        parts.append(f"{ng}@{h:.3g}")
    n = int(tasks.shape[0])
    lmax = int(max(tasks["la_max"].max(), tasks["lb_max"].max())) if n else 0
    zp = np.asarray(tasks["zeta"], dtype=np.float64) + np.asarray(tasks["zetb"], dtype=np.float64)
    z0, z1 = (math.floor(math.log10(zp.min())), math.ceil(math.log10(zp.max()))) if n else (0, 0)
    return f"{'+'.join(parts)}|n2^{max(n, 1).bit_length() - 1}|l{lmax}|z1e{z0}..1e{z1}"


def apply(ts, pab, tasks=None, path: str | None = None, tune: bool = True) -> tuple:
    """Sets the task set's tile shapes from the table, or times them (when tune)
    and records the result.  Returns (tile z per level, "table" | "tuned" | "default")."""
    key = signature(ts.plan.levels, ts.tasks if tasks is None else tasks)
    table = load_table(path)
    ent = table.get(key)
    if ent is not None and len(ent["tile_z"]) == len(ts.plan.levels):
        ts.set_tiles(ent["tile_z"])
        return ts.tiles(), "table"
    if not tune:
        return ts.tiles(), "default"
    tz, ms = ts.autotune(pab)
    table[key] = {"tile_z": tz, "ms": [[round(float(v), 3) for v in row] for row in ms], "candidates_tz": [8, 4, 0]}
    try:
        save_table(table, path)
    except OSError:
        pass  # a read-only install still uses the tuned shapes
    return tz, "tuned"
