"""Fills the tile-shape table of the autotuner for the benchmark workloads.

    python -m libgpw_gb300.tune_tiles --configs 1 2 4 5 [--out tile_table.json]

Each workload is built with its default size, its task set is timed for every
tile shape on cuda:0 (gpw_taskset_autotune) and the fastest shapes are stored
under the workload's signature.
"""
from __future__ import annotations

import argparse
import time

import torch

from . import autotune, capi, tasks as T


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", type=int, nargs="+", default=[1, 2, 3, 4, 5])
    ap.add_argument("--npairs", type=int, default=None)
    ap.add_argument("--out", default=None, help="table file (default: the package table)")
    args = ap.parse_args(argv)
    dev = torch.device("cuda:0")
    table = autotune.load_table(args.out)
    for c in args.configs:
        wl = T.config(c, npairs=args.npairs)
        plan = capi.Plan(wl.levels)
        ts = capi.TaskSet.from_workload(plan, wl)
        pab = torch.from_numpy(wl.pab).to(dev)
        key = autotune.signature(wl.levels, wl.tasks)
        t0 = time.perf_counter()
        tz, ms = ts.autotune(pab)
        table[key] = {"tile_z": tz, "ms": [[round(float(v), 3) for v in row] for row in ms],
                      "candidates_tz": [8, 4, 0], "workload": wl.name}
        print(f"config {c} {wl.name}: tile z {tz}  ms {ms.tolist()}  ({time.perf_counter() - t0:.1f} s)", flush=True)
        autotune.save_table(table, args.out)
        ts.close()
        plan.close()


if __name__ == "__main__":
    main()
