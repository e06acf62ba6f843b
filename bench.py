#!/usr/bin/env python
"""Benchmark: collocate + integrate pairs/s on one GB300.

A step is one collocate (density blocks -> grid) plus one integrate (potential
grid -> matrix elements) over every pair of the workload, through the C ABI.
Default workload: 1,000,000 pairs, la,lb in {0..4}, exponents log-uniform in
[0.05, 200], 30-bohr cubic cell, 256^3 grid (seeded synthetic inputs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config 1..5] [--precision mixed|fp64] [--npairs n]

--impl reference times the CPU implementation of the same path on the host
cores (the oracle port of the reference's FP64 collocate; the reference's own
library where it was built) on a bounded sample of the same workload.
Multi-GPU runs are independent replicas (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "collocate+integrate pairs/s on 1 GB300: batched FP32/3xTF32 vs plain FP64, ≤1e-8 err"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=5)
    ap.add_argument("--npairs", type=int, default=None)
    ap.add_argument("--precision", default="auto", choices=["auto", "mixed", "fp64"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-error", action="store_true", help="skip the FP64 error check of the mixed path")
    ap.add_argument("--no-graph", action="store_true", help="launch the step directly instead of replaying a CUDA graph")
    ap.add_argument("--no-tune", action="store_true",
                    help="tile shapes from the autotuner's table or the default, never timed here")
    ap.add_argument("--dropin", type=int, default=0, metavar="CALLS",
                    help="instead: time CALLS calls of the single-pair drop-in entry on each of the reference's "
                         "task fixtures (host grid in and out, as the reference's replay calls it)")
    ap.add_argument("--ref-calibration", type=int, default=0, metavar="PAIRS",
                    help="instead: where the reference's library was built here (oracle/_ref), time one-core "
                         "collocation of PAIRS random pairs of the workload with the CPU baseline's code and with "
                         "the reference's own code, built as its Makefile builds it and with its asserts")
    return ap.parse_args()


def ref_calibration(args) -> None:
    """The CPU baseline's code (the C restatement) against the reference's own
    grid_collocate_pgf_product_rspace on the same pairs, grids and core: how far
    the baseline's speed stands from the reference's.  Needs the reference
    library built from its sources (oracle/_ref), which exists only where the
    reference tree does; prints one JSON line."""
    from libgpw_gb300 import tasks as T
    from oracle import oracle as O

    O.build()
    need = [os.path.join(ROOT, "oracle", "_ref", f) for f in ("libgpwref.so", "libgpwref_ndebug.so")]
    if not all(os.path.exists(f) for f in need):
        print(json.dumps({"metric": "CPU collocate ms per pair", "unavailable": "reference library not built here"}))
        return
    wl = T.config(args.config, npairs=args.npairs)
    idx = np.random.default_rng(1).choice(wl.ntasks, size=min(args.ref_calibration, wl.ntasks), replace=False)
    tasks = [O.task_dict(wl, int(i)) for i in idx]
    kinds = {"restatement": False, "reference": "ndebug", "reference_with_asserts": True}
    grids = {k: [np.zeros(T.grid_shape(g)) for g in wl.levels] for k in kinds}
    levels = [int(wl.tasks[int(i)]["level"]) for i in idx]

    def run(kind):
        for t, lvl in zip(tasks, levels):
            if O.collocate(t, grids[kind][lvl], use_ref=kinds[kind]):
                raise RuntimeError(f"{kind}: collocate failed")

    ms = {k: [] for k in kinds}
    for k in kinds:  # warm-up pass (page faults of the grids)
        run(k)
    for _ in range(2):
        for k in kinds:
            t0 = time.perf_counter()
            run(k)
            ms[k].append((time.perf_counter() - t0) / len(tasks) * 1e3)
    ref_grids = grids["reference"]
    err = max(float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
              for a, b in zip(grids["restatement"], ref_grids))
    print(json.dumps({"metric": "CPU collocate ms per pair", "config": {"workload": wl.name, "pairs": len(tasks)},
                      "cores": 1, "ms_per_pair": {k: min(v) for k, v in ms.items()},
                      "restatement_vs_reference_grid_rel_l2": err,
                      "reference_build": "grid_base_ref_c.cc with -O2 -DNDEBUG, as the reference's Makefile "
                                         "builds its library (without its x86 -mavx2 and MKL flags); "
                                         "reference_with_asserts: the build the parity fixtures use"}))


def dropin_bench(calls: int) -> None:
    """Microseconds per call of gpw_collocate_pgf_product_rspace (the drop-in for the
    reference's grid_collocate_pgf_product_rspace) on the reference's four task
    fixtures, against the CPU restatement of the same call (oracle, one thread)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from golden_io import TASK_NAMES, load_task
    from libgpw_gb300 import capi
    from oracle import oracle as O

    out = {}
    for name in TASK_NAMES:
        d = load_task(name)
        grid = np.zeros((int(d["ngrid"][2]), int(d["ngrid"][1]), int(d["ngrid"][0])))
        for _ in range(20):
            capi.collocate_pgf_product_rspace(d, grid)
        t0 = time.perf_counter()
        for _ in range(calls):
            capi.collocate_pgf_product_rspace(d, grid)
        gpu_us = (time.perf_counter() - t0) / calls * 1e6
        g2 = np.zeros_like(grid)
        n_cpu = max(10, min(calls, 2000))
        t0 = time.perf_counter()
        for _ in range(n_cpu):
            O.collocate(d, g2)
        cpu_us = (time.perf_counter() - t0) / n_cpu * 1e6
        out[name] = {"gpu_us_per_call": gpu_us, "cpu_oracle_us_per_call": cpu_us, "calls": calls,
                     "grid": list(grid.shape)}
    print(json.dumps({"metric": "drop-in single-pair collocate, us per call", "tasks": out}))


# ----------------------------------------------------------------------------
class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict:
        rows = []
        for ln in (self.out or "").splitlines():
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                rows.append((float(p[1]), float(p[2]), p[5], p[6], p[7], p[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = sorted(r[0] for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[2:]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": rows[0][1], "reasons": sorted(reasons),
                "samples": len(rows)}


# ----------------------------------------------------------------------------
# DRAM bytes (read + write) of one launch of each tiled kernel on the 1M-pair
# workload (256^3, tile 32 x 16 x 8, 79,272,268 (tile, pair) items), from a
# single-pass ncu capture of dram__bytes_read.sum + dram__bytes_write.sum with
# gpu__time_duration.sum.  Other workloads scale it by their item count (an
# estimate: the share of a pair's record and coefficients served by L2 depends
# on the workload).
TRAFFIC_1M = {"k_collocate_tiled": (9.028e9 + 0.193e9, 79_272_268),
              "k_integrate_tiled": (9.510e9 + 2.966e9, 79_272_268)}


def algorithmic_flops(wl) -> tuple:
    """Collocate flops of the dense three-stage contraction per pair,
    2L*nx*ny*nz + 2L^2*nz*ny + 2L^3*nz, with n the cube extents of the library's
    cube rule (box of the general cell); integrate is symmetric.  Also returns
    the cube points."""
    from libgpw_gb300 import tasks as T

    t = wl.tasks
    L = (t["la_max"] + t["lb_max"] + 1 + 2 * (wl.compute_tau != 0)).astype(np.float64)
    n = np.zeros((t.shape[0], 3))
    for lev_i, g in enumerate(wl.levels):
        m = t["level"] == lev_i
        if g["ortho"]:
            for d in range(3):
                n[m, d] = 2 * np.floor(t["radius"][m] / g["dh"][d][d]) + 2
        else:
            inv = np.abs(np.asarray(g["dh_inv"]))
            span = t["radius"][m][:, None] * inv.sum(axis=0)[None, :]
            n[m] = 2 * np.ceil(span) + 1
    nz, ny, nx = n[:, 2], n[:, 1], n[:, 0]
    fl = 2 * L * nx * ny * nz + 2 * L ** 2 * nz * ny + 2 * L ** 3 * nz
    return float(fl.sum()), float((nx * ny * nz).sum())


def subsample(wl, idx):
    """A Workload holding the pairs idx with a compact density-block buffer."""
    from libgpw_gb300 import tasks as T

    t = wl.tasks[idx].copy()
    nsa = (t["maxco"]).astype(np.int64)
    nsb = ((t["lb_max"] + 1) * (t["lb_max"] + 2) // 2).astype(np.int64)
    blk = nsa * nsb
    off = np.zeros(len(idx), np.int64)
    off[1:] = np.cumsum(blk[:-1])
    pab = np.concatenate([wl.pab[int(o): int(o) + int(b)] for o, b in zip(wl.tasks["pab_offset"][idx], blk)])
    t["pab_offset"] = off
    return T.Workload(wl.name + "_sample", t, wl.levels, pab, compute_tau=wl.compute_tau)


def cpu_baseline(wl, seconds: float, seed: int = 0) -> dict:
    """The CPU FP64 path (oracle port) on a random pair sample, all host threads."""
    from oracle import oracle as O

    O.build()
    kind = "port"
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    V = None
    n = 16
    elapsed = 0.0
    while True:
        idx = np.sort(rng.choice(wl.ntasks, size=min(n, wl.ntasks), replace=False))
        sw = subsample(wl, idx)
        if V is None:
            V = [np.random.default_rng(1).uniform(-1, 1, size=g.shape) for g in
                 [np.zeros((int(l["ngrid"][2]), int(l["ngrid"][1]), int(l["ngrid"][0])), dtype=np.int8)
                  for l in wl.levels]]
        t0 = time.perf_counter()
        O.batch(sw, nthreads=threads)
        O.batch(sw, V=V, nthreads=threads)
        elapsed = time.perf_counter() - t0
        if elapsed >= seconds * 0.4 or n >= wl.ntasks:
            break
        n = int(min(wl.ntasks, max(2 * n, n * seconds * 0.6 / max(elapsed, 1e-3))))
    # the same on one core, on a sample of about the same duration
    idx1 = idx[: max(4, len(idx) // threads)]
    sw1 = subsample(wl, idx1)
    t0 = time.perf_counter()
    O.batch(sw1, nthreads=1)
    O.batch(sw1, V=V, nthreads=1)
    el1 = time.perf_counter() - t0
    return {"value": len(idx) / elapsed, "unit": "pairs/s", "cores": threads, "kind": kind,
            "value_1core": len(idx1) / el1,
            "sample": f"{len(idx)} random pairs of the {wl.ntasks}-pair workload, collocate+integrate FP64, "
                      f"{threads} threads with private grids, {elapsed:.1f} s; 1 core: the first {len(idx1)} "
                      f"of them, {el1:.1f} s"}


def fp64_gemm_rate(dev) -> float:
    """FP64 GEMM rate of this GPU (cuBLAS through torch.matmul, 4096^3, best of
    5 after one warm-up), TFLOP/s: the rate an FP64 implementation of the
    contraction could reach at best."""
    import torch

    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    c = a @ b
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The maximum over the ranks of a per-rank time (the rank itself on one rank)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from libgpw_gb300 import tasks as T

    wl = T.config(args.config, npairs=args.npairs)
    vals = []
    base = None
    for k in range(args.warmup + args.steps):
        b = cpu_baseline(wl, max(2.0, args.cpu_seconds / 2), seed=k)
        if k >= args.warmup:
            vals.append(b["value"])
            base = b
    value = float(np.median(vals))
    base["value"] = value
    line = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wl.ntasks / value,
            "ms_per_step_basis": "extrapolated: the whole workload at the pair rate of the timed sample "
                                 "(each step times a bounded random sample of the pairs, cpu_baseline.sample)",
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference", "config": {"workload": wl.name, "npairs": wl.ntasks, "precision": "fp64-cpu"},
            "cpu_baseline": base, "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ----------------------------------------------------------------------------
def main():
    args = parse()
    if args.ref_calibration:
        ref_calibration(args)
        return
    if args.dropin:
        dropin_bench(args.dropin)
        return
    if args.impl == "reference":
        reference_arm(args)
        return
    import torch

    from libgpw_gb300 import capi, tasks as T

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    wl = T.config(args.config, npairs=args.npairs)
    t0 = time.perf_counter()
    plan = capi.Plan(wl.levels, device=local)
    ts = capi.TaskSet.from_workload(plan, wl)
    plan_s = time.perf_counter() - t0
    # a geometry step of the same pairs: centres moved (device set-up and re-binning,
    # gpw_taskset_update_geometry), then moved back to the benchmark's geometry; the
    # second update is the one reported (the first also allocates its buffers)
    geo_ms = []
    if wl.ntasks > 0:
        rng = np.random.default_rng(7)
        ra_h = np.ascontiguousarray(wl.tasks["ra"])
        moved_ra = torch.from_numpy(ra_h + rng.normal(0.0, 0.1, size=ra_h.shape)).to(dev)
        orig_ra = torch.from_numpy(ra_h.copy()).to(dev)
        for r in (moved_ra, orig_ra):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            ts.update_geometry(ra=r)
            geo_ms.append((time.perf_counter() - t1) * 1e3)
        del moved_ra, orig_ra
    prec = args.precision
    pab = torch.from_numpy(wl.pab).to(dev)
    grids = [torch.zeros(T.grid_shape(g), dtype=torch.float64, device=dev) for g in wl.levels]
    Vh = wl.potentials(seed=1)
    V = [torch.from_numpy(v).to(dev) for v in Vh]
    hab = torch.zeros(ts.pab_extent, dtype=torch.float64, device=dev)
    if prec == "auto":
        prec = "mixed"  # the path the metric is quoted on; a failure is an error, not a fallback
    # tile shapes of the mixed path: the autotuner's table, else timed once here (before any timed region)
    tiles, tile_src, tune_s = None, None, 0.0
    if prec == "mixed":
        from libgpw_gb300 import autotune

        t0 = time.perf_counter()
        tiles, tile_src = autotune.apply(ts, pab, tasks=wl.tasks, tune=not args.no_tune)
        tune_s = time.perf_counter() - t0
    items, units = ts.bins()  # of the tile shapes in use
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    def step():
        ts.collocate(pab, grids, prec)
        ts.integrate(V, hab, prec)

    for _ in range(args.warmup):
        step()
    ts.check()
    torch.cuda.synchronize()
    # the whole step as one CUDA graph (collocate + integrate: set-up, tiled
    # kernels, queue resets, back-transform)
    graph = None
    if not args.no_graph:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream().wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step()
        graph.replay()
        torch.cuda.synchronize()
    ts.stats()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            starts[k].record()
            if graph is not None:
                graph.replay()
            else:
                step()
            ends[k].record()
        torch.cuda.synchronize()
    barrier()
    ts.check()
    ms = float(np.median([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    # per-kernel device time of the same step, measured on one direct step
    ts.stats()
    ts.profile(True)
    flush.zero_()
    ts.collocate(pab, grids, prec)
    torch.cuda.synchronize()
    coll_ms, coll_launches, n_kernels = ts.stats()
    ts.integrate(V, hab, prec)
    torch.cuda.synchronize()
    int_ms, int_launches, n_kernels_i = ts.stats()
    ts.profile(False)
    n_kernels += n_kernels_i
    kern_ms = (coll_ms + int_ms) * args.steps
    kern_launches = (coll_launches + int_launches) * args.steps
    ms = max_over_ranks(ms, world, dev)
    value = world * wl.ntasks / (ms * 1e-3)

    # end to end through the host-buffer C ABI calls (pinned host memory, copies inside the timed region),
    # right after the device-timed steps and before the long FP64 error check
    e2e = None
    if not args.no_e2e:
        pab_h = torch.from_numpy(wl.pab).pin_memory().numpy()
        grids_h = [torch.zeros(T.grid_shape(g), dtype=torch.float64).pin_memory().numpy() for g in wl.levels]
        V_h = [torch.from_numpy(v).pin_memory().numpy() for v in Vh]
        hab_h = torch.zeros(ts.pab_extent, dtype=torch.float64).pin_memory().numpy()
        ts.collocate_host(pab_h, grids_h, prec)
        ts.integrate_host(V_h, hab_h, prec)
        ne = max(2, min(args.steps, 5))
        barrier()
        with Clocks(local) as clk_e2e:
            t0 = time.perf_counter()
            for _ in range(ne):
                ts.collocate_host(pab_h, grids_h, prec)
                ts.integrate_host(V_h, hab_h, prec)
            torch.cuda.synchronize()
            barrier()
            e2e_s = max_over_ranks((time.perf_counter() - t0) / ne, world, dev)
        gbytes = sum(g.nbytes for g in grids_h)
        e2e = {"value": world * wl.ntasks / e2e_s, "unit": "pairs/s",
               "h2d_bytes_per_step": int(pab_h.nbytes + gbytes + sum(v.nbytes for v in V_h) + hab_h.nbytes),
               "d2h_bytes_per_step": int(gbytes + hab_h.nbytes), "ms_per_step": e2e_s * 1e3,
               "clocks": clk_e2e.summary()}
        del pab_h, grids_h, V_h, hab_h


    # error of this precision against the plain FP64 path (relative grid L2, max-abs matrix element)
    err = {}
    if not args.no_error:
        g1 = [torch.zeros_like(g) for g in grids]
        g2 = [torch.zeros_like(g) for g in grids]
        h1 = torch.zeros_like(hab)
        h2 = torch.zeros_like(hab)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ts.collocate(pab, g1, prec)
        ts.integrate(V, h1, prec)
        torch.cuda.synchronize()
        ev[0].record()
        ts.collocate(pab, g2, "fp64")
        ts.integrate(V, h2, "fp64")
        ev[1].record()
        torch.cuda.synchronize()
        fp64_ms = ev[0].elapsed_time(ev[1])
        num = sum(float(torch.sum((a - b) ** 2)) for a, b in zip(g1, g2))
        den = sum(float(torch.sum(b ** 2)) for b in g2)
        err = {"grid_rel_l2_vs_fp64": (num / den) ** 0.5 if den > 0 else 0.0,
               "hab_max_abs_vs_fp64": float(torch.max(torch.abs(h1 - h2))),
               "hab_max_abs_scale": float(torch.max(torch.abs(h2))),
               "fp64_path": {"value": wl.ntasks / (fp64_ms * 1e-3), "unit": "pairs/s", "ms_per_step": fp64_ms,
                             "timing": "one collocate+integrate of the plain FP64 kernels, CUDA events"}}
        del g1, g2, h1, h2
        err["fp64_gemm_tflops"] = fp64_gemm_rate(dev)

    if rank != 0:
        return
    flops, points = algorithmic_flops(wl)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    # dominant kernel: the slower of the two contraction kernels; its algorithmic
    # flops (the collocate count, integrate is symmetric) over its average launch
    # time on the launching stream
    dom, dom_ms, dom_n = ("integrate", int_ms, int_launches) if int_ms >= coll_ms else ("collocate", coll_ms, coll_launches)
    per_launch_flops = flops / max(dom_n, 1)
    avg_launch_ms = dom_ms / max(dom_n, 1)
    achieved_tf = per_launch_flops / (avg_launch_ms * 1e-3) / 1e12 if avg_launch_ms > 0 else 0.0
    if prec == "mixed":
        peak = peaks.get("bf16_tflops_sustained") or 1700.0
        kname = f"k_{dom}_tiled"
        roof = {"bound": "tensor", "kernel": kname, "achieved": achieved_tf, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved_tf / peak,
                "traffic": TRAFFIC_1M[kname][0] * items / TRAFFIC_1M[kname][1],
                "traffic_basis": "measured on the 1M-pair workload (one-pass ncu capture), scaled by this "
                                 "launch's (tile, pair) items",
                "items_per_launch": items,
                "peak_source": "bf16 sustained, MEASURED_PEAKS.json (of measured)",
                "limiter": "FP32/integer instruction issue of the float-float stages, not the tensor pipe "
                           "(tensor pipe active ~5%, issue slots busy 62% collocate / 52% integrate in the ncu captures)"}
    else:
        hbm = peaks.get("hbm_gbs") or 6800.0
        gbytes_alg = 16.0 * points  # FP64 read+write per cube point (no reuse)
        per_launch_b = 2 * gbytes_alg / max(kern_launches / args.steps, 1)
        ach = per_launch_b / (avg_launch_ms * 1e-3) / 1e9 if avg_launch_ms > 0 else 0.0
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": None, "peak_source": "hbm_gbs, MEASURED_PEAKS.json (of measured)"}
    roof["kernel_ms_per_step"] = kern_ms / args.steps
    roof["collocate_ms_per_launch"] = coll_ms / max(coll_launches, 1)
    roof["integrate_ms_per_launch"] = int_ms / max(int_launches, 1)
    roof["kernel_launches_per_step"] = kern_launches / args.steps
    roof["algorithmic_tflop_per_step"] = 2 * flops / 1e12
    # speed-up over the plain FP64 GPU path, and over the time an FP64 code would
    # need at this GPU's FP64 GEMM rate for the same algorithmic flops
    vs_fp64 = None
    if err.get("fp64_path"):
        bound_ms = 2 * flops / (err["fp64_gemm_tflops"] * 1e12) * 1e3
        vs_fp64 = {"fp64_gpu_path": err["fp64_path"]["ms_per_step"] / ms,
                   "fp64_path_tflops": 2 * flops / (err["fp64_path"]["ms_per_step"] * 1e-3) / 1e12,
                   "fp64_path_frac_of_fp64_gemm": 2 * flops / (err["fp64_path"]["ms_per_step"] * 1e-3) / 1e12
                   / err["fp64_gemm_tflops"],
                   "fp64_gemm_rate_bound_ms": bound_ms, "fp64_gemm_rate_bound": bound_ms / ms,
                   "note": "ratios of step times: plain FP64 GPU path / this step, and the algorithmic "
                           "flops at the measured FP64 GEMM rate / this step"}
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(wl, args.cpu_seconds)
    lv = wl.levels[0]
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp16 fixed-point slices (tcgen05, exact f32 sums) + float-float + f64 grid" if prec == "mixed" else "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": wl.name, "npairs": wl.ntasks,
                   "grids": ["x".join(str(int(v)) for v in l["ngrid"]) for l in wl.levels],
                   "precision": prec, "compute_tau": wl.compute_tau,
                   "l2": "grid and potential exceed L2; a 512 MB buffer is written between timed steps",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "launch": "CUDA graph replay of the step" if graph is not None else "direct launches",
                   "plan_seconds": plan_s, "items": items, "units": units, "geometry_update_ms": geo_ms[-1] if geo_ms else None, "tile_z": tiles, "tile_source": tile_src, "tune_seconds": tune_s},
        "gpu_launches": int(n_kernels * args.steps),
        "roofline": roof, "error": err, "vs_fp64": vs_fp64, "clocks": clk.summary(), "cpu_baseline": cpu,
        "e2e": e2e,
        "algorithmic_cube_points": points,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
