"""The CPU parts of bench.py: two gloo ranks (one process each, as torchrun
launches them) take the maximum of their per-rank times, the reference arm
prints its line from rank 0 only, and --ref-calibration compares the CPU
baseline's code with the reference's own."""
import contextlib
import io
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(1.5 + rank, world)  # rank 1 is the slower one
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    world, port = 2, _free_port()
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_max_over_ranks_single():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25, 1) == 3.25


def test_reference_arm_prints_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    args = types.SimpleNamespace(config=1, npairs=50, warmup=0, steps=1, cpu_seconds=0.5, gpus=2)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.reference_arm(args)
    assert buf.getvalue() == ""


def test_reference_arm_line(monkeypatch, oracle_lib):
    """Rank 0 of the reference arm: one JSON line with the contract's keys."""
    import json

    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "0")
    args = types.SimpleNamespace(config=1, npairs=50, warmup=0, steps=1, cpu_seconds=0.5, gpus=1)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.reference_arm(args)
    lines = [ln for ln in buf.getvalue().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "pairs/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["workload"] and d["metric"] == bench.METRIC


def test_ref_calibration_line():
    """bench.py --ref-calibration: the CPU baseline's code against the reference's
    own collocate on the same pairs (where the reference library was built)."""
    import json

    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle as O

    if not O.ref_available():
        pytest.skip("reference library not built on this machine")
    args = types.SimpleNamespace(ref_calibration=12, config=1, npairs=None)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.ref_calibration(args)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert set(line["ms_per_pair"]) == {"restatement", "reference", "reference_with_asserts"}
    assert all(v > 0 for v in line["ms_per_pair"].values())
    assert line["restatement_vs_reference_grid_rel_l2"] <= 1e-13
    assert line["config"]["pairs"] == 12
