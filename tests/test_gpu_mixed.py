"""Tiled mixed-precision path (split-fp16 tensor-core contraction, float-float
stages, FP64 grid and matrix-element accumulation) against the FP64 oracle.
Bar: relative grid L2 and max-abs matrix-element error <= 1e-8."""
import numpy as np
import pytest

from golden_io import SET_NAMES, TASK_NAMES, load_set, load_task, rel_l2, task_as_workload
from gpu_util import run_collocate, run_integrate
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu

TOL = 1e-8


@pytest.mark.parametrize("name", SET_NAMES)
def test_mixed_collocate_sets(name, oracle_lib):
    wl, grids_ref, _, _ = load_set(name)
    got = run_collocate(wl, "mixed")
    want = oracle_lib.batch(wl)
    for g, w in zip(got, want):
        assert rel_l2(g, w) <= TOL


@pytest.mark.parametrize("name", SET_NAMES)
def test_mixed_integrate_sets(name, oracle_lib):
    wl, _, V, _ = load_set(name)
    if V is None:
        V = wl.potentials(seed=3)
    got = run_integrate(wl, V, "mixed")
    want = oracle_lib.batch(wl, V=V)
    assert np.abs(got - want).max() <= TOL * max(np.abs(want).max(), 1e-300)


@pytest.mark.parametrize("name", [n for n in TASK_NAMES if "ortho" in n])
def test_mixed_task_files(name):
    d = load_task(name)
    wl = task_as_workload(d)
    got = run_collocate(wl, "mixed")[0]
    assert rel_l2(got, d["grid_ref"]) <= TOL


def test_mixed_config1(oracle_lib):
    wl = T.config(1)
    got = run_collocate(wl, "mixed")[0]
    want = oracle_lib.batch(wl, nthreads=8)[0]
    assert rel_l2(got, want) <= TOL
    V = wl.potentials(seed=2)
    h = run_integrate(wl, V, "mixed")
    hw = oracle_lib.batch(wl, V=V, nthreads=8)
    assert np.abs(h - hw).max() <= TOL * np.abs(hw).max()


def test_mixed_vs_fp64_256(oracle_lib):
    """A sample of the 1M-pair workload's distributions on its 256^3 grid, tau too."""
    for tau in (0, 1):
        wl = T.config(5, npairs=400, seed=77)
        wl.compute_tau = tau
        plan = capi.Plan(wl.levels)
        ts = capi.TaskSet.from_workload(plan, wl)
        g64 = run_collocate(wl, "fp64", ts=ts, plan=plan)[0]
        gmx = run_collocate(wl, "mixed", ts=ts, plan=plan)[0]
        assert rel_l2(gmx, g64) <= TOL
        V = wl.potentials(seed=5)
        h64 = run_integrate(wl, V, "fp64", ts=ts, plan=plan)
        hmx = run_integrate(wl, V, "mixed", ts=ts, plan=plan)
        assert np.abs(hmx - h64).max() <= TOL * np.abs(h64).max()


def test_mixed_multigrid(oracle_lib):
    wl = T.config(2, npairs=300)
    got = run_collocate(wl, "mixed")
    want = oracle_lib.batch(wl, nthreads=8)
    for g, w in zip(got, want):
        assert rel_l2(g, w) <= TOL


@pytest.mark.parametrize("tz", [0, 8])
def test_mixed_general_cell(oracle_lib, tz):
    """General-cell pairs of a mixed call: tz = 0 runs the float-float general
    kernel, tz = 8 the tiled tensor-core kernels (cross factor per point)."""
    wl = T.config(3, npairs=40)
    wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 4.0)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    ts.set_tiles([tz])
    assert ts.tiles() == [tz]
    got = run_collocate(wl, "mixed", ts=ts, plan=plan)[0]
    want = oracle_lib.batch(wl, nthreads=8)[0]
    assert rel_l2(got, want) <= TOL
    V = wl.potentials(seed=6)
    h = run_integrate(wl, V, "mixed", ts=ts, plan=plan)
    hw = oracle_lib.batch(wl, V=V, nthreads=8)
    assert np.abs(h - hw).max() <= TOL * np.abs(hw).max()


@pytest.mark.parametrize("tz", [0, 8])
@pytest.mark.parametrize("name", [n for n in SET_NAMES if n.startswith("general")])
def test_mixed_general_sets_vs_fp64(name, tz):
    """The general-cell golden sets: mixed against the FP64 path of the same task set."""
    wl, _, V, _ = load_set(name)
    if V is None:
        V = wl.potentials(seed=3)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    ts.set_tiles([tz] * len(wl.levels))
    g64 = run_collocate(wl, "fp64", ts=ts, plan=plan)
    gmx = run_collocate(wl, "mixed", ts=ts, plan=plan)
    for a, b in zip(gmx, g64):
        assert rel_l2(a, b) <= TOL
    h64 = run_integrate(wl, V, "fp64", ts=ts, plan=plan)
    hmx = run_integrate(wl, V, "mixed", ts=ts, plan=plan)
    assert np.abs(hmx - h64).max() <= TOL * np.abs(h64).max()


def test_mixed_empty_and_repeat():
    """No pairs: the grid stays zero; a second call accumulates (grid += rho)."""
    wl = T.config(1, npairs=1)
    wl.tasks = wl.tasks[:0]
    assert not np.any(run_collocate(wl, "mixed")[0])
    import torch

    wl = T.config(4, npairs=60)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    dev = torch.device("cuda:0")
    pab = torch.from_numpy(wl.pab).to(dev)
    g = torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)
    ts.collocate(pab, [g], "mixed")
    once = g.clone()
    ts.collocate(pab, [g], "mixed")
    ts.check()
    assert rel_l2(g.cpu().numpy(), 2 * once.cpu().numpy()) <= 1e-15


def test_mixed_cubes_larger_than_the_cell(oracle_lib):
    """Broad Gaussians on a small periodic cell: a cube wraps several times, so a
    tile sees several images of one pair (the multi-image path)."""
    wl = T.synthetic("wrap", 40, 2, (0.2, 0.6), 6.0, [(32, 32, 32)], seed=11)
    got = run_collocate(wl, "mixed")[0]
    want = oracle_lib.batch(wl, nthreads=8)[0]
    assert rel_l2(got, want) <= TOL
    V = wl.potentials(seed=8)
    h = run_integrate(wl, V, "mixed")
    hw = oracle_lib.batch(wl, V=V, nthreads=8)
    assert np.abs(h - hw).max() <= TOL * np.abs(hw).max()


def test_mixed_linearity_and_adjointness_at_scale():
    """Size-independent properties on 20k pairs of the 1M-pair distributions
    (256^3): collocate is linear in the density blocks, and
    <V, collocate(P)> = <integrate(V), P>."""
    import torch

    wl = T.config(5, npairs=20000, seed=99)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    dev = torch.device("cuda:0")
    pab = torch.from_numpy(wl.pab).to(dev)
    shape = T.grid_shape(wl.levels[0])
    g1 = torch.zeros(shape, dtype=torch.float64, device=dev)
    g2 = torch.zeros(shape, dtype=torch.float64, device=dev)
    ts.collocate(pab, [g1], "mixed")
    ts.collocate(-2.0 * pab, [g2], "mixed")  # a power of two scales every slice exactly
    ts.check()
    n1 = torch.linalg.vector_norm(g1)
    assert float(torch.linalg.vector_norm(g2 + 2.0 * g1) / n1) <= 1e-15
    g2.zero_()
    ts.collocate(-3.0 * pab, [g2], "mixed")  # otherwise within the path's precision
    ts.check()
    assert float(torch.linalg.vector_norm(g2 + 3.0 * g1) / n1) <= TOL
    V = torch.from_numpy(wl.potentials(seed=12)[0]).to(dev)
    hab = torch.zeros(ts.pab_extent, dtype=torch.float64, device=dev)
    ts.integrate([V], hab, "mixed")
    ts.check()
    lhs = float(torch.sum(V * g1))
    rhs = float(torch.sum(hab * pab[: ts.pab_extent]))
    assert abs(lhs - rhs) <= TOL * max(abs(lhs), float(torch.sum(torch.abs(V * g1))) * 1e-3)
