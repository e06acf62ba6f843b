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


def test_mixed_general_cell(oracle_lib):
    """General-cell pairs of a mixed call run on the float-float general kernel
    (the reference's row i-ranges, float-float polynomial and exponential)."""
    wl = T.config(3, npairs=40)
    wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 4.0)
    got = run_collocate(wl, "mixed")[0]
    want = oracle_lib.batch(wl, nthreads=8)[0]
    assert rel_l2(got, want) <= TOL
    V = wl.potentials(seed=6)
    h = run_integrate(wl, V, "mixed")
    hw = oracle_lib.batch(wl, V=V, nthreads=8)
    assert np.abs(h - hw).max() <= TOL * np.abs(hw).max()


@pytest.mark.parametrize("name", [n for n in SET_NAMES if n.startswith("general")])
def test_mixed_general_sets_vs_fp64(name):
    """The general-cell golden sets: mixed against the FP64 path of the same task set."""
    wl, _, V, _ = load_set(name)
    if V is None:
        V = wl.potentials(seed=3)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    g64 = run_collocate(wl, "fp64", ts=ts, plan=plan)
    gmx = run_collocate(wl, "mixed", ts=ts, plan=plan)
    for a, b in zip(gmx, g64):
        assert rel_l2(a, b) <= TOL
    h64 = run_integrate(wl, V, "fp64", ts=ts, plan=plan)
    hmx = run_integrate(wl, V, "mixed", ts=ts, plan=plan)
    assert np.abs(hmx - h64).max() <= TOL * np.abs(h64).max()