"""Tile shapes of the mixed path: every shape gives the FP64 results within the
mixed-path bar, the shapes agree with each other, and the autotuner picks one
of them and leaves the caller's buffers alone."""
import numpy as np
import pytest
import torch

from golden_io import rel_l2
from gpu_util import run_collocate, run_integrate
from libgpw_gb300 import autotune, capi, tasks as T

pytestmark = pytest.mark.gpu

TOL = 1e-8


@pytest.mark.parametrize("tz", [8, 4])
def test_shapes_match_fp64(tz):
    wl = T.config(5, npairs=300, seed=21)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    g64 = run_collocate(wl, "fp64", ts=ts, plan=plan)[0]
    V = wl.potentials(seed=4)
    h64 = run_integrate(wl, V, "fp64", ts=ts, plan=plan)
    ts.set_tiles([tz])
    assert ts.tiles() == [tz]
    gmx = run_collocate(wl, "mixed", ts=ts, plan=plan)[0]
    assert rel_l2(gmx, g64) <= TOL
    hmx = run_integrate(wl, V, "mixed", ts=ts, plan=plan)
    assert np.abs(hmx - h64).max() <= TOL * np.abs(h64).max()


def test_multigrid_per_level_shapes(oracle_lib):
    wl = T.config(2, npairs=300)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    ts.set_tiles([4, 8, 4])
    got = run_collocate(wl, "mixed", ts=ts, plan=plan)
    want = oracle_lib.batch(wl, nthreads=8)
    for g, w in zip(got, want):
        assert rel_l2(g, w) <= TOL


def test_bad_shape_rejected():
    wl = T.config(1, npairs=20)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    for bad in (0, 16, 32):  # tz = 0 is for general-cell levels only
        with pytest.raises(capi.GpwError):
            ts.set_tiles([bad])
    assert ts.tiles() == [8]  # the default shape


def test_autotune_picks_a_candidate(tmp_path):
    wl = T.config(5, npairs=2000, seed=5)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    dev = torch.device("cuda:0")
    pab = torch.from_numpy(wl.pab).to(dev)
    pab_before = pab.clone()
    tz, ms = ts.autotune(pab)
    assert tz[0] in (4, 8, 16) and ts.tiles() == tz
    assert (ms[0][:2] > 0).all() and ms[0][2] == -1.0  # tz = 0 is not a candidate on an orthorhombic level
    assert torch.equal(pab, pab_before)
    # the table path: first call tunes and records, the second reads it back
    path = str(tmp_path / "tiles.json")
    tz1, src1 = autotune.apply(ts, pab, path=path)
    ts.set_tiles([4])
    tz2, src2 = autotune.apply(ts, pab, path=path)
    assert src1 == "tuned" and src2 == "table" and tz1 == tz2 == ts.tiles()
    # results after tuning still match FP64
    g64 = run_collocate(wl, "fp64", ts=ts, plan=plan)[0]
    gmx = run_collocate(wl, "mixed", ts=ts, plan=plan)[0]
    assert rel_l2(gmx, g64) <= TOL


def test_bins_follow_the_tile_shapes():
    """gpw_taskset_bins: every pair meets at least one tile; smaller tiles (tz = 4
    on one level is 32 x 32 x 4) give a different item count; a general-cell
    level left untiled (tz = 0) has no items, and tiled it has at most as many
    as the tiles its pairs' index boxes can span (an upper bound; the culling
    itself is checked by the parity tests on the same distribution)."""
    wl = T.config(5, npairs=400, seed=23)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    ts.set_tiles([8])
    items8, units8 = ts.bins()
    assert items8 >= wl.ntasks and units8 >= 1
    ts.set_tiles([4])
    items4, _ = ts.bins()
    assert items4 >= wl.ntasks and items4 != items8

    wg = T.config(3, npairs=200, seed=24)
    plan_g = capi.Plan(wg.levels)
    ts_g = capi.TaskSet.from_workload(plan_g, wg)
    ts_g.set_tiles([0])
    assert ts_g.bins() == (0, 0)
    ts_g.set_tiles([8])
    items_g, units_g = ts_g.bins()
    assert items_g >= wg.ntasks and units_g >= 1
    # tiles of 32 x 16 x 8 that each index box spans, without culling
    g = wg.levels[0]
    span = 2 * np.ceil(wg.tasks["radius"][:, None] * np.abs(np.asarray(g["dh_inv"])).sum(axis=0)[None, :]) + 1
    n = np.asarray(g["npts"], dtype=np.float64)
    boxes = np.prod(np.minimum(np.ceil(span / np.array([32.0, 16.0, 8.0])) + 1, n / np.array([32.0, 16.0, 8.0])), axis=1)
    assert items_g <= boxes.sum()
