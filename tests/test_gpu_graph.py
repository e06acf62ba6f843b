"""The collocate + integrate step is capturable in a CUDA graph: replays give
the same result as direct calls (the tiled kernels reset their work queues with
memset nodes, nothing is allocated)."""
import numpy as np
import pytest

from golden_io import rel_l2
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_graph_replay(precision):
    import torch

    dev = torch.device("cuda:0")
    wl = T.config(1, npairs=200, seed=5)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    pab = torch.from_numpy(wl.pab).to(dev)
    V = [torch.from_numpy(v).to(dev) for v in wl.potentials(seed=2)]
    grid = torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)
    hab = torch.zeros(ts.pab_extent, dtype=torch.float64, device=dev)
    ref_g = torch.zeros_like(grid)
    ref_h = torch.zeros_like(hab)
    ts.collocate(pab, [ref_g], precision)
    ts.integrate(V, ref_h, precision)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        ts.collocate(pab, [grid], precision)
        ts.integrate(V, hab, precision)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    grid.zero_()
    hab.zero_()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        ts.collocate(pab, [grid], precision)
        ts.integrate(V, hab, precision)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    ts.check()
    assert rel_l2(grid.cpu().numpy(), 2 * ref_g.cpu().numpy()) <= 1e-14
    assert np.abs(hab.cpu().numpy() - 2 * ref_h.cpu().numpy()).max() <= 1e-13 * np.abs(ref_h.cpu().numpy()).max()
