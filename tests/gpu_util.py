"""Helpers of the GPU tests: run a Workload through the C ABI on cuda:0."""
import numpy as np

from libgpw_gb300 import capi, tasks as T


def torch_dev():
    import torch

    return torch, torch.device("cuda:0")


def run_collocate(wl, precision="fp64", ts=None, plan=None):
    torch, dev = torch_dev()
    plan = plan or capi.Plan(wl.levels)
    ts = ts or capi.TaskSet.from_workload(plan, wl)
    pab = torch.from_numpy(np.ascontiguousarray(wl.pab)).to(dev)
    grids = [torch.zeros(T.grid_shape(g), dtype=torch.float64, device=dev) for g in wl.levels]
    ts.collocate(pab, grids, precision)
    ts.check()
    return [g.cpu().numpy() for g in grids]


def run_integrate(wl, V, precision="fp64", ts=None, plan=None):
    torch, dev = torch_dev()
    plan = plan or capi.Plan(wl.levels)
    ts = ts or capi.TaskSet.from_workload(plan, wl)
    grids = [torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in V]
    hab = torch.zeros(max(ts.pab_extent, wl.pab.size), dtype=torch.float64, device=dev)
    ts.integrate(grids, hab, precision)
    ts.check()
    return hab.cpu().numpy()[: wl.pab.size]
