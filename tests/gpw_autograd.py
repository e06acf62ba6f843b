"""Test-harness-only torch.autograd.Function over the C ABI: the energy
E = sum_levels <V, rho(pab, ra, rb, zeta, zetb)> with the library's forward
(gpw_collocate) and backward (gpw_backward) kernels.  One task set serves every
evaluation: each forward moves its pairs with gpw_taskset_update_geometry (on the
device) instead of rebuilding it on the host."""
import torch

from libgpw_gb300 import capi, tasks as T


class PairSet:
    """The task set of a workload, created once and moved by every forward."""

    def __init__(self, wl):
        self.wl = wl
        self.plan = capi.Plan(wl.levels)
        self.ts = capi.TaskSet.from_workload(self.plan, wl)


class Energy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pab, ra, rb, zeta, zetb, V, pairs):
        ts, wl = pairs.ts, pairs.wl
        ts.update_geometry(ra.detach().contiguous(), (rb - ra).detach().contiguous(), zeta.detach().contiguous(),
                           zetb.detach().contiguous())
        dev = pab.device
        grids = [torch.zeros(T.grid_shape(g), dtype=torch.float64, device=dev) for g in wl.levels]
        ts.collocate(pab.detach().contiguous(), grids, "fp64")
        E = sum((g * v).sum() for g, v in zip(grids, V))
        ctx.ts, ctx.V = ts, V
        ctx.save_for_backward(pab)
        return E

    @staticmethod
    def backward(ctx, gE):
        (pab,) = ctx.saved_tensors
        n = ctx.ts.tasks.shape[0]
        dev = pab.device
        hab = torch.zeros_like(pab)
        dra = torch.zeros((n, 3), dtype=torch.float64, device=dev)
        drb = torch.zeros_like(dra)
        dza = torch.zeros(n, dtype=torch.float64, device=dev)
        dzb = torch.zeros_like(dza)
        ctx.ts.backward(pab.detach().contiguous(), list(ctx.V), hab, dra, drb, dza, dzb)
        ctx.ts.check()
        return gE * hab, gE * dra, gE * drb, gE * dza, gE * dzb, None, None


def energy(pab, ra, rb, zeta, zetb, V, pairs):
    return Energy.apply(pab, ra, rb, zeta, zetb, V, pairs)
