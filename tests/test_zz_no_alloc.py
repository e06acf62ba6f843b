"""gpw_collocate_noalloc: the collocation entry point that allocates no device
memory, for callers whose device memory belongs to their own pool allocator.
Its scratch is a fixed device array inside the library; the test allocates the
input and output buffers itself, as such a caller would, and checks two calls
in a row against the task-set entry point (gpw_collocate, FP64)."""
import ctypes as C

import numpy as np
import pytest

from golden_io import rel_l2
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 path's parity bar


def _workload(tau):
    wl = T.synthetic("noalloc", 40, 3, (0.3, 30.0), 9.0, [(36, 40, 44)], seed=123, compute_tau=tau)
    return wl


@pytest.mark.parametrize("tau", [0, 1])
def test_noalloc_matches_taskset_path(tau):
    import torch

    dev = torch.device("cuda:0")
    wl = _workload(tau)
    level = np.array([wl.levels[0]], dtype=T.GRID_DTYPE)
    tasks = np.ascontiguousarray(wl.tasks)
    pab = torch.from_numpy(wl.pab).to(dev)
    shape = T.grid_shape(wl.levels[0])
    # reference: the task-set entry point
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    ref = torch.zeros(shape, dtype=torch.float64, device=dev)
    ts.collocate(pab, [ref], "fp64")
    ts.check()
    ref1 = ref.cpu().numpy()
    # the no-allocation entry, twice in a row into the same grid
    grid = torch.zeros(shape, dtype=torch.float64, device=dev)
    L = capi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for call in (1, 2):
        st = L.gpw_collocate_noalloc(level.ctypes.data, tasks.ctypes.data, tasks.shape[0], tau, pab.data_ptr(),
                                     grid.data_ptr(), stream)
        capi.check(st, "gpw_collocate_noalloc")
        torch.cuda.synchronize()
        assert rel_l2(grid.cpu().numpy(), call * ref1) <= TOL


def test_noalloc_rejects_oversized_batch():
    import torch

    dev = torch.device("cuda:0")
    wl = T.synthetic("noalloc_big", 65, 1, (1.0, 10.0), 8.0, [(24, 24, 24)], seed=5)
    level = np.array([wl.levels[0]], dtype=T.GRID_DTYPE)
    tasks = np.ascontiguousarray(wl.tasks)
    pab = torch.from_numpy(wl.pab).to(dev)
    grid = torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)
    st = capi.lib().gpw_collocate_noalloc(level.ctypes.data, tasks.ctypes.data, 65, 0, pab.data_ptr(),
                                          grid.data_ptr(), None)
    assert st == 1
    assert "GPW_NOALLOC_MAX_TASKS" in capi.last_error()
    assert not torch.any(grid)
