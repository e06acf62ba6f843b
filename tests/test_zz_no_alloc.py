"""gpw_collocate_noalloc: the collocation entry point that allocates no device
memory, for callers whose device memory belongs to their own pool allocator.
Its scratch is a fixed device array inside the library; the test allocates the
input and output buffers itself, as such a caller would, and checks two calls
in a row against the CPU oracle (oracle/gpw_oracle.c), not against another GPU
entry point, so a fault shared by the GPU kernels cannot pass unnoticed."""
import numpy as np
import pytest

from golden_io import rel_l2
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 path's parity bar


def _call(level, tasks, tau, pab, grid, stream=None):
    return capi.lib().gpw_collocate_noalloc(level.ctypes.data, tasks.ctypes.data, tasks.shape[0], tau,
                                            pab.data_ptr(), grid.data_ptr(), stream)


@pytest.mark.parametrize("tau", [0, 1])
def test_noalloc_matches_oracle(tau, oracle_lib):
    import torch

    dev = torch.device("cuda:0")
    wl = T.synthetic("noalloc", 40, 3, (0.3, 30.0), 9.0, [(36, 40, 44)], seed=123, compute_tau=tau)
    level = np.array([wl.levels[0]], dtype=T.GRID_DTYPE)
    tasks = np.ascontiguousarray(wl.tasks)
    pab = torch.from_numpy(wl.pab).to(dev)
    want = oracle_lib.batch(wl, nthreads=4)[0]
    grid = torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for call in (1, 2):  # the second call accumulates onto the first
        capi.check(_call(level, tasks, tau, pab, grid, stream), "gpw_collocate_noalloc")
        torch.cuda.synchronize()
        assert rel_l2(grid.cpu().numpy(), call * want) <= TOL


def test_noalloc_reports_out_of_window():
    """A cube that crosses a non-periodic face of the local window is an error
    (the reference asserts, grid_base_ref_c.cc:345-346), and the grid stays untouched."""
    import torch

    dev = torch.device("cuda:0")
    wl = T.synthetic("noalloc_oow", 4, 1, (0.5, 1.0), 10.0, [(32, 32, 32)], seed=3)
    wl.levels[0]["periodic"] = (0, 1, 1)
    wl.tasks["ra"][:, 0] = 0.2  # next to the face: the cube crosses it
    level = np.array([wl.levels[0]], dtype=T.GRID_DTYPE)
    tasks = np.ascontiguousarray(wl.tasks)
    pab = torch.from_numpy(wl.pab).to(dev)
    grid = torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)
    assert _call(level, tasks, 0, pab, grid) == 3  # GPW_ERR_OUT_OF_WINDOW
    assert "local grid" in capi.last_error()
    assert not torch.any(grid)


def test_noalloc_rejects_oversized_batch():
    import torch

    dev = torch.device("cuda:0")
    wl = T.synthetic("noalloc_big", 65, 1, (1.0, 10.0), 8.0, [(24, 24, 24)], seed=5)
    level = np.array([wl.levels[0]], dtype=T.GRID_DTYPE)
    tasks = np.ascontiguousarray(wl.tasks)
    pab = torch.from_numpy(wl.pab).to(dev)
    grid = torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)
    assert _call(level, tasks, 0, pab, grid) == 1
    assert "GPW_NOALLOC_MAX_TASKS" in capi.last_error()
    assert not torch.any(grid)
