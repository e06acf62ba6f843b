"""FP64 GPU path against the reference (committed fixtures) and the oracle.
Bar: relative grid L2 and max-abs matrix-element error <= 1e-12 (FP64 path)."""
import numpy as np
import pytest

from golden_io import SET_NAMES, TASK_NAMES, load_set, load_task, rel_l2, task_as_workload
from gpu_util import run_collocate, run_integrate, torch_dev
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu

TOL = 1e-12


def ref_tol(name):
    # the reference's general-cell exponential recurrence drifts to ~2e-12
    return 1e-11 if name.startswith("general") or name.startswith("collocate_general") else TOL


@pytest.mark.parametrize("name", SET_NAMES)
def test_collocate_vs_reference(name, oracle_lib):
    wl, grids_ref, _, _ = load_set(name)
    got = run_collocate(wl)
    want = oracle_lib.batch(wl)
    for g, r, o in zip(got, grids_ref, want):
        assert rel_l2(g, r) <= ref_tol(name)
        assert rel_l2(g, o) <= TOL


@pytest.mark.parametrize("name", SET_NAMES)
def test_integrate_vs_oracle(name, oracle_lib):
    wl, _, V, hab_ref = load_set(name)
    if V is None:
        V = wl.potentials(seed=3)
    got = run_integrate(wl, V)
    want = oracle_lib.batch(wl, V=V)
    scale = max(np.abs(want).max(), 1e-300)
    assert np.abs(got - want).max() <= TOL * scale
    if hab_ref is not None:
        assert np.abs(got - hab_ref).max() <= 10 * TOL * max(np.abs(hab_ref).max(), 1e-300)


@pytest.mark.parametrize("name", TASK_NAMES)
def test_task_files_explicit_cube(name):
    """The reference's task files through the batch API with their own cube lists."""
    d = load_task(name)
    wl = task_as_workload(d)
    got = run_collocate(wl)[0]
    assert rel_l2(got, d["grid_ref"]) <= ref_tol(name)
    scale = max(np.abs(d["grid_ref"]).max(), 1e-300)
    for z, y, x, v in d["grid_values"]:
        assert abs(got[int(z), int(y), int(x)] - v) <= 1e-12 * scale


@pytest.mark.parametrize("name", TASK_NAMES)
def test_dropin_entry(name):
    """gpw_collocate_pgf_product_rspace: same arguments as the reference, accumulates."""
    d = load_task(name)
    grid = np.ascontiguousarray(d["grid_ref"]).copy()  # accumulates onto what is there
    capi.collocate_pgf_product_rspace(d, grid)
    assert rel_l2(grid, 2.0 * d["grid_ref"]) <= ref_tol(name)


def test_adjoint_identity_gpu():
    wl, _, _, _ = load_set("ortho_tau")
    V = wl.potentials(seed=9)
    grids = run_collocate(wl)
    hab = run_integrate(wl, V)
    lhs = sum(float(np.sum(g * v)) for g, v in zip(grids, V))
    rhs = float(np.sum(wl.pab * hab))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


def test_config1_full(oracle_lib):
    """The 1,000-pair 64^3 workload in full, both directions."""
    wl = T.config(1)
    got = run_collocate(wl)[0]
    want = oracle_lib.batch(wl, nthreads=8)[0]
    assert rel_l2(got, want) <= TOL
    V = wl.potentials(seed=2)
    h = run_integrate(wl, V)
    hw = oracle_lib.batch(wl, V=V, nthreads=8)
    assert np.abs(h - hw).max() <= TOL * np.abs(hw).max()


def test_multigrid_sample(oracle_lib):
    """Three-level multigrid routing (sampled pairs)."""
    wl = T.config(2, npairs=300)
    got = run_collocate(wl)
    want = oracle_lib.batch(wl, nthreads=8)
    for g, w in zip(got, want):
        assert rel_l2(g, w) <= TOL


def test_general_cell_sample(oracle_lib):
    wl = T.config(3, npairs=40)
    wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 5.0)
    got = run_collocate(wl)
    want = oracle_lib.batch(wl, nthreads=8)
    assert rel_l2(got[0], want[0]) <= TOL
    V = wl.potentials(seed=4)
    h = run_integrate(wl, V)
    hw = oracle_lib.batch(wl, V=V, nthreads=8)
    assert np.abs(h - hw).max() <= TOL * np.abs(hw).max()


def test_empty_taskset():
    wl = T.config(1, npairs=1)
    wl.tasks = wl.tasks[:0]
    got = run_collocate(wl)
    assert not np.any(got[0])


def test_repeat_accumulates():
    torch, dev = torch_dev()
    wl = T.config(4, npairs=50)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    pab = torch.from_numpy(wl.pab).to(dev)
    g = torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)
    ts.collocate(pab, [g])
    once = g.clone()
    ts.collocate(pab, [g])
    torch.cuda.synchronize()
    assert rel_l2(g.cpu().numpy(), 2 * once.cpu().numpy()) <= 1e-15


def test_invalid_tasks_rejected():
    wl = T.config(1, npairs=4)
    plan = capi.Plan(wl.levels)
    bad = wl.tasks.copy()
    bad["la_max"][1] = 7
    with pytest.raises(capi.GpwError) as e:
        capi.TaskSet(plan, bad)
    assert e.value.status == 1
    bad = wl.tasks.copy()
    bad["level"][0] = 3
    with pytest.raises(capi.GpwError):
        capi.TaskSet(plan, bad)
    bad = wl.tasks.copy()
    bad["zeta"][2] = -1.0
    with pytest.raises(capi.GpwError):
        capi.TaskSet(plan, bad)


def test_out_of_window_rejected():
    """A non-periodic cube that leaves the local grid is an error, not a fault
    (the reference asserts: grid_base_ref_c.cc:345-346)."""
    wl = T.synthetic("oow", 4, 1, (0.5, 1.0), 10.0, [(32, 32, 32)], seed=3)
    wl.levels[0]["periodic"] = (0, 1, 1)
    wl.tasks["ra"][:, 0] = 0.2  # next to the face: the cube crosses it
    plan = capi.Plan(wl.levels)
    with pytest.raises(capi.GpwError) as e:
        capi.TaskSet(plan, wl.tasks)
    assert e.value.status == 3


@pytest.mark.parametrize("shape", [(14, 23, 17, 3), (14, 23, 17, 1), (1, 12, 29, 5), (13, 45, 29, 7)])
def test_core_contractions(shape):
    """collocate_core / integrate_core known answers with the reference's test
    shapes (collocate.cc:1185-1212), random U(-1,1) inputs, naive sums as truth."""
    torch, dev = torch_dev()
    nz, ny, nx, L = shape
    rng = np.random.default_rng(1)
    ld = max(nz, ny, nx)
    pol = rng.uniform(-1, 1, size=(3, L, ld))
    co = rng.uniform(-1, 1, size=(L, L, L))
    want = np.einsum("agb,gz,by,ax->zyx", co, pol[0, :, :nz], pol[1, :, :ny], pol[2, :, :nx])
    d_pol = torch.from_numpy(pol).to(dev)
    d_co = torch.from_numpy(co).to(dev)
    out = torch.zeros((nz, ny, nx), dtype=torch.float64, device=dev)
    L_ = capi.lib()
    import ctypes as C
    length = (C.c_int * 3)(nz, ny, nx)
    s = torch.cuda.current_stream().cuda_stream
    capi.check(L_.gpw_collocate_core(length, L, d_co.data_ptr(), d_pol.data_ptr(), ld, out.data_ptr(), s))
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy() - want).max() <= 1e-14 * max(1.0, np.abs(want).max())
    V = rng.uniform(-1, 1, size=(nz, ny, nx))
    want2 = np.einsum("zyx,gz,by,ax->gba", V, pol[0, :, :nz], pol[1, :, :ny], pol[2, :, :nx])
    d_V = torch.from_numpy(V).to(dev)
    co2 = torch.zeros((L, L, L), dtype=torch.float64, device=dev)
    capi.check(L_.gpw_integrate_core(length, L, d_pol.data_ptr(), ld, d_V.data_ptr(), co2.data_ptr(), s))
    torch.cuda.synchronize()
    assert np.abs(co2.cpu().numpy() - want2).max() <= 1e-13 * max(1.0, np.abs(want2).max())
