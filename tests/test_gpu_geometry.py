"""gpw_taskset_update_geometry: new centres and exponents for the pairs of an
existing task set, set up and re-binned on the device.  After an update the
FP64 and mixed paths match the CPU oracle on the moved pairs, and a task set
built from scratch for them; bad input leaves the task set as it was."""
import numpy as np
import pytest

from golden_io import rel_l2
from gpu_util import run_collocate, run_integrate, torch_dev
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu


def moved(wl, seed, step=0.4):
    """The same pairs with centres moved by up to a few grid spacings and the
    exponents scaled by a few percent (radii kept, as the update keeps them)."""
    rng = np.random.default_rng(seed)
    t = wl.tasks.copy()
    n = t.shape[0]
    t["ra"] = t["ra"] + rng.normal(0.0, step, size=(n, 3))
    t["rab"] = t["rab"] + rng.normal(0.0, step / 2, size=(n, 3))
    t["zeta"] = t["zeta"] * np.exp(rng.normal(0.0, 0.05, size=n))
    t["zetb"] = t["zetb"] * np.exp(rng.normal(0.0, 0.05, size=n))
    return T.Workload(wl.name + "_moved", t, wl.levels, wl.pab, compute_tau=wl.compute_tau)


def update(ts, w):
    torch, dev = torch_dev()
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)  # noqa: E731
    ts.update_geometry(f(w.tasks["ra"]), f(w.tasks["rab"]), f(w.tasks["zeta"]), f(w.tasks["zetb"]))


@pytest.mark.parametrize("cfg,npairs,tiles", [(5, 1500, None), (2, 1500, None), (3, 200, [0]), (3, 200, [8])])
def test_update_matches_oracle_and_fresh_taskset(cfg, npairs, tiles, oracle_lib):
    wl = T.config(cfg, npairs=npairs, seed=800 + cfg)
    w1 = moved(wl, seed=900 + cfg, step=0.4 if cfg != 3 else 0.2)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    if tiles is not None:
        ts.set_tiles(tiles)
    run_collocate(wl, "mixed", ts=ts, plan=plan)  # the binned state in use before the update
    update(ts, w1)
    want = oracle_lib.batch(w1, nthreads=16)
    V = w1.potentials(seed=5)
    want_h = oracle_lib.batch(w1, V=V, nthreads=16)
    fresh = capi.TaskSet.from_workload(plan, w1)
    g_fresh = run_collocate(w1, "fp64", ts=fresh, plan=plan)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-8)):
        got = run_collocate(w1, prec, ts=ts, plan=plan)
        for g, w in zip(got, want):
            assert rel_l2(g, w) <= tol, prec
        if prec == "fp64":
            for g, f in zip(got, g_fresh):
                assert rel_l2(g, f) <= 1e-14
        h = run_integrate(w1, V, prec, ts=ts, plan=plan)
        assert np.abs(h - want_h).max() <= tol * np.abs(want_h).max(), prec
    # tiles set after the update re-bin from the updated host copy of the geometry
    if cfg == 5:
        ts.set_tiles([4])
        got = run_collocate(w1, "mixed", ts=ts, plan=plan)[0]
        assert rel_l2(got, want[0]) <= 1e-8


def test_update_partial_arrays(oracle_lib):
    """NULL arrays keep their values: moving only ra (rab kept) moves both centres."""
    torch, dev = torch_dev()
    wl = T.config(4, npairs=300, seed=11)
    t = wl.tasks.copy()
    t["ra"] = t["ra"] + 0.3
    w1 = T.Workload("ra_only", t, wl.levels, wl.pab)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    ts.update_geometry(ra=torch.from_numpy(np.ascontiguousarray(t["ra"])).to(dev))
    got = run_collocate(w1, "mixed", ts=ts, plan=plan)[0]
    assert rel_l2(got, oracle_lib.batch(w1, nthreads=16)[0]) <= 1e-8


def test_update_rejects_bad_input_and_keeps_the_taskset():
    torch, dev = torch_dev()
    wl = T.config(4, npairs=200, seed=12)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    before = run_collocate(wl, "mixed", ts=ts, plan=plan)[0]
    z = torch.from_numpy(np.ascontiguousarray(wl.tasks["zeta"])).to(dev)
    z[3] = -1.0
    with pytest.raises(capi.GpwError) as e:
        ts.update_geometry(zeta=z)
    assert e.value.status == 1
    ra = torch.from_numpy(np.ascontiguousarray(wl.tasks["ra"])).to(dev)
    ra[0, 1] = float("nan")
    with pytest.raises(capi.GpwError):
        ts.update_geometry(ra=ra)
    after = run_collocate(wl, "mixed", ts=ts, plan=plan)[0]
    assert rel_l2(after, before) <= 1e-15


def test_update_out_of_window_rejected():
    """A move that would take a cube across a non-periodic face is an error."""
    torch, dev = torch_dev()
    wl = T.synthetic("oow_upd", 4, 1, (4.0, 8.0), 10.0, [(32, 32, 32)], seed=3)
    wl.levels[0]["periodic"] = (0, 1, 1)
    wl.tasks["rab"] *= 0.1
    wl.tasks["ra"][:, 0] = 5.0  # well inside
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    ra = wl.tasks["ra"].copy()
    ra[:, 0] = 0.2  # next to the face
    with pytest.raises(capi.GpwError) as e:
        ts.update_geometry(ra=torch.from_numpy(np.ascontiguousarray(ra)).to(dev))
    assert e.value.status == 3
