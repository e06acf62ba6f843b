"""The collocated functions other than rho on the GPU (gpw_function 1-4: tau and
phi_a d phi_b - d phi_a phi_b along x, y, z): FP64 and mixed collocate and
integrate against the CPU oracle, and the backward pass of tau with la = lb = 4
(moments to degree 12) against central differences of the oracle's energy.
Bars: FP64 1e-12, mixed 1e-8, gradients 1e-6 of the pair's largest."""
import numpy as np
import pytest

from golden_io import rel_l2
from gpu_util import run_collocate, run_integrate
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("func", [1, 2, 3, 4])
def test_functions_vs_oracle(func, oracle_lib):
    O = oracle_lib
    for wl in (T.config(4, npairs=300, seed=61), T.config(5, npairs=200, seed=62)):
        wl.compute_tau = func
        want = O.batch(wl, nthreads=16)[0]
        V = wl.potentials(seed=63)
        want_h = O.batch(wl, V=V, nthreads=16)
        plan = capi.Plan(wl.levels)
        ts = capi.TaskSet.from_workload(plan, wl)
        for prec, tol in (("fp64", 1e-12), ("mixed", 1e-8)):
            got = run_collocate(wl, prec, ts=ts, plan=plan)[0]
            assert rel_l2(got, want) <= tol, (wl.name, prec)
            h = run_integrate(wl, V, prec, ts=ts, plan=plan)
            assert np.abs(h - want_h).max() <= tol * np.abs(want_h).max(), (wl.name, prec)


def test_tau_backward_l4_vs_fd(oracle_lib):
    from fd_util import fd_gradients, gpu_gradients

    wl = T.synthetic("bwd_tau4", 400, 4, (0.3, 30.0), 12.0, [(64, 64, 64)], seed=71, lmin=3)
    wl.compute_tau = 1
    V = wl.potentials(seed=72)
    hab, grads = gpu_gradients(wl, V)
    want = oracle_lib.batch(wl, V=V, nthreads=16)
    assert np.abs(hab - want).max() <= 1e-12 * np.abs(want).max()
    idx = np.sort(np.random.default_rng(73).choice(wl.ntasks, size=30, replace=False))
    fd, stable = fd_gradients(oracle_lib, wl, V, idx)
    assert stable.mean() >= 0.9
    for s, i in enumerate(idx):
        if stable[s]:
            scale = np.abs(fd[s]).max()
            assert np.all(np.abs(grads[i] - fd[s]) <= 1e-6 * scale), (i, grads[i], fd[s])
