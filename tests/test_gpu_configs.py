"""Parity on the benchmark workloads' own distributions, with no cap on the cube
radius: seeded subsamples of the multigrid workload (200k pairs, l <= 3,
180^3/90^3/45^3), the general-cell workload (50k pairs, l <= 4, 15-bohr cell at
60-90 degrees, 128^3: cubes larger than the cell wrap around it), the
differentiation workload (20k pairs, l <= 2, 96^3: forces and exponent
gradients against central finite differences of the oracle's energy) and the
1M-pair workload (l <= 4, 256^3), each compared directly with the CPU oracle
(oracle/gpw_oracle.c, itself pinned to the reference's grid_base_ref_c.cc).

Bars: FP64 path <= 1e-12, mixed path <= 1e-8 (relative grid L2, max-abs matrix
element over the largest), forces <= 1e-6 of the pair's largest gradient."""
import numpy as np
import pytest

from golden_io import rel_l2
from gpu_util import run_collocate, run_integrate
from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOLMX = 1e-8
NTHR = 16


def _max_rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _check(wl, precisions, tiles=None):
    """Collocate and integrate of wl on the GPU in each precision against the oracle."""
    from oracle import oracle as O

    want_g = O.batch(wl, nthreads=NTHR)
    V = wl.potentials(seed=31)
    want_h = O.batch(wl, V=V, nthreads=NTHR)
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    if tiles is not None:
        ts.set_tiles(tiles)
    out = {}
    for prec in precisions:
        tol = TOL64 if prec == "fp64" else TOLMX
        got = run_collocate(wl, prec, ts=ts, plan=plan)
        errs = [rel_l2(g, w) for g, w in zip(got, want_g)]
        h = run_integrate(wl, V, prec, ts=ts, plan=plan)
        herr = _max_rel(h, want_h)
        out[prec] = (max(errs), herr)
        assert max(errs) <= tol, (prec, errs)
        assert herr <= tol, (prec, herr)
    return out


def test_multigrid_workload_sample():
    wl = T.config(2, npairs=3000, seed=202)
    _check(wl, ["fp64", "mixed"])


def _general_sample():
    wl = T.config(3, npairs=300, seed=303)
    g = wl.levels[0]
    # box extent per lattice axis (points) of each pair: some exceed the cell
    span = 2 * np.ceil(wl.tasks["radius"][:, None] * np.abs(np.asarray(g["dh_inv"])).sum(axis=0)[None, :]) + 1
    assert (span > np.asarray(g["npts"])[None, :]).any(), "the sample must hold cubes that wrap the cell"
    return wl


def test_general_cell_workload_fp64():
    _check(_general_sample(), ["fp64"])


@pytest.mark.parametrize("tz", [0, 8])
def test_general_cell_workload_mixed(tz):
    """tz = 0: the float-float general-cell kernel; tz = 8: the tiled tensor-core kernels."""
    _check(_general_sample(), ["mixed"], tiles=[tz])


def test_1m_pair_workload_sample():
    wl = T.config(5, npairs=2000, seed=505)
    _check(wl, ["fp64", "mixed"])


def test_1m_pair_workload_sample_tau():
    wl = T.config(5, npairs=1000, seed=506)
    wl.compute_tau = 1
    _check(wl, ["fp64", "mixed"])


# ---------------------------------------------------------------------------
# differentiation workload: forces and exponent gradients vs central differences
TOLF = 1e-6
NSAMPLE = 60


def test_differentiation_workload_forces_vs_fd():
    """gpw_backward on all 20,000 pairs of the differentiation workload (96^3);
    the gradients of 60 random pairs against central differences (h = 1e-5) of
    the oracle's energy E_i = sum(pab_i * <V | basis_i>).  On an orthorhombic grid
    a pair's point set is fixed by its cube centre; a pair whose centre moves
    under a step would make the difference quotient meaningless, so such pairs
    are skipped, and at most 5% may be."""
    from fd_util import fd_gradients, gpu_gradients
    from oracle import oracle as O

    wl = T.config(4)
    V = wl.potentials(seed=6)
    hab, grads = gpu_gradients(wl, V)
    idx = np.sort(np.random.default_rng(404).choice(wl.ntasks, size=NSAMPLE, replace=False))
    fd, stable = fd_gradients(O, wl, V, idx, nthreads=NTHR)
    assert stable.mean() >= 0.95, f"{(~stable).sum()} of {NSAMPLE} pairs change cube centre under a step"
    for s, i in enumerate(idx):
        if not stable[s]:
            continue
        scale = np.abs(fd[s]).max()  # 0 only where the prefactor underflows
        assert np.all(np.abs(grads[i] - fd[s]) <= TOLF * scale), (i, grads[i], fd[s])
    # dE/dpab of the whole workload is the oracle's integrate
    want = O.batch(wl, V=V, nthreads=NTHR)
    assert _max_rel(hab, want) <= TOL64
