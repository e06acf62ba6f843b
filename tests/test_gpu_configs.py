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
H = 1e-5
TOLF = 1e-6
NSAMPLE = 60


def _variants(wl, idx):
    """Per sampled pair: the pair itself and its 16 central-difference variants
    (ra, rb +-h along x, y, z; zeta, zetb +-h), each with its own copy of the
    density block, as one Workload for one oracle call."""
    t0 = wl.tasks
    nsa = t0["maxco"].astype(np.int64)
    nsb = ((t0["lb_max"] + 1) * (t0["lb_max"] + 2) // 2).astype(np.int64)
    rows, blocks = [], []
    for i in idx:
        ra = t0["ra"][i].copy()
        rb = ra + t0["rab"][i]
        za, zb = float(t0["zeta"][i]), float(t0["zetb"][i])
        var = [dict()]
        for d in range(3):
            e = np.zeros(3)
            e[d] = H
            var += [dict(ra=ra + e), dict(ra=ra - e), dict(rb=rb + e), dict(rb=rb - e)]
        var += [dict(za=za + H), dict(za=za - H), dict(zb=zb + H), dict(zb=zb - H)]
        blk = wl.pab[int(t0["pab_offset"][i]): int(t0["pab_offset"][i]) + int(nsa[i] * nsb[i])]
        for v in var:
            t = t0[i:i + 1].copy()
            a = v.get("ra", ra)
            b = v.get("rb", rb)
            t["ra"][0] = a
            t["rab"][0] = b - a
            t["zeta"][0] = v.get("za", za)
            t["zetb"][0] = v.get("zb", zb)
            rows.append(t)
            blocks.append(blk)
    tasks = np.concatenate(rows)
    off = np.zeros(len(blocks), np.int64)
    off[1:] = np.cumsum([b.size for b in blocks[:-1]])
    tasks["pab_offset"] = off
    return T.Workload("fd", tasks, wl.levels, np.concatenate(blocks)), off, [b.size for b in blocks]


def _cube_centre(t, h):
    zp = t["zeta"] + t["zetb"]
    rp = t["ra"] + (t["zetb"] / zp)[:, None] * t["rab"]
    return np.floor(rp / h[None, :]).astype(np.int64)


def test_differentiation_workload_forces_vs_fd():
    """gpw_backward on all 20,000 pairs of the differentiation workload (96^3);
    the gradients of 60 random pairs against central differences (h = 1e-5) of
    the oracle's energy E_i = sum(pab_i * <V | basis_i>).  On an orthorhombic grid
    a pair's point set is fixed by its cube centre; a pair whose centre moves
    under a step would make the difference quotient meaningless, so such pairs
    are skipped, and at most 5% may be."""
    import torch

    from oracle import oracle as O

    wl = T.config(4)
    V = wl.potentials(seed=6)
    dev = torch.device("cuda:0")
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    n = wl.ntasks
    pab = torch.from_numpy(wl.pab).to(dev)
    Vd = [torch.from_numpy(v).to(dev) for v in V]
    hab = torch.zeros_like(pab)
    dra = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    drb = torch.zeros_like(dra)
    dza = torch.zeros(n, dtype=torch.float64, device=dev)
    dzb = torch.zeros_like(dza)
    ts.backward(pab, Vd, hab, dra, drb, dza, dzb)
    ts.check()
    dra, drb, dza, dzb = (x.cpu().numpy() for x in (dra, drb, dza, dzb))
    idx = np.sort(np.random.default_rng(404).choice(n, size=NSAMPLE, replace=False))
    fdw, off, size = _variants(wl, idx)
    hab_v = O.batch(fdw, V=V, nthreads=NTHR)
    E = np.array([float(np.dot(hab_v[o:o + s], fdw.pab[o:o + s])) for o, s in zip(off, size)]).reshape(NSAMPLE, 17)
    h = np.diag(np.asarray(wl.levels[0]["dh"]))
    cc = _cube_centre(fdw.tasks, h).reshape(NSAMPLE, 17, 3)
    stable = np.all(cc == cc[:, :1, :], axis=(1, 2))
    assert stable.mean() >= 0.95, f"{(~stable).sum()} of {NSAMPLE} pairs change cube centre under a step"
    checked = 0
    for s, i in enumerate(idx):
        if not stable[s]:
            continue
        e = E[s]
        fd = {}
        for d in range(3):
            fd[("ra", d)] = (e[1 + 4 * d] - e[2 + 4 * d]) / (2 * H)
            fd[("rb", d)] = (e[3 + 4 * d] - e[4 + 4 * d]) / (2 * H)
        fd[("za", 0)] = (e[13] - e[14]) / (2 * H)
        fd[("zb", 0)] = (e[15] - e[16]) / (2 * H)
        got = {("ra", d): dra[i, d] for d in range(3)}
        got.update({("rb", d): drb[i, d] for d in range(3)})
        got[("za", 0)] = dza[i]
        got[("zb", 0)] = dzb[i]
        scale = max(abs(v) for v in fd.values())  # 0 only where the prefactor underflows
        for k in fd:
            assert abs(got[k] - fd[k]) <= TOLF * scale, (i, k, got[k], fd[k])
        checked += 1
    assert checked >= int(0.95 * NSAMPLE)
    # dE/dpab of the whole workload is the oracle's integrate
    want = O.batch(wl, V=V, nthreads=NTHR)
    assert _max_rel(hab.cpu().numpy(), want) <= TOL64
