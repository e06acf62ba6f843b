"""Backward kernels: dE/dpab (= integrate), forces dE/dRa, dE/dRb and exponent
gradients dE/dzeta, dE/dzetb against FP64 central finite differences (h = 1e-5)
of the CPU oracle's energy, <= 1e-6 relative, for rho, tau and
phi_a d_x phi_b - d_x phi_a phi_b (gpw_function 0, 1, 2)."""
import numpy as np
import pytest

from libgpw_gb300 import capi, tasks as T

pytestmark = pytest.mark.gpu

H = 1e-5
TOL = 1e-6


def workload(ortho=True, n=10, seed=41, func=0):
    wl = _workload(ortho, n, seed)
    wl.compute_tau = func
    return wl


def _workload(ortho, n, seed):
    if ortho:
        wl = T.synthetic("bwd", n, 2, (0.3, 20.0), 8.0, [(40, 40, 40)], seed=seed)
    else:
        wl = T.synthetic("bwd_g", n, 2, (0.5, 20.0), T.lattice_15(length=8.0), [(36, 36, 36)], seed=seed,
                         ortho=False)
        wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 4.0)
    return wl


def energy_cpu(O, wl, V, i, ra=None, rb=None, za=None, zb=None):
    """E of pair i alone: sum over its block of pab * <V | basis> (oracle)."""
    t = wl.tasks[i:i + 1].copy()
    ra0 = t["ra"][0].copy()
    rb0 = ra0 + t["rab"][0]
    ra1 = ra0 if ra is None else ra
    rb1 = rb0 if rb is None else rb
    t["ra"][0] = ra1
    t["rab"][0] = rb1 - ra1
    if za is not None:
        t["zeta"][0] = za
    if zb is not None:
        t["zetb"][0] = zb
    hab = O.batch(wl, V=V, tasks=t)
    return float(np.sum(hab * wl.pab))


def point_set(O, wl, i, **kw):
    """Grid points pair i touches (the oracle's nonzero pattern), with perturbed
    centres or exponents."""
    t = wl.tasks[i:i + 1].copy()
    ra0 = t["ra"][0].copy()
    rb0 = ra0 + t["rab"][0]
    ra1 = kw.get("ra", ra0)
    rb1 = kw.get("rb", rb0)
    t["ra"][0] = ra1
    t["rab"][0] = rb1 - ra1
    if "za" in kw:
        t["zeta"][0] = kw["za"]
    if "zb" in kw:
        t["zetb"][0] = kw["zb"]
    sub = T.Workload("one", t, wl.levels, np.ones_like(wl.pab), compute_tau=wl.compute_tau)
    return [g != 0 for g in O.batch(sub)]


def stable(O, wl, i):
    """True if the pair's point set is the same for every finite-difference step
    (the cube is fixed by the centre cell on orthorhombic grids; on general cells
    the row bounds move with the centre)."""
    t = wl.tasks[i]
    ra = t["ra"].copy()
    rb = ra + t["rab"]
    base = point_set(O, wl, i)
    steps = []
    for d in range(3):
        e = np.zeros(3)
        e[d] = H
        steps += [dict(ra=ra + e), dict(ra=ra - e), dict(rb=rb + e), dict(rb=rb - e)]
    steps += [dict(za=float(t["zeta"]) + H), dict(za=float(t["zeta"]) - H), dict(zb=float(t["zetb"]) + H),
              dict(zb=float(t["zetb"]) - H)]
    for kw in steps:
        for a, b in zip(base, point_set(O, wl, i, **kw)):
            if not np.array_equal(a, b):
                return False
    return True


@pytest.mark.parametrize("func", [0, 1, 2])
@pytest.mark.parametrize("ortho", [True, False])
def test_forces_and_exponents_vs_fd(ortho, func, oracle_lib):
    import torch

    O = oracle_lib
    wl = workload(ortho, func=func)
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
    hab_ref = O.batch(wl, V=V)
    assert np.abs(hab.cpu().numpy() - hab_ref).max() <= 1e-12 * np.abs(hab_ref).max()
    checked = 0
    for i in range(n):
        if not stable(O, wl, i):
            continue
        t = wl.tasks[i]
        ra = t["ra"].copy()
        rb = ra + t["rab"]
        scale = 0.0
        fd = {}
        for d in range(3):
            e = np.zeros(3)
            e[d] = H
            fd[("ra", d)] = (energy_cpu(O, wl, V, i, ra=ra + e) - energy_cpu(O, wl, V, i, ra=ra - e)) / (2 * H)
            fd[("rb", d)] = (energy_cpu(O, wl, V, i, rb=rb + e) - energy_cpu(O, wl, V, i, rb=rb - e)) / (2 * H)
        za, zb = float(t["zeta"]), float(t["zetb"])
        fd[("za", 0)] = (energy_cpu(O, wl, V, i, za=za + H) - energy_cpu(O, wl, V, i, za=za - H)) / (2 * H)
        fd[("zb", 0)] = (energy_cpu(O, wl, V, i, zb=zb + H) - energy_cpu(O, wl, V, i, zb=zb - H)) / (2 * H)
        scale = max(abs(v) for v in fd.values())
        if scale < 1e-8:
            continue
        got = {("ra", d): dra[i, d] for d in range(3)}
        got.update({("rb", d): drb[i, d] for d in range(3)})
        got[("za", 0)] = dza[i]
        got[("zb", 0)] = dzb[i]
        for k in fd:
            assert abs(got[k] - fd[k]) <= TOL * scale, (i, k, got[k], fd[k])
        checked += 1
    assert checked >= 3


def test_autograd_function(oracle_lib):
    """The torch.autograd.Function of the test harness: gradients of E with respect
    to the density blocks, centres and exponents through gpw_backward."""
    import torch

    from gpw_autograd import PairSet, energy

    wl = workload(True, n=6, seed=43)
    V = wl.potentials(seed=8)
    dev = torch.device("cuda:0")
    pab = torch.from_numpy(wl.pab).to(dev).requires_grad_(True)
    ra = torch.from_numpy(wl.tasks["ra"].copy()).to(dev).requires_grad_(True)
    rb = torch.from_numpy((wl.tasks["ra"] + wl.tasks["rab"]).copy()).to(dev).requires_grad_(True)
    za = torch.from_numpy(wl.tasks["zeta"].copy()).to(dev).requires_grad_(True)
    zb = torch.from_numpy(wl.tasks["zetb"].copy()).to(dev).requires_grad_(True)
    Vd = [torch.from_numpy(v).to(dev) for v in V]
    pairs = PairSet(wl)
    E = energy(pab, ra, rb, za, zb, Vd, pairs)
    gp, gra, grb, gza, gzb = torch.autograd.grad(E, [pab, ra, rb, za, zb])
    # dE/dpab is the oracle's integrate; E itself is the oracle's <V, rho>
    hab = oracle_lib.batch(wl, V=V)
    assert np.abs(gp.cpu().numpy() - hab).max() <= 1e-12 * np.abs(hab).max()
    E_cpu = sum(float(np.sum(g * v)) for g, v in zip(oracle_lib.batch(wl), V))
    assert abs(float(E.detach()) - E_cpu) <= 1e-12 * max(abs(E_cpu), 1.0)
    assert torch.all(torch.isfinite(gra)) and torch.all(torch.isfinite(gza))
    # a second evaluation at moved centres through the same task set (device update)
    shift = torch.full_like(ra, 0.05)
    ra2 = (ra.detach() + shift).requires_grad_(True)
    rb2 = (rb.detach() + shift).requires_grad_(True)
    E2 = energy(pab, ra2, rb2, za, zb, Vd, pairs)
    t2 = wl.tasks.copy()
    t2["ra"] = t2["ra"] + 0.05
    w2 = T.Workload("moved", t2, wl.levels, wl.pab)
    E2_cpu = sum(float(np.sum(g * v)) for g, v in zip(oracle_lib.batch(w2), V))
    assert abs(float(E2.detach()) - E2_cpu) <= 1e-12 * max(abs(E2_cpu), 1.0)


def test_backward_tau_high_l_general_cell_rejected():
    """tau with la = lb = 4 needs moments to degree 12; on a general cell they go
    through the lattice transform, built to degree 10: reported, not computed."""
    import torch

    wl = T.synthetic("bwd_g4", 3, 4, (0.5, 20.0), T.lattice_15(length=8.0), [(36, 36, 36)], seed=2,
                     ortho=False, lmin=4)
    wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 3.0)
    wl.compute_tau = 1
    plan = capi.Plan(wl.levels)
    ts = capi.TaskSet.from_workload(plan, wl)
    dev = torch.device("cuda:0")
    pab = torch.from_numpy(wl.pab).to(dev)
    V = [torch.zeros(T.grid_shape(wl.levels[0]), dtype=torch.float64, device=dev)]
    dra = torch.zeros((3, 3), dtype=torch.float64, device=dev)
    with pytest.raises(capi.GpwError) as e:
        ts.backward(pab, V, None, dra)
    assert e.value.status == 4
