"""Central differences of the oracle's pair energies E_i = sum(pab_i * <V | f(phi_a, phi_b)>)
with respect to the two centres and the two exponents, for checking gpw_backward."""
import numpy as np

from libgpw_gb300 import tasks as T

H = 1e-5


def variants(wl, idx):
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
    return T.Workload("fd", tasks, wl.levels, np.concatenate(blocks), compute_tau=wl.compute_tau), off, \
        [b.size for b in blocks]


def cube_centre(t, h):
    zp = t["zeta"] + t["zetb"]
    rp = t["ra"] + (t["zetb"] / zp)[:, None] * t["rab"]
    return np.floor(rp / h[None, :]).astype(np.int64)


def fd_gradients(O, wl, V, idx, nthreads=16):
    """(fd[k][8] = dRa xyz, dRb xyz, dzeta, dzetb; stable[k]) for the sampled
    pairs of an orthorhombic workload.  A pair whose cube centre moves under a
    step has a different point set on each side and is marked unstable."""
    fdw, off, size = variants(wl, idx)
    hab_v = O.batch(fdw, V=V, nthreads=nthreads)
    n = len(idx)
    E = np.array([float(np.dot(hab_v[o:o + s], fdw.pab[o:o + s])) for o, s in zip(off, size)]).reshape(n, 17)
    h = np.diag(np.asarray(wl.levels[0]["dh"]))
    cc = cube_centre(fdw.tasks, h).reshape(n, 17, 3)
    stable = np.all(cc == cc[:, :1, :], axis=(1, 2))
    fd = np.zeros((n, 8))
    for d in range(3):
        fd[:, d] = (E[:, 1 + 4 * d] - E[:, 2 + 4 * d]) / (2 * H)
        fd[:, 3 + d] = (E[:, 3 + 4 * d] - E[:, 4 + 4 * d]) / (2 * H)
    fd[:, 6] = (E[:, 13] - E[:, 14]) / (2 * H)
    fd[:, 7] = (E[:, 15] - E[:, 16]) / (2 * H)
    return fd, stable


def gpu_gradients(wl, V):
    """gpw_backward on the whole workload: (hab, grads[n][8]) on the host."""
    import torch

    from libgpw_gb300 import capi

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
    g = np.concatenate([dra.cpu().numpy(), drb.cpu().numpy(), dza.cpu().numpy()[:, None],
                        dzb.cpu().numpy()[:, None]], axis=1)
    return hab.cpu().numpy(), g
