"""The derivative functions of the CPU oracle (oracle/gpw_oracle.c) against
their definitions.  tau = 1/2 grad phi_a . grad phi_b is pinned by the
reference's own fixtures (test_oracle.py); phi_a d phi_b - d phi_a phi_b
(compute_polynomial_coefficients_ADBmDAB, coefficient.hpp:209-354) has no
runnable counterpart in the reference, so it is checked here against
  * the centre derivatives of rho: since d/dx phi_a = -d phi_a / d ax,
    phi_a d_x phi_b - d_x phi_a phi_b = d rho / d ax - d rho / d bx
    (central differences, h = 1e-5, all pairs moved together), and
  * antisymmetry: exchanging the two primitives (centres, exponents, shells and
    the transposed block) flips its sign and leaves rho unchanged."""
import numpy as np
import pytest

from golden_io import rel_l2
from libgpw_gb300 import tasks as T

H = 1e-5


def _workload(func, seed=5):
    wl = T.synthetic("fn", 8, 2, (0.5, 8.0), 10.0, [(40, 40, 40)], seed=seed)
    wl.compute_tau = func
    return wl


def _shift(wl, which, d, h):
    w = T.Workload(wl.name, wl.tasks.copy(), wl.levels, wl.pab, compute_tau=0)
    if which == "a":
        w.tasks["ra"][:, d] += h
        w.tasks["rab"][:, d] -= h
    else:
        w.tasks["rab"][:, d] += h
    return w


def _centres(wl, h):
    t = wl.tasks
    zp = t["zeta"] + t["zetb"]
    rp = t["ra"] + (t["zetb"] / zp)[:, None] * t["rab"]
    return np.floor(rp / h[None, :]).astype(np.int64)


@pytest.mark.parametrize("d", [0, 1, 2])
def test_adbmdab_is_the_centre_derivative_difference(oracle_lib, d):
    O = oracle_lib
    wl = _workload(2 + d)
    got = O.batch(wl)[0]
    h = np.diag(np.asarray(wl.levels[0]["dh"]))
    shifted = [_shift(wl, s, d, sg * H) for s in ("a", "b") for sg in (1, -1)]
    cc0 = _centres(wl, h)
    for w in shifted:  # the point sets stay the same under every step
        assert np.array_equal(_centres(w, h), cc0)
    g = [O.batch(w)[0] for w in shifted]
    fd = (g[0] - g[1]) / (2 * H) - (g[2] - g[3]) / (2 * H)
    assert np.linalg.norm(got) > 0
    assert rel_l2(got, fd) <= 1e-6


def _swapped(wl):
    """The same pairs with the two primitives exchanged."""
    from libgpw_gb300.tasks import ncoset

    t0 = wl.tasks
    t = t0.copy()
    rb = t0["ra"] + t0["rab"]
    t["ra"], t["rab"] = rb, -t0["rab"]
    t["zeta"], t["zetb"] = t0["zetb"], t0["zeta"]
    for k0, k1 in (("la_max", "lb_max"), ("la_min", "lb_min")):
        t[k0], t[k1] = t0[k1], t0[k0]
    blocks, off = [], 0
    for i in range(t0.shape[0]):
        la, lb = int(t0["la_max"][i]), int(t0["lb_max"][i])
        nsa, nsb = (la + 1) * (la + 2) // 2, (lb + 1) * (lb + 2) // 2
        blk = wl.pab[int(t0["pab_offset"][i]): int(t0["pab_offset"][i]) + nsa * nsb].reshape(nsb, nsa)
        blocks.append(blk.T.reshape(-1))
        t["pab_offset"][i] = off
        t["maxco"][i] = nsb
        t["o1"][i] = -ncoset(lb - 1)
        t["o2"][i] = -ncoset(la - 1)
        off += nsa * nsb
    return T.Workload(wl.name + "_swap", t, wl.levels, np.concatenate(blocks), compute_tau=wl.compute_tau)


@pytest.mark.parametrize("func", [0, 1, 2, 3, 4])
def test_exchange_symmetry(oracle_lib, func):
    O = oracle_lib
    wl = _workload(func, seed=9)
    g = O.batch(wl)[0]
    gs = O.batch(_swapped(wl))[0]
    sign = -1.0 if func >= 2 else 1.0
    assert np.linalg.norm(g) > 0
    assert rel_l2(gs, sign * g) <= 1e-13
