"""The loop bounds of the pair set-up and back-transform kernels
(forward_coef / adjoint_coef in libgpw_gb300/csrc/gpw_coef.cuh), restated in
Python: the three one-axis contractions skip the products whose lattice-power
factor is structurally zero.  A power lx of T1[(lya,lza)][(lyb,lzb)] is zero
beyond (A-lya-lza) + (B-lyb-lzb), and T2[lza][lzb][ly][lx] beyond
lx + ly = (A-lza) + (B-lzb), for any local block whose shells lie within A and
B (the derivative functions raise them by one).  The pruned and full loops give
the same coefficients; the kernels themselves are compared with the oracle in
the GPU tests."""
import itertools

import numpy as np
import pytest


def tri(A):
    return [(ly, lz) for s in range(A + 1) for lz in range(s + 1) for ly in [s - lz]]


def alpha(L, A, B, rng):
    # any values: the bounds come from the structure (k <= i + j), not the numbers
    al = np.zeros((3, A + 1, B + 1, L))
    for ax, i, j in itertools.product(range(3), range(A + 1), range(B + 1)):
        al[ax, i, j, : i + j + 1] = rng.uniform(-1, 1, i + j + 1)
    return al


def forward(P, al, A, B, la_min, lb_min, prune):
    L = A + B + 1
    ta_l, tb_l = tri(A), tri(B)
    T1 = {}
    for (lya, lza), (lyb, lzb) in itertools.product(ta_l, tb_l):
        for lx in range(L):
            s = 0.0
            for lxa in range(max(la_min - lya - lza, 0), A - lya - lza + 1):
                for lxb in range(max(lb_min - lyb - lzb, 0), B - lyb - lzb + 1):
                    if lx <= lxa + lxb:
                        s += P[(lxa, lya, lza, lxb, lyb, lzb)] * al[0, lxa, lxb, lx]
            T1[(lya, lza, lyb, lzb, lx)] = s
            if lx > (A - lya - lza) + (B - lyb - lzb):
                assert s == 0.0
    T2 = {}
    n_y = 0
    for lza, lzb, ly, lx in itertools.product(range(A + 1), range(B + 1), range(L), range(L)):
        s = 0.0
        cap = A + B - lza - lzb - lx
        for lya in range(A - lza + 1):
            lo = max(ly - lya, 0)
            hi = min(B - lzb, cap - lya) if prune else B - lzb
            for lyb in range(lo, hi + 1):
                s += T1[(lya, lza, lyb, lzb, lx)] * al[1, lya, lyb, ly]
                n_y += 1
        T2[(lza, lzb, ly, lx)] = s
        if lx + ly > A + B - lza - lzb:
            assert s == 0.0
    c = {}
    n_z = 0
    lp = A + B
    for lz, ly, lx in itertools.product(range(L), range(L), range(L)):
        if lx + ly + lz > lp:
            continue
        s = 0.0
        cap = A + B - lx - ly
        for lza in range(A + 1):
            lo = max(lz - lza, 0)
            hi = min(B, cap - lza) if prune else B
            for lzb in range(lo, hi + 1):
                s += T2[(lza, lzb, ly, lx)] * al[2, lza, lzb, lz]
                n_z += 1
        c[(lz, ly, lx)] = s
    return c, n_y + n_z


@pytest.mark.parametrize("A,B,la_min,lb_min", [(0, 0, 0, 0), (1, 2, 1, 2), (3, 3, 3, 3), (4, 4, 4, 4),
                                               (5, 3, 3, 2), (5, 5, 3, 3), (4, 2, 0, 0)])
def test_pruned_contractions_equal_full(A, B, la_min, lb_min):
    rng = np.random.default_rng(10 * A + B)
    L = A + B + 1
    al = alpha(L, A, B, rng)
    P = {}
    for lxa, lya, lza in itertools.product(range(A + 1), repeat=3):
        if not la_min <= lxa + lya + lza <= A:
            continue
        for lxb, lyb, lzb in itertools.product(range(B + 1), repeat=3):
            if lb_min <= lxb + lyb + lzb <= B:
                P[(lxa, lya, lza, lxb, lyb, lzb)] = rng.uniform(-1, 1)
    full, n_full = forward(P, al, A, B, la_min, lb_min, prune=False)
    pruned, n_pruned = forward(P, al, A, B, la_min, lb_min, prune=True)
    assert pruned == full  # the skipped terms are exact zeros: bit-identical sums
    assert n_pruned <= n_full
