"""Generates the committed golden fixtures from the reference itself.

Run in a tree where the reference sources exist (it reads the reference's task
fixtures and calls the reference's own grid_collocate_pgf_product_rspace,
compiled by oracle/ref/Makefile):

    python tests/golden/make_golden.py --ref-root <reference checkout>

Outputs (tests/golden/):
  reference_tasks.npz  the four "Grid collocate task v1" files of the reference
                       (src/lib/collocate_{ortho,general}_{density,tau}.task):
                       every argument, the values each file pins, and the full
                       grid the reference computes for it
  reference_sets.npz   seeded synthetic pair sets (orthorhombic / general cell,
                       rho / tau, periodic / non-periodic) with the reference's
                       full grids; two sets also carry matrix elements built
                       from the reference by adjointness
                       (h[j,i] = <V, collocate(unit block e_ji)>)
"""
from __future__ import annotations

import argparse
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libgpw_gb300 import tasks as T  # noqa: E402
from oracle import oracle as O  # noqa: E402


def task_files(ref_root):
    out = {}
    for path in sorted(glob.glob(os.path.join(ref_root, "src", "lib", "collocate_*.task"))):
        name = os.path.basename(path)[: -len(".task")]
        t = T.read_task_file(path)
        grid = np.zeros((t["ngrid"][2], t["ngrid"][1], t["ngrid"][0]))
        O.collocate(t, grid, use_ref=True)
        p = name + "/"
        for k in ("compute_tau", "use_ortho", "la_max", "la_min", "lb_max", "lb_min", "lmax",
                  "nspheres", "maxco", "o1", "o2"):
            out[p + k] = np.int32(t[k])
        for k in ("zeta", "zetb", "rscale", "radius"):
            out[p + k] = np.float64(t[k])
        for k in ("dh", "dh_inv", "ra", "rab", "npts", "ngrid", "lb_grid", "periodic", "lb_cube",
                  "ub_cube", "sphere_bounds", "pab", "grid_values"):
            out[p + k] = np.asarray(t[k])
        out[p + "grid_ref"] = grid
    return out


def set_arrays(prefix, wl, grids, V=None, hab=None):
    out = {
        prefix + "tasks": wl.tasks,
        prefix + "levels": wl.level_array(),
        prefix + "pab": wl.pab,
        prefix + "compute_tau": np.int32(wl.compute_tau),
    }
    for l, g in enumerate(grids):
        out[prefix + f"grid_ref_{l}"] = g
    if V is not None:
        for l, v in enumerate(V):
            out[prefix + f"V_{l}"] = v
        out[prefix + "hab_ref"] = hab
    return out


def ref_collocate_set(wl):
    grids = [np.zeros(T.grid_shape(g)) for g in wl.levels]
    for i in range(wl.ntasks):
        d = O.task_dict(wl, i)
        O.collocate(d, grids[int(wl.tasks[i]["level"])], use_ref=True)
    return grids


def ref_integrate_set(wl, V):
    """Matrix elements from the reference by adjointness: one reference collocation
    per block element with a unit block."""
    hab = np.zeros_like(wl.pab)
    for i in range(wl.ntasks):
        tk = wl.tasks[i]
        d = O.task_dict(wl, i)
        v = V[int(tk["level"])]
        la, lb = int(tk["la_max"]), int(tk["lb_max"])
        for jco in range(T.ncoset(int(tk["lb_min"]) - 1), T.ncoset(lb)):
            for ico in range(T.ncoset(int(tk["la_min"]) - 1), T.ncoset(la)):
                unit = np.zeros_like(d["pab"])
                unit[jco, ico] = 1.0
                d2 = dict(d, pab=unit)
                g = np.zeros_like(v)
                O.collocate(d2, g, use_ref=True)
                idx = int(tk["pab_offset"]) + (int(tk["o2"]) + jco) * int(tk["maxco"]) + int(tk["o1"]) + ico
                hab[idx] += float(np.sum(g * v))
    return hab


def synthetic_sets():
    out = {}
    # orthorhombic, rho, large exponent range: cubes wrap the 24^3 period
    wl = T.synthetic("ortho_rho", 24, 4, (0.1, 50.0), 10.0, [(24, 24, 24)], seed=11)
    out.update(set_arrays("ortho_rho/", wl, ref_collocate_set(wl)))
    # orthorhombic, tau, non-cubic box and grid
    wl = T.synthetic("ortho_tau", 16, 3, (0.2, 30.0), (9.0, 10.0, 11.0), [(20, 24, 28)], seed=12,
                     compute_tau=1)
    out.update(set_arrays("ortho_tau/", wl, ref_collocate_set(wl)))
    # orthorhombic, two levels, integrate goldens by adjointness
    wl = T.synthetic("ortho_int", 8, 2, (0.3, 20.0), 8.0, [(24, 24, 24), (16, 16, 16)], seed=13,
                     route=lambda z: (np.asarray(z) < 3.0).astype(np.int32))
    V = wl.potentials(seed=14)
    out.update(set_arrays("ortho_int/", wl, ref_collocate_set(wl), V, ref_integrate_set(wl, V)))
    # general cell, rho and tau (radius capped: the reference visits the whole box)
    for name, tau, seed in (("general_rho", 0, 15), ("general_tau", 1, 16)):
        wl = T.synthetic(name, 12, 3 if tau else 4, (0.5, 40.0), T.lattice_15(length=9.0),
                         [(20, 20, 20)], seed=seed, ortho=False, compute_tau=tau)
        wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 4.0)
        out.update(set_arrays(name + "/", wl, ref_collocate_set(wl)))
    wl = T.synthetic("general_int", 6, 2, (0.5, 20.0), T.lattice_15(length=8.0), [(16, 16, 16)],
                     seed=17, ortho=False)
    wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 3.5)
    V = wl.potentials(seed=18)
    out.update(set_arrays("general_int/", wl, ref_collocate_set(wl), V, ref_integrate_set(wl, V)))
    # non-periodic x axis: centres kept away from the x faces so every cube fits
    wl = T.synthetic("ortho_nonperiodic", 10, 2, (1.0, 30.0), 10.0, [(32, 32, 32)], seed=19)
    g = wl.levels[0]
    g["periodic"] = (0, 1, 1)
    wl.tasks["ra"][:, 0] = np.random.default_rng(20).uniform(4.0, 6.0, size=wl.ntasks)
    wl.tasks["rab"][:, 0] = np.random.default_rng(21).uniform(-0.5, 0.5, size=wl.ntasks)
    wl.tasks["radius"] = np.minimum(wl.tasks["radius"], 3.0)
    out.update(set_arrays("ortho_nonperiodic/", wl, ref_collocate_set(wl)))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", required=True, help="root of the reference checkout (holds src/lib)")
    args = ap.parse_args()
    O.build(ref_src=os.path.join(args.ref_root, "src", "lib"))
    if not O.ref_available():
        sys.exit("reference library not built (reference sources absent?)")
    np.savez_compressed(os.path.join(HERE, "reference_tasks.npz"), **task_files(args.ref_root))
    np.savez_compressed(os.path.join(HERE, "reference_sets.npz"), **synthetic_sets())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
