"""Loads the committed golden fixtures (tests/golden/*.npz) as Workloads."""
import os

import numpy as np

from libgpw_gb300 import tasks as T

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SET_NAMES = ["ortho_rho", "ortho_tau", "ortho_int", "general_rho", "general_tau", "general_int",
             "ortho_nonperiodic"]
TASK_NAMES = ["collocate_general_density", "collocate_general_tau", "collocate_ortho_density",
              "collocate_ortho_tau"]


def load_set(name):
    z = np.load(os.path.join(GOLDEN, "reference_sets.npz"))
    p = name + "/"
    levels = [z[p + "levels"][i] for i in range(z[p + "levels"].shape[0])]
    wl = T.Workload(name, z[p + "tasks"].copy(), levels, z[p + "pab"].copy(),
                    compute_tau=int(z[p + "compute_tau"]))
    grids = [z[p + f"grid_ref_{l}"] for l in range(len(levels))]
    V = hab = None
    if p + "hab_ref" in z.files:
        V = [z[p + f"V_{l}"] for l in range(len(levels))]
        hab = z[p + "hab_ref"]
    return wl, grids, V, hab


def load_task(name):
    z = np.load(os.path.join(GOLDEN, "reference_tasks.npz"))
    p = name + "/"
    d = {k[len(p):]: z[k] for k in z.files if k.startswith(p)}
    for k in ("compute_tau", "use_ortho", "la_max", "la_min", "lb_max", "lb_min", "lmax",
              "nspheres", "maxco", "o1", "o2"):
        d[k] = int(d[k])
    for k in ("zeta", "zetb", "rscale", "radius"):
        d[k] = float(d[k])
    return d


def task_as_workload(d):
    """A task-v1 fixture as a one-task Workload: cube from its own sphere list."""
    g = np.zeros((), dtype=T.GRID_DTYPE)
    g["npts"], g["ngrid"], g["lb_grid"], g["periodic"] = d["npts"], d["ngrid"], d["lb_grid"], d["periodic"]
    g["dh"], g["dh_inv"], g["ortho"] = d["dh"], d["dh_inv"], d["use_ortho"]
    t = np.zeros(1, dtype=T.TASK_DTYPE)
    for k in ("zeta", "zetb", "rscale", "radius", "la_max", "la_min", "lb_max", "lb_min", "maxco", "o1", "o2"):
        t[k] = d[k]
    t["ra"], t["rab"] = d["ra"], d["rab"]
    t["lb_cube"], t["ub_cube"] = d["lb_cube"], d["ub_cube"]
    t["pab_offset"] = 0
    t["level"] = 0
    t["sphere_offset"] = 0 if d["use_ortho"] else -1
    table = np.asarray(d["sphere_bounds"], dtype=np.int32)
    if table.size == 0:
        table = np.zeros(1, dtype=np.int32)
    return T.Workload(d.get("name", "task"), t, [g], np.ascontiguousarray(d["pab"]).reshape(-1).copy(),
                      compute_tau=d["compute_tau"], sphere_table=table)


def rel_l2(a, b):
    a = np.asarray(a); b = np.asarray(b)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / n) if n > 0 else float(np.linalg.norm(a - b))
