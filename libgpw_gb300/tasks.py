"""Task and grid descriptions on the host: numpy mirrors of the C structs in
include/gpw.h, the seeded synthetic workloads, and a reader and a writer for
the reference's "Grid collocate task v1" text format.

Reference anchors (mtaillefumier/libgpw):
  * per-call arguments of grid_collocate_pgf_product_rspace -> gpw_task / gpw_grid_desc
    (src/lib/grid_base_ref_c.h:40-67)
  * task v1 format: writer src/lib/grid_base_ref_c.cc:1047-1183,
    reader src/lib/grid_base_ref_replay.cc:18-273.  This reader reads the whole
    file, keeps the cube of general-cell tasks absent instead of dereferencing it,
    and reports which grid values the file pins (the writer only visits the x=0
    plane, grid_base_ref_c.cc:1160,1171).  write_task_file writes the same lines
    in the same order but pins every nonzero grid value.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

NCOSET = [1, 4, 10, 20, 35, 56, 84, 120, 165, 220, 286, 364, 455, 560]

TASK_DTYPE = np.dtype(
    [
        ("zeta", "<f8"), ("zetb", "<f8"), ("rscale", "<f8"),
        ("ra", "<f8", (3,)), ("rab", "<f8", (3,)), ("radius", "<f8"),
        ("pab_offset", "<i8"), ("sphere_offset", "<i8"),
        ("la_max", "<i4"), ("la_min", "<i4"), ("lb_max", "<i4"), ("lb_min", "<i4"),
        ("level", "<i4"), ("maxco", "<i4"), ("o1", "<i4"), ("o2", "<i4"),
        ("lb_cube", "<i4", (3,)), ("ub_cube", "<i4", (3,)),
    ],
    align=True,
)
assert TASK_DTYPE.itemsize == 152

GRID_DTYPE = np.dtype(
    [
        ("npts", "<i4", (3,)), ("ngrid", "<i4", (3,)), ("lb_grid", "<i4", (3,)),
        ("periodic", "<i4", (3,)), ("dh", "<f8", (3, 3)), ("dh_inv", "<f8", (3, 3)),
        ("ortho", "<i4"), ("pad_", "<i4"),
    ],
    align=True,
)
assert GRID_DTYPE.itemsize == 200


def ncoset(l: int) -> int:
    return 0 if l < 0 else NCOSET[l]


def coset(lx: int, ly: int, lz: int) -> int:
    """Cartesian index, the coset order of grid_base_ref_c.cc:39-46."""
    l = lx + ly + lz
    if l == 0:
        return 0
    return NCOSET[l - 1] + ((l - lx) * (l - lx + 1)) // 2 + lz


def make_grid(cell, npts, ortho=True, periodic=(1, 1, 1), ngrid=None, lb_grid=(0, 0, 0)):
    """One grid level.  `cell` is a 3x3 matrix whose rows are the lattice vectors
    (or a scalar / 3-vector for an orthorhombic box).  dh rows are the step vectors."""
    cell = np.asarray(cell, dtype=np.float64)
    if cell.ndim == 0:
        cell = np.eye(3) * float(cell)
    elif cell.ndim == 1:
        cell = np.diag(cell)
    npts = np.asarray(npts, dtype=np.int32).reshape(3)
    g = np.zeros((), dtype=GRID_DTYPE)
    g["npts"] = npts
    g["ngrid"] = npts if ngrid is None else np.asarray(ngrid, dtype=np.int32)
    g["lb_grid"] = lb_grid
    g["periodic"] = periodic
    dh = cell / npts[:, None]
    g["dh"] = dh
    g["dh_inv"] = np.linalg.inv(dh)
    g["ortho"] = 1 if ortho else 0
    return g


def grid_shape(g) -> tuple:
    """numpy shape (z, y, x) of a level's grid array."""
    n = g["ngrid"]
    return (int(n[2]), int(n[1]), int(n[0]))


def radius_rule(zetp, eps=1e-10):
    """Cube radius used by the synthetic workloads: exp(-zetp r^2) = eps."""
    return np.sqrt(np.log(1.0 / eps) / np.asarray(zetp, dtype=np.float64))


@dataclass
class Workload:
    """A batch of pairs over one or more grid levels, with density blocks
    (pab) and potentials (V) as the benchmarks and tests use them."""

    name: str
    tasks: np.ndarray                       # TASK_DTYPE[n]
    levels: list                            # GRID_DTYPE scalars
    pab: np.ndarray                         # float64[extent]
    compute_tau: int = 0                    # gpw_function: 0 rho, 1 tau, 2-4 ADBmDAB x/y/z
    sphere_table: np.ndarray | None = None  # int32, CP2K-format lists
    meta: dict = field(default_factory=dict)

    @property
    def ntasks(self) -> int:
        return int(self.tasks.shape[0])

    def level_array(self) -> np.ndarray:
        return np.array([np.asarray(l) for l in self.levels], dtype=GRID_DTYPE).reshape(-1)

    def potentials(self, seed: int = 1) -> list:
        rng = np.random.default_rng(seed)
        return [rng.uniform(-1.0, 1.0, size=grid_shape(g)) for g in self.levels]


def _blocks(rng, la, lb):
    """Compact per-shell blocks: block element P(jco, ico) of shells la x lb lives
    at pab[off + (o2 + jco) * maxco + (o1 + ico)] with o1 = -ncoset(la-1),
    o2 = -ncoset(lb-1), maxco = shell size of a."""
    nsa = (la + 1) * (la + 2) // 2
    nsb = (lb + 1) * (lb + 2) // 2
    sizes = nsa * nsb
    offsets = np.zeros_like(sizes, dtype=np.int64)
    offsets[1:] = np.cumsum(sizes[:-1])
    extent = int(sizes.sum())
    pab = rng.uniform(-1.0, 1.0, size=extent)
    return nsa, offsets, pab


def synthetic(
    name: str,
    npairs: int,
    lmax: int,
    zeta_range,
    cell,
    levels_npts,
    seed: int,
    route=None,
    ortho=True,
    eps=1e-10,
    compute_tau=0,
    lmin: int = 0,
):
    """Seeded synthetic pairs: la, lb uniform in {lmin..lmax} (one Cartesian shell
    per primitive, la_min = la_max), exponents log-uniform in zeta_range, both
    centres uniform in the cell (fractional coordinates), rab the minimum-image
    vector, rscale 1, density blocks uniform in [-1, 1], radius by radius_rule.
    `route(zetp) -> level` picks the grid level (multigrid); default level 0."""
    rng = np.random.default_rng(seed)
    cellm = np.asarray(cell, dtype=np.float64)
    if cellm.ndim == 0:
        cellm = np.eye(3) * float(cellm)
    elif cellm.ndim == 1:
        cellm = np.diag(cellm)
    levels = [make_grid(cellm, n, ortho=ortho) for n in levels_npts]
    la = rng.integers(lmin, lmax + 1, size=npairs)
    lb = rng.integers(lmin, lmax + 1, size=npairs)
    lo, hi = math.log(zeta_range[0]), math.log(zeta_range[1])
    zeta = np.exp(rng.uniform(lo, hi, size=npairs))
    zetb = np.exp(rng.uniform(lo, hi, size=npairs))
    fa = rng.uniform(0.0, 1.0, size=(npairs, 3))
    fb = rng.uniform(0.0, 1.0, size=(npairs, 3))
    df = fb - fa
    df -= np.round(df)
    ra = fa @ cellm
    rab = df @ cellm
    zetp = zeta + zetb
    t = np.zeros(npairs, dtype=TASK_DTYPE)
    t["zeta"], t["zetb"], t["rscale"] = zeta, zetb, 1.0
    t["ra"], t["rab"] = ra, rab
    t["radius"] = radius_rule(zetp, eps)
    t["la_max"], t["la_min"], t["lb_max"], t["lb_min"] = la, la, lb, lb
    t["level"] = 0 if route is None else np.asarray(route(zetp), dtype=np.int32)
    nsa, offsets, pab = _blocks(rng, la, lb)
    t["pab_offset"] = offsets
    t["maxco"] = nsa
    t["o1"] = -np.array([ncoset(int(x) - 1) for x in la], dtype=np.int32)
    t["o2"] = -np.array([ncoset(int(x) - 1) for x in lb], dtype=np.int32)
    t["sphere_offset"] = -1
    return Workload(name, t, levels, pab, compute_tau=compute_tau,
                    meta={"seed": seed, "eps": eps, "zeta_range": list(zeta_range)})


def multigrid_route(zetp):
    """Level routing of the 3-level multigrid workload: zetp > 20 -> level 0 (finest),
    2 < zetp <= 20 -> level 1, else level 2 (coarsest)."""
    zetp = np.asarray(zetp)
    return np.where(zetp > 20.0, 0, np.where(zetp > 2.0, 1, 2)).astype(np.int32)


def lattice_15(rng_seed=3, length=15.0):
    """Lattice vectors of length `length`, angles uniform in [60, 90] degrees."""
    rng = np.random.default_rng(rng_seed)
    al, be, ga = np.radians(rng.uniform(60.0, 90.0, size=3))
    a = np.array([length, 0.0, 0.0])
    b = np.array([length * math.cos(ga), length * math.sin(ga), 0.0])
    cx = math.cos(be)
    cy = (math.cos(al) - math.cos(be) * math.cos(ga)) / math.sin(ga)
    cz = math.sqrt(max(1.0 - cx * cx - cy * cy, 1e-12))
    c = length * np.array([cx, cy, cz])
    return np.stack([a, b, c])


# Workloads of the benchmark suite (seeded; no dataset is involved).
def config(idx: int, npairs: int | None = None, seed: int | None = None) -> Workload:
    """idx 1..5: the five workloads; npairs overrides the pair count (smaller
    parity cases with the same distributions)."""
    if idx == 1:
        return synthetic("pairs1k_l2_64cubed", npairs or 1000, 2, (0.1, 50.0), 10.0, [(64, 64, 64)],
                         seed or 101)
    if idx == 2:
        return synthetic("pairs200k_l3_multigrid180", npairs or 200_000, 3, (0.05, 200.0), 20.0,
                         [(180,) * 3, (90,) * 3, (45,) * 3], seed or 102, route=multigrid_route)
    if idx == 3:
        return synthetic("pairs50k_l4_general128", npairs or 50_000, 4, (0.1, 100.0), lattice_15(),
                         [(128,) * 3], seed or 103, ortho=False)
    if idx == 4:
        return synthetic("pairs20k_l2_96cubed", npairs or 20_000, 2, (0.1, 50.0), 12.0, [(96,) * 3],
                         seed or 104)
    if idx == 5:
        return synthetic("pairs1M_l4_256cubed", npairs or 1_000_000, 4, (0.05, 200.0), 30.0,
                         [(256,) * 3], seed or 105)
    raise ValueError(idx)


# ---------------------------------------------------------------------------
# Task v1 files
def read_task_file(path: str) -> dict:
    """Parses a "#Grid collocate task v1" file into a dict of numpy values:
    scalar fields, dh/dh_inv (3x3), sphere_bounds (dense, nspheres long),
    pab (maxco x maxco) and the listed grid values (z, y, x, value)."""
    with open(path) as fh:
        lines = [ln.rstrip("\n") for ln in fh]
    if not lines or lines[0] != "#Grid collocate task v1":
        raise ValueError(f"{path}: not a task v1 file")
    out: dict = {"dh": np.zeros((3, 3)), "dh_inv": np.zeros((3, 3))}
    grid_vals = []
    pab_vals = {}
    sb_vals = {}
    for ln in lines[1:]:
        if ln == "#THE_END":
            break
        parts = ln.split()
        key = parts[0]
        if key in ("dh", "dh_inv"):
            out[key][int(parts[1])] = [float(x) for x in parts[2:5]]
        elif key in ("ra", "rab"):
            out[key] = np.array([float(x) for x in parts[1:4]])
        elif key in ("npts", "ngrid", "lb_grid", "periodic", "lb_cube", "ub_cube"):
            out[key] = np.array([int(x) for x in parts[1:4]], dtype=np.int32)
        elif key in ("zeta", "zetb", "rscale", "radius"):
            out[key] = float(parts[1])
        elif key == "sphere_bounds":
            sb_vals[int(parts[1])] = int(parts[2])
        elif key == "pab":
            pab_vals[(int(parts[1]), int(parts[2]))] = float(parts[3])
        elif key == "grid":
            grid_vals.append((int(parts[1]), int(parts[2]), int(parts[3]), float(parts[4])))
        else:
            out[key] = int(parts[1])
    ns = out["nspheres"]
    sb = np.zeros(ns, dtype=np.int32)
    for i, v in sb_vals.items():
        sb[i] = v
    out["sphere_bounds"] = sb
    m = out["maxco"]
    pab = np.zeros((m, m))
    for (i, j), v in pab_vals.items():
        pab[i, j] = v
    out["pab"] = pab
    out["grid_values"] = np.array(grid_vals, dtype=np.float64).reshape(-1, 4)
    if "lb_cube" not in out:
        out["lb_cube"] = np.zeros(3, dtype=np.int32)
        out["ub_cube"] = np.zeros(3, dtype=np.int32)
    return out


_TASK_INT_KEYS = ("compute_tau", "use_ortho", "la_max", "la_min", "lb_max", "lb_min")


def write_task_file(path: str, task: dict, grid=None) -> int:
    """Writes a "#Grid collocate task v1" file: the lines of the reference's dump
    (grid_base_ref_c.cc:1105-1179, same keys and order), doubles with 17
    significant digits (exact round trip), and every nonzero value of `grid`
    (the task's own contribution, shape (ngrid[2], ngrid[1], ngrid[0])) as
    "grid z y x value" - all planes, where the reference's loop visits x = 0 only.
    `task` holds the fields read_task_file returns.  Returns the number of grid
    lines written."""

    def f(x):
        return "%.16e" % float(x)

    def v3(key, conv):
        return f"{key} " + " ".join(conv(x) for x in np.asarray(task[key]).reshape(3))

    lines = ["#Grid collocate task v1"]
    lines += [f"{k} {int(task[k])}" for k in _TASK_INT_KEYS]
    lines += [f"{k} {f(task[k])}" for k in ("zeta", "zetb", "rscale")]
    dh, dhi = np.asarray(task["dh"]).reshape(3, 3), np.asarray(task["dh_inv"]).reshape(3, 3)
    lines += [f"dh {i} " + " ".join(f(x) for x in dh[i]) for i in range(3)]
    lines += [f"dh_inv {i} " + " ".join(f(x) for x in dhi[i]) for i in range(3)]
    lines += [v3("ra", f), v3("rab", f)]
    lines += [v3(k, lambda x: str(int(x))) for k in ("npts", "ngrid", "lb_grid", "periodic")]
    lines += [f"lmax {int(task['lmax'])}", f"radius {f(task['radius'])}"]
    if int(task["use_ortho"]):
        lines += [v3(k, lambda x: str(int(x))) for k in ("lb_cube", "ub_cube")]
    # the first nspheres entries, as the reference's dump loop (i < nspheres)
    sb = np.asarray(task["sphere_bounds"], dtype=np.int64).reshape(-1)[: int(task["nspheres"])]
    lines += [f"nspheres {int(task['nspheres'])}", f"nspheres_nonzero {int(np.count_nonzero(sb))}"]
    lines += [f"sphere_bounds {i} {int(v)}" for i, v in enumerate(sb) if v != 0]
    lines += [f"{k} {int(task[k])}" for k in ("maxco", "o1", "o2")]
    pab = np.asarray(task["pab"], dtype=np.float64)
    m = int(task["maxco"])
    lines += [f"pab {i} {j} {f(pab[i, j])}" for i in range(m) for j in range(m)]
    nz = np.argwhere(grid != 0.0) if grid is not None else np.zeros((0, 3), dtype=np.int64)
    lines.append(f"ngrid_nonzero {len(nz)}")
    lines += [f"grid {z} {y} {x} {f(grid[z, y, x])}" for z, y, x in nz]
    lines.append("#THE_END")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    return len(nz)
