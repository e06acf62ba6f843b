"""The CPU oracle (oracle/gpw_oracle.c) against the reference's own fixtures and
outputs.  These pins are what every GPU parity test leans on."""
import numpy as np
import pytest

from golden_io import SET_NAMES, TASK_NAMES, load_set, load_task, rel_l2, task_as_workload
from libgpw_gb300 import tasks as T


@pytest.mark.parametrize("name", TASK_NAMES)
def test_task_file_pinned_values(oracle_lib, name):
    """The values each reference task file stores (grid_base_ref_replay.cc:260-272
    compares the same ones) are reproduced, and so is the reference's full grid."""
    d = load_task(name)
    grid = np.zeros((d["ngrid"][2], d["ngrid"][1], d["ngrid"][0]))
    assert oracle_lib.collocate(d, grid) == 0
    gv = d["grid_values"]
    scale = max(np.abs(d["grid_ref"]).max(), 1e-300)
    for z, y, x, v in gv:
        assert abs(grid[int(z), int(y), int(x)] - v) <= 1e-12 * scale
    assert rel_l2(grid, d["grid_ref"]) <= (1e-11 if not d["use_ortho"] else 1e-13)
    # pinned counts: the writer only visits the x = 0 plane (grid_base_ref_c.cc:1160)
    expected = {"collocate_ortho_density": 388, "collocate_general_tau": 108}.get(name, 0)
    assert len(gv) == expected


@pytest.mark.parametrize("name", TASK_NAMES)
def test_task_file_batch_path(oracle_lib, name):
    """The same fixtures through the batch entry (gpw_task + explicit sphere table)."""
    d = load_task(name)
    wl = task_as_workload(d)
    grids = oracle_lib.batch(wl)
    assert rel_l2(grids[0], d["grid_ref"]) <= (1e-11 if not d["use_ortho"] else 1e-13)


@pytest.mark.parametrize("name", SET_NAMES)
def test_sets_match_reference(oracle_lib, name):
    """Seeded pair sets: the oracle's grids against the reference's full grids.
    General-cell tolerance is looser because the reference's row exponential
    recurrence (grid_base_ref_c.cc:816-834) drifts to ~2e-12."""
    wl, grids_ref, V, hab_ref = load_set(name)
    grids = oracle_lib.batch(wl)
    tol = 1e-11 if name.startswith("general") else 1e-13
    for g, r in zip(grids, grids_ref):
        assert rel_l2(g, r) <= tol
    if hab_ref is not None:
        hab = oracle_lib.batch(wl, V=V)
        assert np.abs(hab - hab_ref).max() <= 1e-12 * max(np.abs(hab_ref).max(), 1.0)


@pytest.mark.parametrize("name", ["ortho_rho", "ortho_tau", "general_rho", "general_tau"])
def test_adjoint_identity(oracle_lib, name):
    """<V, collocate(P)> == sum P * integrate(V): integrate is the adjoint."""
    wl, _, _, _ = load_set(name)
    V = wl.potentials(seed=7)
    grids = oracle_lib.batch(wl)
    hab = oracle_lib.batch(wl, V=V)
    lhs = sum(float(np.sum(g * v)) for g, v in zip(grids, V))
    rhs = float(np.sum(wl.pab * hab))
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + np.sqrt(sum(float(np.sum(g * g)) for g in grids)))


def test_threads_match_serial(oracle_lib):
    wl, _, _, _ = load_set("ortho_rho")
    g1 = oracle_lib.batch(wl, nthreads=1)
    g4 = oracle_lib.batch(wl, nthreads=4)
    assert rel_l2(g4[0], g1[0]) <= 1e-14


def test_sphere_rule_shape(oracle_lib):
    """Rule lists are well formed, mirror-symmetric cubes inside [lb_cube, ub_cube]."""
    rng = np.random.default_rng(0)
    for _ in range(50):
        h = rng.uniform(0.05, 0.5, size=3)
        r = float(rng.uniform(0.01, 6.0))
        lb, ub, sb = oracle_lib.sphere_bounds(r, np.diag(h))
        assert np.all(ub == 1 - lb)
        kgmin = sb[0]
        assert kgmin == lb[2]
        pos = 1
        for kg in range(kgmin, 1):
            jg = sb[pos]; pos += 1
            assert jg >= lb[1]
            for _j in range(jg, 1):
                assert sb[pos] >= lb[0]
                pos += 1
        assert pos == sb.size


def test_reference_direct(oracle_lib):
    """Where the reference library was built here, compare on fresh random pairs."""
    if not oracle_lib.ref_available():
        pytest.skip("reference library not built on this machine")
    wl = T.synthetic("direct", 12, 4, (0.1, 50.0), 9.0, [(18, 18, 18)], seed=99)
    for i in range(wl.ntasks):
        d = oracle_lib.task_dict(wl, i)
        a = np.zeros(T.grid_shape(wl.levels[0])); b = np.zeros_like(a)
        oracle_lib.collocate(d, a, use_ref=True)
        oracle_lib.collocate(d, b)
        assert rel_l2(b, a) <= 1e-13


@pytest.mark.parametrize("cfg,npairs,tol", [(1, 16, 1e-13), (2, 24, 1e-13), (3, 12, 1e-11), (5, 24, 1e-13)])
def test_reference_on_benchmark_workloads(oracle_lib, cfg, npairs, tol):
    """The restatement against the reference's own collocate, pair by pair, on
    random pairs of the benchmark workloads (their own exponent, radius, l and
    cell distributions: multigrid levels, the general cell's wrapping cubes, the
    256^3 grid), and the reference's -DNDEBUG build (the one bench.py
    --ref-calibration times) against its parity build.  General cells: the
    reference's row recurrence drifts up to ~2e-12 from exact exponentials."""
    if not oracle_lib.ref_available():
        pytest.skip("reference library not built on this machine")
    wl = T.config(cfg, npairs=2000 if cfg in (2, 5) else None, seed=31 + cfg)
    rng = np.random.default_rng(cfg)
    for i in rng.choice(wl.ntasks, size=npairs, replace=False):
        d = oracle_lib.task_dict(wl, int(i))
        lvl = wl.levels[int(wl.tasks[int(i)]["level"])]
        ref, nd, port = (np.zeros(T.grid_shape(lvl)) for _ in range(3))
        assert oracle_lib.collocate(d, ref, use_ref=True) == 0
        assert oracle_lib.collocate(d, nd, use_ref="ndebug") == 0
        assert oracle_lib.collocate(d, port) == 0
        assert np.array_equal(nd, ref)
        assert rel_l2(port, ref) <= tol


@pytest.mark.parametrize("name", TASK_NAMES)
def test_task_file_writer_round_trip(oracle_lib, name, tmp_path):
    """write_task_file writes the reference's task lines with every nonzero grid
    value (the reference's dump loop visits x = 0 only): read back, the fields
    are identical, the file pins the reference's whole grid, and the oracle
    reproduces it from the file alone."""
    d = load_task(name)
    path = str(tmp_path / (name + ".task"))
    n = T.write_task_file(path, d, d["grid_ref"])
    assert n == int(np.count_nonzero(d["grid_ref"])) > 0
    r = T.read_task_file(path)
    for k in ("compute_tau", "use_ortho", "la_max", "la_min", "lb_max", "lb_min", "lmax", "nspheres",
              "maxco", "o1", "o2", "zeta", "zetb", "rscale", "radius"):
        assert r[k] == d[k], k
    for k in ("dh", "dh_inv", "ra", "rab", "npts", "ngrid", "lb_grid", "periodic", "sphere_bounds", "pab"):
        assert np.array_equal(np.asarray(r[k]), np.asarray(d[k])), k
    if d["use_ortho"]:
        assert np.array_equal(r["lb_cube"], d["lb_cube"]) and np.array_equal(r["ub_cube"], d["ub_cube"])
    pinned = np.zeros_like(d["grid_ref"])
    gv = r["grid_values"]
    pinned[gv[:, 0].astype(int), gv[:, 1].astype(int), gv[:, 2].astype(int)] = gv[:, 3]
    assert np.array_equal(pinned, d["grid_ref"])
    grid = np.zeros_like(d["grid_ref"])
    assert oracle_lib.collocate(r, grid) == 0
    assert rel_l2(grid, d["grid_ref"]) <= (1e-11 if not d["use_ortho"] else 1e-13)


@pytest.mark.parametrize("name", TASK_NAMES)
def test_task_file_writer_read_by_reference(oracle_lib, name, tmp_path):
    """Files from write_task_file pass the reference's own reader and replay
    (grid_collocate_replay, grid_base_ref_replay.cc:18-274, built from the
    reference sources into oracle/_ref): it parses every line with its asserts,
    recollocates the task and finds the pinned values it compares equal.  Run in
    a child process, since a reader assert aborts."""
    import os
    import subprocess
    import sys

    from oracle import oracle as O

    if not O.ref_available():
        pytest.skip("the reference library is built only where the reference sources are")
    d = load_task(name)
    if not d["use_ortho"]:
        # the reference's replay prints ub_cube[0] of a general-cell task, whose
        # cube it has set to NULL (grid_base_ref_replay.cc:226): it crashes on
        # the reference's own general-cell files as well
        pytest.skip("the reference's replay dereferences the absent cube of general-cell tasks")
    path = str(tmp_path / (name + ".task"))
    T.write_task_file(path, d, d["grid_ref"])
    lib = os.path.join(os.path.dirname(O.__file__), "_ref", "libgpwref.so")
    code = ("import ctypes, sys; L = ctypes.CDLL(sys.argv[1]); L.gpwref_replay.restype = ctypes.c_double; "
            "print('MAXDIFF', L.gpwref_replay(sys.argv[2].encode(), 1))")
    r = subprocess.run([sys.executable, "-c", code, lib, path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    diff = float([ln for ln in r.stdout.splitlines() if ln.startswith("MAXDIFF")][-1].split()[1])
    assert diff <= 1e-12 * max(float(np.abs(d["grid_ref"]).max()), 1e-300)
