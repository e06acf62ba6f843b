"""TEST INFRASTRUCTURE ONLY: ctypes bindings of the CPU oracle.

  * liboracle.so       -- the C restatement in gpw_oracle.c (always built)
  * _ref/libgpwref.so  -- the reference's own grid_collocate_pgf_product_rspace
                          (src/lib/grid_base_ref_c.cc:1018), built from the
                          reference sources by ref/Makefile where they exist

Only tests, the smoke check and the CPU-baseline leg of bench.py use this
module; the library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_ref = None
_ref_ndebug = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

_ARGS = [C.c_int] * 6 + [C.c_double] * 3 + [_dp, _dp, _dp, _dp, _ip, _ip, _ip, _ip, C.c_int,
                                            C.c_double, _ip, _ip, C.c_int, _ip, C.c_int, C.c_int,
                                            C.c_int, _dp, _dp]


def build(quiet: bool = True, ref_src: str | None = None) -> None:
    """Compiles liboracle.so, and _ref/libgpwref.so from the reference's src/lib
    directory when one is given (ref_src, or the GPW_REFERENCE_SRC environment
    variable) and holds the reference sources."""
    ref_src = ref_src or os.environ.get("GPW_REFERENCE_SRC", "")
    cmd = ["make", "-s", "-C", HERE, "all"] + ([f"REF={ref_src}"] if ref_src else [])
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL if quiet else None)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.gpwo_collocate.argtypes = _ARGS
        L.gpwo_collocate.restype = C.c_int
        L.gpwo_integrate.argtypes = _ARGS
        L.gpwo_integrate.restype = C.c_int
        L.gpwo_sphere_bounds.argtypes = [C.c_double, _dp, _ip, _ip, _ip, C.c_int]
        L.gpwo_sphere_bounds.restype = C.c_int
        L.gpwo_batch.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int,
                                 C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p),
                                 C.POINTER(C.c_void_p), C.c_void_p, C.c_int64, C.c_int]
        L.gpwo_batch.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libgpwref.so"))


def ref(ndebug: bool = False):
    """The reference's own collocate: built with its asserts (parity), or with
    -DNDEBUG as the reference's Makefile builds its library (timing)."""
    global _ref, _ref_ndebug
    if (_ref_ndebug if ndebug else _ref) is None:
        L = C.CDLL(os.path.join(HERE, "_ref", "libgpwref_ndebug.so" if ndebug else "libgpwref.so"))
        L.gpwref_collocate.argtypes = _ARGS
        L.gpwref_collocate.restype = C.c_int
        if ndebug:
            _ref_ndebug = L
        else:
            _ref = L
    return _ref_ndebug if ndebug else _ref


def _i3(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.int32).reshape(3))


def _args(t: dict, pab_or_v, out):
    sb = np.ascontiguousarray(np.asarray(t.get("sphere_bounds", np.zeros(1)), dtype=np.int32))
    if sb.size == 0:
        sb = np.zeros(1, dtype=np.int32)
    return (int(t["compute_tau"]), int(t["use_ortho"]), int(t["la_max"]), int(t["la_min"]),
            int(t["lb_max"]), int(t["lb_min"]), float(t["zeta"]), float(t["zetb"]),
            float(t["rscale"]), np.ascontiguousarray(t["dh"], dtype=np.float64).reshape(9),
            np.ascontiguousarray(t["dh_inv"], dtype=np.float64).reshape(9),
            np.ascontiguousarray(t["ra"], dtype=np.float64), np.ascontiguousarray(t["rab"], dtype=np.float64),
            _i3(t["npts"]), _i3(t["ngrid"]), _i3(t["lb_grid"]), _i3(t["periodic"]), int(t["lmax"]),
            float(t["radius"]), _i3(t.get("lb_cube", (0, 0, 0))), _i3(t.get("ub_cube", (0, 0, 0))),
            int(t.get("nspheres", sb.size)), sb, int(t["maxco"]), int(t["o1"]), int(t["o2"]),
            np.ascontiguousarray(pab_or_v, dtype=np.float64).reshape(-1), out)


def collocate(t: dict, grid: np.ndarray, use_ref: bool | str = False) -> int:
    """grid += rho of one task (dict in the task-v1 vocabulary): the restatement,
    the reference (use_ref=True) or its -DNDEBUG build (use_ref="ndebug")."""
    assert grid.dtype == np.float64 and grid.flags.c_contiguous
    f = ref(ndebug=use_ref == "ndebug").gpwref_collocate if use_ref else lib().gpwo_collocate
    return f(*_args(t, t["pab"], grid.reshape(-1)))


def integrate(t: dict, V: np.ndarray, hab: np.ndarray) -> int:
    """hab (maxco x maxco) += <V | basis> of one task (the adjoint of collocate)."""
    assert hab.dtype == np.float64 and hab.flags.c_contiguous
    return lib().gpwo_integrate(*_args(t, V, hab.reshape(-1)))


def sphere_bounds(radius: float, dh) -> tuple:
    """The library's cube rule restated: (lb_cube, ub_cube, sphere_bounds)."""
    dh9 = np.ascontiguousarray(np.asarray(dh, dtype=np.float64).reshape(9))
    lb = np.zeros(3, dtype=np.int32)
    ub = np.zeros(3, dtype=np.int32)
    buf = np.zeros(1, dtype=np.int32)
    n = lib().gpwo_sphere_bounds(radius, dh9, lb, ub, buf, 1)
    if n < 0:
        buf = np.zeros(-n, dtype=np.int32)
        n = lib().gpwo_sphere_bounds(radius, dh9, lb, ub, buf, -n)
    if n <= 0:
        raise ValueError("bad radius / dh")
    return lb, ub, buf[:n]


def batch(wl, V=None, nthreads: int = 1, tasks=None):
    """Runs a Workload on the CPU.  Without V: returns the collocated grids.
    With V (list per level): returns hab (same layout as wl.pab)."""
    from libgpw_gb300.tasks import grid_shape

    tasks = wl.tasks if tasks is None else tasks
    tasks = np.ascontiguousarray(tasks)
    lv = wl.level_array()
    st = wl.sphere_table if wl.sphere_table is not None else np.zeros(1, dtype=np.int32)
    st = np.ascontiguousarray(st, dtype=np.int32)
    nl = len(wl.levels)
    if V is None:
        grids = [np.zeros(grid_shape(g)) for g in wl.levels]
        gp = (C.c_void_p * nl)(*[g.ctypes.data for g in grids])
        s = lib().gpwo_batch(0, int(wl.compute_tau), tasks.ctypes.data, tasks.shape[0], lv.ctypes.data,
                             nl, st.ctypes.data, wl.pab.ctypes.data, gp, None, None, 0, nthreads)
        if s:
            raise RuntimeError(f"oracle batch status {s}")
        return grids
    Vc = [np.ascontiguousarray(v, dtype=np.float64) for v in V]
    vp = (C.c_void_p * nl)(*[v.ctypes.data for v in Vc])
    hab = np.zeros_like(wl.pab)
    s = lib().gpwo_batch(1, int(wl.compute_tau), tasks.ctypes.data, tasks.shape[0], lv.ctypes.data, nl,
                         st.ctypes.data, None, None, vp, hab.ctypes.data, hab.size, nthreads)
    if s:
        raise RuntimeError(f"oracle batch status {s}")
    return hab


def task_dict(wl, i: int, level=None) -> dict:
    """One task of a Workload in the reference's call vocabulary, with a square
    maxco x maxco block (o1 = o2 = 0) as grid_collocate_pgf_product_rspace wants,
    and the library's cube rule for orthorhombic levels."""
    from libgpw_gb300.tasks import ncoset

    T = wl.tasks[i]
    g = wl.levels[int(T["level"])] if level is None else level
    la, lb = int(T["la_max"]), int(T["lb_max"])
    m = max(ncoset(la), ncoset(lb))
    if wl.compute_tau:
        m = max(m, ncoset(la + 1), ncoset(lb + 1))
    pab = np.zeros((m, m))
    la_min, lb_min = int(T["la_min"]), int(T["lb_min"])
    for jco in range(ncoset(lb_min - 1), ncoset(lb)):
        for ico in range(ncoset(la_min - 1), ncoset(la)):
            idx = int(T["pab_offset"]) + (int(T["o2"]) + jco) * int(T["maxco"]) + int(T["o1"]) + ico
            pab[jco, ico] = wl.pab[idx]
    d = dict(compute_tau=wl.compute_tau, use_ortho=int(g["ortho"]), la_max=la, la_min=la_min,
             lb_max=lb, lb_min=lb_min, zeta=float(T["zeta"]), zetb=float(T["zetb"]),
             rscale=float(T["rscale"]), dh=np.array(g["dh"]), dh_inv=np.array(g["dh_inv"]),
             ra=np.array(T["ra"]), rab=np.array(T["rab"]), npts=np.array(g["npts"]),
             ngrid=np.array(g["ngrid"]), lb_grid=np.array(g["lb_grid"]),
             periodic=np.array(g["periodic"]), lmax=max(la, lb) + 1,
             radius=float(T["radius"]), maxco=m, o1=0, o2=0, pab=pab)
    if int(g["ortho"]):
        lbc, ubc, sb = sphere_bounds(float(T["radius"]), g["dh"])
        d.update(lb_cube=lbc, ub_cube=ubc, sphere_bounds=sb, nspheres=sb.size)
    else:
        d.update(lb_cube=np.zeros(3, np.int32), ub_cube=np.zeros(3, np.int32),
                 sphere_bounds=np.zeros(1, np.int32), nspheres=0)
    return d
