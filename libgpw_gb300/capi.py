"""ctypes bindings of the C ABI (include/gpw.h) and a thin host-side layer.

The device buffers are torch tensors (plumbing only: device memory and the
stream); all computation happens in libgpw_gb300/_lib/libgpw_gb300.so.  There
is no CPU fallback: if the library is missing or a call fails, an exception is
raised.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

from . import tasks as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgpw_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "gpw.h")

PREC = {"fp64": 0, "mixed": 1}
STATUS = {0: "GPW_SUCCESS", 1: "GPW_ERR_INVALID_ARG", 2: "GPW_ERR_CUDA", 3: "GPW_ERR_OUT_OF_WINDOW",
          4: "GPW_ERR_UNSUPPORTED", 5: "GPW_ERR_NO_DEVICE", 6: "GPW_ERR_ALLOC", 7: "GPW_ERR_TIMEOUT"}

_lib = None


class GpwError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def header_functions() -> list:
    """Names of every function include/gpw.h declares."""
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(gpw_[a-z_0-9]+)\s*\(", src, re.M)))


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
    sig = {
        "gpw_last_error_string": ([], C.c_char_p),
        "gpw_version": ([], C.c_char_p),
        "gpw_sphere_bounds": ([dbl, vp, vp, vp, vp, i32], i32),
        "gpw_plan_create": ([C.POINTER(vp), i32, vp, i32], i32),
        "gpw_plan_destroy": ([vp], i32),
        "gpw_taskset_create": ([vp, vp, i64, i32, vp, i64, C.POINTER(vp)], i32),
        "gpw_taskset_destroy": ([vp], i32),
        "gpw_taskset_pab_extent": ([vp], i64),
        "gpw_collocate": ([vp, i32, vp, vp, vp], i32),
        "gpw_integrate": ([vp, i32, vp, vp, vp], i32),
        "gpw_backward": ([vp, vp, vp, vp, vp, vp, vp, vp, vp], i32),
        "gpw_taskset_check": ([vp, vp], i32),
        "gpw_taskset_update_geometry": ([vp, vp, vp, vp, vp, vp], i32),
        "gpw_collocate_host": ([vp, i32, vp, vp], i32),
        "gpw_integrate_host": ([vp, i32, vp, vp], i32),
        "gpw_collocate_pgf_product_rspace": ([i32] * 6 + [dbl] * 3 + [vp] * 8 + [i32, dbl, vp, vp, i32, vp, i32,
                                                                                i32, i32, vp, vp], i32),
        "gpw_taskset_profile": ([vp, i32], i32),
        "gpw_taskset_bins": ([vp, C.POINTER(i64), C.POINTER(i64)], i32),
        "gpw_taskset_stats": ([vp, C.POINTER(dbl), C.POINTER(i64), C.POINTER(i64)], i32),
        "gpw_taskset_set_tiles": ([vp, vp], i32),
        "gpw_taskset_get_tiles": ([vp, vp], i32),
        "gpw_taskset_autotune": ([vp, vp, vp, vp, vp], i32),
        "gpw_selftest_tensorcore": ([C.POINTER(i64)], i32),
        "gpw_selftest_ff_exp": ([i64, C.POINTER(dbl), C.POINTER(dbl)], i32),
        "gpw_collocate_noalloc": ([vp, vp, i32, i32, vp, vp, vp], i32),
        "gpw_collocate_core": ([vp, i32, vp, vp, i32, vp, vp], i32),
        "gpw_integrate_core": ([vp, i32, vp, i32, vp, vp, vp], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def last_error() -> str:
    return lib().gpw_last_error_string().decode()


def check(status: int, what: str = "") -> None:
    if status != 0:
        raise GpwError(status, f"{what}: {last_error()}")


def sphere_bounds(radius: float, dh) -> tuple:
    """The library's cube rule (gpw_sphere_bounds): (lb_cube, ub_cube, list)."""
    dh = np.ascontiguousarray(np.asarray(dh, dtype=np.float64).reshape(3, 3))
    lb = np.zeros(3, np.int32)
    ub = np.zeros(3, np.int32)
    n = lib().gpw_sphere_bounds(float(radius), dh.ctypes.data, lb.ctypes.data, ub.ctypes.data, None, 0)
    if n == 0:
        raise GpwError(1, last_error())
    buf = np.zeros(-n if n < 0 else n, np.int32)
    n = lib().gpw_sphere_bounds(float(radius), dh.ctypes.data, lb.ctypes.data, ub.ctypes.data, buf.ctypes.data,
                                buf.size)
    return lb, ub, buf[:n]


def _stream_handle(stream) -> int | None:
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Plan:
    """Grid levels bound to one device (gpw_plan_create)."""

    def __init__(self, levels, device: int = 0):
        self.levels = [np.asarray(l) for l in levels]
        arr = np.array(self.levels, dtype=T.GRID_DTYPE).reshape(-1)
        self._arr = arr
        h = C.c_void_p()
        check(lib().gpw_plan_create(C.byref(h), len(self.levels), arr.ctypes.data, device), "gpw_plan_create")
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            lib().gpw_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# the collocated function of a task set (enum gpw_function): 0 rho, 1 tau, and
# phi_a d phi_b - d phi_a phi_b along x, y, z
FUNC = {"ab": 0, "dadb": 1, "adbmdab_x": 2, "adbmdab_y": 3, "adbmdab_z": 4}


class TaskSet:
    """Uploaded, sorted and binned pairs (gpw_taskset_create).  compute_tau is
    the gpw_function of the task set (0 / 1: the reference's compute_tau)."""

    def __init__(self, plan: Plan, tasks, compute_tau: int = 0, sphere_table=None):
        self.plan = plan
        self.tasks = np.ascontiguousarray(tasks, dtype=T.TASK_DTYPE)
        tab = None if sphere_table is None else np.ascontiguousarray(sphere_table, dtype=np.int32)
        self._tab = tab
        h = C.c_void_p()
        check(lib().gpw_taskset_create(plan.handle, self.tasks.ctypes.data, self.tasks.shape[0], int(compute_tau),
                                       None if tab is None else tab.ctypes.data, 0 if tab is None else tab.size,
                                       C.byref(h)), "gpw_taskset_create")
        self.handle = h
        self.pab_extent = int(lib().gpw_taskset_pab_extent(h))

    @classmethod
    def from_workload(cls, plan: Plan, wl: "T.Workload"):
        return cls(plan, wl.tasks, wl.compute_tau, wl.sphere_table)

    def close(self):
        if self.handle:
            lib().gpw_taskset_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _ptrs(grids):
        for g in grids:
            assert g.is_cuda and g.dtype.is_floating_point and g.element_size() == 8 and g.is_contiguous()
        return (C.c_void_p * len(grids))(*[g.data_ptr() for g in grids])

    def collocate(self, pab, grids, precision: str = "fp64", stream=None):
        """grids[l] += rho (device tensors, float64)."""
        assert pab.is_cuda and pab.numel() >= self.pab_extent
        check(lib().gpw_collocate(self.handle, PREC[precision], pab.data_ptr(), self._ptrs(grids),
                                  _stream_handle(stream)), "gpw_collocate")

    def integrate(self, grids, hab, precision: str = "fp64", stream=None):
        """hab += <V | basis> (device tensors, float64)."""
        assert hab.is_cuda and hab.numel() >= self.pab_extent
        check(lib().gpw_integrate(self.handle, PREC[precision], self._ptrs(grids), hab.data_ptr(),
                                  _stream_handle(stream)), "gpw_integrate")

    def backward(self, pab, grids, hab=None, dra=None, drb=None, dzeta=None, dzetb=None, stream=None):
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        check(lib().gpw_backward(self.handle, pab.data_ptr(), self._ptrs(grids), p(hab), p(dra), p(drb), p(dzeta),
                                 p(dzetb), _stream_handle(stream)), "gpw_backward")

    def update_geometry(self, ra=None, rab=None, zeta=None, zetb=None, stream=None):
        """New centres / exponents of the same pairs (device tensors in task order;
        None keeps the current values): gpw_taskset_update_geometry."""
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        for t in (ra, rab, zeta, zetb):
            assert t is None or (t.is_cuda and t.dtype.is_floating_point and t.element_size() == 8
                                 and t.is_contiguous())
        check(lib().gpw_taskset_update_geometry(self.handle, p(ra), p(rab), p(zeta), p(zetb),
                                                _stream_handle(stream)), "gpw_taskset_update_geometry")

    def profile(self, enable: bool = True):
        check(lib().gpw_taskset_profile(self.handle, int(enable)), "gpw_taskset_profile")

    def stats(self) -> tuple:
        """(contraction ms, contraction launches, kernel launches) since the last call."""
        ms, nc, nk = C.c_double(), C.c_int64(), C.c_int64()
        check(lib().gpw_taskset_stats(self.handle, C.byref(ms), C.byref(nc), C.byref(nk)), "gpw_taskset_stats")
        return ms.value, nc.value, nk.value

    def bins(self) -> tuple:
        """(tile, pair) items and work units of the tiled path (gpw_taskset_bins)."""
        a, b = C.c_int64(), C.c_int64()
        check(lib().gpw_taskset_bins(self.handle, C.byref(a), C.byref(b)), "gpw_taskset_bins")
        return a.value, b.value

    def check(self, stream=None):
        check(lib().gpw_taskset_check(self.handle, _stream_handle(stream)), "device status")

    # tile shapes of the mixed path (z extent per level: 4 or 8; 0 = a general-cell
    # level on the float-float kernel instead of tiles)
    def set_tiles(self, tile_z):
        tz = np.ascontiguousarray(np.asarray(tile_z, dtype=np.int32).reshape(-1))
        assert tz.size == len(self.plan.levels)
        check(lib().gpw_taskset_set_tiles(self.handle, tz.ctypes.data), "gpw_taskset_set_tiles")

    def tiles(self) -> list:
        tz = np.zeros(len(self.plan.levels), np.int32)
        check(lib().gpw_taskset_get_tiles(self.handle, tz.ctypes.data), "gpw_taskset_get_tiles")
        return [int(v) for v in tz]

    def autotune(self, pab, stream=None) -> tuple:
        """Times each tile shape (gpw_taskset_autotune) and keeps the fastest:
        (tile z per level, ms[level][candidate tz = 8, 4, 0]; 0 only on general-cell levels)."""
        nl = len(self.plan.levels)
        tz = np.zeros(nl, np.int32)
        ms = np.zeros(3 * nl, np.float64)
        check(lib().gpw_taskset_autotune(self.handle, pab.data_ptr(), tz.ctypes.data, ms.ctypes.data,
                                         _stream_handle(stream)), "gpw_taskset_autotune")
        return [int(v) for v in tz], ms.reshape(nl, 3)

    # host-buffer calls (numpy in, numpy out; copies inside the library)
    def collocate_host(self, pab: np.ndarray, grids: list, precision: str = "fp64"):
        ptrs = (C.c_void_p * len(grids))(*[g.ctypes.data for g in grids])
        pab = np.ascontiguousarray(pab, dtype=np.float64)
        check(lib().gpw_collocate_host(self.handle, PREC[precision], pab.ctypes.data, ptrs), "gpw_collocate_host")

    def integrate_host(self, grids: list, hab: np.ndarray, precision: str = "fp64"):
        gr = [np.ascontiguousarray(g, dtype=np.float64) for g in grids]
        ptrs = (C.c_void_p * len(gr))(*[g.ctypes.data for g in gr])
        check(lib().gpw_integrate_host(self.handle, PREC[precision], ptrs, hab.ctypes.data), "gpw_integrate_host")


def selftest_tensorcore() -> int:
    """Runs gpw_selftest_tensorcore; returns the number of wrong MMA elements."""
    n = C.c_int64(-1)
    check(lib().gpw_selftest_tensorcore(C.byref(n)), "gpw_selftest_tensorcore")
    return n.value


def selftest_ff_exp(npoints: int = 1 << 22) -> tuple:
    """Runs gpw_selftest_ff_exp: (largest relative error where the result's low
    part is normal, largest relative error below that)."""
    a, b = C.c_double(-1.0), C.c_double(-1.0)
    check(lib().gpw_selftest_ff_exp(int(npoints), C.byref(a), C.byref(b)), "gpw_selftest_ff_exp")
    return a.value, b.value


def collocate_pgf_product_rspace(t: dict, grid: np.ndarray) -> None:
    """The drop-in single-pair entry (gpw_collocate_pgf_product_rspace) with the
    argument dictionary of the task-v1 vocabulary; grid (numpy, host) += rho."""
    i3 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.int32).reshape(3))  # noqa: E731
    d9 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(3, 3))  # noqa: E731
    d3 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(3))  # noqa: E731
    keep = [d9(t["dh"]), d9(t["dh_inv"]), d3(t["ra"]), d3(t["rab"]), i3(t["npts"]), i3(t["ngrid"]),
            i3(t["lb_grid"]), i3(t["periodic"]), i3(t.get("lb_cube", (0, 0, 0))), i3(t.get("ub_cube", (0, 0, 0))),
            np.ascontiguousarray(t.get("sphere_bounds", np.zeros(1)), dtype=np.int32),
            np.ascontiguousarray(t["pab"], dtype=np.float64)]
    assert grid.dtype == np.float64 and grid.flags.c_contiguous
    st = lib().gpw_collocate_pgf_product_rspace(
        int(t["compute_tau"]), int(t["use_ortho"]), int(t["la_max"]), int(t["la_min"]), int(t["lb_max"]),
        int(t["lb_min"]), float(t["zeta"]), float(t["zetb"]), float(t["rscale"]), keep[0].ctypes.data,
        keep[1].ctypes.data, keep[2].ctypes.data, keep[3].ctypes.data, keep[4].ctypes.data, keep[5].ctypes.data,
        keep[6].ctypes.data, keep[7].ctypes.data, int(t["lmax"]), float(t["radius"]), keep[8].ctypes.data,
        keep[9].ctypes.data, int(t.get("nspheres", keep[10].size)), keep[10].ctypes.data, int(t["maxco"]),
        int(t["o1"]), int(t["o2"]), keep[11].ctypes.data, grid.ctypes.data)
    check(st, "gpw_collocate_pgf_product_rspace")
