"""libgpw_gb300: collocate / integrate of Gaussian-pair densities on periodic
real-space grids, native to one NVIDIA GB300 (sm_103a).

The compute path is the CUDA library libgpw_gb300/_lib/libgpw_gb300.so behind
the C ABI of include/gpw.h; this package only binds it (capi) and describes
tasks and grids (tasks).
"""
from . import tasks  # noqa: F401
from .capi import GpwError, Plan, TaskSet, collocate_pgf_product_rspace, lib, sphere_bounds  # noqa: F401

__all__ = ["tasks", "GpwError", "Plan", "TaskSet", "collocate_pgf_product_rspace", "lib", "sphere_bounds"]
