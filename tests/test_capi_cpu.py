"""C ABI checks that need no GPU: the library loads, exports what include/gpw.h
declares, the host-side cube rule equals the oracle's restatement, and calls
that need a device fail cleanly."""
import ctypes as C

import numpy as np
import pytest

from libgpw_gb300 import capi, tasks as T


def test_exports_every_declared_symbol():
    L = capi.lib()
    names = capi.header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n


def test_sphere_rule_matches_oracle(oracle_lib):
    rng = np.random.default_rng(5)
    for _ in range(300):
        h = np.diag(rng.uniform(0.03, 0.9, size=3))
        r = float(np.exp(rng.uniform(np.log(0.01), np.log(20.0))))
        a = capi.sphere_bounds(r, h)
        b = oracle_lib.sphere_bounds(r, h)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_sphere_rule_rejects_bad_input():
    with pytest.raises(capi.GpwError):
        capi.sphere_bounds(-1.0, np.eye(3))
    with pytest.raises(capi.GpwError):
        capi.sphere_bounds(1.0, np.zeros((3, 3)))


def test_struct_layouts():
    # sizes the C side assumes (static_assert-like check through numpy)
    assert T.TASK_DTYPE.itemsize == 152
    assert T.GRID_DTYPE.itemsize == 200


def test_version_string():
    assert b"sm_103a" in capi.lib().gpw_version()


def test_null_arguments_rejected():
    L = capi.lib()
    assert L.gpw_collocate(None, 0, None, None, None) == 1
    assert L.gpw_integrate(None, 0, None, None, None) == 1
    assert L.gpw_taskset_check(None, None) == 1
    h = C.c_void_p()
    assert L.gpw_plan_create(C.byref(h), 0, None, 0) == 1


def test_task_file_reader_roundtrip():
    from golden_io import load_task

    d = load_task("collocate_ortho_density")
    assert d["grid_values"].shape == (388, 4)
    assert d["nspheres"] == 234
