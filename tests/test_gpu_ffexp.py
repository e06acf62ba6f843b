"""The float-float exponential of the mixed path (libgpw_gb300/csrc/gpw_ff.cuh,
Tang's table method) swept on the device against FP64 exp: its stated bound is a
relative error of about 2^-45 while the result's low part is a normal float
(arguments above -60); below, the low part and then the high part become float
subnormals, so the error there is measured against max(exp(a), 2^-126) and is
bounded by about one subnormal step (2^-149) over 2^-126, i.e. 2^-23."""
import pytest

from libgpw_gb300 import capi

pytestmark = pytest.mark.gpu


def test_ff_exp_sweep():
    err, err_low = capi.selftest_ff_exp(1 << 22)
    assert 0.0 < err <= 2.0 ** -44, err
    assert err_low <= 2.0 ** -22, err_low
