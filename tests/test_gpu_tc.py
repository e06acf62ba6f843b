"""Tensor-core building blocks on the device."""
import pytest

from libgpw_gb300 import capi

pytestmark = pytest.mark.gpu


def test_tensorcore_selftest_exact():
    """One fp16 MMA with FP32 accumulation in the mixed path's operand layout
    reproduces the exact integer products (|slice| <= 2^10, K = 16)."""
    assert capi.selftest_tensorcore() == 0
