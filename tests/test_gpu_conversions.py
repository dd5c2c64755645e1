"""The mixed form converts FP64 state, metrics and registers to FP32 (and back) with integer
arithmetic on the IEEE-754 encodings instead of the FP64 pipe. Its results must be the hardware
conversions' bit for bit, over raw encodings, the float range and its edges, and rounding ties."""
import pytest

pytestmark = pytest.mark.gpu


def test_conversions_match_hardware():
    from plens_gb300.api import selftest_conversions

    assert selftest_conversions(1 << 24, seed=1) == 0
    assert selftest_conversions(1 << 22, seed=12345) == 0
