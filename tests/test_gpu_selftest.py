"""Device self-test: the integer-arithmetic binary64 <-> binary32 conversions
that the certified mode uses instead of the FP64-pipe hardware conversions
must agree with the hardware bit for bit."""
import pytest

pytestmark = pytest.mark.gpu


def test_integer_conversions_match_hardware(ctx):
    d2f_fail, f2d_fail = ctx.self_test(1 << 26)
    assert d2f_fail == 0
    assert f2d_fail == 0
