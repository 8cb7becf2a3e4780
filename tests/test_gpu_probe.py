"""The FP64 FMA rate probe (tmvg_probe_fp64_rate), the denominator of the
benchmark's FP64 roofline fractions: a plausible rate for a GB300 (whose FP64
runs at about two FMAs per SM per clock) that repeats within a few percent."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_rate_is_plausible_and_repeatable(dev):
    from tmv_gb300 import linalg

    h = linalg.handle(dev.index or 0)
    a, b = h.fp64_rate(), h.fp64_rate()
    assert 0.3 < a < 5.0 and 0.3 < b < 5.0, (a, b)
    assert abs(a - b) <= 0.1 * max(a, b)
