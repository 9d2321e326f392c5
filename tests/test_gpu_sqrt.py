"""The kernels' square root (sqrt_rn: approximate reciprocal square root,
one coupled Newton step, Markstein's fused residual correction) against the
IEEE single-precision routine, bit for bit over every positive float."""
import pytest

from pmmc_gb300 import capi

pytestmark = pytest.mark.gpu


def test_sqrt_rn_matches_ieee_on_every_positive_float(ctx):
    lo, hi = 0x00000000, 0x7F800001          # +0 .. +inf, subnormals included
    step = 1 << 30
    total = 0
    for a in range(lo, hi, step):
        bad, first = capi.selftest_sqrt(ctx, a, min(step, hi - a))
        assert bad == 0, f"{bad} mismatches, first at bit pattern {first:#010x}"
        total += min(step, hi - a)
    assert total == hi - lo
