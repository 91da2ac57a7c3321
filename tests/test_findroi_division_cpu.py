"""The filters' fast division by the recurrence constant b0 is enabled per
divisor by a host check (no GPU needed): Markstein's sequence through
RN(1/b0) must equal IEEE division for every significand of [1, 2)."""
import pytest

from bamf_gb300 import frontend


@pytest.mark.parametrize("sigma", [0.5, 0.8, 1.0, 1.3, 1.6, 2.0, 2.6, 3.2, 5.2])
def test_host_check_passes_for_the_usual_filter_widths(sigma):
    assert frontend.division_check(sigma)["host_exact"]
