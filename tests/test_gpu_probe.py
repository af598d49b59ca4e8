"""The integer-ALU probe behind the Smith-Waterman rooflines returns plausible rates:
above a trillion instructions per second on a GB300 and below what its SMs could issue
at one instruction per lane per clock."""
import pytest

pytestmark = pytest.mark.gpu


def test_measure_int_alu():
    import torch
    import strobealign_gb300 as sa
    r = sa.measure_int_alu()
    p = torch.cuda.get_device_properties(0)
    ceiling = p.multi_processor_count * 128 * 2.2e9  # lanes per SM x a clock above the maximum
    for k in ("viaddmax_per_s", "max_xor_per_s"):
        assert 1e12 < r[k] < ceiling, (k, r[k])
