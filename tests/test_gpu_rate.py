"""mmf_fp64_rate: the FP64 instruction rate the benchmark divides by is
measured on the GPU it runs on.  GB300 issues about two FP64 instructions
per SM and clock (152 SMs at up to 2.07 GHz: at most 630 G/s), and the
varying-operand mix cannot beat the reused-operand DFMA stream by much."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_rate_is_measured(mmf):
    best, mixed = mmf.capi.fp64_rate(0)
    assert 1e10 < best < 2e12
    assert 1e10 < mixed < 1.2 * best
