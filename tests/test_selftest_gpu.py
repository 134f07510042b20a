"""The library's integer-pipe FP64<->FP32 conversions (fpconv.cuh), used by
the precision form, equal the hardware conversion instructions bit for bit on
edge cases (signed zeros, subnormals, range limits, rounding ties at every
float exponent, infinities, NaNs) and on 2^26 random bit patterns; the
line-solve factor table that the allocation-free x-line solve builds on the
device equals the host's table bit for bit (several lengths up to 512 and
seven betadx values); the integer-pipe sums of FP64 values that the stencils
use (sum3_diff, sum6, sum3_abs_pair, sum3_abs) give FP64 arithmetic's bits
where that arithmetic is exact and agree with it to their error bound on
2^24 random sextuples, with exact zeros and NaN for non-finite inputs."""
import pytest

pytestmark = pytest.mark.gpu


def test_conversions_and_factor_table_match(gpu_lib):
    assert gpu_lib.mibm_selftest_() == 0
