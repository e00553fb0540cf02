"""The integer-pipe binary64 routines (py-orbit_gb300/csrc/softf64.cuh) as
compiled for the GPU, against the FP64 instructions on the same device: the
multiply, add, fused multiply-add, x 2^+-1 and the double-to-float and
float-to-double conversions must return the same bits on every generated
case (random normal operands over exponent spreads of
+-1000, +-60, +-5 and 0, total and near cancellations, close significands,
rounding ties, fma ties, zeros and random bit patterns covering subnormals,
infinities and NaN).  The host build of the same header is checked in
test_softf64_host.py; the device build differs (the 64-bit high multiply is
an intrinsic there)."""
import pytest

pytestmark = pytest.mark.gpu


def test_soft_binary64_matches_the_fp64_instructions_bit_for_bit():
    import orbit_gb300 as og
    for seed in (1, 2):
        counts = og.softf64_check(100_000_000, seed=seed)
        assert counts == (0, 0, 0, 0, 0, 0), (seed, counts)
