"""The integer FP64 <-> FP32 conversions of the mixed form's state update
(rgpu_internal.h widen_f32, narrow_mirror) equal the hardware conversions
bit for bit: the FP32 -> FP64 widening of the accumulated flux difference,
and the FP32 mirror of U^{n+1} that the last sweep writes for the next
step's CFL pass (which the full CFL pass forms with the hardware
conversion). Values: doubles of every exponent, doubles at and next to the
FP32 rounding ties, around FLT_MIN and FLT_MAX, signed zeros, and FP32
values of every exponent."""
import pytest

from rhyme_gb300 import gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_integer_conversions_match_hardware(seed):
    assert gpu.check_conversions(1 << 26, seed) == 0
