"""The assembly's FP64 division and square root (researchuv_gb300/csrc/fp64rn.cuh: integer and
FP32 pipes, Newton corrections with an exact 128-bit residual, remainder-based rounding) must
give the IEEE round-to-nearest bits of the hardware operations for every input: checked bit
for bit on 2^26 seeded inputs per class -- moderate exponents, arbitrary bit patterns
(zeros, subnormals, infinities, NaNs, out-of-range quotients through the hardware path),
quotients near midpoints, square roots near perfect squares."""
import pytest

import researchuv_gb300 as R

pytestmark = pytest.mark.gpu

CLASSES = {0: "quotients, exponents within +-60", 1: "quotients of arbitrary bit patterns",
           2: "quotients near a midpoint", 3: "square roots, exponents within +-60",
           4: "square roots of arbitrary bit patterns", 5: "square roots near perfect squares"}


@pytest.mark.parametrize("mode", sorted(CLASSES))
def test_div_sqrt_bitwise(mode):
    ctx = R.Context(0)
    for seed in (1, 0x5EED0000 + mode):
        bad, first = R.selftest_fp64(ctx, mode, seed, 1 << 26)
        assert bad == 0, (CLASSES[mode], bad, [float.hex(v) for v in first])


def test_selftest_rejects_bad_mode():
    ctx = R.Context(0)
    with pytest.raises(R.RuvError):
        R.selftest_fp64(ctx, 9, 1, 10)
