"""The snorm16 read of the CUDA kernels (Store<TSF_STORE_SNORM16>::load in
csrc/tsf_common.cuh) replaces the division s / 32767 of the OpenCL
CL_SNORM_INT16 read (kernels_no_3d_write.cl:9-21) by a multiply and one fma
correction (Markstein's correction step).  Here the three IEEE operations are
evaluated with exact rational arithmetic, each rounded to FP32, for every one
of the 65,536 stored values, and compared with the correctly rounded quotient:
the kernels' read gives the bits of the division the oracle performs."""
from fractions import Fraction

import numpy as np


def _rn32(x: Fraction) -> Fraction:
    """x rounded to the nearest FP32 value, ties to even (normal range)."""
    if x == 0:
        return Fraction(0)
    sign = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while Fraction(2) ** e > a:
        e -= 1
    while Fraction(2) ** (e + 1) <= a:
        e += 1
    scale = Fraction(2) ** (e - 23)
    m = a / scale
    fl = m.numerator // m.denominator
    rem = m - fl
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and fl % 2 == 1):
        fl += 1
    return sign * fl * scale


def test_reciprocal_constant():
    r = np.array([0x38000100], np.uint32).view(np.float32)[0]
    assert Fraction(float(r)) == _rn32(Fraction(1, 32767))


def test_corrected_quotient_is_exact_for_every_input():
    r = Fraction(float(np.array([0x38000100], np.uint32).view(np.float32)[0]))
    for s in range(-32768, 32768):
        x = Fraction(s)
        q0 = _rn32(x * r)                        # __fmul_rn(x, r)
        e = _rn32(-q0 * 32767 + x)               # __fmaf_rn(-q0, 32767, x)
        assert e == -q0 * 32767 + x              # the residual is exact
        q = _rn32(e * r + q0)                    # __fmaf_rn(e, r, q0)
        assert q == _rn32(x / 32767), s
        # and the oracle's FP32 division agrees
        assert float(q) == float(np.float32(s) / np.float32(32767)), s
