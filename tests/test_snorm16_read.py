"""The snorm16 read of the CUDA kernels (snorm16_from_bits in
csrc/tsf_common.cuh) replaces the division s / 32767 of the OpenCL
CL_SNORM_INT16 read (kernels_no_3d_write.cl:9-21) by bit operations, one
subtraction and one fma: t = (bits 0x43C00000 | (s + 2^15)) - 385, then
max(-1, RN(t + t * c)) with c = 2^-15 + 2^-30.  Here every step is evaluated
with exact rational arithmetic, each rounded to FP32, for every one of the
65,536 stored values, and compared with the correctly rounded quotient: the
kernels' read gives the bits of the division the oracle performs."""
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


def _f32(bits: int) -> Fraction:
    return Fraction(float(np.array([bits], np.uint32).view(np.float32)[0]))


def test_constant_is_the_rounded_reciprocal():
    c = _f32(0x38000100)
    assert c == Fraction(1, 2 ** 15) + Fraction(1, 2 ** 30)
    assert c == _rn32(Fraction(1, 32767))


def test_bit_pattern_gives_385_plus_t():
    s = np.arange(-32768, 32768, dtype=np.int64)
    u16 = (s & 0xFFFF).astype(np.uint32)                 # the stored 16 bits
    lo = (u16 ^ 0x43C08000).astype(np.uint32)            # low half of a word
    word = (u16 << 16).astype(np.uint32)                 # the same value as a high half
    hi = ((word >> 16) & 0xFFFF) ^ 0x43C08000
    assert np.array_equal(lo, hi)
    v = lo.view(np.float32).astype(np.float64)
    assert np.array_equal(v, 385.0 + s * 2.0 ** -15)
    # the subtraction of 385 is exact (same binade as the operand)
    t = (lo.view(np.float32) - np.float32(385.0)).astype(np.float64)
    assert np.array_equal(t, s * 2.0 ** -15)


def test_fma_read_is_exact_for_every_input():
    c = _f32(0x38000100)
    for s in range(-32768, 32768):
        t = Fraction(s, 2 ** 15)
        q = _rn32(t + t * c)                              # __fmaf_rn(t, c, t)
        q = max(q, Fraction(-1))                          # fmaxf(-1, .)
        assert q == max(_rn32(Fraction(s, 32767)), Fraction(-1)), s
        # and the oracle's FP32 division agrees
        ref = np.float32(s) / np.float32(32767)
        assert float(q) == float(max(ref, np.float32(-1.0))), s


def test_paired_read_bits():
    """snorm16_pair2 (csrc/packed.cuh): a paired 16-bit max clamps s to >= -32767
    (both -32768 and -32767 read as -1), flipping bit 15 of each half gives
    s + 2^15, and two byte permutations place each half under 384.0f's
    exponent: the FP32 values 385 + t, t = max(s, -32767) 2^-15."""
    s = np.arange(-32768, 32768, dtype=np.int64)
    lo16 = (s & 0xFFFF).astype(np.uint32)
    hi16 = lo16[::-1].copy()                               # another value in the high half
    w = lo16 | (hi16 << 16)

    def vmaxs2(a, b):
        def half(x, sh):
            v = ((x >> sh) & 0xFFFF).astype(np.int64)
            return np.where(v >= 32768, v - 65536, v)
        lo = np.maximum(half(a, 0), half(np.full_like(a, b), 0)) & 0xFFFF
        hi = np.maximum(half(a, 16), half(np.full_like(a, b), 16)) & 0xFFFF
        return (lo | (hi << 16)).astype(np.uint32)

    def byte_perm(x, y, sel):
        src = [(x >> (8 * i)) & 0xFF for i in range(4)] + [(np.uint32(y) >> (8 * i)) & 0xFF for i in range(4)]
        out = np.zeros_like(x)
        for i in range(4):
            out |= (src[(sel >> (4 * i)) & 0x7] << (8 * i)).astype(np.uint32)
        return out

    x = vmaxs2(w, 0x80018001) ^ np.uint32(0x80008000)
    tl = byte_perm(x, 0x43C00000, 0x7610).view(np.float32) - np.float32(385.0)
    th = byte_perm(x, 0x43C00000, 0x7632).view(np.float32) - np.float32(385.0)
    s_hi = np.where(hi16 >= 32768, hi16.astype(np.int64) - 65536, hi16.astype(np.int64))
    assert np.array_equal(tl.astype(np.float64), np.maximum(s, -32767) * 2.0 ** -15)
    assert np.array_equal(th.astype(np.float64), np.maximum(s_hi, -32767) * 2.0 ** -15)
    # the fma read of -32767 is exactly -1, the value max(-1, s / 32767) gives for -32768
    c = _f32(0x38000100)
    t = Fraction(-32767, 2 ** 15)
    assert _rn32(t + t * c) == -1


def test_offset_form_reads():
    """snorm16_offset2 / snorm16_offset_lo (csrc/tsf_common.cuh), used by the
    TDF's x-paired copy: the copy stores max(s, -32767) + 2^15 per half; its
    low-half read (byte permutation under 384.0f, minus 385, the fma) gives
    t = max(s, -32767) 2^-15 and then the same value as the clamped read of
    s, with no clamp left (the fma read of -32767 is exactly -1)."""
    s = np.arange(-32768, 32768, dtype=np.int64)
    off = (np.maximum(s, -32767) + 32768).astype(np.uint32)              # the stored offset half
    x = ((np.maximum(s, -32767) & 0xFFFF) ^ 0x8000).astype(np.uint32)    # vmaxs2, then the xor
    assert np.array_equal(x, off) and off.min() == 1
    t = (off | np.uint32(0x43C00000)).view(np.float32) - np.float32(385.0)
    assert np.array_equal(t.astype(np.float64), np.maximum(s, -32767) * 2.0 ** -15)
    c = _f32(0x38000100)
    for si in (-32768, -32767, -32766, -1, 0, 1, 12345, 32767):
        ti = Fraction(max(si, -32767), 2 ** 15)
        assert _rn32(ti + ti * c) == max(_rn32(Fraction(si, 32767)), Fraction(-1)), si
