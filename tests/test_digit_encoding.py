"""The digit-to-bf16 encoding of the mixed form's images (bsg_ozaki.cuh,
OzDigits::digit_f32), restated on the host in IEEE float32: the FP32 product
or fma is exact and its high half equals the bf16 that the integer form (float
bits of d with the exponent lowered by 8i, zero kept zero) gives, for every
digit the split can produce.  Host arithmetic only; the device kernels are
covered by the mixed-form parity tests."""
import numpy as np


def _bits(x):
    return int(np.float32(x).view(np.uint32))


def _integer_form(d, i):
    """bf16 bits of d * 2^(-8i) from the float bits of d, exponent lowered by 8i"""
    if d == 0:
        return 0
    return ((_bits(np.float32(d)) - ((8 * i) << 23)) & 0xFFFFFFFF) >> 16


def _byte_perm(x, y, sel):
    b = [(x >> (8 * k)) & 255 for k in range(4)] + [(y >> (8 * k)) & 255 for k in range(4)]
    return sum(b[(sel >> (4 * n)) & 7] << (8 * n) for n in range(4))


def test_scaled_digit_is_exact_bf16():
    for i in range(8):
        sc = np.float32(2.0 ** (-8 * i))
        for d in range(-256, 257):
            f = _bits(np.float32(d) * sc)
            assert f & 0xFFFF == 0, (d, i)  # the float's low half is empty: the bf16 is exact
            assert f >> 16 == _integer_form(d, i), (d, i)


def test_low_digit_by_byte_permute_and_fma():
    rng = np.random.default_rng(7)
    for nd in range(2, 6):
        lowb = 8 * (nd - 1)
        Ts = [int(t) for t in rng.integers(-(1 << (lowb + 7)), 1 << (lowb + 7), 3000)] + [0, (1 << lowb) - 1, -1]
        for T in Ts:
            lo = T & 0xFFFFFFFF
            for i in range(1, nd):
                d = ((lo >> (lowb - 8 * i)) & 255) - 128  # the integer digit
                b = _byte_perm(lo, 0, 0x4440 | ((lowb >> 3) - i))
                assert b == d + 128
                sc = np.float32(2.0 ** (-8 * i))
                # fma(b, sc, -128 sc): the exact value (b - 128) sc is representable,
                # so the fused result equals it; float64 holds it exactly
                fused = np.float32(np.float64(b) * np.float64(sc) - 128.0 * np.float64(sc))
                assert _bits(fused) == _bits(np.float32(d) * sc)


def test_bf16_pair_packing():
    # two bf16 = the high halves of two floats: byte permute selector 0x7632
    for x, y in [(0x12345678, 0x9ABCDEF0), (0x3F800000, 0xBF800000), (0, 0xFFFF0000)]:
        assert _byte_perm(x, y, 0x7632) == (x >> 16) | ((y >> 16) << 16)
