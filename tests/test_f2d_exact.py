"""The bit construction behind f2d_exact (csrc/ofd_common.cuh), the float ->
double conversion that the generated space-order-4 ghost sums use instead of
the FP64 unit's: for normal floats the double's bits are the sign, the
exponent rebiased by 1023 - 127 = 896 and the mantissa shifted left by 29;
zeros keep their sign; subnormal, infinite and NaN inputs take the hardware
conversion.  Checked here against numpy's conversion on every exponent with
65,536 mantissas each (both mantissa ends included), both signs."""
import numpy as np


def f2d_bits(b):
    b = b.astype(np.uint64)
    e = (b >> np.uint64(23)) & np.uint64(0xFF)
    sgn = (b >> np.uint64(31)) << np.uint64(63)
    normal = sgn | ((e + np.uint64(896)) << np.uint64(52)) | ((b & np.uint64(0x7FFFFF)) << np.uint64(29))
    zero = (b & np.uint64(0x7FFFFFFF)) == 0
    out = np.where((e >= 1) & (e <= 254), normal, np.uint64(0))
    return np.where(zero, sgn, out), ((e >= 1) & (e <= 254)) | zero


def test_f2d_bits_equal_numpy_conversion():
    rng = np.random.default_rng(3)
    for e in range(256):
        m = rng.integers(0, 1 << 23, size=65536, dtype=np.uint64)
        m[:2] = (0, (1 << 23) - 1)
        for s in (0, 1):
            b = (np.uint64(s) << np.uint64(31)) | (np.uint64(e) << np.uint64(23)) | m
            bits, handled = f2d_bits(b)
            ref = b.astype(np.uint32).view(np.float32).astype(np.float64).view(np.uint64)
            assert np.array_equal(bits[handled], ref[handled]), (s, e)
            if 1 <= e <= 254:
                assert handled.all()
