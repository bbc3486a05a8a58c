"""The mixed LJ pair's bin shift, formed from a packed list entry's code bits.

A packed entry is (j << 6) | (kx << 4) | (ky << 2) | kz with k = bin_j -
bin_i + 1 per dimension (3 = padding).  The pair kernel (csrc/lj_pair.cuh,
lj_geo) reads the code bits where they sit, ORed under the exponent of 2^23,
so the float is 2^23 + m k (m = 16, 4, 1), and forms the shift as
fma(m k, -w / m, w).  These checks run the same float32 steps in numpy: the
shift must equal (1 - k) w exactly for k = 0, 1, 2 (the table it replaced held
float(1 - k) * w), and the padding code must land beyond every cutoff.
"""
import numpy as np

EXP = np.uint32(0x4B000000)  # bits of 2^23


def _code_float(e: np.ndarray, mask: int) -> np.ndarray:
    bits = (e.astype(np.uint32) & np.uint32(mask)) | EXP
    return bits.view(np.float32) - np.float32(8388608.0)


def _shift(t: np.ndarray, w: np.ndarray, m: int) -> np.ndarray:
    # fma(t, -w / m, w) in float32: the product of two float32 values and the
    # sum with w are exact in float64 at these magnitudes, so one rounding to
    # float32 afterwards is the fused multiply-add's single rounding
    nw = (-w / np.float32(m)).astype(np.float32)
    return (t.astype(np.float64) * nw.astype(np.float64) + w.astype(np.float64)).astype(np.float32)


def test_code_bits_read_as_exact_multiples():
    ks = np.arange(4)
    for shift_bits, mask, m in ((4, 0x30, 16), (2, 0x0C, 4), (0, 0x03, 1)):
        e = (np.arange(1 << 10, dtype=np.int64)[:, None] << 6) | (ks[None, :] << shift_bits)
        t = _code_float(e.ravel(), mask)
        np.testing.assert_array_equal(t, np.tile(np.float32(m) * ks.astype(np.float32), 1 << 10))


def test_shift_equals_table_value():
    rng = np.random.default_rng(20261204)
    w = np.concatenate([rng.uniform(0.5, 20.0, 20000), [2.8, 2.8470, 5.734, 1.0, 3.0]]).astype(np.float32)
    for m in (16, 4, 1):
        for k in (0, 1, 2):
            t = np.full_like(w, np.float32(m * k))
            got = _shift(t, w, m)
            want = (np.float32(1 - k) * w).astype(np.float32)
            np.testing.assert_array_equal(got, want)
            if k == 1:
                assert not np.any(np.signbit(got)), "the zero shift must be +0, as in the table"


def test_padding_code_is_beyond_the_cutoff():
    # k = 3 gives -2 w per dimension; a bin is at least the neighbour cutoff
    # wide, so the padding pair (i with itself) sits at 2 w sqrt(3) > cutoff
    rng = np.random.default_rng(7)
    cut = rng.uniform(0.5, 10.0, 1000).astype(np.float32)
    w = (cut * rng.uniform(1.0, 3.0, 1000)).astype(np.float32)
    for m in (16, 4, 1):
        s = _shift(np.full_like(w, np.float32(3 * m)), w, m)
        np.testing.assert_array_equal(s, (-2 * w).astype(np.float32))
    r2 = 3 * (2 * w.astype(np.float64)) ** 2
    assert np.all(r2 > cut.astype(np.float64) ** 2 * (1 + 4e-6))
