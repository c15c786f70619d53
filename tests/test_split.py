"""The FP32 high/low split of FP64 values behind the mixed solver's dense
copies (A_hi = fl32(A), A_lo = fl32(A - A_hi)) is computed with integer
operations on the FP64 bits.  CPU only: the library's host build of the same
source, checked bit for bit against numpy's round-to-nearest conversions."""
import ctypes

import numpy as np

import tasktorrent_gb300 as t


def split(v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    hi = np.empty(v.size, np.float32)
    lo = np.empty(v.size, np.float32)
    st = t.lib().ttg_split_f64_f32(v.ctypes.data_as(ctypes.c_void_p), v.size, hi.ctypes.data_as(ctypes.c_void_p),
                                   lo.ctypes.data_as(ctypes.c_void_p))
    assert st == t.TTG_OK
    return hi, lo


def reference(v):
    with np.errstate(all="ignore"):  # 1e39 overflows FP32 to inf in both
        hi = v.astype(np.float32)
        lo = (v - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def check(v):
    v = np.asarray(v, dtype=np.float64)
    hi, lo = split(v)
    rh, rl = reference(v)
    fin = np.isfinite(v)
    assert np.array_equal(hi.view(np.uint32)[fin], rh.view(np.uint32)[fin])
    assert np.array_equal(lo.view(np.uint32)[fin], rl.view(np.uint32)[fin])


def test_random_magnitudes():
    rng = np.random.default_rng(7)
    n = 400_000
    check(rng.standard_normal(n) * np.exp2(rng.integers(-70, 110, n)))
    check(rng.uniform(-1, 1, n))


def test_ties_and_carries():
    rng = np.random.default_rng(8)
    top = rng.integers(0, 1 << 23, 50_000).astype(np.uint64)
    for rem in ((1 << 28) - 1, 1 << 28, (1 << 28) + 1, 0, (1 << 29) - 1):  # below, at and above the half-way point
        bits = (np.uint64(1023 + 5) << np.uint64(52)) | (top << np.uint64(29)) | np.uint64(rem)
        check(bits.view(np.float64))
        check(-bits.view(np.float64))
    # all-ones mantissa: rounding up carries into the exponent
    carry = (np.uint64(1023) << np.uint64(52)) | (np.uint64((1 << 23) - 1) << np.uint64(29)) | \
        np.arange(1 << 28, 1 << 29, 4096, dtype=np.uint64)
    check(carry.view(np.float64))


def test_edges_take_the_fp64_formula():
    check([0.0, -0.0, 1.0, -1.0, 2.0 ** -60, 2.0 ** -61, 2.0 ** 100, 2.0 ** 101, 1e-300, 5e-324, 3.0, 1 / 3, -2 / 3, 1e38, 1e39])
