"""The grouped tensor-core GEMM's epilogue converts its FP32 sums to FP64 by
bit fields on the integer pipe (f32_to_f64_int, csrc/umma_gemm.cu): the same
formula in numpy against numpy's float32 -> float64 conversion, on normal
values of every exponent, signed zeros, infinities and NaNs (exact), and on
subnormals (flushed to zero)."""
import numpy as np


def f32_to_f64_int(f):
    u = np.asarray(f, np.float32).view(np.uint32).astype(np.uint64)
    sign = u & 0x80000000
    e = (u >> 23) & 0xff
    m = u & 0x7fffff
    ed = np.where(e == 0xff, 0x7ff, e + (1023 - 127))
    hi = np.where(e == 0, sign, sign | (ed << 20) | (m >> 3))
    lo = np.where(e == 0, 0, (m << 29) & 0xffffffff)
    return ((hi << 32) | lo).astype(np.uint64).view(np.float64)


def test_normal_values_are_exact():
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 2 ** 32, size=200000, dtype=np.uint64).astype(np.uint32)
    f = bits.view(np.float32)
    normal = np.isfinite(f) & (np.abs(f) >= np.finfo(np.float32).tiny)
    got = f32_to_f64_int(f[normal])
    ref = f[normal].astype(np.float64)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    ext = np.array([1.0, -1.0, np.finfo(np.float32).max, -np.finfo(np.float32).max, np.finfo(np.float32).tiny,
                    3.1415927, -2.5e-20, 6.0e30], np.float32)
    assert np.array_equal(f32_to_f64_int(ext).view(np.uint64), ext.astype(np.float64).view(np.uint64))


def test_zeros_infinities_nans_and_subnormals():
    f = np.array([0.0, -0.0, np.inf, -np.inf], np.float32)
    got = f32_to_f64_int(f)
    assert np.array_equal(got.view(np.uint64), f.astype(np.float64).view(np.uint64))
    nans = np.array([1, 7, 0x400000, 0x7fffff], np.uint32) | np.uint32(0x7f800000)
    assert np.isnan(f32_to_f64_int(nans.view(np.float32))).all()
    sub = np.array([1, 0x7fffff, 0x80000001], np.uint32).view(np.float32)
    assert (f32_to_f64_int(sub) == 0.0).all()
