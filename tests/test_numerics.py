"""The integer-arithmetic building blocks of the kernels, restated in numpy and
checked against exact arithmetic (CPU only; the GPU parity tests check the
kernels themselves).  The invariant division is also checked in its shipped
form: tests/cpp/idx_div_check.cpp compiles ttv_kernels.cuh's make_idx_div and
idx_div as host code.

* ttv_kernels.cuh make_idx_div / idx_div: division by an invariant divisor
  (Granlund and Montgomery's round-up method) for every 32-bit dividend.
* ttv_device.cuh split_double: a double in [2^-60, 2^61) as hi + lo floats
  built from its bits (lo = (1.m - 1) 2^k, exact), |x - hi - lo| < 2^-46 |x|.
* ttv_device.cuh f2d: float -> double from the float's bits for normal floats.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def idx_div_params(d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    return m, min(l, 1), max(l - 1, 0)


def idx_div(n, params):
    m, s1, s2 = params
    t = (m * n) >> 32
    return ((t + (((n - t) & 0xFFFFFFFF) >> s1)) & 0xFFFFFFFF) >> s2


def test_invariant_division_exact_for_32_bit_dividends():
    rng = np.random.default_rng(3)
    divisors = list(range(1, 1100)) + [(1 << k) + e for k in range(1, 32) for e in (-1, 0, 1)
                                       if 1 <= (1 << k) + e < (1 << 32)]
    divisors += [int(x) for x in rng.integers(1, 1 << 32, 500)] + [(1 << 32) - 1]
    for d in divisors:
        params = idx_div_params(d)
        assert params[0] < (1 << 32)
        ns = [0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 31) - 1, 1 << 31, (1 << 32) - 1]
        ns += [int(x) for x in rng.integers(0, 1 << 32, 60)]
        for n in ns:
            if 0 <= n < (1 << 32):
                assert idx_div(n, params) == n // d, (n, d)


def split_double(x):
    bits = x.view(np.uint64)
    hi32 = (bits >> np.uint64(32)).astype(np.uint32)
    lo32 = (bits & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    ok = ((hi32 & np.uint32(0x7FF00000)) - np.uint32(963 << 20)).astype(np.uint32) < np.uint32(121 << 20)
    top = ((hi32.astype(np.uint64) << np.uint64(3)) | (lo32.astype(np.uint64) >> np.uint64(29))) \
        & np.uint64(0xFFFFFFFF)
    top = (top.astype(np.uint32) + np.uint32(128 << 23)).astype(np.uint32)
    hb = ((top & np.uint32(0x7FFFFFFF)) | (hi32 & np.uint32(0x80000000))).astype(np.uint32)
    sgnexp = ((hb & np.uint32(0xFF800000)) - np.uint32(23 << 23)).astype(np.uint32)
    lo = ((sgnexp | ((lo32 >> np.uint32(6)) & np.uint32(0x7FFFFF))).astype(np.uint32).view(np.float32)
          - sgnexp.view(np.float32))
    return hb.view(np.float32), lo.astype(np.float32), ok


def test_double_split_error_and_window():
    rng = np.random.default_rng(5)
    x = rng.standard_normal(200000) * 10.0 ** rng.integers(-20, 20, 200000)
    x = np.concatenate([x, [1.0, -1.0, 2.0 ** -60, -(2.0 ** 61) * 0.999, 2.0 ** -61, 2.0 ** 61, 0.0]])
    hi, lo, ok = split_double(x)
    e = (x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    assert np.array_equal(ok, (e >= 963) & (e < 1084))   # the exponent window, no more, no less
    rec = hi[ok].astype(np.float64) + lo[ok].astype(np.float64)
    assert (np.abs(rec - x[ok]) < 2.0 ** -46 * np.abs(x[ok])).all()
    # lo is exactly the next 23 significand bits of x
    exact = ((x.view(np.uint64) & np.uint64(0x1FFFFFFF)) >> np.uint64(6)).astype(np.float64) * \
        np.ldexp(1.0, e.astype(np.int64) - 1069) * np.sign(x)
    assert np.array_equal(lo[ok].astype(np.float64), exact[ok])


def f2d(f):
    u = f.view(np.uint32)
    m = u & np.uint32(0x7FFFFFFF)
    hi = (((m >> np.uint32(3)) + np.uint32(896 << 20)) | (u & np.uint32(0x80000000))).astype(np.uint64)
    lo = (u.astype(np.uint64) << np.uint64(29)) & np.uint64(0xFFFFFFFF)
    normal = (m - np.uint32(0x00800000)).astype(np.uint32) < np.uint32(0x7F000000)
    return ((hi << np.uint64(32)) | lo).view(np.float64), normal


def test_float_to_double_from_bits():
    rng = np.random.default_rng(6)
    f = (rng.standard_normal(100000) * 10.0 ** rng.integers(-35, 35, 100000)).astype(np.float32)
    f = np.concatenate([f[np.isfinite(f)], np.array([1.0, -1.0, 2.0 ** -126, 3.0e38, -3.0e38], np.float32)])
    d, normal = f2d(f)
    assert np.array_equal(d[normal], f[normal].astype(np.float64))
    # zeros and subnormals are not normal: the kernels build or convert those separately
    _, n0 = f2d(np.array([0.0, -0.0, 1e-45, 1e-40], np.float32))
    assert not n0.any()


def test_shipped_invariant_division_on_the_host(tmp_path):
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if not gxx or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers missing")
    exe = str(tmp_path / "idx_div_check")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", cuda_inc,
                        os.path.join(ROOT, "tests", "cpp", "idx_div_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("PASSED"), r.stdout + r.stderr
