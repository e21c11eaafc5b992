"""f32_of_difference (csrc/f32_diff.cuh): fl32(x - a) rounded once to
nearest-even with integer arithmetic, checked on the host against exact
rational arithmetic (the leaf frames use it in place of a float64
subtraction and conversion; the filters' error bounds need one correct
rounding).  Cases it declines must be the ones the header names."""

import ctypes
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def helper(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("f32diff") / "libf32diff.so")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC",
                    os.path.join(HERE, "f32_diff_host.cpp"), "-o", out], check=True)
    lib = ctypes.CDLL(out)
    fn = lib.f32_of_differences
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                   ctypes.c_void_p]

    def run(x, a):
        x = np.ascontiguousarray(x, dtype=np.float64)
        a = np.ascontiguousarray(a, dtype=np.float64)
        r = np.empty(len(x), dtype=np.float32)
        ok = np.empty(len(x), dtype=np.int32)
        fn(x.ctypes.data, a.ctypes.data, len(x), r.ctypes.data, ok.ctypes.data)
        return r, ok.astype(bool)
    return run


def round_f32(fr):
    """Fraction -> float32, one rounding to nearest-even (normal range)."""
    if fr == 0:
        return np.float32(0.0)
    sign = -1 if fr < 0 else 1
    a = abs(fr)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    # a in [2^e, 2^(e+1)); 24 significant bits
    q = a / Fraction(2) ** (e - 23)
    qi = q.numerator // q.denominator
    rem = q - qi
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and qi % 2 == 1):
        qi += 1
    if qi == 1 << 24:
        qi >>= 1
        e += 1
    return np.float32(sign * float(Fraction(qi) * Fraction(2) ** (e - 23)))


def exact(x, a):
    return np.array([round_f32(Fraction(float(u)) - Fraction(float(v))) for u, v in zip(x, a)],
                    dtype=np.float32)


def test_random_offsets_match_one_rounding(helper):
    rng = np.random.default_rng(5)
    xs, as_ = [], []
    for mag in (1e-3, 1.0, 700.0, 1e4, 5e6):
        for r in (1e-12, 1e-7, 1e-3, 1.0, 3e2):
            a = rng.uniform(-mag, mag, 400)
            xs.append(a + rng.uniform(-r, r, 400) * mag)
            as_.append(a)
    x, a = np.concatenate(xs), np.concatenate(as_)
    got, ok = helper(x, a)
    assert ok.mean() > 0.9
    want = exact(x[ok], a[ok])
    np.testing.assert_array_equal(got[ok].view(np.uint32), want.view(np.uint32))
    # where the exact difference is a float64, one rounding equals the
    # float64 subtraction followed by the conversion
    d = x[ok] - a[ok]
    same = np.array([Fraction(float(u)) - Fraction(float(v)) == Fraction(float(w))
                     for u, v, w in zip(x[ok], a[ok], d)])
    np.testing.assert_array_equal(got[ok][same].view(np.uint32),
                                  d[same].astype(np.float32).view(np.uint32))


def test_ties_round_to_even(helper):
    # x - a = (2^24 + 1) ulp and (2^24 + 3) ulp: halfway cases at 25 bits
    a = np.full(4, 1.0)
    ulp = 2.0 ** -52
    x = a + np.array([(2 ** 24 + 1) * ulp * 2, (2 ** 24 + 3) * ulp * 2,
                      -(2 ** 24 + 1) * ulp * 2, (2 ** 25 + 2) * ulp])
    got, ok = helper(x, a)
    assert ok.all()
    np.testing.assert_array_equal(got.view(np.uint32), exact(x, a).view(np.uint32))


def test_declined_cases(helper):
    inf, nan = float("inf"), float("nan")
    x = np.array([0.0, 1.0, inf, 1.0, nan, 1e-310, 1.0, 3.0, 3e38])
    a = np.array([1.0, 0.0, 1.0, inf, 1.0, 1.0, 2048.0, 3.0, -3e38])
    got, ok = helper(x, a)
    # zeros, non-finite, subnormal inputs, exponents more than 9 apart, and a
    # result beyond float32's range are declined; equal values give +0
    assert ok.tolist() == [False, False, False, False, False, False, False, True, False]
    assert got[7] == 0.0 and not np.signbit(got[7])
