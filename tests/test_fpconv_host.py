"""The integer-pipe arithmetic the kernels use (melt_ibm_gb300/csrc/fpconv.cuh),
built for the host by g++ from the same source and checked on the CPU against
exact rational arithmetic and numpy:

* sum3_diff_f64, sum6_f64, sum3_abs_pair_f64, sum3_abs_f64 and sum3_diff_f32
  give the correctly rounded exact sum when every input is a multiple of the
  last bit's weight of the largest, and are within 6 * 2^-52 of the largest
  |input| plus half a unit of the result otherwise;
* zeros give +0, an infinite or NaN input gives NaN;
* d2f_bits and f2d_bits equal numpy's IEEE conversions on edge cases and on
  random bit patterns.
"""
from __future__ import annotations

import ctypes as C
import math
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SUMS = {"sum3_diff_f64": 0, "sum6_f64": 1, "sum3_abs_pair_f64": 2, "sum3_abs_f64": 3, "sum3_diff_f32": 4}


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    out = tmp_path_factory.mktemp("fpconv") / "libfpconv_host.so"
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(ROOT / "melt_ibm_gb300" / "csrc"),
                    str(ROOT / "tests" / "fpconv_host.cpp"), "-o", str(out)], check=True)
    L = C.CDLL(str(out))
    L.fpconv_sums.argtypes = [C.c_int, C.c_longlong, C.c_void_p, C.c_void_p]
    L.fpconv_d2f.argtypes = [C.c_longlong, C.c_void_p, C.c_void_p]
    L.fpconv_f2d.argtypes = [C.c_longlong, C.c_void_p, C.c_void_p]
    return L


def run_sums(lib, which: str, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(x.shape[0])
    lib.fpconv_sums(SUMS[which], x.shape[0], x.ctypes.data, out.ctypes.data)
    return out


def exact(which: str, v) -> Fraction:
    f = [Fraction(float(a)) for a in v]
    if which in ("sum3_diff_f64", "sum3_diff_f32"):
        return (f[0] - f[1]) + (f[2] - f[3]) + (f[4] - f[5])
    if which == "sum6_f64":
        return sum(f, Fraction(0))
    if which == "sum3_abs_pair_f64":
        return abs(f[0] + f[1]) + abs(f[2] + f[3]) + abs(f[4] + f[5])
    return abs(f[0]) + abs(f[2]) + abs(f[4])


def grid_inputs(rng, n):
    """k * 2^s, |k| < 2^50 with spread magnitudes, one s per sextuple: every
    exact sum is a double."""
    k = rng.integers(-(1 << 49), 1 << 49, size=(n, 6), dtype=np.int64) >> rng.integers(0, 32, size=(n, 6))
    s = rng.integers(-60, 21, size=(n, 1))
    return np.ldexp(k.astype(np.float64), s)


def spread_inputs(rng, n):
    m = 1.0 + rng.random((n, 6))
    sign = np.where(rng.random((n, 6)) < 0.5, -1.0, 1.0)
    x = sign * np.ldexp(m, rng.integers(-40, 41, size=(n, 6)))
    x[::7, 1] = x[::7, 0]                 # exact cancellations
    x[::11, 3] = x[::11, 2]
    return x


@pytest.mark.parametrize("which", sorted(SUMS))
def test_correctly_rounded_on_the_grid(lib, which):
    x = grid_inputs(np.random.default_rng(11), 3000)
    got = run_sums(lib, which, x)
    for t in range(x.shape[0]):
        e = exact(which, x[t])
        want = float(e)                                   # the exact sum is a double here
        if which == "sum3_diff_f32":
            want = float(np.float32(want))
        assert got[t] == want, (which, t, x[t], got[t], want)


@pytest.mark.parametrize("which", sorted(SUMS))
def test_error_bound_on_spread_inputs(lib, which):
    x = spread_inputs(np.random.default_rng(12), 3000)
    got = run_sums(lib, which, x)
    for t in range(x.shape[0]):
        e = exact(which, x[t])
        amax = max(abs(Fraction(float(a))) for a in x[t])
        if which == "sum3_diff_f32":
            half_unit = Fraction(float(np.spacing(np.float32(abs(got[t]))))) / 2
        else:
            half_unit = Fraction(math.ulp(got[t])) / 2
        assert abs(Fraction(float(got[t])) - e) <= Fraction(6, 1 << 52) * amax + half_unit, (which, t, x[t])


def test_zeros_and_non_finite(lib):
    inf, nan = float("inf"), float("nan")
    x = np.array([[0.0] * 6, [0.0, -0.0, 0.0, -0.0, 0.0, 0.0], [inf, 1.0, 0, 0, 0, 0], [1.0, 1.0, nan, 0, 0, 0]])
    for which in SUMS:
        got = run_sums(lib, which, x)
        assert got[0] == 0.0 and math.copysign(1.0, got[0]) == 1.0, which
        assert got[1] == 0.0, which
        assert math.isnan(got[2]) and math.isnan(got[3]), which


def test_conversions_match_numpy(lib):
    rng = np.random.default_rng(13)
    edge = np.array([0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38, 1.1754943508222875e-38,
                     1.401298464324817e-45, 7.006492321624085e-46, 7.006492321624087e-46, 1e-300, 4.9e-324,
                     float("inf"), -float("inf"), float("nan")]).view(np.uint64)
    rand = rng.integers(0, 1 << 63, size=200000, dtype=np.int64).astype(np.uint64)
    rand[::2] = (rand[::2] & np.uint64(0x800FFFFFFFFFFFFF)) | (
        (np.uint64(0x340) + rand[::2] % np.uint64(0x140)) << np.uint64(52))   # near the float range
    bits = np.concatenate([edge, rand])
    out = np.empty(bits.shape[0], dtype=np.uint32)
    lib.fpconv_d2f(bits.shape[0], bits.ctypes.data, out.ctypes.data)
    d = bits.view(np.float64)
    with np.errstate(over="ignore", invalid="ignore"):
        want = d.astype(np.float32)
    got = out.view(np.float32)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))

    fb = (rng.integers(0, 1 << 32, size=200000, dtype=np.int64)).astype(np.uint32)
    fb = np.concatenate([np.array([0, 0x80000000, 1, 0x7FFFFF, 0x800000, 0x7F7FFFFF, 0x7F800000, 0xFF800000,
                                   0x7FC00000], dtype=np.uint32), fb])
    out64 = np.empty(fb.shape[0], dtype=np.uint64)
    lib.fpconv_f2d(fb.shape[0], fb.ctypes.data, out64.ctypes.data)
    with np.errstate(invalid="ignore"):
        want64 = fb.view(np.float32).astype(np.float64)
    got64 = out64.view(np.float64)
    nan = np.isnan(want64)
    assert np.array_equal(np.isnan(got64), nan)
    assert np.array_equal(got64[~nan].view(np.uint64), want64[~nan].view(np.uint64))
