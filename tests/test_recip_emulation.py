"""The FP64 reciprocal of the flux kernels (rcp in ldg_device.cuh) restated
on the CPU in exact arithmetic:

* the operand's high and low words become an FP32 value by rebiasing the
  exponent field and truncating the significand to 23 bits (integer
  operations, exact);
* the FP32 seed is modelled as the correctly rounded FP32 reciprocal of that
  value, moved by up to +-2 FP32 ulp.  This covers the special-function
  approximation's error with margin;
* the seed comes back to FP64 by the inverse rebias (exact), and one
  third-order correction y = y0 (1 + e + e^2), e = 1 - x y0, runs as three
  FMAs, each computed exactly here and rounded once to FP64.

The result must be faithful (below one ulp of 1/x) for every seed in that
range, and almost always the correctly rounded value.  The GPU test
(tests/test_gpu_recip.py) checks the device code itself."""
import struct
from fractions import Fraction

import numpy as np
import pytest

REBIAS = (1023 - 127) << 20


def f64_bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def bits_f64(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def f32_of_bits(b):
    return struct.unpack("<f", struct.pack("<I", b & 0xFFFFFFFF))[0]


def f32_bits(f):
    return struct.unpack("<I", struct.pack("<f", f))[0]


def in_range(x):
    hi = f64_bits(x) >> 32
    return ((hi >> 20) - 898) & 0xFFFFFFFF <= 250


def to_f32(x):
    b = f64_bits(x)
    hi, lo = b >> 32, b & 0xFFFFFFFF
    return f32_of_bits((((hi - REBIAS) & 0xFFFFFFFF) << 3 | (lo >> 29)) & 0xFFFFFFFF)


def to_f64(f):
    b = f32_bits(f)
    hi = (b >> 3) + REBIAS
    lo = (b << 29) & 0xFFFFFFFF
    return bits_f64((hi << 32) | lo)


def fma(a, b, c):
    """a*b + c exactly, rounded once to the nearest double."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def rcp(x, seed_ulps):
    xf = to_f32(x)
    s = np.float32(1.0) / np.float32(xf)  # correctly rounded FP32 reciprocal
    sb = f32_bits(float(s)) + seed_ulps     # moved by whole FP32 ulps
    y0 = to_f64(f32_of_bits(sb))
    e = fma(-x, y0, 1.0)
    t = fma(e, e, e)
    return fma(y0, t, y0)


def ulp_error(y, x):
    exact = Fraction(1) / Fraction(x)
    r = float(exact)
    ulp = abs(np.spacing(r))
    return float(abs(Fraction(y) - exact) / Fraction(ulp))


@pytest.fixture(scope="module")
def operands():
    rng = np.random.default_rng(11)
    wide = np.exp2(rng.uniform(-124.9, 125.9, 1500))
    physical = rng.uniform(0.05, 400.0, 1500)
    edge = np.array([2.0 ** -125, 2.0 ** 126 * (1 - 2 ** -53), 1.0, 1.5, 2.0 - 2 ** -52, 3.0])
    return [float(v) for v in np.concatenate([wide, physical, edge])]


def test_format_changes_are_exact(operands):
    for x in operands[:500]:
        assert in_range(x)
        # the FP32 operand is x truncated to 23 significand bits
        trunc = bits_f64(f64_bits(x) & ~((1 << 29) - 1))
        assert float(np.float32(to_f32(x))) == trunc
        # an FP32 value comes back unchanged
        f = np.float32(1.0) / np.float32(to_f32(x))
        assert to_f64(float(f)) == float(f)


@pytest.mark.parametrize("seed_ulps", [-2, -1, 0, 1, 2])
def test_faithful_for_seeds_within_two_fp32_ulps(operands, seed_ulps):
    errs = [ulp_error(rcp(x, seed_ulps), x) for x in operands]
    assert max(errs) < 1.0, max(errs)
    assert np.mean(np.array(errs) <= 0.5) > 0.99


def test_range_test_excludes_what_fp32_cannot_hold():
    for x in (0.0, -1.0, 2.0 ** -126, 2.0 ** 126, 1e300, 5e-324, float("inf"), float("nan")):
        assert not in_range(x)
    for x in (2.0 ** -125, 1.0, 2.0 ** 126 * (1 - 2 ** -53)):
        assert in_range(x)
