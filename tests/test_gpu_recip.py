"""The flux kernels' FP64 reciprocal (an FP32 special-function seed with one
third-order correction, ldg_device.cuh) against correctly rounded values:
faithful (below one ulp) wherever the seeded form runs, and IEEE behaviour
(CUDA's own 1.0/x) on zero, negative, non-finite, subnormal and
out-of-range operands.  The reciprocal square root the fluxes use is CUDA's
rsqrt, checked against its documented bound (one ulp)."""
import numpy as np
import pytest

import ldg

pytestmark = pytest.mark.gpu


def ulp_error(got, x, f):
    """|got - f(x)| in units of the last place of the correctly rounded
    value; f evaluated in extended precision."""
    ref = f(x.astype(np.longdouble))
    ulp = np.spacing(np.abs(ref.astype(np.float64))).astype(np.longdouble)
    return np.abs((got.astype(np.longdouble) - ref) / ulp).astype(np.float64)


def recip(v):
    return 1 / v


def rsqrt(v):
    return 1 / np.sqrt(v)


@pytest.fixture(scope="module")
def operands():
    rng = np.random.default_rng(7)
    wide = np.exp2(rng.uniform(-124.9, 125.9, 400_000))        # the seeded range
    physical = rng.uniform(0.05, 400.0, 400_000)                # densities, c^2, rho_N rho_K
    near_one = 1.0 + rng.uniform(-1e-6, 1e-6, 50_000)
    powers = np.exp2(np.arange(-125.0, 126.0))                 # exact powers of two
    return np.concatenate([wide, physical, near_one, powers])


def test_faithful_in_the_seeded_range(operands):
    x = operands
    r, rs = ldg.probe_recip(x)
    er, ers = ulp_error(r, x, recip), ulp_error(rs, x, rsqrt)
    assert er.max() < 1.0, (er.max(), x[er.argmax()])
    # almost always the correctly rounded value
    assert np.mean(er <= 0.5) > 0.99
    assert ers.max() <= 1.0, (ers.max(), x[ers.argmax()])


def test_special_and_out_of_range_operands():
    x = np.array([0.0, -0.0, -1.0, -3.5e-200, np.inf, -np.inf, np.nan, 5e-324, 1e-310,
                  2.0 ** -126, 2.0 ** -125.5, 2.0 ** 126, 2.0 ** 127, 1e300, 1.7e308, 2.0 ** -1000])
    r, rs = ldg.probe_recip(x)
    with np.errstate(divide="ignore", invalid="ignore"):
        r_ieee = 1.0 / x
        rs_ieee = 1.0 / np.sqrt(x)
    # every operand here is outside the seeded range; 1.0/x is correctly
    # rounded, so the fallback matches numpy's division bit for bit
    nan = np.isnan(r_ieee)
    assert np.array_equal(np.isnan(r), nan)
    assert np.array_equal(r[~nan].view(np.int64), r_ieee[~nan].view(np.int64))
    assert np.array_equal(np.isnan(rs), np.isnan(rs_ieee))
    assert np.array_equal(np.signbit(rs[~np.isnan(rs)]), np.signbit(rs_ieee[~np.isnan(rs_ieee)]))
    fin = np.isfinite(rs_ieee) & (rs_ieee != 0)
    with np.errstate(divide="ignore", invalid="ignore"):
        e = ulp_error(rs[fin], x[fin], rsqrt)
    assert e.max() <= 1.0, e  # CUDA's rsqrt: within one ulp
    assert np.array_equal(rs[~fin & ~np.isnan(rs_ieee)], rs_ieee[~fin & ~np.isnan(rs_ieee)])


def test_empty_and_invalid_calls():
    r, rs = ldg.probe_recip(np.zeros(0))
    assert r.size == 0 and rs.size == 0
