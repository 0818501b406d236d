"""GPU parity: the CUDA library against the CPU oracle on the same inputs.

Bit-exact for the stages that are integer/byte work or IEEE-exact arithmetic
(split, compaction, scan, two-level error, compensated sums, and the region
evaluation of integrands built from + - * / alone).  For integrands that call
exp/cos/pow, the device math library and glibc may differ in the last bit, so
estimates are compared at 1e-12 relative and error estimates at 1e-12 of the
region's absolute estimate scale: the null rules are differences of nearly equal
rule sums, so a last-bit difference of f can move a region's error estimate by
far more than one ulp of the error itself.
"""
import math

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from tests.reference_cases import BOX, CONFIG1, CONFIG1_VALUE, EASY

pytestmark = pytest.mark.gpu

EXACT_FAMILIES = (pg.CONSTANT, pg.PRODUCT_PEAK, pg.CORNER_PEAK, pg.PRODUCT)
TRANSC_FAMILIES = (pg.OSCILLATORY, pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS, pg.GAUSSIAN_SUM)


def _random_integrand(rng, family, d):
    a = rng.random(d) * 5 + 0.5
    u = rng.random(d)
    return pg.Integrand(family, d, list(a), list(u), c=1.7)


def _random_regions(rng, d, n):
    # dyadic boxes like the ones the iteration produces
    depth = rng.integers(0, 6, size=(d, n))
    length = 0.5 ** depth
    left = np.floor(rng.random((d, n)) / length) * length
    return left, length


def _bits_equal(a, b):
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()


@pytest.mark.parametrize("d", range(2, 11))
@pytest.mark.parametrize("family", EXACT_FAMILIES)
def test_evaluate_exact_families_bitwise(ctx, orc, d, family):
    rng = np.random.default_rng(100 * d + family)
    f = _random_integrand(rng, family, d)
    n = 300 if d < 9 else 60
    left, length = _random_regions(rng, d, n)
    est, err, bis = ctx.evaluate_regions(f, left, length)
    oest, oerr, obis = orc.evaluate_regions(f, left, length)
    assert _bits_equal(est, oest)
    assert _bits_equal(err, oerr)
    assert (bis == obis).all()


@pytest.mark.parametrize("d", [2, 3, 5, 8, 10])
@pytest.mark.parametrize("family", TRANSC_FAMILIES)
def test_evaluate_transcendental_families(ctx, orc, d, family):
    rng = np.random.default_rng(7 * d + family)
    f = _random_integrand(rng, family, d)
    n = 200 if d < 9 else 40
    left, length = _random_regions(rng, d, n)
    est, err, bis = ctx.evaluate_regions(f, left, length)
    oest, oerr, obis = orc.evaluate_regions(f, left, length)
    scale = np.abs(oest) + oerr + 1e-300
    assert np.all(np.abs(est - oest) <= 1e-12 * np.abs(oest) + 1e-300)
    assert np.all(np.abs(err - oerr) <= 1e-12 * scale)
    # split axes agree except where two fourth differences tie to rounding
    assert np.mean(bis == obis) >= 0.97


@pytest.mark.parametrize("d", [2, 4, 6])
def test_evaluate_general_box(ctx, orc, d):
    rng = np.random.default_rng(d)
    f = _random_integrand(rng, pg.PRODUCT_PEAK, d)
    lows = -1.0 - rng.random(d)
    highs = 0.5 + 2 * rng.random(d)
    vol = pg.Volume(list(lows), list(highs))
    left, length = _random_regions(rng, d, 100)
    est, err, bis = ctx.evaluate_regions(f, left, length, vol)
    oest, oerr, obis = orc.evaluate_regions(f, left, length, lows, highs)
    assert _bits_equal(est, oest) and _bits_equal(err, oerr) and (bis == obis).all()


@pytest.mark.parametrize("value", [15.37, -15.37, 0.0])
def test_constant_region_estimates_gpu(ctx, orc, value):
    """RegionSampling.cu:48-171 on the GPU."""
    for splits in range(5, 15):
        left, length = orc.uniform_split(2, splits)
        est, _, _ = ctx.evaluate_regions(pg.constant(2, value), left, length)
        assert np.allclose(est, value / left.shape[1], rtol=1e-6, atol=0)


@pytest.mark.parametrize("n", [2, 64, 4096, 2 * 2048 + 6, 300000])
def test_two_level_bitwise(ctx, orc, n):
    rng = np.random.default_rng(n)
    est = rng.standard_normal(n)
    err = np.abs(rng.standard_normal(n)) * 1e-3
    err[::7] = 0.0
    par = rng.standard_normal(n // 2)
    for relerr in (True, False):
        ne, act = ctx.two_level(est, err, par, 1e-3, relerr)
        one, oact = orc.two_level(est, err, par, 1e-3, relerr)
        assert _bits_equal(ne, one)
        assert (act == oact).all()


@pytest.mark.parametrize("n,d", [(1, 2), (100, 2), (5000, 5), (70000, 8), (3000, 10)])
def test_filter_split_bitwise(ctx, orc, n, d):
    rng = np.random.default_rng(n + d)
    left, length = _random_regions(rng, d, n)
    act = (rng.random(n) < 0.6).astype(np.uint8)
    act[0] = 1
    bis = rng.integers(0, d, n).astype(np.int32)
    est, err = rng.standard_normal(n), rng.random(n)
    gl, gln, gpe, gpr = ctx.filter_split(left, length, act, bis, est, err)
    ol, oln, ope, opr = orc.filter_split(left, length, act, bis, est, err)
    assert _bits_equal(gl, ol) and _bits_equal(gln, oln)
    assert _bits_equal(gpe, ope) and _bits_equal(gpr, opr)


def test_scan_known_answer(ctx):
    """Exclusive scan of 0/1 flags (prefix_sum.cu:19-103 checks the same primitive)."""
    f = np.array([1, 0, 1, 1, 0, 0, 1, 1], dtype=np.uint8)
    out, tot = ctx.exclusive_scan_flags(f)
    assert list(out) == [0, 1, 1, 2, 3, 3, 3, 4] and tot == 5
    rng = np.random.default_rng(0)
    for n in (1, 2047, 2048, 2049, 1 << 20):
        g = (rng.random(n) < 0.3).astype(np.uint8)
        out, tot = ctx.exclusive_scan_flags(g)
        ref = np.concatenate([[0], np.cumsum(g)[:-1]])
        assert (out == ref).all() and tot == g.sum()


@pytest.mark.parametrize("n", [0, 1, 2, 2048, 2049, 1 << 16, 3 * (1 << 20) + 17])
def test_reduce_sum_bitwise(ctx, orc, n):
    """Reduction.cu:49-157 sums iota arrays; here the compensated sum must equal
    the oracle's (same fixed order) bit for bit."""
    x = np.arange(n, dtype=np.float64) * 0.1 + np.sin(np.arange(n))
    assert _bits_equal(ctx.reduce_sum(x), orc.canon_sum(x))
    if n:
        assert ctx.reduce_sum(np.arange(1, n + 1, dtype=np.float64)) == n * (n + 1) / 2


# ---------------------------------------------------------------------------
# Full iteration
# ---------------------------------------------------------------------------
def _same_result(r, o):
    return (r.estimate == o.estimate and r.errorest == o.errorest and r.nregions == o.nregions
            and r.status == o.status and r.iters == o.iters and r.neval == o.neval)


def test_config1_bitwise_and_analytic(ctx, orc):
    r = ctx.integrate(CONFIG1, 1e-3, 0.0)
    o, _ = orc.integrate(CONFIG1, 1e-3, 0.0)
    assert _same_result(r, o)
    assert r.status == 0 and abs(r.estimate - CONFIG1_VALUE) / CONFIG1_VALUE <= 1e-3


@pytest.mark.parametrize("epsrel", [1e-3, 1e-4, 1e-5, 1e-6])
def test_product_peak_8d_bitwise(ctx, orc, epsrel):
    rng = np.random.default_rng(8)
    a = rng.random(8)
    a *= 9.0 / a.sum()
    f = pg.genz(pg.PRODUCT_PEAK, a, rng.random(8))
    r = ctx.integrate(f, epsrel, 0.0)
    o, _ = orc.integrate(f, epsrel, 0.0)
    assert _same_result(r, o)
    exact = np.prod(a * (np.arctan(a * (1 - np.asarray(f.u[:8]))) + np.arctan(a * np.asarray(f.u[:8]))))
    assert r.status == 0 and abs(r.estimate - exact) / exact <= epsrel


@pytest.mark.parametrize("name,f,true", EASY + BOX, ids=[c[0] for c in EASY + BOX])
def test_reference_known_integrals_gpu(ctx, name, f, true):
    """Easy_Integrals.cu / BoxIntegrals.cu at epsrel 1e-3 on the GPU."""
    r = ctx.integrate(f, 1e-3, 1e-12)
    assert r.status == 0
    assert abs(r.estimate - true) / abs(true) <= 1e-3


def test_corner_peak_full_loop_bitwise(ctx, orc):
    f = EASY[1][1]
    r = ctx.integrate(f, 1e-3, 1e-12)
    o, _ = orc.integrate(f, 1e-3, 1e-12)
    assert _same_result(r, o)


def test_nan_and_constant_gpu(ctx):
    r = ctx.integrate(pg.Integrand(pg.NAN_VALUE, 2), 1e-3, 1e-12)
    assert math.isnan(r.estimate)
    r = ctx.integrate(pg.constant(2, 15.37), 1e-3, 1e-12)
    assert r.status == 0 and r.estimate == pytest.approx(15.37, rel=1e-12)


def test_do_integration_from_c(lib):
    import ctypes
    res = ctypes.c_double(0.0)
    rc = lib.do_integration_from_c(ctypes.byref(res))
    assert rc == 0 and abs(res.value - 0.25) / 0.25 <= 1e-6


def test_accuracy_improves_with_epsrel_gpu(ctx):
    eps, prev = 1e-3, 1.0
    while eps > 1e-6:
        r = ctx.integrate(pg.Integrand(pg.FUN6, 6), eps, 1e-40)
        assert r.status == 0 and r.errorest / r.estimate <= eps and r.errorest <= prev
        prev = r.errorest
        eps /= 2


def test_transcendental_full_loop_close_to_oracle(ctx, orc):
    f = EASY[3][1]  # 8-D C0, 2M regions
    r = ctx.integrate(f, 1e-3, 1e-12)
    o, _ = orc.integrate(f, 1e-3, 1e-12)
    assert r.status == o.status == 0
    assert abs(r.estimate - o.estimate) <= 1e-10 * abs(o.estimate)
    assert r.nregions == o.nregions


def test_bad_arguments(ctx):
    with pytest.raises(pg.PaganiError):
        ctx.integrate(pg.Integrand(pg.PRODUCT_PEAK, 1, [1.0], [0.5]), 1e-3, 0.0)
    with pytest.raises(pg.PaganiError):
        ctx.integrate(pg.Integrand(99, 3), 1e-3, 0.0)
    with pytest.raises(pg.PaganiError):
        ctx.integrate(CONFIG1, -1.0, 0.0)
