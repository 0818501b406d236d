"""Pins the CPU oracle against the known answers and golden behaviour of the
reference's own tests (test/cuda/pagani/*.cu).  No GPU needed."""
import math

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from tests.reference_cases import BOX, CONFIG1, CONFIG1_VALUE, EASY


@pytest.mark.parametrize("value", [15.37, -15.37, 0.0])
@pytest.mark.parametrize("splits", range(5, 15))
def test_constant_region_estimates(orc, value, splits):
    """RegionSampling.cu:48-171: every region of a uniform 2-D split of a
    constant integrand estimates value / nregions (1e-6)."""
    left, length = orc.uniform_split(2, splits)
    est, err, bis = orc.evaluate_regions(pg.constant(2, value), left, length)
    n = left.shape[1]
    assert np.allclose(est, value / n, rtol=1e-6, atol=0)


@pytest.mark.parametrize("d", [3, 5, 8])
def test_uniform_split_volumes(orc, d):
    """Uniform_sub_division.cu:23-95: the initial split tiles the unit cube."""
    parts = 4 if d < 5 else 2
    left, length = orc.uniform_split(d, parts)
    assert left.shape[1] == parts ** d
    assert abs(np.prod(length, axis=0).sum() - 1.0) < 1e-14
    assert set(np.unique(left)) == {k / parts for k in range(parts)}


def test_split_layout_dim1(orc):
    """RegionSplitting.cu:41-116: split every region on axis 1; parent i gives
    children i and n+i; axis 0 intact, axis 1 halved."""
    left, length = orc.uniform_split(2, 5)
    n = left.shape[1]
    act = np.ones(n, dtype=np.uint8)
    bis = np.ones(n, dtype=np.int32)
    ol, oln, pe, pr = orc.filter_split(left, length, act, bis, np.zeros(n), np.zeros(n))
    for i in range(n):
        assert ol[0, i] == left[0, i] and ol[0, n + i] == left[0, i]
        assert oln[0, i] == length[0, i] and oln[0, n + i] == length[0, i]
        assert ol[1, i] == left[1, i] and ol[1, n + i] == left[1, i] + length[1, i] / 2
        assert oln[1, i] == length[1, i] / 2 and oln[1, n + i] == length[1, i] / 2


def test_split_first_region_dim0(orc):
    """RegionSplitting.cu:118-203: region 0 split on axis 0, the rest on axis 1."""
    left, length = orc.uniform_split(2, 5)
    n = left.shape[1]
    bis = np.ones(n, dtype=np.int32)
    bis[0] = 0
    ol, oln, _, _ = orc.filter_split(left, length, np.ones(n, np.uint8), bis, np.zeros(n), np.zeros(n))
    assert ol[0, n] == left[0, 0] + length[0, 0] / 2 and ol[1, n] == left[1, 0]
    assert oln[0, 0] == length[0, 0] / 2 and oln[1, 0] == length[1, 0]


@pytest.mark.parametrize("inactive", [[], [15], [0, 99]])
def test_filter_compaction(orc, inactive):
    """RegionFiltering.cu:42-494: active count, compacted coordinates, parent
    estimates/errors in order."""
    rng = np.random.default_rng(1)
    n, d = 100, 2
    left, length = rng.random((d, n)), rng.random((d, n))
    est, err = rng.random(n), rng.random(n)
    act = np.ones(n, dtype=np.uint8)
    act[inactive] = 0
    bis = np.zeros(n, dtype=np.int32)
    ol, oln, pe, pr = orc.filter_split(left, length, act, bis, est, err)
    keep = np.nonzero(act)[0]
    A = keep.size
    assert ol.shape[1] == 2 * A
    assert (pe == est[keep]).all() and (pr == err[keep]).all()
    assert (ol[1, :A] == left[1, keep]).all() and (ol[1, A:] == left[1, keep]).all()


def test_single_region_filter(orc):
    left, length = np.array([[0.0], [0.0]]), np.array([[1.0], [1.0]])
    ol, oln, pe, pr = orc.filter_split(left, length, np.array([1], np.uint8), np.array([1], np.int32),
                                       np.array([2.0]), np.array([0.1]))
    assert ol.shape == (2, 2) and pe[0] == 2.0 and ol[1, 1] == 0.5


def test_integration_from_c_known_answer(orc):
    """test_integration_from_c.c:17-23: integral of x*y over the unit square is 1/4 at 1e-6."""
    r, _ = orc.integrate(pg.Integrand(pg.PRODUCT, 2), 1e-6, 1e-12)
    assert r.status == 0 and abs(r.estimate - 0.25) / 0.25 <= 1e-6


def test_constant_integral(orc):
    r, _ = orc.integrate(pg.constant(2, 15.37), 1e-3, 1e-12)
    assert r.status == 0 and r.estimate == pytest.approx(15.37, rel=1e-12)


def test_nan_integral(orc):
    """NanIntegral.cu:25-37."""
    r, _ = orc.integrate(pg.Integrand(pg.NAN_VALUE, 2), 1e-3, 1e-12)
    assert math.isnan(r.estimate)


FAST_EASY = [c for c in EASY if c[0] in ("genz3_8d", "genz6_6d")]


@pytest.mark.parametrize("name,f,true", FAST_EASY + BOX, ids=[c[0] for c in FAST_EASY + BOX])
def test_known_integrals(orc, name, f, true):
    """Easy_Integrals.cu:74-149 and BoxIntegrals.cu:15-65 at epsrel 1e-3."""
    r, _ = orc.integrate(f, 1e-3, 1e-12)
    assert r.status == 0
    assert abs(r.estimate - true) / abs(true) <= 1e-3


@pytest.mark.slow
@pytest.mark.parametrize("name,f,true", [c for c in EASY if c not in FAST_EASY], ids=lambda c: str(c))
def test_known_integrals_slow(orc, name, f, true):
    r, _ = orc.integrate(f, 1e-3, 1e-12)
    assert r.status == 0
    assert abs(r.estimate - true) / abs(true) <= 1e-3


def test_accuracy_improves_with_epsrel(orc):
    """accuracy_improves_with_epsrel.cu:38-67: status 0, err/est <= epsrel, and
    a non-increasing error estimate as epsrel halves."""
    eps, prev = 1e-3, 1.0
    f = pg.Integrand(pg.FUN6, 6)
    while eps > 1e-6:
        r, _ = orc.integrate(f, eps, 1e-40)
        assert r.status == 0
        assert r.errorest / r.estimate <= eps
        assert r.errorest <= prev
        prev = r.errorest
        eps /= 2


def test_config1_analytic(orc):
    r, _ = orc.integrate(CONFIG1, 1e-3, 0.0)
    assert r.status == 0
    assert abs(r.estimate - CONFIG1_VALUE) / CONFIG1_VALUE <= 1e-3
    assert r.errorest / r.estimate <= 1e-3


def test_canonical_sum_is_compensated(orc):
    x = np.array([1e16, 1.0, -1e16, 1.0] * 3000)
    assert orc.canon_sum(x) == 6000.0
    rng = np.random.default_rng(3)
    y = rng.standard_normal(50000)
    assert abs(orc.canon_sum(y) - math.fsum(y)) <= 1e-12 * np.abs(y).sum()


def test_oracle_regions_entry_equals_plain(orc):
    """The oracle's first-list entry with no list is its plain integrate."""
    import gpuintegration_gb300 as pg
    for fam, d in ((pg.PRODUCT_PEAK, 3), (pg.CORNER_PEAK, 4)):
        f = pg.genz(fam, [4.0] * d, [0.3] * d)
        a, _ = orc.integrate(f, 1e-5, 0.0)
        b, _ = orc.integrate_regions(f, None, None, 1e-5, 0.0)
        assert (a.estimate, a.errorest, a.nregions, a.iters) == (b.estimate, b.errorest, b.nregions, b.iters)


def test_oracle_predict_split_keeps_iteration_15(orc):
    """predict_split (Workspace.cuh:415-441): with classification off for 15
    iterations every region splits, so the list of iteration 15 of a 2-D run
    holds 16 * 2^15 regions covering the unit square."""
    import numpy as np
    import gpuintegration_gb300 as pg
    f = pg.genz(pg.GAUSSIAN, [20.0, 20.0], [0.37, 0.61])
    r, snap = orc.integrate_regions(f, None, None, 1e-12, 0.0, predict_split=True, snap_cap=1 << 20)
    assert r.status == 0 and snap[0] == 16 * 2 ** 15
    left, length = snap[1]
    assert abs(np.prod(length, axis=0).sum() - 1.0) < 1e-12


@pytest.mark.parametrize("d", [2, 4, 6])
def test_gaussian_sum_family(orc, d):
    """GAUSSIAN_SUM is the Gaussian family formed as one exponential of the sum of
    squares, the form of the reference's m-Cubes Gaussian functors
    (cuda/mcubes/demos/Gauss9D.cu:8-24): pointwise it equals the product form
    to rounding (1e-12 relative: the sum's rounding scales with its size), and
    the oracle integrates it to the analytic value."""
    from gpuintegration_gb300 import workloads as W
    rng = np.random.default_rng(12 + d)
    a, u = list(rng.random(d) * 4 + 0.5), list(rng.random(d))
    fs = pg.Integrand(pg.GAUSSIAN_SUM, d, a, u, c=1.3)
    fp = pg.Integrand(pg.GAUSSIAN, d, a, u, c=1.3)
    for _ in range(100):
        x = rng.random(d)
        vs, vp = orc.eval_point(fs, x), orc.eval_point(fp, x)
        assert abs(vs - vp) <= 1e-12 * abs(vp) + 1e-300
    exact = W.analytic(fs)
    r, _ = orc.integrate(fs, 1e-6, 0.0)
    assert r.status == 0 and abs(r.estimate - exact) <= 1e-6 * abs(exact)
