"""Rare paths of the iteration, GPU against the oracle bit for bit: the
memory-pressure heuristic classifier (forced with a small memory model), the
relative-error classification switched off, and the iteration cap."""
import numpy as np
import pytest

import gpuintegration_gb300 as pg

pytestmark = pytest.mark.gpu


def _same(r, o):
    return (r.estimate == o.estimate and r.errorest == o.errorest and r.nregions == o.nregions
            and r.status == o.status and r.iters == o.iters and r.neval == o.neval)


@pytest.mark.parametrize("mem", [1e6, 2e6, 4e6, 8e6])
def test_heuristic_classifier_path_bitwise(ctx, orc, mem):
    """heuristic_classifier.cuh:362-451 via Workspace.cuh:74-118.  With these
    memory models the classifier runs its threshold search: it terminates the
    integral (1e6) or thins the region list (2e6..8e6)."""
    rng = np.random.default_rng(0)
    a = rng.random(5) * 8 + 2
    f = pg.genz(pg.PRODUCT_PEAK, a, rng.random(5))
    opt = pg.default_options(device_mem_model=mem)
    r = ctx.integrate(f, 1e-7, 0.0, options=opt)
    o, tr = orc.integrate(f, 1e-7, 0.0, device_mem=mem, trace_cap=800)
    assert _same(r, o)


def test_classifier_terminates_like_the_oracle(ctx, orc):
    f = pg.genz(pg.CORNER_PEAK, [2.0, 1.0, 3.0, 1.5, 0.5, 1.0], [0.0] * 6)
    opt = pg.default_options(device_mem_model=3e6)
    r = ctx.integrate(f, 1e-9, 0.0, options=opt)
    o, _ = orc.integrate(f, 1e-9, 0.0, device_mem=3e6)
    assert _same(r, o)


def test_relerr_classification_off_bitwise(ctx, orc):
    f = pg.genz(pg.PRODUCT_PEAK, [3.0, 2.0, 4.0], [0.3, 0.6, 0.5])
    r = ctx.integrate(f, 1e-5, 0.0, relerr_classification=False)
    o, _ = orc.integrate(f, 1e-5, 0.0, relerr_classification=False)
    assert _same(r, o)


@pytest.mark.parametrize("cap", [1, 3, 7])
def test_iteration_cap_bitwise(ctx, orc, cap):
    f = pg.genz(pg.PRODUCT_PEAK, [20.0] * 4, [0.5] * 4)
    opt = pg.default_options(max_iters=cap)
    r = ctx.integrate(f, 1e-9, 0.0, options=opt)
    o, _ = orc.integrate(f, 1e-9, 0.0, max_iters=cap)
    assert _same(r, o)
    assert r.status == 1


def test_general_box_full_loop_bitwise(ctx, orc):
    f = pg.genz(pg.PRODUCT_PEAK, [4.0, 3.0, 5.0], [0.1, -0.5, 1.5])
    lows, highs = [-1.0, -2.0, 0.5], [1.0, 0.5, 2.5]
    r = ctx.integrate(f, 1e-6, 0.0, vol=pg.Volume(lows, highs))
    o, _ = orc.integrate(f, 1e-6, 0.0, lows=np.array(lows), highs=np.array(highs))
    assert _same(r, o)


def test_empty_batch_and_bad_requests(ctx):
    assert ctx.batch_integrate([], [], []) == []
    with pytest.raises(pg.PaganiError):
        ctx.batch_integrate([pg.Integrand(pg.PRODUCT_PEAK, 13, [1.0] * 13, [0.5] * 13)], [1e-3], [0.0])
    with pytest.raises(pg.PaganiError):
        ctx.serve([pg.constant(2, 1.0)] * 2, [1e-3] * 2, [0.0] * 2, [5.0, 1.0])  # arrivals not ascending


@pytest.mark.parametrize("d", [9, 10, 11, 12])
def test_high_dimensions_bitwise(ctx, orc, d):
    rng = np.random.default_rng(d)
    a = rng.random(d)
    a *= 9.0 / a.sum()
    f = pg.genz(pg.PRODUCT_PEAK, a, rng.random(d))
    r = ctx.integrate(f, 1e-3, 0.0)
    o, _ = orc.integrate(f, 1e-3, 0.0)
    assert _same(r, o)


def test_heuristic_classifier_in_a_batch(ctx, orc):
    """Several integrals run the classifier's threshold search in the same
    iterations (a small memory model): each result equals the oracle's alone."""
    rng = np.random.default_rng(21)
    fs = [pg.genz(pg.PRODUCT_PEAK, rng.random(d) * 8 + 2, rng.random(d)) for d in (3, 4, 5, 5, 6)]
    opt = pg.default_options(device_mem_model=2e6)
    batch = ctx.batch_integrate(fs, [1e-7] * len(fs), 0.0, options=opt)
    for f, b in zip(fs, batch):
        o, _ = orc.integrate(f, 1e-7, 0.0, device_mem=2e6)
        assert _same(b, o)
    st = ctx.stats()
    assert st.classify_passes > 0
