"""Caller-given first region lists and the predict_split variant
(cuda/pagani/quad/GPUquad/Workspace.cuh:148-158,415-441) on the GPU against the
oracle."""
import numpy as np
import pytest

import gpuintegration_gb300 as pg

pytestmark = pytest.mark.gpu


def _same(a, b):
    return (a.estimate, a.errorest, a.nregions, a.iters, a.status) == \
           (b.estimate, b.errorest, b.nregions, b.iters, b.status)


@pytest.mark.parametrize("fam,d", [(pg.PRODUCT_PEAK, 3), (pg.GAUSSIAN, 5), (pg.C0, 8)])
def test_uniform_list_equals_plain_call(ctx, orc, fam, d):
    """integrate_regions on the uniform split the plain call starts from gives
    the plain call's result bit for bit."""
    f = pg.genz(fam, [3.0] * d, [0.4] * d)
    parts = 4 if d < 5 else 2
    left, length = orc.uniform_split(d, parts)
    a = ctx.integrate(f, 1e-4, 0.0)
    b = ctx.integrate_regions(f, left, length, 1e-4, 0.0)
    assert _same(a, b)


def test_custom_list_matches_oracle(ctx, orc):
    """A 3 x 3 x 3 first list (not the library's default) on a product peak: the
    GPU run equals the oracle's run from the same list bit for bit."""
    d = 3
    f = pg.genz(pg.PRODUCT_PEAK, [6.0, 4.0, 9.0], [0.3, 0.55, 0.7])
    left, length = orc.uniform_split(d, 3)
    g = ctx.integrate_regions(f, left, length, 1e-6, 0.0)
    o, _ = orc.integrate_regions(f, left, length, 1e-6, 0.0)
    assert (g.estimate, g.errorest, g.nregions, g.iters, g.status) == \
           (o.estimate, o.errorest, o.nregions, o.iters, o.status)


def test_predict_split_matches_oracle_with_snapshot(ctx, orc):
    """predict_split on a 2-D product peak: the result and the region list kept
    at iteration 15 (16 x 2^15 regions) equal the oracle's bit for bit."""
    f = pg.genz(pg.PRODUCT_PEAK, [30.0, 30.0], [0.37, 0.61])
    left, length = orc.uniform_split(2, 4)
    g = ctx.integrate_regions(f, left, length, 1e-13, 0.0, predict_split=True)
    snap = ctx.last_snapshot()
    o, osnap = orc.integrate_regions(f, None, None, 1e-13, 0.0, predict_split=True, snap_cap=1 << 20)
    assert (g.estimate, g.errorest, g.nregions, g.iters, g.status) == \
           (o.estimate, o.errorest, o.nregions, o.iters, o.status)
    assert snap is not None and osnap is not None and osnap[0] == 16 * 2 ** 15
    assert np.array_equal(snap[0], osnap[1][0]) and np.array_equal(snap[1], osnap[1][1])
    # the plain call with predict_split keeps the same snapshot
    g2 = ctx.integrate(f, 1e-13, 0.0, options=pg.default_options(predict_split=1))
    assert _same(g, g2)
    snap2 = ctx.last_snapshot()
    assert np.array_equal(snap[0], snap2[0]) and np.array_equal(snap[1], snap2[1])


def test_predict_split_exp_family_close_to_oracle(ctx, orc):
    f = pg.genz(pg.C0, [8.0, 8.0], [0.37, 0.61])
    g = ctx.integrate(f, 1e-9, 0.0, options=pg.default_options(predict_split=1))
    o, osnap = orc.integrate_regions(f, None, None, 1e-9, 0.0, predict_split=True)
    assert g.status == o.status == 0
    assert abs(g.estimate - o.estimate) <= 1e-12 * abs(o.estimate)
    assert ctx.last_snapshot()[0].shape[1] == osnap[0] == 16 * 2 ** 15


def test_bad_region_list_is_rejected(ctx):
    f = pg.genz(pg.PRODUCT_PEAK, [3.0, 3.0], [0.5, 0.5])
    left = np.array([[0.0, 0.5], [0.0, 0.0]])
    length = np.array([[0.5, -0.5], [1.0, 1.0]])
    with pytest.raises(pg.PaganiError):
        ctx.integrate_regions(f, left, length, 1e-3, 0.0)
