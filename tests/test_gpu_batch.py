"""Batched PAGANI: each integral's result is identical alone and in a batch."""
import numpy as np
import pytest

import gpuintegration_gb300 as pg

pytestmark = pytest.mark.gpu


def _mixed(rng, count):
    fams = list(pg.GENZ_FAMILIES)
    sums = {pg.OSCILLATORY: 6.0, pg.PRODUCT_PEAK: 9.0, pg.CORNER_PEAK: 7.0, pg.GAUSSIAN: 26.0, pg.C0: 12.0,
            pg.DISCONTINUOUS: 6.3}
    out = []
    for _ in range(count):
        d = int(rng.integers(2, 9))
        fam = fams[int(rng.integers(0, 6))]
        a = rng.random(d)
        a *= sums[fam] / a.sum()
        u = rng.random(d)
        out.append(pg.genz(fam, a, u))
    return out


def test_batch_equals_individual_runs(ctx):
    rng = np.random.default_rng(42)
    fs = _mixed(rng, 24)
    eps = 10 ** rng.uniform(-5, -3, size=len(fs))
    batch = ctx.batch_integrate(fs, eps, 0.0)
    for f, e, b in zip(fs, eps, batch):
        r = ctx.integrate(f, float(e), 0.0)
        assert (r.estimate, r.errorest, r.nregions, r.status, r.iters, r.neval) == \
               (b.estimate, b.errorest, b.nregions, b.status, b.iters, b.neval)


@pytest.mark.parametrize("count,pool,seed", [(12, 6000, 7), (40, 2500, 8)])
def test_small_pool_admission_and_spill_keep_results(ctx, count, pool, seed):
    """With a pool far too small for the batch, integrals wait for admission and
    over-capacity region lists move to host memory (pinned spill slices, reused
    across iterations) between iterations; every result must still equal the
    integral's stand-alone result bit for bit."""
    rng = np.random.default_rng(seed)
    fs = _mixed(rng, count)
    eps = 10 ** rng.uniform(-5, -3.5, size=len(fs))
    opt = pg.default_options(max_regions=pool)
    batch = ctx.batch_integrate(fs, eps, 0.0, options=opt)
    for f, e, b in zip(fs, eps, batch):
        r = ctx.integrate(f, float(e), 0.0)
        assert (r.estimate, r.errorest, r.nregions, r.status, r.iters) == \
               (b.estimate, b.errorest, b.nregions, b.status, b.iters)
