"""Served PAGANI: requests arriving while others run are admitted at iteration
boundaries (continuous batching); each result equals the request's own
stand-alone result, bit for bit."""
import numpy as np
import pytest

import gpuintegration_gb300 as pg
from gpuintegration_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_served_results_equal_standalone(ctx):
    cases = W.mixed_cases(40, 77, 3, 10, 1e-5, 1e-3)
    arrivals = np.sort(np.random.default_rng(3).uniform(0.0, 300.0, len(cases)))
    fs = [c.integrand for c in cases]
    eps = [c.epsrel for c in cases]
    # a pool far smaller than the mix: requests wait for admission and spill
    opt = pg.default_options(max_regions=20000)
    served, done = ctx.serve(fs, eps, 0.0, arrivals, options=opt)
    assert np.all(done >= arrivals - 1e-6)
    for f, e, s in zip(fs, eps, served):
        r = ctx.integrate(f, e, 0.0)
        assert (r.estimate, r.errorest, r.nregions, r.status, r.iters) == \
               (s.estimate, s.errorest, s.nregions, s.status, s.iters)


def test_serve_overlaps_requests(ctx):
    """A long request and short ones arriving during it: the short ones finish
    before the long one (they were admitted while it ran)."""
    long = pg.genz(pg.GAUSSIAN, [4.0] * 7, [0.5] * 7)
    short = [pg.genz(pg.PRODUCT_PEAK, [1.0, 2.0, 1.5], [0.3, 0.5, 0.7]) for _ in range(5)]
    fs = [long] + short
    eps = [1e-6] + [1e-4] * 5
    arrivals = np.array([0.0, 5.0, 10.0, 15.0, 20.0, 25.0])
    res, done = ctx.serve(fs, eps, 0.0, arrivals)
    assert all(r.status == 0 for r in res)
    assert done[1:].max() < done[0]


@pytest.mark.parametrize("mode", [pg.EVAL_POINTS, pg.EVAL_SET_SUMS])
def test_served_workload_sample_equals_standalone(ctx, mode):
    """The served configuration's request stream (Genz integrands, dim 3..10,
    epsrel log-uniform [1e-6, 1e-3]) on its own Poisson schedule at 2000
    requests/s, keeping the requests of dimension <= 6 with epsrel >= 1e-5, under
    a 64 MB region-pool budget so requests queue for admission: every request
    finishes after it arrives, and each result is its stand-alone result bit for
    bit."""
    arrivals_all = W.poisson_arrivals(2000.0, 0.25)
    cases_all = W.config5_cases(len(arrivals_all))
    keep = [i for i, c in enumerate(cases_all) if c.integrand.ndim <= 6 and c.epsrel >= 1e-5]
    assert len(keep) >= 100
    cases = [cases_all[i] for i in keep]
    arrivals = arrivals_all[keep]
    fs = [c.integrand for c in cases]
    eps = [c.epsrel for c in cases]
    opt = pg.default_options(eval_mode=mode)
    served, done = ctx.serve(fs, eps, 0.0, arrivals, budget_bytes=64 << 20, options=opt)
    assert np.all(done >= arrivals - 1e-6)
    key = lambda r: (r.estimate, r.errorest, r.nregions, r.status, r.iters, r.neval)  # noqa: E731
    for f, e, s in zip(fs, eps, served):
        assert key(s) == key(ctx.integrate(f, e, 0.0, options=pg.default_options(eval_mode=mode)))
