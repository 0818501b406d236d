"""Failure handling without a GPU fault: allocation failures are made on the
host (pg_context_fail_allocation fails one cudaMalloc/cudaMallocHost before it
is called), the call that needed the buffer returns PG_OOM with the error
text, and the same context then gives the results of a fresh one."""
import numpy as np
import pytest

import gpuintegration_gb300 as pg
from gpuintegration_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _batch():
    rng = np.random.default_rng(404)
    fs = [W.make(pg.GENZ_FAMILIES[i % 6], 3 + i % 6, rng) for i in range(24)]
    eps = list(10 ** rng.uniform(-5, -3, size=len(fs)))
    return fs, eps


def _keys(rs):
    return [(r.estimate, r.errorest, r.nregions, r.status, r.iters) for r in rs]


@pytest.mark.parametrize("after", [0, 1, 3, 7])
@pytest.mark.parametrize("mode", [pg.EVAL_POINTS, pg.EVAL_SET_SUMS])
def test_allocation_failure_returns_oom_and_context_stays_usable(after, mode):
    fs, eps = _batch()
    opt = pg.default_options(eval_mode=mode)
    with pg.Context(0) as fresh:
        expect = _keys(fresh.batch_integrate(fs, eps, 0.0, options=opt))
    with pg.Context(0) as c:
        c.integrate(pg.genz(pg.PRODUCT_PEAK, [2.0] * 3, [0.5] * 3), 1e-3, 0.0)  # buffers of a small run
        c.fail_allocation(after)
        with pytest.raises(pg.PaganiError) as e:
            c.batch_integrate(fs, eps, 0.0, options=opt)
        assert e.value.code == pg.PG_OOM and "injected" in str(e.value)
        c.fail_allocation(-1)
        assert _keys(c.batch_integrate(fs, eps, 0.0, options=opt)) == expect
        f = fs[0]
        assert _keys([c.integrate(f, eps[0], 0.0, options=opt)]) == [expect[0]]
