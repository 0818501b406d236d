"""The benchmark's batched workload (the 4096 screened mixed Genz integrals of
the batched configuration) on the GPU, on a seeded sample of 512 of its
integrals with at most 200 000 regions each, in both evaluation modes:

* the batch gives every integral its stand-alone pg_integrate result bit for
  bit (estimate, error, regions, iterations, status, evaluations);
* every integral converges (status 0) within its epsrel of the analytic value;
* in the point-by-point mode, region and evaluation counts equal those the
  screen recorded (tests/golden/config4_screen.json), which the CPU oracle
  reproduces (tests/test_config4_screen.py).
"""
import json

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from gpuintegration_gb300 import workloads as W
from tests.golden import make_config4_screen as S

pytestmark = pytest.mark.gpu

SAMPLE = 512
MAX_REGIONS = 200000


@pytest.fixture(scope="module")
def sample():
    screen = json.load(open(S.PATH))
    cases = W.config4_cases(4096)
    light = [k for k, r in enumerate(screen["nregions"]) if r <= MAX_REGIONS]
    idx = sorted(int(k) for k in np.random.default_rng(5).choice(light, SAMPLE, replace=False))
    return screen, cases, idx


@pytest.mark.parametrize("mode", [pg.EVAL_POINTS, pg.EVAL_SET_SUMS])
def test_workload_sample_batched_equals_plain_and_converges(ctx, sample, mode):
    screen, cases, idx = sample
    fs = [cases[k].integrand for k in idx]
    eps = [cases[k].epsrel for k in idx]
    batch = ctx.batch_integrate(fs, eps, 0.0, options=pg.default_options(eval_mode=mode))
    key = lambda r: (r.estimate, r.errorest, r.nregions, r.iters, r.status, r.neval)  # noqa: E731
    for k, f, e, b in zip(idx, fs, eps, batch):
        r = ctx.integrate(f, e, 0.0, options=pg.default_options(eval_mode=mode))
        assert key(b) == key(r), (k, key(b), key(r))
        assert b.status == 0 and W.within_tolerance(b.estimate, cases[k].exact, cases[k].epsrel), (k, b)
        if mode == pg.EVAL_POINTS:
            assert (b.nregions, b.neval) == (screen["nregions"][k], screen["neval"][k]), k
