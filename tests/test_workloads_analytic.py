"""The analytic values the benchmark judges convergence against
(gpuintegration_gb300/workloads.py, closed forms of the Genz families as in
cuda/pagani/demos/compute_genz_integrals.cuh:241-340) agree with an independent
adaptive cubature (scipy.integrate.cubature) at d = 2 and 3, on seeded
parameters with the benchmark's sharpness scalings."""
import itertools

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from gpuintegration_gb300 import workloads as W

scipy_integrate = pytest.importorskip("scipy.integrate")
if not hasattr(scipy_integrate, "cubature"):
    pytest.skip("scipy without cubature", allow_module_level=True)


def _vectorised(family, a, u, c):
    a = np.asarray(a)
    u = np.asarray(u)
    if family == pg.OSCILLATORY:
        return lambda x: np.cos(2 * np.pi * u[0] + x @ a)
    if family == pg.PRODUCT_PEAK:
        return lambda x: np.prod(1.0 / (a ** -2.0 + (x - u) ** 2), axis=-1)
    if family == pg.CORNER_PEAK:
        d = len(a)
        return lambda x: (1.0 + x @ a) ** (-(d + 1))
    if family == pg.GAUSSIAN:
        s = c if c else 1.0
        return lambda x: s ** len(a) * np.exp(-np.sum((a * (x - u)) ** 2, axis=-1))
    if family == pg.C0:
        return lambda x: np.exp(-np.sum(a * np.abs(x - u), axis=-1))
    if family == pg.DISCONTINUOUS:
        return lambda x: np.exp(x @ a)
    raise ValueError(family)


def _boxes(family, u, d):
    """Sub-boxes with the integrand smooth inside (kinks and jumps at u)."""
    if family == pg.DISCONTINUOUS:
        return [(np.zeros(d), np.asarray(u[:d]))]
    if family == pg.C0:
        cuts = [[(0.0, u[k]), (u[k], 1.0)] for k in range(d)]
        return [(np.array([c[0] for c in cs]), np.array([c[1] for c in cs])) for cs in itertools.product(*cuts)]
    return [(np.zeros(d), np.ones(d))]


SUMS = {pg.OSCILLATORY: 6.0, pg.PRODUCT_PEAK: 9.0, pg.CORNER_PEAK: 7.0, pg.GAUSSIAN: 26.0, pg.C0: 12.0,
        pg.DISCONTINUOUS: 6.3}


@pytest.mark.parametrize("family", sorted(SUMS))
@pytest.mark.parametrize("d", [2, 3])
def test_analytic_matches_cubature(family, d):
    rng = np.random.default_rng(100 * family + d)
    a = rng.random(d)
    a *= (SUMS[family] * d / 8.0) / a.sum()  # the 8-D sharpness sums, scaled to d
    u = rng.random(d) * 0.8 + 0.1
    f = pg.genz(family, list(a), list(u))
    exact = W.analytic(f)
    g = _vectorised(family, a, u, f.c)
    total = 0.0
    for lo, hi in _boxes(family, u, d):
        r = scipy_integrate.cubature(g, lo, hi, rtol=1e-12, atol=0.0, max_subdivisions=100000)
        assert r.status == "converged"
        total += r.estimate
    assert abs(total - exact) <= 1e-9 * abs(exact), (family, d, total, exact)
