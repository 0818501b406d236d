"""Seeded cases of the reference-kernel golden file (tests/golden/ref_phase1.npz)."""
import numpy as np

import gpuintegration_gb300 as pg

FAMILIES = [pg.PRODUCT_PEAK, pg.CORNER_PEAK, pg.PRODUCT, pg.CONSTANT, pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS,
            pg.OSCILLATORY]
DIMS = [2, 3, 5, 8]
NREG = 128
# (family, ndim, seed, general box?)
CASES = [(fam, d, 1000 * fam + d, False) for fam in FAMILIES for d in DIMS] + \
        [(pg.PRODUCT_PEAK, 4, 77, True), (pg.GAUSSIAN, 6, 78, True)] + \
        [(pg.PRODUCT, d, 7000 + d, False) for d in (4, 6, 7, 9, 10)] + \
        [(fam, d, 9000 + 10 * fam + d, False) for fam in (pg.PRODUCT_PEAK, pg.GAUSSIAN, pg.CORNER_PEAK)
         for d in (4, 6, 7, 9, 10)]


def case_inputs(case):
    fam, d, seed, box = case
    rng = np.random.default_rng(seed)
    a = rng.random(d) * 5 + 0.5
    u = rng.random(d)
    f = pg.Integrand(fam, d, list(a), list(u), c=(1.7 if fam == pg.CONSTANT else 0.0))
    depth = rng.integers(0, 7, size=(d, NREG))
    length = 0.5 ** depth
    left = np.floor(rng.random((d, NREG)) / length) * length
    lows = highs = None
    if box:
        lows = -1.0 - rng.random(d)
        highs = 0.5 + 2 * rng.random(d)
    return f, left, length, lows, highs
