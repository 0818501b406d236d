"""Cases of the reference-iteration golden file (tests/golden/ref_iter.npz):
configuration 1 and 8-D integrals of the configuration-2 families, chosen so
that every iteration stays far below the heuristic classifier's trigger.
`full`: every region's estimate and errors are stored; otherwise only the
decisions (split axes, active flags) and the iteration totals.  Then a 6-D
discontinuous integral with a long trajectory (36 iterations), and three
oscillatory integrals over many periods whose region estimates cancel, so
that the error-budget fix (Workspace.cuh:121-146) marks every region active
again in some iterations."""
import numpy as np

import gpuintegration_gb300 as pg
from gpuintegration_gb300 import workloads as W
from tests.reference_cases import CONFIG1


def cases():
    c2 = {(c.integrand.family, c.epsrel): c for c in W.config2_cases()}
    out = [("config1_product_peak_5d_1e-3", CONFIG1, 1e-3, True)]
    for fam, eps, full in ((pg.CORNER_PEAK, 1e-3, True), (pg.CORNER_PEAK, 1e-4, True), (pg.PRODUCT_PEAK, 1e-4, True),
                           (pg.GAUSSIAN, 1e-3, True), (pg.GAUSSIAN, 1e-4, True), (pg.C0, 1e-3, False)):
        c = c2[(fam, eps)]
        out.append((f"config2_{pg.FAMILY_NAMES[fam]}_8d_{eps:.0e}", c.integrand, eps, full))
    rng = np.random.default_rng([99, 12])
    d = int(rng.integers(2, 7))
    fam = pg.GENZ_FAMILIES[int(rng.integers(0, 6))]
    eps = float(10 ** rng.uniform(-6, -3))
    out.append((f"long_{pg.FAMILY_NAMES[fam]}_{d}d", W.make(fam, d, rng), eps, True))
    for seed in (1, 2, 3):
        rng = np.random.default_rng([55, seed])
        d = int(rng.integers(2, 4))
        a = rng.random(d)
        a *= float(rng.uniform(15, 60)) / a.sum()
        f = pg.Integrand(pg.OSCILLATORY, d, list(a), list(rng.random(d)))
        eps = float(10 ** rng.uniform(-6, -3))
        out.append((f"budgetfix_oscillatory_{d}d_seed{seed}", f, eps, True))
    return out
