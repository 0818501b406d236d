"""Cases of the reference-iteration golden file (tests/golden/ref_iter.npz):
configuration 1 and 8-D integrals of the configuration-2 families, chosen so
that every iteration stays far below the heuristic classifier's trigger.
`full`: every region's estimate and errors are stored; otherwise only the
decisions (split axes, active flags) and the iteration totals."""
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
    return out
