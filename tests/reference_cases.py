"""Integrands and known answers of the reference's own tests, expressed as
library families.  Positional a_i / u_i follow the argument order of each
reference functor."""
import math

import gpuintegration_gb300 as pg

# test/cuda/pagani/Easy_Integrals.cu:54-149 and common/cuda/integrands.cuh
EASY = [
    ("genz2_6d", pg.genz(pg.PRODUCT_PEAK, [50.0] * 6, [0.5] * 6), 1.286889807581113e13),          # F_2_6D :1681-1705
    ("genz3_8d", pg.genz(pg.CORNER_PEAK, [3, 2, 1, 4, 5, 6, 7, 8], [0.0] * 8), 2.2751965817917756076e-10),  # F_3_8D :1368-1389
    ("genz4_5d", pg.genz(pg.GAUSSIAN, [25.0] * 5, [0.5] * 5), 1.79132603674879e-06),              # F_4_5D :1857-1880
    ("genz5_8d", pg.genz(pg.C0, [10.0] * 8, [0.5] * 8), 2.425217625641885e-06),                   # F_5_8D :1427-1452
    ("genz6_6d", pg.genz(pg.DISCONTINUOUS, [10, 9, 8, 7, 6, 5], [.9, .8, .7, .6, .5, .4]), 1.5477367885091207413e8),  # F_6_6D :1756-1774
]
# test/cuda/pagani/BoxIntegrals.cu:15-65, cuda/pagani/demos/function.cuh:113-172
BOX = [
    ("box8_15", pg.Integrand(pg.BOX, 8, c=15.0), 8879.851175413485),
    ("box8_25", pg.Integrand(pg.BOX, 8, c=25.0), 14996089.096112404019),
    ("box8_22", pg.Integrand(pg.BOX, 8, c=22.0), 1495369.283757217694),
]
# Configuration 1: 5-D product peak a_i = 10, u_i = 0.5, analytic (20 atan 5)^5
CONFIG1 = pg.genz(pg.PRODUCT_PEAK, [10.0] * 5, [0.5] * 5)
CONFIG1_VALUE = (20.0 * math.atan(5.0)) ** 5
