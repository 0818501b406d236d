"""m-Cubes CPU oracle: Philox known answers and statistical agreement."""
import pytest

import gpuintegration_gb300 as pg
from gpuintegration_gb300 import workloads as W

# Known-answer vectors of Philox4x32-10 (Salmon et al., SC'11; Random123 kat_vectors)
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_known_answers(orc, ctr, key, expect):
    assert orc.philox(ctr, key) == expect


@pytest.mark.parametrize("f", [
    pg.genz(pg.GAUSSIAN, [5.0, 4.0, 3.0], [0.3, 0.6, 0.5]),
    pg.genz(pg.PRODUCT_PEAK, [3.0, 2.0], [0.4, 0.7]),
    pg.genz(pg.C0, [2.0, 3.0, 1.0, 2.0], [0.5, 0.2, 0.7, 0.4]),
])
def test_mcubes_within_three_sigma(orc, f):
    r, _ = orc.mcubes_integrate(f, 1e-3, 0.0, 2e5, titer=15, itmax=10, skip=3)
    exact = W.analytic(f)
    assert abs(r.estimate - exact) <= 3 * r.errorest + 1e-12
    assert r.errorest / abs(exact) < 1e-2


def test_mcubes_is_reproducible_from_its_seed(orc):
    f = pg.genz(pg.GAUSSIAN, [5.0, 4.0], [0.3, 0.6])
    a, _ = orc.mcubes_integrate(f, 1e-3, 0.0, 5e4, seed=11)
    b, _ = orc.mcubes_integrate(f, 1e-3, 0.0, 5e4, seed=11)
    c, _ = orc.mcubes_integrate(f, 1e-3, 0.0, 5e4, seed=12)
    assert a.estimate == b.estimate and a.errorest == b.errorest
    assert a.estimate != c.estimate
