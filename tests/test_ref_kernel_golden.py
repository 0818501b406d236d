"""Per-region parity with the reference's own CUDA evaluation kernel.

tests/golden/ref_phase1.npz holds the estimate, error and split axis that the
reference's INIT_REGION_POOL / SampleRegionBlock (compiled from the reference
sources for sm_103a, oracle/ref/ref_phase1.cu) computed on the GPU for the
seeded cases of tests/golden/ref_phase1_cases.py (made by
tests/golden/make_ref_phase1_golden.py).  The library must reproduce them bit
for bit; the CPU oracle must too for integrands built from + - * /, and to
1e-12 otherwise (glibc's exp/cos are not CUDA's).
"""
import os

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from tests.golden.ref_phase1_cases import CASES, case_inputs

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_phase1.npz"))
EXACT = (pg.PRODUCT_PEAK, pg.CORNER_PEAK, pg.PRODUCT, pg.CONSTANT)
IDS = [f"{pg.FAMILY_NAMES[c[0]]}-d{c[1]}{'-box' if c[3] else ''}" for c in CASES]


@pytest.mark.parametrize("i", range(len(CASES)), ids=IDS)
def test_oracle_vs_reference_kernel(orc, i):
    f, left, length, lows, highs = case_inputs(CASES[i])
    est, err, bis = orc.evaluate_regions(f, left, length, lows, highs)
    re, rr, rb = GOLD[f"est_{i}"], GOLD[f"err_{i}"], GOLD[f"bis_{i}"]
    if f.family in EXACT:
        assert est.tobytes() == re.tobytes() and err.tobytes() == rr.tobytes()
        assert (bis == rb).all()
    else:
        assert np.all(np.abs(est - re) <= 1e-12 * np.abs(re) + 1e-300)
        assert np.all(np.abs(err - rr) <= 1e-12 * (np.abs(re) + rr) + 1e-300)
        assert np.mean(bis == rb) >= 0.97


@pytest.mark.gpu
@pytest.mark.parametrize("i", range(len(CASES)), ids=IDS)
def test_library_vs_reference_kernel_bitwise(ctx, i):
    f, left, length, lows, highs = case_inputs(CASES[i])
    vol = None if lows is None else pg.Volume(list(lows), list(highs))
    est, err, bis = ctx.evaluate_regions(f, left, length, vol)
    assert est.tobytes() == GOLD[f"est_{i}"].tobytes()
    assert err.tobytes() == GOLD[f"err_{i}"].tobytes()
    assert (bis == GOLD[f"bis_{i}"]).all()
