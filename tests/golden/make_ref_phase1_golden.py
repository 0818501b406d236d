"""Regenerates tests/golden/ref_phase1.npz: per-region estimate, error and split
axis computed by the reference's own evaluation kernel (the cubin that
oracle/ref/build_ref.sh builds from the reference sources), for seeded
integrands of every family on seeded dyadic region lists.  Needs a GPU and the
cubin; see ref_phase1_runner.py.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests.golden.ref_phase1_cases import CASES, case_inputs  # noqa: E402
from tests.golden.ref_phase1_runner import RefKernel  # noqa: E402


def main():
    k = RefKernel()
    out = {}
    for i, case in enumerate(CASES):
        f, left, length, lows, highs = case_inputs(case)
        est, err, bis = k.evaluate(f, left, length, lows, highs)
        out[f"est_{i}"], out[f"err_{i}"], out[f"bis_{i}"] = est, err, bis
    np.savez_compressed(os.path.join(HERE, "ref_phase1.npz"), **out)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
