"""Regenerates tests/golden/ref_iter.npz: the reference's PAGANI iteration run
with the reference's own device stages (tests/golden/ref_iter_runner.py) on the
cases of ref_iter_cases.py.  Needs a GPU and oracle/_ref/ref_phase1.cubin +
ref_stages.cubin (oracle/ref/build_ref.sh)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle  # noqa: E402  (the uniform split of Sub_regions.cuh:11-36)
from tests.golden.ref_iter_cases import cases  # noqa: E402
from tests.golden.ref_iter_runner import RefStages, reference_integrate  # noqa: E402
from tests.golden.ref_phase1_runner import RefKernel  # noqa: E402


def main():
    st = RefStages(RefKernel())
    out = {}
    for name, f, eps, full in cases():
        res, recs = reference_integrate(st, f, eps, 0.0, oracle.uniform_split)
        out[f"{name}/result"] = np.array([res["estimate"], res["errorest"], res["nregions"], res["iters"],
                                          res["status"]], dtype=np.float64)
        out[f"{name}/n"] = np.array([r["n"] for r in recs], dtype=np.int64)
        out[f"{name}/iter_sums"] = np.array([[r["iter_est"], r["iter_err"]] for r in recs])
        out[f"{name}/fixed"] = np.array([r["fixed"] for r in recs], dtype=np.uint8)
        out[f"{name}/bisect"] = np.concatenate([r["bisect"] for r in recs]).astype(np.int8)
        out[f"{name}/act_refine"] = np.concatenate([r["act_refine"] for r in recs]).astype(np.uint8)
        out[f"{name}/act"] = np.concatenate([r["act"] for r in recs]).astype(np.uint8)
        if full:
            for k in ("est", "err_raw", "err"):
                out[f"{name}/{k}"] = np.concatenate([r[k] for r in recs])
        print(name, res, len(recs), "iterations", sum(r["n"] for r in recs), "regions", flush=True)
    np.savez_compressed(os.path.join(HERE, "ref_iter.npz"), **out)


if __name__ == "__main__":
    main()
