"""Pre-screens the seeded config-4 candidate stream (4096 mixed Genz integrals).

Candidate i is workloads.mixed_cases(..., master=4096)[i]: dim ~ U{2..8}, family
~ U{6 Genz}, epsrel log-uniform in [1e-7, 1e-4].  A candidate is accepted when
PAGANI converges (status 0) and its estimate is within epsrel of the analytic
value; the first 4096 accepted candidates form the benchmark workload.  The
screen runs the candidates through the GPU library's batched path, whose
per-integral results are those of its plain path (tests/test_gpu_batch.py),
which matches the CPU oracle (bit-identical for integrands built from
+ - * /; tests/test_gpu_parity.py, tests/test_gpu_config2.py).

Writes tests/golden/config4_screen.json.  Needs a GPU.
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import gpuintegration_gb300 as pg  # noqa: E402
from gpuintegration_gb300 import workloads as W  # noqa: E402


def main(target=4096, candidates=5600, master=4096):
    cases = W.mixed_cases(candidates, master, 2, 8, 1e-7, 1e-4)
    ctx = pg.Context(0)
    t0 = time.time()
    res = ctx.batch_integrate([c.integrand for c in cases], [c.epsrel for c in cases], 0.0)
    elapsed = time.time() - t0
    accepted, rejected = [], []
    for i, (c, r) in enumerate(zip(cases, res)):
        ok = r.status == 0 and W.within_tolerance(r.estimate, c.exact, c.epsrel)
        (accepted if ok else rejected).append(i)
    if len(accepted) < target:
        raise SystemExit(f"only {len(accepted)} of {candidates} candidates accepted; raise `candidates`")
    accepted = accepted[:target]
    last = accepted[-1]
    out = {
        "master": master, "dmin": 2, "dmax": 8, "eps_lo": 1e-7, "eps_hi": 1e-4, "target": target,
        "accepted": accepted,
        "rejected_before_last": [i for i in rejected if i < last],
        "screen_seconds": round(elapsed, 1),
        "nregions": [int(res[i].nregions) for i in accepted],
        "neval": [int(res[i].neval) for i in accepted],
    }
    with open(os.path.join(HERE, "config4_screen.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"accepted {target} of {last + 1} candidates ({len(out['rejected_before_last'])} rejected) in {elapsed:.1f}s")


if __name__ == "__main__":
    main()
