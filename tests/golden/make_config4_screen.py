"""Pre-screens the seeded config-4 candidate stream (4096 mixed Genz integrals).

Candidate i is workloads.mixed_cases(..., master=4096)[i]: dim ~ U{2..8}, family
~ U{6 Genz}, epsrel log-uniform in [1e-7, 1e-4].  A candidate is accepted when
PAGANI converges (status 0) and its estimate is within epsrel of the analytic
value; the first 4096 accepted candidates form the benchmark workload.  The
screen runs the candidates through the GPU library's batched path, whose
per-integral results are those of its plain path (tests/test_gpu_batch.py),
which matches the CPU oracle (bit-identical for integrands built from
+ - * /; tests/test_gpu_parity.py, tests/test_gpu_config2.py).

`python make_config4_screen.py` (needs a GPU) writes
tests/golden/config4_screen.json.  `python make_config4_screen.py
--oracle-check [--max-regions N] [--max-dim D] [--extend]` (CPU only) repeats
the screen's decision with the CPU oracle on the accepted candidates with at
most N regions (default ORACLE_MAX_REGIONS) and the rejected candidates of
dimension at most D (default ORACLE_MAX_REJECTED_DIM), and records the
agreement in the file's `oracle_check` entry; `--extend` runs only the
candidates beyond the bounds already recorded and adds them
(tests/test_config4_screen.py repeats a seeded sample).
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gpuintegration_gb300 import workloads as W  # noqa: E402

PATH = os.path.join(HERE, "config4_screen.json")
ORACLE_MAX_REGIONS = 200000
ORACLE_MAX_REJECTED_DIM = 6


def main(target=4096, candidates=5600, master=4096):
    import gpuintegration_gb300 as pg
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
    with open(PATH, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"accepted {target} of {last + 1} candidates ({len(out['rejected_before_last'])} rejected) in {elapsed:.1f}s")


def candidates_of(screen):
    """The candidate stream up to the last accepted candidate."""
    return W.mixed_cases(screen["accepted"][-1] + 1, screen["master"], screen["dmin"], screen["dmax"],
                         screen["eps_lo"], screen["eps_hi"])


def oracle_decision(oracle, case, threads=None):
    """(accepted, result) of the CPU oracle on one candidate: status 0 and within epsrel of the exact value."""
    r, _ = oracle.integrate(case.integrand, case.epsrel, 0.0, nthreads=threads)
    return r.status == 0 and W.within_tolerance(r.estimate, case.exact, case.epsrel), r


def _record(screen, acc_n, acc_ok, rej_n, rej_ok, max_regions, max_dim, seconds):
    screen["oracle_check"] = {
        "accepted_checked": acc_n, "accepted_agree": acc_ok, "rejected_checked": rej_n, "rejected_agree": rej_ok,
        "max_regions": max_regions, "max_rejected_dim": max_dim,
        "rule": f"CPU oracle on every accepted candidate with <= {max_regions} regions (same decision, "
                f"region and evaluation counts) and every rejected candidate of dimension <= {max_dim} "
                f"(rejected too)",
        "seconds": round(seconds, 1)}
    with open(PATH, "w") as f:
        json.dump(screen, f, separators=(",", ":"))


def oracle_check(max_regions=ORACLE_MAX_REGIONS, max_dim=ORACLE_MAX_REJECTED_DIM, extend=False):
    """Repeats the screen's decisions with the oracle.  With `extend`, only the
    candidates beyond the bounds already recorded are run and their counts added
    (the accepted band first, recorded before the rejected band starts)."""
    from oracle import oracle
    oracle.load()
    screen = json.load(open(PATH))
    cand = candidates_of(screen)
    prev = screen.get("oracle_check") if extend else None
    lo_regions, lo_dim = (prev["max_regions"], prev["max_rejected_dim"]) if prev else (-1, 0)
    acc_n, acc_ok, rej_n, rej_ok, secs = ((prev["accepted_checked"], prev["accepted_agree"], prev["rejected_checked"],
                                           prev["rejected_agree"], prev["seconds"]) if prev else (0, 0, 0, 0, 0.0))
    t0 = time.time()
    for k, i in enumerate(screen["accepted"]):
        if not lo_regions < screen["nregions"][k] <= max_regions:
            continue
        ok, r = oracle_decision(oracle, cand[i])
        acc_n += 1
        acc_ok += ok and r.nregions == screen["nregions"][k] and r.neval == screen["neval"][k]
    _record(screen, acc_n, acc_ok, rej_n, rej_ok, max(max_regions, lo_regions), lo_dim, secs + time.time() - t0)
    for i in screen["rejected_before_last"]:
        if not lo_dim < cand[i].integrand.ndim <= max_dim:
            continue
        ok, _ = oracle_decision(oracle, cand[i])
        rej_n += 1
        rej_ok += not ok
    _record(screen, acc_n, acc_ok, rej_n, rej_ok, max(max_regions, lo_regions), max(max_dim, lo_dim),
            secs + time.time() - t0)
    print(json.dumps(screen["oracle_check"]))


if __name__ == "__main__":
    args = sys.argv[1:]
    if "--oracle-check" in args:
        # optional: --max-regions N --max-dim D --extend
        kw = {}
        if "--max-regions" in args:
            kw["max_regions"] = int(args[args.index("--max-regions") + 1])
        if "--max-dim" in args:
            kw["max_dim"] = int(args[args.index("--max-dim") + 1])
        oracle_check(extend="--extend" in args, **kw)
    else:
        main()
