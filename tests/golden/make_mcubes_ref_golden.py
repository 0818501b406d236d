"""Regenerates tests/golden/mcubes_ref.json: results of the reference's own
m-Cubes codes with recorded seeds, for the library's statistical comparison
(tests/test_mcubes_ref.py).  TEST INFRASTRUCTURE.

"seq" (run with --seq, on any host): the reference's sequential CPU m-Cubes
(cuda/mcubes/mcubesSeq.hh), built from the reference sources by
oracle/ref/build_ref.sh into oracle/_ref/mcubes_seq_run.  Its damping
exponent is 0.5 (cuda/mcubes/seqCodesDefs.hh:7), every iteration adapts the
grid, and the weighted mean covers every iteration.

"gpu" (run with --gpu, on a GPU): the reference's GPU m-Cubes, its own
sampling kernels in its iteration loop (tests/golden/ref_mcubes_runner.py),
damping exponent 1.5, three recorded seeds per case.
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SEQ = os.path.join(ROOT, "oracle", "_ref", "mcubes_seq_run")
OUT = os.path.join(HERE, "mcubes_ref.json")

SEQ_RUNS = [(1, 1000000, 15, s) for s in (11, 12, 13)] + [(2, 1000000, 15, s) for s in (11, 12, 13)] + \
           [(0, 2 ** 24, 20, 11)]


def gpu_cases():
    import gpuintegration_gb300 as pg
    from gpuintegration_gb300 import workloads as W
    return [("gauss6_sigma0.01", W.config3_integrand(), 1e-4, 2.0 ** 24, 20, 20, 5),
            ("corner3", pg.genz(pg.CORNER_PEAK, [3.0, 2.0, 1.0], [0.0, 0.0, 0.0]), 1e-5, 1e6, 15, 10, 3),
            ("c0_4", pg.genz(pg.C0, [2.0, 3.0, 1.0, 2.0], [0.5, 0.2, 0.7, 0.4]), 1e-5, 1e6, 15, 10, 3)]


def main_gpu():
    sys.path.insert(0, ROOT)
    from tests.golden.ref_mcubes_runner import RefMcubes
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    ref = RefMcubes()
    runs = []
    for name, f, eps, ncall, titer, itmax, skip in gpu_cases():
        for base in (1000, 2000, 3000):
            r = ref.integrate(f, eps, 0.0, ncall, titer, itmax, skip, base)
            r.update({"case": name, "epsrel": eps, "ncall": ncall, "titer": titer, "itmax": itmax, "skip": skip,
                      "base_seed": base, "alpha": 1.5})
            runs.append(r)
            print(r, flush=True)
    data["gpu"] = runs
    json.dump(data, open(OUT, "w"), indent=1)


def main():
    if "--gpu" in sys.argv:
        return main_gpu()
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    runs = []
    for case, ncall, itmx, seed in SEQ_RUNS:
        out = subprocess.check_output([SEQ, str(case), str(ncall), str(itmx), str(seed)], text=True)
        r = json.loads(out.strip().splitlines()[-1])
        r.update({"case_id": case, "ncall": ncall, "itmx": itmx, "seed": seed, "alpha": 0.5})
        runs.append(r)
        print(r, flush=True)
    data["seq"] = runs
    json.dump(data, open(OUT, "w"), indent=1)


if __name__ == "__main__":
    sys.exit(main())
