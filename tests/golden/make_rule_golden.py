"""Regenerates tests/golden/rule_tables.json from the reference itself.

Builds oracle/_ref/dump_rule_tables from the reference sources (which must be
present at $REF, else beside this repository) with oracle/ref/build_ref.sh, runs
it, and stores the degree-9 rule tables for ndim 2..10 with every double as a
hex float so the comparison in tests/test_rule_tables.py is bit-exact.
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main(dmax=10):
    subprocess.check_call(["sh", os.path.join(ROOT, "oracle", "ref", "build_ref.sh")])
    exe = os.path.join(ROOT, "oracle", "_ref", "dump_rule_tables")
    out = subprocess.check_output([exe, str(dmax)], text=True)
    tables = {}
    for line in out.splitlines():
        parts = line.split()
        d, name, vals = int(parts[0]), parts[1], parts[2:]
        entry = tables.setdefault(str(d), {})
        if name in ("feval",):
            entry[name] = int(vals[0])
        elif name == "gindex":
            entry[name] = [int(v) for v in vals]
        elif name == "gen":
            # Every coordinate is 0 or +-G[k]; store the signed code k+1 and G once.
            mags = sorted({abs(float.fromhex(v)) for v in vals} - {0.0}, reverse=True)
            entry["gen_mag"] = [m.hex() for m in mags]
            codes = []
            for v in vals:
                x = float.fromhex(v)
                codes.append(0 if x == 0.0 else (mags.index(abs(x)) + 1) * (1 if x > 0 else -1))
            entry["gen_code"] = "".join("0abcdeABCDE"[c if c >= 0 else 5 - c] for c in codes)
        else:
            entry[name] = vals  # hex floats, parsed with float.fromhex
    path = os.path.join(HERE, "rule_tables.json")
    with open(path, "w") as f:
        json.dump({"source": "reference cuda/pagani/quad/GPUquad/Rule.cuh via oracle/ref/dump_rule_tables.cu",
                   "tables": tables}, f, separators=(",", ":"))
    print("wrote", path)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 10)
