"""Degree-9 rule tables: oracle and library against the reference's own tables.

tests/golden/rule_tables.json was produced by running the reference's
quad::Rule<double>::Init (cuda/pagani/quad/GPUquad/Rule.cuh:370-510) through
tests/golden/make_rule_golden.py.  Every double must match bit for bit.
"""
import json
import os

import numpy as np
import pytest

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "rule_tables.json")))["tables"]
DIMS = sorted(int(d) for d in GOLDEN)


def _golden(d):
    t = GOLDEN[str(d)]
    mags = [float.fromhex(v) for v in t["gen_mag"]]
    code = "0abcdeABCDE"
    gen = []
    for ch in t["gen_code"]:
        k = code.index(ch)
        gen.append(0.0 if k == 0 else (mags[k - 1] if k <= 5 else -mags[k - 6]))
    return {
        "feval": t["feval"],
        "w": np.array([float.fromhex(v) for v in t["w"]]),
        "scale": np.array([float.fromhex(v) for v in t["scale"]]),
        "norm": np.array([float.fromhex(v) for v in t["norm"]]),
        "set_of": np.array(t["gindex"], dtype=np.int32),
        "gen": np.array(gen).reshape(t["feval"], d),
    }


def _same(a, b):
    return np.asarray(a, dtype=np.float64).tobytes() == np.asarray(b, dtype=np.float64).tobytes()


@pytest.mark.parametrize("d", DIMS)
def test_oracle_tables_match_reference(orc, d):
    g, o = _golden(d), orc.rule_tables(d)
    assert o["feval"] == g["feval"]
    assert _same(o["w"], g["w"]) and _same(o["scale"], g["scale"]) and _same(o["norm"], g["norm"])
    assert (o["set_of"] == g["set_of"]).all()
    assert _same(o["gen"], g["gen"])


@pytest.mark.parametrize("d", DIMS)
def test_library_tables_match_reference(lib, d):
    import gpuintegration_gb300 as pg
    g, t = _golden(d), pg.rule_tables(d)
    assert t["feval"] == g["feval"]
    assert _same(t["w"], g["w"]) and _same(t["scale"], g["scale"]) and _same(t["norm"], g["norm"])
    assert (t["set_of"] == g["set_of"]).all()
    assert _same(t["gen"], g["gen"])


@pytest.mark.parametrize("d", DIMS)
def test_rule_exact_on_monomials(orc, d):
    """The basic rule integrates monomials of degree <= 9 exactly on [-1/2,1/2]^d (so [0,1]^d)."""
    t = orc.rule_tables(d)
    w = t["w"].reshape(9, 5)[:, 0][t["set_of"]]
    x = t["gen"]
    rng = np.random.default_rng(d)
    for _ in range(20):
        deg = rng.integers(0, 10)
        powers = np.zeros(d, dtype=int)
        for _ in range(deg):
            powers[rng.integers(0, d)] += 1
        got = float(np.sum(w * np.prod(x ** powers, axis=1)))
        exact = np.prod([0.0 if p % 2 else (0.5 ** p) / (p + 1) for p in powers])
        assert abs(got - exact) < 1e-13, (powers, got, exact)


@pytest.mark.parametrize("d", DIMS)
def test_split_axis_point_order(orc, d):
    """Points 1..4d are (+e_k, -e_k) pairs of sets 1 and 2: the fourth-difference
    code of the reference relies on this order (Sample.cuh:204-209)."""
    t = orc.rule_tables(d)
    g = t["gen"]
    for k in range(d):
        for s, base in ((1, 1), (2, 1 + 2 * d)):
            p, m = g[base + 2 * k], g[base + 2 * k + 1]
            assert t["set_of"][base + 2 * k] == s
            assert p[k] > 0 and m[k] < 0 and p[k] == -m[k]
            assert np.count_nonzero(p) == 1 and np.count_nonzero(m) == 1


@pytest.mark.parametrize("d", list(range(2, 13)))
def test_null_rule_norms_non_negative(lib, d):
    """The evaluation kernel takes the null-rule maxima on the bit patterns of
    |.| * norm, which orders them numerically only when every norm is >= 0."""
    import gpuintegration_gb300 as pg
    t = pg.rule_tables(d)
    assert np.all(t["norm"] >= 0.0) and not np.any(np.signbit(t["norm"]))
