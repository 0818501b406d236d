"""The whole PAGANI iteration against the reference's own run.

tests/golden/ref_iter.npz holds, per iteration, the region count, the split
axis of every region, the active flags set by the reference's two-level
stage, the flags the iteration keeps (after the error-budget fix), the
iteration totals, the final result and, for most cases, every region's
estimate, raw error and two-level error.  They were made by running the
reference's compiled device stages (region evaluation, RefineError,
alignRegions, divideIntervalsGPU) in the reference's loop
(tests/golden/make_ref_iter_golden.py).

Each test walks the reference's trajectory: from the uniform split, it
evaluates the iteration's regions with the stage under test, compares split
axes, estimates and errors, runs the two-level stage on the reference's
parents and compares errors and flags, then filters and splits with the
reference's kept flags to reach the next iteration's list.  Split axes and
flags must be identical in every region (zero flips).  Values must be
bit-identical for the integrands built from + - * / and for the library's
device evaluation of every family (CUDA's exp is the reference's); the CPU
oracle's glibc exp may differ from CUDA's in the last bit, so its estimates
and errors of the exp families are compared at 1e-12 (errors at 1e-12 of
|estimate| + error).  The full loops must give the reference's region count
and iteration count; their totals are compensated sums here and plain sums in
the reference, so estimates and errors agree to 1e-12 of the magnitudes
summed, not bitwise.
"""
import os

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from tests.golden.ref_iter_cases import cases

PATH = os.path.join(os.path.dirname(__file__), "golden", "ref_iter.npz")
GOLD = np.load(PATH) if os.path.exists(PATH) else None
CASES = cases()
IEEE_EXACT = (pg.PRODUCT_PEAK, pg.CORNER_PEAK, pg.PRODUCT, pg.CONSTANT)
needs_gold = pytest.mark.skipif(GOLD is None, reason="tests/golden/ref_iter.npz not generated")


def _same(a, b, exact, scale=None, floor=None):
    a, b = np.asarray(a), np.asarray(b)
    if exact:
        return a.tobytes() == b.tobytes()
    s = np.abs(b) if scale is None else scale
    ok = np.abs(a - b) <= 1e-12 * s + 1e-300
    if floor is not None:  # both values at the rounding-noise floor
        ok |= (np.abs(a) <= floor) & (np.abs(b) <= floor)
    return bool(np.all(ok))


def _walk(name, f, eps, full, evaluate, two_level, filter_split, exact_values, noise_floor=0.0):
    from oracle import oracle
    n_it = GOLD[f"{name}/n"]
    d = f.ndim
    parts = 4 if d < 5 else (2 if d <= 10 else 1)
    left, length = oracle.uniform_split(d, parts)
    parent = None
    off = 0
    for i, n in enumerate(n_it):
        n = int(n)
        assert left.shape[1] == n, (name, i)
        sl = slice(off, off + n)
        est, err_raw, bis = evaluate(f, left, length)
        assert (bis == GOLD[f"{name}/bisect"][sl]).all(), (name, i, "split axes")
        if parent is None:
            err, act = err_raw, np.ones(n, dtype=np.uint8)
        else:
            err, act = two_level(est, err_raw, parent, eps)
        assert (np.asarray(act, dtype=np.uint8) == GOLD[f"{name}/act_refine"][sl]).all(), (name, i, "flags")
        if full:
            ge, gr, g2 = GOLD[f"{name}/est"][sl], GOLD[f"{name}/err_raw"][sl], GOLD[f"{name}/err"][sl]
            assert _same(est, ge, exact_values), (name, i, "estimates")
            floor = noise_floor * np.abs(ge) if noise_floor else None
            assert _same(err_raw, gr, exact_values, np.abs(ge) + gr, floor), (name, i, "errors")
            assert _same(err, g2, exact_values, np.abs(ge) + g2, floor), (name, i, "two-level errors")
        keep = GOLD[f"{name}/act"][sl]
        off += n
        if i + 1 == len(n_it) or keep.sum() == 0:
            break
        left, length, parent, _ = filter_split(left, length, keep, GOLD[f"{name}/bisect"][sl], est, err)


def _check_result(name, r):
    # The totals add one finished part per iteration, each the iteration's
    # sum less its active regions' sum (nearly equal sums for the error), so
    # they are compared at 1e-12 of the magnitudes summed: the iterations'
    # estimate and error totals.
    g = GOLD[f"{name}/result"]
    sums = np.abs(GOLD[f"{name}/iter_sums"]).sum(axis=0)
    assert (r.nregions, r.iters, r.status) == (int(g[2]), int(g[3]), int(g[4])), name
    assert abs(r.estimate - g[0]) <= 1e-12 * max(abs(g[0]), sums[0])
    assert abs(r.errorest - g[1]) <= 1e-12 * max(abs(g[1]), sums[1])


@needs_gold
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_walks_the_reference_iteration(orc, case):
    name, f, eps, full = case
    _walk(name, f, eps, full,
          lambda f, l, n: orc.evaluate_regions(f, l, n),
          lambda e, r, p, eps: orc.two_level(e, r, p, eps),
          lambda l, n, a, b, e, r: orc.filter_split(l, n, a, b, e, r),
          exact_values=f.family in IEEE_EXACT)


@needs_gold
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_full_loop_matches_reference_run(orc, case):
    name, f, eps, _ = case
    r, _ = orc.integrate(f, eps, 0.0)
    _check_result(name, r)
    # fix_error_budget_overflow (Workspace.cuh:121-146) fires in as many iterations as in the reference's run
    assert orc.budget_fixes() == int(GOLD[f"{name}/fixed"].sum())


@needs_gold
@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_library_walks_the_reference_iteration(ctx, case):
    name, f, eps, full = case
    _walk(name, f, eps, full,
          lambda f, l, n: ctx.evaluate_regions(f, l, n),
          lambda e, r, p, eps: ctx.two_level(e, r, p, eps),
          lambda l, n, a, b, e, r: ctx.filter_split(l, n, a, b, e, r),
          exact_values=True)


@needs_gold
@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_library_full_loop_matches_reference_run(ctx, case):
    name, f, eps, _ = case
    _check_result(name, ctx.integrate(f, eps, 0.0))


# The set-sum evaluation (PG_EVAL_SET_SUMS) of the product-form families on the
# reference's trajectory: the same split axes and flags in every region;
# estimates and errors at 1e-12, errors also accepted where both sit at the
# null rules' rounding-noise floor (1e-6 of the estimate; see
# tests/test_setsum.py).
SETSUM_CASES = [c for c in CASES if c[1].family in (pg.PRODUCT_PEAK, pg.GAUSSIAN, pg.C0)]


@needs_gold
@pytest.mark.gpu
@pytest.mark.parametrize("case", SETSUM_CASES, ids=[c[0] for c in SETSUM_CASES])
def test_library_setsums_walk_the_reference_iteration(ctx, case):
    name, f, eps, full = case
    _walk(name, f, eps, full,
          lambda f, l, n: ctx.evaluate_regions(f, l, n, eval_mode=pg.EVAL_SET_SUMS),
          lambda e, r, p, eps: ctx.two_level(e, r, p, eps),
          lambda l, n, a, b, e, r: ctx.filter_split(l, n, a, b, e, r),
          exact_values=False, noise_floor=1e-6)


@needs_gold
@pytest.mark.gpu
@pytest.mark.parametrize("case", SETSUM_CASES, ids=[c[0] for c in SETSUM_CASES])
def test_library_setsums_full_loop_matches_reference_run(ctx, case):
    name, f, eps, _ = case
    _check_result(name, ctx.integrate(f, eps, 0.0, options=pg.default_options(eval_mode=pg.EVAL_SET_SUMS)))
