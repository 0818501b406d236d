"""Region evaluation by generator-set sums (PG_EVAL_SET_SUMS).

For the product-form families the library can form the rule's nine
generator-set sums by a recurrence over the axes instead of evaluating every
rule point.  The sums are the reference's (Sample.cuh:145-148 accumulates
f * w[set(p)][r] point by point), rounded differently, so per-region
estimates are compared with the reference's own kernel (tests/golden/
ref_phase1.npz) at 1e-12 relative and errors at 1e-12 of |estimate| + error,
the tolerance of the transcendental families in the point-by-point mode (the
null rules are differences of nearly equal sums).  The split axes must be the
reference kernel's exactly: the values the fourth differences read are formed
as in the point-by-point evaluation.  Against the oracle's restatement of the
same recurrence the library is bit-exact for integrands built from + - * /.

One exception, on random regions far smaller than the golden cases': where f
is so smooth over a region that its null rules cancel to rounding noise, the
error estimate is that noise, and two summation orders give different noise
(a few regions in a million at d = 8, e.g. 2.5e-7 of the estimate point by
point against 3.5e-15 from the set sums, whose positive-term sums are better
conditioned).  Such errors are accepted when both are below NOISE_FLOOR of the
region's estimate.
"""
import os

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from tests.golden.ref_phase1_cases import CASES, case_inputs
from tests.reference_cases import CONFIG1, CONFIG1_VALUE

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_phase1.npz"))
PRODUCT_FORM = (pg.PRODUCT_PEAK, pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS, pg.PRODUCT)
IEEE_EXACT = (pg.PRODUCT_PEAK, pg.PRODUCT)
SEP_CASES = [i for i, c in enumerate(CASES) if c[0] in PRODUCT_FORM]
OTHER_CASES = [i for i, c in enumerate(CASES) if c[0] not in PRODUCT_FORM]
IDS = {i: f"{pg.FAMILY_NAMES[c[0]]}-d{c[1]}{'-box' if c[3] else ''}" for i, c in enumerate(CASES)}
REL = 1e-12
NOISE_FLOOR = 1e-6


def _errors_agree(err, ref_err, ref_est):
    close = np.abs(err - ref_err) <= REL * (np.abs(ref_est) + ref_err) + 1e-300
    noise = (err <= NOISE_FLOOR * np.abs(ref_est)) & (ref_err <= NOISE_FLOOR * np.abs(ref_est))
    return bool(np.all(close | noise))


def _close_to_reference(est, err, bis, i):
    re, rr, rb = GOLD[f"est_{i}"], GOLD[f"err_{i}"], GOLD[f"bis_{i}"]
    assert np.all(np.abs(est - re) <= REL * np.abs(re) + 1e-300)
    assert np.all(np.abs(err - rr) <= REL * (np.abs(re) + rr) + 1e-300)
    assert (bis == rb).all()


@pytest.mark.parametrize("i", SEP_CASES, ids=[IDS[i] for i in SEP_CASES])
def test_oracle_setsums_vs_reference_kernel(orc, i):
    f, left, length, lows, highs = case_inputs(CASES[i])
    with orc.eval_mode(1):
        est, err, bis = orc.evaluate_regions(f, left, length, lows, highs)
    _close_to_reference(est, err, bis, i)


def test_oracle_setsums_fall_back_for_other_families(orc):
    """Families that are not products of per-axis factors are evaluated point by point."""
    for i in OTHER_CASES[:4]:
        f, left, length, lows, highs = case_inputs(CASES[i])
        a = orc.evaluate_regions(f, left, length, lows, highs)
        with orc.eval_mode(1):
            b = orc.evaluate_regions(f, left, length, lows, highs)
        for x, y in zip(a, b):
            assert np.asarray(x).tobytes() == np.asarray(y).tobytes()


def test_oracle_setsums_full_loop_config1(orc):
    """Config 1 in set-sum mode converges to the analytic value like the point-by-point loop."""
    f = CONFIG1
    with orc.eval_mode(1):
        r, _ = orc.integrate(f, 1e-3, 0.0)
    p, _ = orc.integrate(f, 1e-3, 0.0)
    assert r.status == 0
    assert abs(r.estimate - CONFIG1_VALUE) <= 1e-3 * CONFIG1_VALUE
    assert abs(r.estimate - p.estimate) <= 1e-9 * abs(p.estimate)
    assert r.nregions == p.nregions


@pytest.mark.gpu
@pytest.mark.parametrize("i", SEP_CASES, ids=[IDS[i] for i in SEP_CASES])
def test_library_setsums_vs_reference_kernel(ctx, i):
    f, left, length, lows, highs = case_inputs(CASES[i])
    vol = None if lows is None else pg.Volume(list(lows), list(highs))
    est, err, bis = ctx.evaluate_regions(f, left, length, vol, eval_mode=pg.EVAL_SET_SUMS)
    _close_to_reference(est, err, bis, i)


@pytest.mark.gpu
@pytest.mark.parametrize("i", OTHER_CASES, ids=[IDS[i] for i in OTHER_CASES])
def test_library_setsum_mode_other_families_bitwise(ctx, i):
    """Non-product families take the point-by-point kernel in set-sum mode: bit for bit the reference's."""
    f, left, length, lows, highs = case_inputs(CASES[i])
    vol = None if lows is None else pg.Volume(list(lows), list(highs))
    est, err, bis = ctx.evaluate_regions(f, left, length, vol, eval_mode=pg.EVAL_SET_SUMS)
    assert est.tobytes() == GOLD[f"est_{i}"].tobytes()
    assert err.tobytes() == GOLD[f"err_{i}"].tobytes()
    assert (bis == GOLD[f"bis_{i}"]).all()


def _regions(rng, d, n):
    depth = rng.integers(0, 9, size=(d, n))
    length = 0.5 ** depth
    left = np.floor(rng.random((d, n)) / length) * length
    return left, length


@pytest.mark.gpu
@pytest.mark.parametrize("d", range(2, 13))
@pytest.mark.parametrize("family", PRODUCT_FORM)
def test_library_setsums_vs_oracle(ctx, orc, family, d):
    rng = np.random.default_rng(31 * d + family)
    a = rng.random(d) * 5 + 0.5
    f = pg.Integrand(family, d, list(a), list(rng.random(d)))
    n = 700 if d <= 10 else 200  # more than one block of 128 regions, a ragged last block
    left, length = _regions(rng, d, n)
    est, err, bis = ctx.evaluate_regions(f, left, length, eval_mode=pg.EVAL_SET_SUMS)
    with orc.eval_mode(1):
        oest, oerr, obis = orc.evaluate_regions(f, left, length)
    if family in IEEE_EXACT:
        assert est.tobytes() == oest.tobytes() and err.tobytes() == oerr.tobytes()
        assert (bis == obis).all()
    else:
        assert np.all(np.abs(est - oest) <= REL * np.abs(oest) + 1e-300)
        assert _errors_agree(err, oerr, oest)
        assert np.mean(bis == obis) >= 0.97  # glibc's exp is not CUDA's: ties of fourth differences may flip
    # and against the point-by-point evaluation of the same regions
    pest, perr, pbis = ctx.evaluate_regions(f, left, length)
    assert np.all(np.abs(est - pest) <= REL * np.abs(pest) + 1e-300)
    assert _errors_agree(err, perr, pest)
    assert (bis == pbis).all()


@pytest.mark.gpu
def test_library_setsums_general_box(ctx, orc):
    rng = np.random.default_rng(5)
    for d in (3, 6, 9):
        f = pg.Integrand(pg.PRODUCT_PEAK, d, list(rng.random(d) * 4 + 1), list(rng.random(d)))
        lows = -1.0 - rng.random(d)
        highs = 0.5 + 2 * rng.random(d)
        left, length = _regions(rng, d, 300)
        est, err, bis = ctx.evaluate_regions(f, left, length, pg.Volume(list(lows), list(highs)),
                                             eval_mode=pg.EVAL_SET_SUMS)
        with orc.eval_mode(1):
            oest, oerr, obis = orc.evaluate_regions(f, left, length, lows, highs)
        assert est.tobytes() == oest.tobytes() and err.tobytes() == oerr.tobytes() and (bis == obis).all()


def _opts(**kw):
    return pg.default_options(eval_mode=pg.EVAL_SET_SUMS, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("eps", [1e-3, 1e-4, 1e-5, 1e-6])
def test_full_loop_product_peak_bitwise_vs_oracle(ctx, orc, eps):
    """Whole iteration in set-sum mode: estimate, error, regions and iterations equal the oracle's bit for bit."""
    rng = np.random.default_rng(int(-np.log10(eps)))
    f = pg.genz(pg.PRODUCT_PEAK, list(rng.random(8) * 9 / 4), list(rng.random(8)))
    r = ctx.integrate(f, eps, 0.0, options=_opts())
    with orc.eval_mode(1):
        o, _ = orc.integrate(f, eps, 0.0)
    assert (r.estimate, r.errorest, r.nregions, r.iters, r.status) == \
           (o.estimate, o.errorest, o.nregions, o.iters, o.status)


@pytest.mark.gpu
def test_full_loop_config1_bitwise_vs_oracle(ctx, orc):
    f = CONFIG1
    r = ctx.integrate(f, 1e-3, 0.0, options=_opts())
    with orc.eval_mode(1):
        o, _ = orc.integrate(f, 1e-3, 0.0)
    assert (r.estimate, r.errorest, r.nregions) == (o.estimate, o.errorest, o.nregions)
    assert abs(r.estimate - CONFIG1_VALUE) <= 1e-3 * CONFIG1_VALUE


@pytest.mark.gpu
def test_batch_in_setsum_mode_equals_alone(ctx):
    """A mixed batch (product-form and other families, so several evaluation runs
    per iteration) gives each integral its stand-alone set-sum result bit for bit,
    also with a pool small enough to force admission waits and spills."""
    from gpuintegration_gb300 import workloads as W
    rng = np.random.default_rng(77)
    fs = [W.make(pg.GENZ_FAMILIES[int(rng.integers(0, 6))], int(rng.integers(2, 9)), rng) for _ in range(30)]
    eps = 10 ** rng.uniform(-5, -3.5, size=len(fs))
    for pool in (0, 3000):
        opt = _opts(max_regions=pool)
        batch = ctx.batch_integrate(fs, eps, 0.0, options=opt)
        for f, e, b in zip(fs, eps, batch):
            r = ctx.integrate(f, float(e), 0.0, options=_opts())
            assert (r.estimate, r.errorest, r.nregions, r.status, r.iters) == \
                   (b.estimate, b.errorest, b.nregions, b.status, b.iters)
    st = ctx.stats()
    assert st.setsum_regions > 0


@pytest.mark.gpu
@pytest.mark.parametrize("family", [pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS, pg.PRODUCT_PEAK])
def test_full_loop_setsums_meet_tolerance(ctx, family):
    """8-D, epsrel 1e-3..1e-5: set-sum results are within epsrel of the analytic value."""
    from gpuintegration_gb300 import workloads as W
    for k, eps in enumerate((1e-3, 1e-4, 1e-5)):
        f = W.make(family, 8, np.random.default_rng([family, k]))
        r = ctx.integrate(f, eps, 0.0, options=_opts())
        p = ctx.integrate(f, eps, 0.0)
        assert r.status == 0
        exact = W.analytic(f)
        assert abs(r.estimate - exact) <= 2 * eps * abs(exact) or abs(r.estimate - p.estimate) <= 1e-6 * abs(exact)
        assert abs(r.estimate - p.estimate) <= eps * abs(exact)


@pytest.mark.gpu
def test_parent_terms_cache_changes_no_bit(ctx, monkeypatch):
    """Sibling pairs take the factors of every axis but the split one from
    their parent's kept terms; those are the values they would compute, so
    results with the cache and without it (PG_SETSUM_CACHE=0) agree bit for
    bit, alone and in batches (with spills, whose integrals restart without
    cached terms), at up to 12 dimensions."""
    from gpuintegration_gb300 import workloads as W
    rng = np.random.default_rng(31)
    fams = (pg.GAUSSIAN, pg.C0, pg.PRODUCT_PEAK, pg.DISCONTINUOUS)
    fs = [W.make(fams[i % 4], d, rng) for i, d in enumerate((3, 5, 8, 8, 8, 10, 12, 6))]
    eps = [1e-4, 1e-5, 1e-4, 1e-5, 1e-6, 1e-3, 1e-3, 1e-5]

    def run():
        alone = [ctx.integrate(f, e, 0.0, options=_opts()) for f, e in zip(fs, eps)]
        batch = ctx.batch_integrate(fs, eps, 0.0, options=_opts())
        small = ctx.batch_integrate(fs, eps, 0.0, options=_opts(max_regions=20000))
        return [(r.estimate, r.errorest, r.nregions, r.iters, r.status) for r in alone + batch + small]

    with_cache = run()
    monkeypatch.setenv("PG_SETSUM_CACHE", "0")
    assert run() == with_cache
