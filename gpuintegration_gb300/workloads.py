"""Seeded Genz test-integral workloads and their analytic values.

The six Genz families (oscillatory, product peak, corner peak, Gaussian, C0,
discontinuous) with u_i ~ U[0,1) and a_i ~ U[0,1) rescaled so that sum a_i is
the family's difficulty: 6, 9, 7, 26, 12 and 6.3 respectively.  The
discontinuous family follows the reference's shape (zero when any x_i > u_i,
common/cuda/integrands.cuh:1459-1486).  Every integral is seeded by
(master seed, index) so a workload is reproducible from its seed alone.

Analytic values are closed forms from the mathematics, evaluated so that the
result is accurate to far better than 1e-7 relative:
  oscillatory    Re[ exp(i 2 pi u_1) prod_j (exp(i a_j) - 1) / (i a_j) ]
  product peak   prod a_i (atan(a_i (1 - u_i)) + atan(a_i u_i))
  corner peak    1/(d! prod a_i) sum_{v in {0,1}^d} (-1)^|v| / (1 + a.v)   (exact rationals)
  Gaussian       prod sqrt(pi)/(2 a_i) (erf(a_i (1 - u_i)) + erf(a_i u_i))
  C0             prod (2 - exp(-a_i u_i) - exp(-a_i (1 - u_i))) / a_i
  discontinuous  prod (exp(a_i u_i) - 1) / a_i
"""
import cmath
import math
from dataclasses import dataclass
from fractions import Fraction
from typing import List

import numpy as np

from . import (C0, CORNER_PEAK, DISCONTINUOUS, GAUSSIAN, GAUSSIAN_SUM, GENZ_FAMILIES, OSCILLATORY, PRODUCT_PEAK,
               Integrand)

DIFFICULTY = {OSCILLATORY: 6.0, PRODUCT_PEAK: 9.0, CORNER_PEAK: 7.0, GAUSSIAN: 26.0, C0: 12.0, DISCONTINUOUS: 6.3}


def _erf(x):
    return math.erf(x)


def analytic(f: Integrand) -> float:
    """Exact integral of a Genz-family integrand over the unit cube."""
    d = f.ndim
    a = [float(v) for v in f.a[:d]]
    u = [float(v) for v in f.u[:d]]
    if f.family == OSCILLATORY:
        z = cmath.exp(1j * 2.0 * math.pi * u[0])
        for aj in a:
            z *= (cmath.exp(1j * aj) - 1.0) / (1j * aj)
        return z.real
    if f.family == PRODUCT_PEAK:
        return math.prod(ai * (math.atan(ai * (1 - ui)) + math.atan(ai * ui)) for ai, ui in zip(a, u))
    if f.family == CORNER_PEAK and d > 8:
        # alternating sum over the 2^d vertices, summed exactly (math.fsum) from rounded terms
        terms = []
        for mask in range(1 << d):
            s = math.fsum(a[k] for k in range(d) if mask >> k & 1)
            terms.append((-1.0 if bin(mask).count("1") % 2 else 1.0) / (1.0 + s))
        return math.fsum(terms) / (math.factorial(d) * math.prod(a))
    if f.family == CORNER_PEAK:
        fa = [Fraction(x) for x in a]
        total = Fraction(0)
        for mask in range(1 << d):
            s = Fraction(1)
            for k in range(d):
                if mask >> k & 1:
                    s += fa[k]
            total += (-1 if bin(mask).count("1") % 2 else 1) / s
        return float(total / (math.factorial(d) * math.prod(fa)))
    if f.family in (GAUSSIAN, GAUSSIAN_SUM):  # the same function; GAUSSIAN_SUM forms one exponential
        scale = float(f.c) if f.c else 1.0
        return math.prod(scale * math.sqrt(math.pi) / (2 * ai) * (_erf(ai * (1 - ui)) + _erf(ai * ui))
                         for ai, ui in zip(a, u))
    if f.family == C0:
        return math.prod((2 - math.exp(-ai * ui) - math.exp(-ai * (1 - ui))) / ai for ai, ui in zip(a, u))
    if f.family == DISCONTINUOUS:
        return math.prod(math.expm1(ai * ui) / ai for ai, ui in zip(a, u))
    raise ValueError("not a Genz family")


def oscillatory_conditioning(f: Integrand) -> float:
    """|value| / |complex amplitude|: small when the real part cancels."""
    z = cmath.exp(1j * 2.0 * math.pi * float(f.u[0]))
    for aj in f.a[:f.ndim]:
        z *= (cmath.exp(1j * aj) - 1.0) / (1j * aj)
    return abs(z.real) / abs(z)


def make(family: int, d: int, rng: np.random.Generator) -> Integrand:
    a = rng.random(d)
    a *= DIFFICULTY[family] / a.sum()
    u = rng.random(d)
    return Integrand(family, d, [float(x) for x in a], [float(x) for x in u])


@dataclass
class Case:
    integrand: Integrand
    epsrel: float
    exact: float
    seed: tuple


def _rng(master: int, index: int) -> np.random.Generator:
    return np.random.default_rng([master, index])


def _accept(f: Integrand) -> bool:
    # An oscillatory integral whose value cancels to < 1e-3 of its amplitude has
    # no meaningful relative tolerance; redraw it (deterministically).
    return f.family != OSCILLATORY or oscillatory_conditioning(f) >= 1e-3


def config2_cases(master: int = 2024) -> List[Case]:
    """8-D, the six families, epsrel in {1e-3, 1e-4, 1e-5, 1e-6}: one seeded integral per (family, epsrel)."""
    out = []
    for fi, fam in enumerate(GENZ_FAMILIES):
        for ei, eps in enumerate((1e-3, 1e-4, 1e-5, 1e-6)):
            k = 0
            while True:
                f = make(fam, 8, _rng(master, 1000 * fi + 10 * ei + k))
                if _accept(f):
                    break
                k += 1
            out.append(Case(f, eps, analytic(f), (master, 1000 * fi + 10 * ei + k)))
    return out


def mixed_cases(count: int, master: int, dmin: int, dmax: int, eps_lo: float, eps_hi: float) -> List[Case]:
    """dim ~ U{dmin..dmax}, family ~ U{6}, epsrel log-uniform in [eps_lo, eps_hi]."""
    out = []
    for i in range(count):
        k = 0
        while True:
            rng = _rng(master, i * 64 + k)
            d = int(rng.integers(dmin, dmax + 1))
            fam = GENZ_FAMILIES[int(rng.integers(0, 6))]
            eps = float(10 ** rng.uniform(math.log10(eps_lo), math.log10(eps_hi)))
            f = make(fam, d, rng)
            if _accept(f):
                break
            k += 1
        out.append(Case(f, eps, analytic(f), (master, i * 64 + k)))
    return out


def config4_candidates(count: int, master: int = 4096) -> List[Case]:
    """Unscreened config-4 stream: dim 2..8, epsrel log-uniform [1e-7, 1e-4]."""
    return mixed_cases(count, master, 2, 8, 1e-7, 1e-4)


def config4_cases(count: int = 4096, screen_path: str = None) -> List[Case]:
    """Batched workload: the first `count` candidates of the config-4 stream that
    PAGANI converges within tolerance (list of accepted candidate indices in
    tests/golden/config4_screen.json, made by tests/golden/make_config4_screen.py)."""
    import json
    import os
    path = screen_path or os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests",
                                       "golden", "config4_screen.json")
    screen = json.load(open(path))
    idx = screen["accepted"][:count]
    cand = mixed_cases(idx[-1] + 1, screen["master"], screen["dmin"], screen["dmax"], screen["eps_lo"],
                       screen["eps_hi"])
    return [cand[i] for i in idx]


def config5_cases(count: int, master: int = 5000) -> List[Case]:
    """Served workload requests: dim 3..10, epsrel log-uniform [1e-6, 1e-3]."""
    return mixed_cases(count, master, 3, 10, 1e-6, 1e-3)


def within_tolerance(estimate: float, exact: float, epsrel: float) -> bool:
    return abs(estimate - exact) <= epsrel * abs(exact)


def config3_integrand(sigma: float = 0.01, d: int = 6) -> Integrand:
    """m-Cubes configuration: exp(-sum (x_i - 0.5)^2 / (2 sigma^2)) / (sigma sqrt(2 pi))^d on [0,1]^d, one
    exponential of the sum as in the reference's m-Cubes Gaussian functors (GAUSSIAN_SUM)."""
    a = 1.0 / (sigma * math.sqrt(2.0))
    return Integrand(GAUSSIAN_SUM, d, [a] * d, [0.5] * d, c=1.0 / (sigma * math.sqrt(2.0 * math.pi)))


def poisson_arrivals(rate_per_s: float, duration_s: float, seed: int = 5005) -> "np.ndarray":
    """Arrival times in milliseconds of a Poisson process, ascending."""
    rng = np.random.default_rng(seed)
    n = int(rate_per_s * duration_s * 1.2) + 16
    t = np.cumsum(rng.exponential(1000.0 / rate_per_s, size=n))
    return t[t < duration_s * 1000.0]
