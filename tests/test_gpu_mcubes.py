"""m-Cubes on the GPU: against the CPU oracle (same Philox stream, same work
split, same order of the bin sums), against cuRAND's Philox, bit-for-bit
repeatability from the seed, and on the 6-D sigma=0.01 Gaussian."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import gpuintegration_gb300 as pg
from gpuintegration_gb300 import workloads as W

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_philox_matches_curand(orc):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    rng = np.random.default_rng(5)
    cases = [[int(v) for v in rng.integers(0, 2 ** 32, 6, dtype=np.uint64)] for _ in range(16)]
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "philox")
        subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                               os.path.join(HERE, "curand_philox_check.cu")])
        args = [f"{v:x}" for c in cases for v in c]
        out = subprocess.check_output([exe] + args, text=True).split("\n")
    for c, line in zip(cases, out):
        assert orc.philox(c[:4], c[4:]) == [int(w, 16) for w in line.split()]


@pytest.mark.parametrize("f,ncall", [
    (pg.genz(pg.GAUSSIAN, [5.0, 4.0, 3.0], [0.3, 0.6, 0.5]), 2e5),
    (pg.genz(pg.PRODUCT_PEAK, [3.0, 2.0], [0.4, 0.7]), 1e5),
    (pg.genz(pg.C0, [2.0, 3.0, 1.0, 2.0], [0.5, 0.2, 0.7, 0.4]), 3e5),
    (pg.genz(pg.OSCILLATORY, [1.0, 2.0, 1.5, 0.5, 1.0], [0.1] * 5), 5e5),
    (pg.genz(pg.GAUSSIAN_SUM, [5.0, 4.0, 3.0, 6.0], [0.3, 0.6, 0.5, 0.45]), 4e5),
])
def test_gpu_matches_oracle(ctx, orc, f, ncall):
    r = ctx.mcubes_integrate(f, 1e-3, 0.0, ncall, titer=12, itmax=8, skip=3, seed=99)
    o, _ = orc.mcubes_integrate(f, 1e-3, 0.0, ncall, titer=12, itmax=8, skip=3, seed=99)
    assert r.iters == o.iters and r.status == o.status
    assert abs(r.estimate - o.estimate) <= 1e-9 * abs(o.estimate)
    assert abs(r.errorest - o.errorest) <= 1e-6 * o.errorest
    exact = W.analytic(f)
    assert abs(r.estimate - exact) <= 3 * r.errorest + 1e-12


def test_config3_gaussian_6d(ctx):
    """6-D Gaussian sigma = 0.01 normalised to 1, 500 bins, ncall 2^24
    (15,059,072 calls per iteration by the reference geometry), 20 iterations,
    fixed seed, target relative error 1e-4."""
    f = W.config3_integrand()
    r = ctx.mcubes_integrate(f, 1e-4, 0.0, 2.0 ** 24, titer=20, itmax=20, skip=5, seed=2024)
    assert r.nregions == 14 ** 6
    assert abs(r.estimate - 1.0) <= 3 * r.errorest
    assert r.status == 0 and r.errorest <= 1e-4


@pytest.mark.parametrize("f,ncall", [
    (W.config3_integrand(), 2.0 ** 24),
    (pg.genz(pg.C0, [2.0, 3.0, 1.0, 2.0], [0.5, 0.2, 0.7, 0.4]), 3e5),
])
def test_same_seed_repeats_bit_for_bit(ctx, f, ncall):
    """The per-bin sums that adapt the grid are formed in a fixed order, so two
    runs from one seed agree in every bit; another seed gives another run."""
    runs = [ctx.mcubes_integrate(f, 1e-4, 0.0, ncall, titer=20, itmax=20, skip=5, seed=s) for s in (7, 7, 8)]
    a, b, c = [(r.estimate, r.errorest, r.chi_sq, r.iters, r.status) for r in runs]
    assert a == b
    assert a != c


def test_early_stop_counts_iterations(ctx, orc):
    """After convergence the remaining iterations are skipped on the device:
    the iteration count and result are those of the oracle's loop, which stops."""
    f = pg.genz(pg.PRODUCT_PEAK, [3.0, 2.0], [0.4, 0.7])
    r = ctx.mcubes_integrate(f, 1e-2, 0.0, 1e5, titer=30, itmax=10, skip=2, seed=3)
    o, _ = orc.mcubes_integrate(f, 1e-2, 0.0, 1e5, titer=30, itmax=10, skip=2, seed=3)
    assert r.status == 0 and r.iters == o.iters and r.iters < 30
    assert abs(r.estimate - o.estimate) <= 1e-9 * abs(o.estimate)
