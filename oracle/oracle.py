"""ctypes wrapper of the CPU oracle (oracle/pagani_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the oracle the GB300 library is tested against.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import this.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["pagani_oracle.cpp"]

_lib = None
_D = ctypes.POINTER(ctypes.c_double)


class OrcResult(ctypes.Structure):
    _fields_ = [("estimate", ctypes.c_double), ("errorest", ctypes.c_double), ("chi_sq", ctypes.c_double),
                ("neval", ctypes.c_uint64), ("nregions", ctypes.c_uint64), ("nfinished", ctypes.c_uint64),
                ("iters", ctypes.c_uint64), ("status", ctypes.c_int32), ("last_phase", ctypes.c_int32)]


def build():
    """Compiles the oracle with g++ (no contraction: results identical on x86-64 and aarch64)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", "-o", LIB] + srcs
    subprocess.check_call(cmd)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(LIB)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    lib.orc_feval.restype = ctypes.c_int
    lib.orc_set_eval_mode.argtypes = [ctypes.c_int]
    lib.orc_set_eval_mode.restype = ctypes.c_int
    lib.orc_budget_fixes.restype = ctypes.c_int
    lib.orc_rule_tables.argtypes = [ctypes.c_int, _D, _D, _D, P(ctypes.c_int32), _D]
    lib.orc_eval_point.restype = ctypes.c_double
    lib.orc_eval_point.argtypes = [vp, _D]
    lib.orc_evaluate_regions.argtypes = [vp, _D, _D, ctypes.c_uint64, _D, _D, _D, _D, P(ctypes.c_int32), ctypes.c_int]
    lib.orc_two_level.argtypes = [ctypes.c_uint64, _D, _D, _D, _D, P(ctypes.c_uint8), ctypes.c_double, ctypes.c_int]
    lib.orc_canon_sum.restype = ctypes.c_double
    lib.orc_canon_sum.argtypes = [_D, ctypes.c_uint64]
    lib.orc_uniform_split.restype = ctypes.c_uint64
    lib.orc_uniform_split.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D]
    lib.orc_filter_split.restype = ctypes.c_uint64
    lib.orc_filter_split.argtypes = [ctypes.c_int, ctypes.c_uint64, _D, _D, P(ctypes.c_uint8), P(ctypes.c_int32), _D,
                                     _D, _D, _D, _D, _D]
    lib.orc_integrate.restype = ctypes.c_int
    lib.orc_integrate.argtypes = [vp, ctypes.c_double, ctypes.c_double, _D, _D, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_int, P(OrcResult), _D, ctypes.c_int]
    lib.orc_integrate_regions.restype = ctypes.c_int
    lib.orc_integrate_regions.argtypes = [vp, ctypes.c_double, ctypes.c_double, _D, _D, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_int, _D, _D, ctypes.c_uint64,
                                          ctypes.c_int, _D, _D, ctypes.c_uint64, P(ctypes.c_uint64), P(OrcResult),
                                          _D, ctypes.c_int]
    lib.orc_philox.argtypes = [P(ctypes.c_uint32), P(ctypes.c_uint32), P(ctypes.c_uint32)]
    if hasattr(lib, "orc_mcubes_integrate"):
        lib.orc_mcubes_integrate.restype = ctypes.c_int
        lib.orc_mcubes_integrate.argtypes = [vp, ctypes.c_double, ctypes.c_double, _D, _D, ctypes.c_double,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                             ctypes.c_double, P(OrcResult), _D, ctypes.c_int]
    _lib = lib
    return lib


def _p(a, t=ctypes.c_double):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(t))


def _integrand_struct(f):
    # Same layout as pg_integrand; accepts a gpuintegration_gb300.Integrand.
    return f.to_c()


def rule_tables(ndim):
    lib = load()
    fe = lib.orc_feval(ndim)
    w, sc, nm = np.zeros(45), np.zeros(45), np.zeros(45)
    so = np.zeros(fe, dtype=np.int32)
    gen = np.zeros(fe * ndim)
    lib.orc_rule_tables(ndim, _p(w), _p(sc), _p(nm), _p(so, ctypes.c_int32), _p(gen))
    return {"w": w, "scale": sc, "norm": nm, "set_of": so, "gen": gen.reshape(fe, ndim), "feval": fe}


def eval_point(f, x):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    s = _integrand_struct(f)
    return lib.orc_eval_point(ctypes.byref(s), _p(x))


class eval_mode:
    """Context manager: the oracle's region-evaluation mode inside the block
    (0 point by point, 1 generator-set sums for the product-form families)."""

    def __init__(self, mode):
        self.mode = mode

    def __enter__(self):
        assert load().orc_set_eval_mode(self.mode) == 0
        return self

    def __exit__(self, *a):
        load().orc_set_eval_mode(0)


def budget_fixes():
    """Iterations of the last integration in which fix_error_budget_overflow fired."""
    return load().orc_budget_fixes()


def evaluate_regions(f, left, length, lows=None, highs=None, nthreads=None):
    lib = load()
    left = np.ascontiguousarray(left, dtype=np.float64)
    length = np.ascontiguousarray(length, dtype=np.float64)
    d = f.ndim
    n = left.size // d
    lows = np.zeros(d) if lows is None else np.ascontiguousarray(lows, dtype=np.float64)
    highs = np.ones(d) if highs is None else np.ascontiguousarray(highs, dtype=np.float64)
    est, err = np.zeros(n), np.zeros(n)
    bis = np.zeros(n, dtype=np.int32)
    s = _integrand_struct(f)
    rc = lib.orc_evaluate_regions(ctypes.byref(s), _p(lows), _p(highs), n, _p(left), _p(length), _p(est), _p(err),
                                  _p(bis, ctypes.c_int32), nthreads or os.cpu_count() or 1)
    assert rc == 0
    return est, err, bis


def two_level(est, err, parent_est, epsrel, relerr_classification=True):
    lib = load()
    est = np.ascontiguousarray(est, dtype=np.float64)
    err = np.ascontiguousarray(err, dtype=np.float64)
    par = np.ascontiguousarray(parent_est, dtype=np.float64)
    n = est.size
    ne, act = np.zeros(n), np.zeros(n, dtype=np.uint8)
    lib.orc_two_level(n, _p(est), _p(err), _p(par), _p(ne), _p(act, ctypes.c_uint8), epsrel,
                      1 if relerr_classification else 0)
    return ne, act


def canon_sum(x):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib.orc_canon_sum(_p(x), x.size)


def uniform_split(ndim, parts):
    lib = load()
    n = lib.orc_uniform_split(ndim, parts, None, None)
    left, length = np.zeros((ndim, n)), np.zeros((ndim, n))
    lib.orc_uniform_split(ndim, parts, _p(left), _p(length))
    return left, length


def filter_split(left, length, active, bisect, est, err):
    lib = load()
    left = np.ascontiguousarray(left, dtype=np.float64)
    length = np.ascontiguousarray(length, dtype=np.float64)
    d, n = left.shape
    active = np.ascontiguousarray(active, dtype=np.uint8)
    bisect = np.ascontiguousarray(bisect, dtype=np.int32)
    est = np.ascontiguousarray(est, dtype=np.float64)
    err = np.ascontiguousarray(err, dtype=np.float64)
    A = int(active.astype(bool).sum())
    ol, oln = np.zeros((d, 2 * A)), np.zeros((d, 2 * A))
    pe, pr = np.zeros(A), np.zeros(A)
    lib.orc_filter_split(d, n, _p(left), _p(length), _p(active, ctypes.c_uint8), _p(bisect, ctypes.c_int32), _p(est),
                         _p(err), _p(ol), _p(oln), _p(pe), _p(pr))
    return ol, oln, pe, pr


def integrate(f, epsrel, epsabs, lows=None, highs=None, relerr_classification=True, device_mem=16e9, max_iters=700,
              nthreads=None, trace_cap=0):
    lib = load()
    d = f.ndim
    lows = np.zeros(d) if lows is None else np.ascontiguousarray(lows, dtype=np.float64)
    highs = np.ones(d) if highs is None else np.ascontiguousarray(highs, dtype=np.float64)
    r = OrcResult()
    tr = np.zeros((max(trace_cap, 1), 6))
    s = _integrand_struct(f)
    nt = lib.orc_integrate(ctypes.byref(s), epsrel, epsabs, _p(lows), _p(highs), 1 if relerr_classification else 0,
                           device_mem, max_iters, nthreads or os.cpu_count() or 1, ctypes.byref(r), _p(tr), trace_cap)
    assert nt >= 0, nt
    return r, tr[:nt]


def integrate_regions(f, left, length, epsrel, epsabs, lows=None, highs=None, relerr_classification=True,
                      predict_split=False, device_mem=16e9, max_iters=700, nthreads=None, snap_cap=0):
    """Workspace::integrate from a first region list (None: the uniform split),
    with the predict_split variant; returns (result, snapshot or None)."""
    lib = load()
    d = f.ndim
    lows = np.zeros(d) if lows is None else np.ascontiguousarray(lows, dtype=np.float64)
    highs = np.ones(d) if highs is None else np.ascontiguousarray(highs, dtype=np.float64)
    n = 0
    if left is not None:
        left = np.ascontiguousarray(left, dtype=np.float64)
        length = np.ascontiguousarray(length, dtype=np.float64)
        n = left.shape[1]
    sl = np.zeros(d * max(snap_cap, 1))  # filled as SoA (d, n) over the first d * n entries
    sn = np.zeros(d * max(snap_cap, 1))
    snap_n = ctypes.c_uint64()
    r = OrcResult()
    s = _integrand_struct(f)
    nt = lib.orc_integrate_regions(ctypes.byref(s), epsrel, epsabs, _p(lows), _p(highs),
                                   1 if relerr_classification else 0, device_mem, max_iters,
                                   nthreads or os.cpu_count() or 1, _p(left), _p(length), n,
                                   1 if predict_split else 0, _p(sl), _p(sn), snap_cap, ctypes.byref(snap_n),
                                   ctypes.byref(r), None, 0)
    assert nt >= 0, nt
    snap = None
    if snap_n.value:
        k = snap_n.value
        snap = (k, (sl[:d * k].reshape(d, k).copy(), sn[:d * k].reshape(d, k).copy()) if snap_cap >= k else None)
    return r, snap


def philox(ctr, key):
    lib = load()
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib.orc_philox(c, k, o)
    return list(o)


def mcubes_integrate(f, epsrel, epsabs, ncall, titer=15, itmax=15, skip=5, nbins=500, seed=0x5EED, alpha=1.5,
                     lows=None, highs=None, trace_cap=0):
    lib = load()
    d = f.ndim
    lows = np.zeros(d) if lows is None else np.ascontiguousarray(lows, dtype=np.float64)
    highs = np.ones(d) if highs is None else np.ascontiguousarray(highs, dtype=np.float64)
    r = OrcResult()
    tr = np.zeros((max(trace_cap, 1), 4))
    s = _integrand_struct(f)
    nt = lib.orc_mcubes_integrate(ctypes.byref(s), epsrel, epsabs, _p(lows), _p(highs), ncall, titer, itmax, skip,
                                  nbins, seed, alpha, ctypes.byref(r), _p(tr), trace_cap)
    assert nt >= 0, nt
    return r, tr[:nt]
