"""GB300-native PAGANI adaptive cubature and m-Cubes VEGAS, Python side.

This module is a thin ctypes layer over the C ABI in include/pagani_gb300.h
(libpagani_gb300.so, built in-tree by gpuintegration_gb300/_build.py).  It
mirrors the reference's C++ interface so that code written against it reads
the same:

    Workspace(ndim).integrate(integrand, epsrel, epsabs, vol)
        -> IntegrationResult        # cuda/pagani/quad/GPUquad/Workspace.cuh:361-368
    mcubes_integrate(integrand, epsrel, epsabs, ncall, vol, titer, itmax, skip)
        -> IntegrationResult        # cuda/mcubes/vegasT.cuh:999-1030

Integrands are described by family and parameters (Integrand), because a
device functor cannot cross a C ABI.  There is no CPU fallback: if the CUDA
library cannot be loaded, every call raises.
"""
import ctypes
import os
import re
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpagani_gb300.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "pagani_gb300.h")

MAX_DIM = 16
MIN_NDIM = 2
MAX_NDIM = 12

PG_OK = 0
PG_NOT_CONVERGED = 1
PG_BAD_ARG = -1
PG_OOM = -2
PG_CUDA_ERROR = -3
PG_TIMEOUT = -4
PG_UNSUPPORTED = -5

# Region-evaluation modes (pg_options.eval_mode): every rule point in the
# reference's order, or generator-set sums for the product-form families.
EVAL_POINTS = 0
EVAL_SET_SUMS = 1

(CONSTANT, OSCILLATORY, PRODUCT_PEAK, CORNER_PEAK, GAUSSIAN, C0, DISCONTINUOUS, PRODUCT, NAN_VALUE, BOX, FUN6,
 GAUSSIAN_SUM) = range(12)
FAMILY_NAMES = {
    CONSTANT: "constant", OSCILLATORY: "oscillatory", PRODUCT_PEAK: "product_peak", CORNER_PEAK: "corner_peak",
    GAUSSIAN: "gaussian", C0: "c0", DISCONTINUOUS: "discontinuous", PRODUCT: "product", NAN_VALUE: "nan",
    BOX: "box", FUN6: "fun6", GAUSSIAN_SUM: "gaussian_sum",
}
GENZ_FAMILIES = (OSCILLATORY, PRODUCT_PEAK, CORNER_PEAK, GAUSSIAN, C0, DISCONTINUOUS)


class PgIntegrand(ctypes.Structure):
    _fields_ = [("family", ctypes.c_int32), ("ndim", ctypes.c_int32), ("a", ctypes.c_double * MAX_DIM),
                ("u", ctypes.c_double * MAX_DIM), ("c", ctypes.c_double)]


class PgResult(ctypes.Structure):
    _fields_ = [("estimate", ctypes.c_double), ("errorest", ctypes.c_double), ("chi_sq", ctypes.c_double),
                ("neval", ctypes.c_uint64), ("nregions", ctypes.c_uint64), ("nfinished", ctypes.c_uint64),
                ("iters", ctypes.c_uint64), ("status", ctypes.c_int32), ("last_phase", ctypes.c_int32)]


class PgOptions(ctypes.Structure):
    _fields_ = [("relerr_classification", ctypes.c_int32), ("max_iters", ctypes.c_int32),
                ("device_mem_model", ctypes.c_double), ("max_regions", ctypes.c_uint64),
                ("eval_mode", ctypes.c_int32), ("predict_split", ctypes.c_int32)]


class PgStats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint64), ("eval_launches", ctypes.c_uint64),
                ("regions_evaluated", ctypes.c_uint64), ("points_evaluated", ctypes.c_uint64),
                ("eval_ms", ctypes.c_double), ("stage_ms", ctypes.c_double), ("stage_bytes", ctypes.c_uint64),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("tune_warps", ctypes.c_int32 * 2), ("tune_ctas_per_sm", ctypes.c_int32 * 2),
                ("eval_bytes", ctypes.c_uint64), ("host_ms", ctypes.c_double), ("sync_ms", ctypes.c_double),
                ("spill_ms", ctypes.c_double), ("admit_ms", ctypes.c_double),
                ("setsum_regions", ctypes.c_uint64), ("classify_ms", ctypes.c_double),
                ("classify_passes", ctypes.c_uint64), ("setsum_pairs", ctypes.c_uint64),
                ("setsum_cached_pairs", ctypes.c_uint64)]


class PgIterationRecord(ctypes.Structure):
    _fields_ = [("regions", ctypes.c_uint64), ("integrals", ctypes.c_uint32), ("eval_launches", ctypes.c_uint32),
                ("eval_ms", ctypes.c_double), ("stage_ms", ctypes.c_double)]


class PgMcubesOptions(ctypes.Structure):
    _fields_ = [("ncall", ctypes.c_double), ("titer", ctypes.c_int32), ("itmax", ctypes.c_int32),
                ("skip", ctypes.c_int32), ("nbins", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("alpha", ctypes.c_double)]


_lib = None
_D = ctypes.POINTER(ctypes.c_double)


def _ptr(a, ctype=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ctype)) if a is not None else None


def load_library(path: str = LIB_PATH):
    """Loads libpagani_gb300.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with gpuintegration_gb300._build.build() "
                           "(the GB300 library has no CPU fallback)")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    c_ctx = ctypes.c_void_p
    sig = {
        "pg_options_default": (None, [P(PgOptions)]),
        "pg_feval": (ctypes.c_int, [ctypes.c_int]),
        "pg_context_create": (ctypes.c_int, [ctypes.c_int, P(c_ctx)]),
        "pg_context_destroy": (ctypes.c_int, [c_ctx]),
        "pg_last_error": (ctypes.c_char_p, [c_ctx]),
        "pg_context_set_profiling": (ctypes.c_int, [c_ctx, ctypes.c_int]),
        "pg_context_stats": (ctypes.c_int, [c_ctx, P(PgStats)]),
        "pg_context_reset_stats": (ctypes.c_int, [c_ctx]),
        "pg_context_iterations": (ctypes.c_int, [c_ctx, P(PgIterationRecord), ctypes.c_uint64,
                                                 P(ctypes.c_uint64)]),
        "pg_context_fail_allocation": (ctypes.c_int, [c_ctx, ctypes.c_int64]),
        "pg_context_stream": (ctypes.c_void_p, [c_ctx]),
        "pg_synchronize": (ctypes.c_int, [c_ctx]),
        "pg_integrate_regions": (ctypes.c_int, [c_ctx, P(PgIntegrand), _D, _D, ctypes.c_uint64, ctypes.c_double,
                                                ctypes.c_double, _D, _D, P(PgOptions), P(PgResult)]),
        "pg_last_snapshot": (ctypes.c_int, [c_ctx, P(ctypes.c_int32), P(ctypes.c_uint64), _D, _D, ctypes.c_uint64]),
        "pg_integrate": (ctypes.c_int, [c_ctx, P(PgIntegrand), ctypes.c_double, ctypes.c_double, _D, _D,
                                        P(PgOptions), P(PgResult)]),
        "pg_evaluate_regions": (ctypes.c_int, [c_ctx, P(PgIntegrand), _D, _D, ctypes.c_uint64, _D, _D, _D, _D,
                                               P(ctypes.c_int32), ctypes.c_int32]),
        "pg_evaluate_regions_device": (ctypes.c_int, [c_ctx, P(PgIntegrand), _D, _D, ctypes.c_uint64,
                                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
        "pg_two_level": (ctypes.c_int, [c_ctx, ctypes.c_uint64, _D, _D, _D, _D, P(ctypes.c_uint8), ctypes.c_double,
                                        ctypes.c_int32]),
        "pg_filter_split": (ctypes.c_int, [c_ctx, ctypes.c_int, ctypes.c_uint64, _D, _D, P(ctypes.c_uint8),
                                           P(ctypes.c_int32), _D, _D, _D, _D, _D, _D, P(ctypes.c_uint64)]),
        "pg_reduce_sum": (ctypes.c_int, [c_ctx, _D, ctypes.c_uint64, _D]),
        "pg_exclusive_scan_flags": (ctypes.c_int, [c_ctx, P(ctypes.c_uint8), ctypes.c_uint64, P(ctypes.c_uint64),
                                                   P(ctypes.c_uint64)]),
        "pg_rule_tables": (ctypes.c_int, [ctypes.c_int, _D, _D, _D, P(ctypes.c_int32), _D]),
        "do_integration_from_c": (ctypes.c_int, [_D]),
        "pg_mcubes_options_default": (None, [P(PgMcubesOptions)]),
        "pg_mcubes_integrate": (ctypes.c_int, [c_ctx, P(PgIntegrand), ctypes.c_double, ctypes.c_double, _D, _D,
                                               P(PgMcubesOptions), P(PgResult)]),
        "pg_batch_integrate": (ctypes.c_int, [c_ctx, ctypes.c_uint64, P(PgIntegrand), _D, _D, P(PgOptions),
                                              P(PgResult)]),
        "pg_batch_integrate_timed": (ctypes.c_int, [c_ctx, ctypes.c_uint64, P(PgIntegrand), _D, _D, P(PgOptions),
                                                    P(PgResult), _D]),
        "pg_probe_fp64_peak": (ctypes.c_int, [c_ctx, _D]),
        "pg_serve": (ctypes.c_int, [c_ctx, ctypes.c_uint64, P(PgIntegrand), _D, _D, _D, ctypes.c_uint64,
                                    ctypes.c_double, P(PgOptions), P(PgResult), _D]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def declared_symbols(header: str = HEADER_PATH) -> List[str]:
    """Names of the functions include/pagani_gb300.h declares."""
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_\w+|do_integration_from_c)\s*\(", text)) - {"pg_status"})


# ---------------------------------------------------------------------------
@dataclass
class Integrand:
    """An integrand of one of the library's families (see include/pagani_gb300.h)."""
    family: int
    ndim: int
    a: Sequence[float] = ()
    u: Sequence[float] = ()
    c: float = 0.0

    def to_c(self) -> PgIntegrand:
        s = PgIntegrand()
        s.family = int(self.family)
        s.ndim = int(self.ndim)
        for i, v in enumerate(self.a):
            s.a[i] = float(v)
        for i, v in enumerate(self.u):
            s.u[i] = float(v)
        s.c = float(self.c)
        return s


def genz(family: int, a: Sequence[float], u: Sequence[float]) -> Integrand:
    return Integrand(family, len(a), list(a), list(u))


def constant(ndim: int, value: float) -> Integrand:
    return Integrand(CONSTANT, ndim, c=value)


@dataclass
class Volume:
    """quad::Volume<T, ndim> (common/cuda/Volume.cuh:9-52): per-axis lows/highs."""
    lows: Sequence[float]
    highs: Sequence[float]

    @staticmethod
    def unit(ndim: int) -> "Volume":
        return Volume([0.0] * ndim, [1.0] * ndim)


@dataclass
class IntegrationResult:
    """numint::integration_result (common/integration_result.hh:11-21)."""
    estimate: float = 0.0
    errorest: float = 0.0
    neval: int = 0
    nregions: int = 0
    nFinishedRegions: int = 0
    status: int = -1
    lastPhase: int = -1
    chi_sq: float = 0.0
    iters: int = 0

    @staticmethod
    def from_c(r: PgResult) -> "IntegrationResult":
        return IntegrationResult(r.estimate, r.errorest, r.neval, r.nregions, r.nfinished, r.status, r.last_phase,
                                 r.chi_sq, r.iters)


class PaganiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pagani_gb300 error {code}: {msg}")
        self.code = code


def default_options(**kw) -> PgOptions:
    lib = load_library()
    o = PgOptions()
    lib.pg_options_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Context:
    """Owns one pg_context (device memory pool + stream) on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.pg_context_create(device, ctypes.byref(h))
        if rc != PG_OK:
            raise PaganiError(rc, "pg_context_create failed (no usable CUDA device?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.pg_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, allow=(PG_OK, PG_NOT_CONVERGED)):
        if rc not in allow:
            raise PaganiError(rc, self.lib.pg_last_error(self.h).decode())
        return rc

    # -- statistics ---------------------------------------------------------
    def set_profiling(self, on: bool):
        self.lib.pg_context_set_profiling(self.h, 1 if on else 0)

    def stats(self) -> PgStats:
        s = PgStats()
        self.lib.pg_context_stats(self.h, ctypes.byref(s))
        return s

    def reset_stats(self):
        self.lib.pg_context_reset_stats(self.h)

    def fail_allocation(self, after: int):
        """Testing hook: the allocation after `after` more fails with PG_OOM (negative: off)."""
        self._check(self.lib.pg_context_fail_allocation(self.h, int(after)), allow=(PG_OK,))

    def iterations(self) -> np.ndarray:
        """Per-iteration records since the last reset_stats (profiling on): a structured
        array with fields regions, integrals, eval_launches, eval_ms, stage_ms."""
        n = ctypes.c_uint64()
        self._check(self.lib.pg_context_iterations(self.h, None, 0, ctypes.byref(n)))
        buf = (PgIterationRecord * max(n.value, 1))()
        self._check(self.lib.pg_context_iterations(self.h, buf, n.value, ctypes.byref(n)))
        dt = np.dtype([("regions", np.uint64), ("integrals", np.uint32), ("eval_launches", np.uint32),
                       ("eval_ms", np.float64), ("stage_ms", np.float64)])
        return np.frombuffer(bytes(buf), dtype=dt, count=n.value).copy()

    # -- PAGANI -------------------------------------------------------------
    def integrate(self, f: Integrand, epsrel: float, epsabs: float, vol: Optional[Volume] = None,
                  relerr_classification: bool = True, options: Optional[PgOptions] = None) -> IntegrationResult:
        o = options if options is not None else default_options()
        o.relerr_classification = 1 if relerr_classification else 0
        lo = hi = None
        if vol is not None:
            lo = np.ascontiguousarray(vol.lows, dtype=np.float64)
            hi = np.ascontiguousarray(vol.highs, dtype=np.float64)
        r = PgResult()
        self._check(self.lib.pg_integrate(self.h, ctypes.byref(f.to_c()), epsrel, epsabs, _ptr(lo), _ptr(hi),
                                          ctypes.byref(o), ctypes.byref(r)))
        return IntegrationResult.from_c(r)

    def integrate_regions(self, f: Integrand, left, length, epsrel: float, epsabs: float,
                          vol: Optional[Volume] = None, relerr_classification: bool = True,
                          predict_split: bool = False, options: Optional[PgOptions] = None) -> IntegrationResult:
        """Workspace::integrate(f, subregions, ...) (Workspace.cuh:148-158): PAGANI from
        the given first region list, SoA arrays of shape (ndim, n) in unit coordinates."""
        o = options if options is not None else default_options()
        o.relerr_classification = 1 if relerr_classification else 0
        o.predict_split = 1 if predict_split else 0
        left = np.ascontiguousarray(left, dtype=np.float64)
        length = np.ascontiguousarray(length, dtype=np.float64)
        if left.shape != length.shape or left.ndim != 2 or left.shape[0] != f.ndim:
            raise ValueError("left and length must have shape (ndim, n)")
        lo = hi = None
        if vol is not None:
            lo = np.ascontiguousarray(vol.lows, dtype=np.float64)
            hi = np.ascontiguousarray(vol.highs, dtype=np.float64)
        r = PgResult()
        self._check(self.lib.pg_integrate_regions(self.h, ctypes.byref(f.to_c()), _ptr(left), _ptr(length),
                                                  left.shape[1], epsrel, epsabs, _ptr(lo), _ptr(hi),
                                                  ctypes.byref(o), ctypes.byref(r)))
        return IntegrationResult.from_c(r)

    def last_snapshot(self):
        """The region list kept at iteration 15 by the last predict_split run
        (Sub_regions::take_snapshot), as (left, length) of shape (ndim, n), or None."""
        d = ctypes.c_int32()
        n = ctypes.c_uint64()
        self._check(self.lib.pg_last_snapshot(self.h, ctypes.byref(d), ctypes.byref(n), None, None, 0))
        if n.value == 0:
            return None
        left = np.zeros((d.value, n.value))
        length = np.zeros((d.value, n.value))
        self._check(self.lib.pg_last_snapshot(self.h, ctypes.byref(d), ctypes.byref(n), _ptr(left), _ptr(length),
                                              n.value))
        return left, length

    def batch_integrate(self, fs: Sequence[Integrand], epsrel, epsabs, options: Optional[PgOptions] = None,
                        completion_ms: Optional[np.ndarray] = None):
        n = len(fs)
        arr = fs if isinstance(fs, ctypes.Array) else (PgIntegrand * n)(*[f.to_c() for f in fs])
        er = np.ascontiguousarray(np.broadcast_to(np.asarray(epsrel, dtype=np.float64), (n,)))
        ea = np.ascontiguousarray(np.broadcast_to(np.asarray(epsabs, dtype=np.float64), (n,)))
        out = (PgResult * n)()
        o = options if options is not None else default_options()
        self._check(self.lib.pg_batch_integrate_timed(self.h, n, arr, _ptr(er), _ptr(ea), ctypes.byref(o), out,
                                                      _ptr(completion_ms)))
        return [IntegrationResult.from_c(out[i]) for i in range(n)]

    def serve(self, fs, epsrel, epsabs, arrival_ms, budget_bytes: int = 0, options: Optional[PgOptions] = None,
              deadline_ms: float = 0.0):
        """Continuous-batching run over an arrival schedule; returns (results, completion_ms)."""
        n = len(fs)
        arr = fs if isinstance(fs, ctypes.Array) else (PgIntegrand * n)(*[f.to_c() for f in fs])
        er = np.ascontiguousarray(np.broadcast_to(np.asarray(epsrel, dtype=np.float64), (n,)))
        ea = np.ascontiguousarray(np.broadcast_to(np.asarray(epsabs, dtype=np.float64), (n,)))
        arrival = np.ascontiguousarray(arrival_ms, dtype=np.float64)
        done = np.zeros(n)
        out = (PgResult * n)()
        o = options if options is not None else default_options()
        self._check(self.lib.pg_serve(self.h, n, arr, _ptr(er), _ptr(ea), _ptr(arrival), int(budget_bytes),
                                      float(deadline_ms), ctypes.byref(o), out, _ptr(done)))
        return [IntegrationResult.from_c(out[i]) for i in range(n)], done

    def probe_fp64_peak(self) -> float:
        """Measured FP64 FMA rate of this GPU in TFLOP/s."""
        v = ctypes.c_double()
        self._check(self.lib.pg_probe_fp64_peak(self.h, ctypes.byref(v)))
        return v.value

    def stream_handle(self) -> int:
        return self.lib.pg_context_stream(self.h) or 0

    def evaluate_regions(self, f: Integrand, left: np.ndarray, length: np.ndarray, vol: Optional[Volume] = None,
                         eval_mode: int = 0):
        """Per-region estimate, error and split axis of a SoA region list [ndim, n]."""
        left = np.ascontiguousarray(left, dtype=np.float64)
        length = np.ascontiguousarray(length, dtype=np.float64)
        n = left.shape[1] if left.ndim == 2 else left.size // f.ndim
        est = np.zeros(n)
        err = np.zeros(n)
        bis = np.zeros(n, dtype=np.int32)
        lo = hi = None
        if vol is not None:
            lo = np.ascontiguousarray(vol.lows, dtype=np.float64)
            hi = np.ascontiguousarray(vol.highs, dtype=np.float64)
        self._check(self.lib.pg_evaluate_regions(self.h, ctypes.byref(f.to_c()), _ptr(lo), _ptr(hi), n, _ptr(left),
                                                 _ptr(length), _ptr(est), _ptr(err), _ptr(bis, ctypes.c_int32),
                                                 eval_mode))
        return est, err, bis

    def two_level(self, est, err, parent_est, epsrel, relerr_classification=True):
        est = np.ascontiguousarray(est, dtype=np.float64)
        err = np.ascontiguousarray(err, dtype=np.float64)
        par = None if parent_est is None else np.ascontiguousarray(parent_est, dtype=np.float64)
        n = est.size
        new_err = np.zeros(n)
        act = np.zeros(n, dtype=np.uint8)
        self._check(self.lib.pg_two_level(self.h, n, _ptr(est), _ptr(err), _ptr(par), _ptr(new_err),
                                          _ptr(act, ctypes.c_uint8), epsrel, 1 if relerr_classification else 0))
        return new_err, act

    def filter_split(self, left, length, active, bisect, est, err=None):
        left = np.ascontiguousarray(left, dtype=np.float64)
        length = np.ascontiguousarray(length, dtype=np.float64)
        ndim, n = left.shape
        active = np.ascontiguousarray(active, dtype=np.uint8)
        bisect = np.ascontiguousarray(bisect, dtype=np.int32)
        est = np.ascontiguousarray(est, dtype=np.float64)
        err = None if err is None else np.ascontiguousarray(err, dtype=np.float64)
        A = int(active.astype(bool).sum())
        out_left = np.zeros((ndim, 2 * A))
        out_len = np.zeros((ndim, 2 * A))
        par_est = np.zeros(A)
        par_err = np.zeros(A) if err is not None else None
        na = ctypes.c_uint64()
        self._check(self.lib.pg_filter_split(self.h, ndim, n, _ptr(left), _ptr(length), _ptr(active, ctypes.c_uint8),
                                             _ptr(bisect, ctypes.c_int32), _ptr(est), _ptr(err), _ptr(out_left),
                                             _ptr(out_len), _ptr(par_est), _ptr(par_err), ctypes.byref(na)))
        assert na.value == A
        return out_left, out_len, par_est, par_err

    def reduce_sum(self, x) -> float:
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = ctypes.c_double()
        self._check(self.lib.pg_reduce_sum(self.h, _ptr(x), x.size, ctypes.byref(out)))
        return out.value

    def exclusive_scan_flags(self, flags):
        flags = np.ascontiguousarray(flags, dtype=np.uint8)
        out = np.zeros(flags.size, dtype=np.uint64)
        tot = ctypes.c_uint64()
        self._check(self.lib.pg_exclusive_scan_flags(self.h, _ptr(flags, ctypes.c_uint8), flags.size,
                                                     _ptr(out, ctypes.c_uint64), ctypes.byref(tot)))
        return out, tot.value

    # -- m-Cubes ------------------------------------------------------------
    def mcubes_integrate(self, f: Integrand, epsrel: float, epsabs: float, ncall: float = 1e6,
                         vol: Optional[Volume] = None, titer: int = 15, itmax: int = 15, skip: int = 5,
                         seed: int = 0x5EED, nbins: int = 500, alpha: float = 1.5) -> IntegrationResult:
        o = PgMcubesOptions()
        self.lib.pg_mcubes_options_default(ctypes.byref(o))
        o.ncall, o.titer, o.itmax, o.skip, o.seed, o.nbins, o.alpha = ncall, titer, itmax, skip, seed, nbins, alpha
        lo = hi = None
        if vol is not None:
            lo = np.ascontiguousarray(vol.lows, dtype=np.float64)
            hi = np.ascontiguousarray(vol.highs, dtype=np.float64)
        r = PgResult()
        self._check(self.lib.pg_mcubes_integrate(self.h, ctypes.byref(f.to_c()), epsrel, epsabs, _ptr(lo), _ptr(hi),
                                                 ctypes.byref(o), ctypes.byref(r)))
        return IntegrationResult.from_c(r)


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class Workspace:
    """Mirror of Workspace<double, ndim> (cuda/pagani/quad/GPUquad/Workspace.cuh:23-71)."""

    def __init__(self, ndim: int, ctx: Optional[Context] = None):
        self.ndim = ndim
        self.ctx = ctx or default_context()

    def integrate(self, integrand: Integrand, epsrel: float, epsabs: float, vol: Optional[Volume] = None,
                  relerr_classification: bool = True) -> IntegrationResult:
        if integrand.ndim != self.ndim:
            raise ValueError("integrand dimension does not match the workspace")
        return self.ctx.integrate(integrand, epsrel, epsabs, vol, relerr_classification)


def mcubes_integrate(integrand: Integrand, epsrel: float, epsabs: float, ncall: float, vol: Optional[Volume] = None,
                     totalIters: int = 15, adjustIters: int = 15, skipIters: int = 5, seed: int = 0x5EED,
                     ctx: Optional[Context] = None) -> IntegrationResult:
    """Mirror of cuda_mcubes::integrate (cuda/mcubes/vegasT.cuh:999-1030), with a fixed seed."""
    return (ctx or default_context()).mcubes_integrate(integrand, epsrel, epsabs, ncall, vol, totalIters,
                                                        adjustIters, skipIters, seed)


def rule_tables(ndim: int):
    """The library's degree-9 rule tables (host-side; no GPU needed)."""
    lib = load_library()
    fe = lib.pg_feval(ndim)
    if fe < 0:
        raise ValueError("ndim out of range")
    w = np.zeros(45)
    sc = np.zeros(45)
    nm = np.zeros(45)
    so = np.zeros(fe, dtype=np.int32)
    gen = np.zeros(fe * ndim)
    lib.pg_rule_tables(ndim, _ptr(w), _ptr(sc), _ptr(nm), _ptr(so, ctypes.c_int32), _ptr(gen))
    return {"w": w, "scale": sc, "norm": nm, "set_of": so, "gen": gen.reshape(fe, ndim), "feval": fe}
