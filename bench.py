#!/usr/bin/env python3
"""Benchmark of the GB300 PAGANI library on the batched Genz workload.

Workload (one step): the 4096 pre-screened mixed Genz integrals of the
batched configuration -- dim ~ U{2..8}, family ~ U{6 Genz families}, seeded
a_i/u_i scaled per family, epsrel log-uniform in [1e-7, 1e-4], FP64, unit
cube -- integrated together by one pg_batch_integrate call (one device region
pool of 2^26 regions, one evaluation launch per kernel run per iteration).
Region evaluation uses generator-set sums for the product-form families
(PG_EVAL_SET_SUMS; `--eval-mode points` selects the reference's
point-by-point order).

Metric: converged integrals per second, where an integral counts when PAGANI
reports status 0 and the estimate lies within its epsrel of the analytic
value.  `value` is timed with CUDA events on the library's stream around each
step (inputs already on the host side are a few MB of descriptors; the region
pool lives on the device); `e2e` is the same metric by host wall clock around
the C-ABI call, including the descriptor upload, the result download and the
pinned-host traffic of region lists that leave the pool.  p50/p99 are the
per-integral completion latencies inside a step.  After the timed steps the
plain per-call path runs the same integrals one pg_integrate call at a time
(the batched-over-plain ratio), and the CPU oracle runs a bounded sample; a
wall-time budget bounds both legs so the whole run ends in time.

The reference arm (--impl reference) times the CPU restatement of the
reference's PAGANI iteration (oracle/, point by point, every host thread) on a
fixed bounded sample of the workload per step, and reports its throughput
extrapolated to the whole workload by evaluation count.

`--config eval` times one evaluation kernel on a synthetic region list (the
target of the ncu captures under profiles/); `--config 3` m-Cubes; `--config
5` the served workload.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "integrals/s at rel err <=1e-6, batched vs plain PAGANI on 1 GB300; p50/p99 latency"
WORKLOAD = "batched PAGANI: 4096 pre-screened mixed Genz integrals, dim 2..8, 6 families, epsrel log-U[1e-7,1e-4]"
SCREEN = os.path.join(ROOT, "tests", "golden", "config4_screen.json")
EVAL_MODES = {"points": 0, "sets": 1}
# DRAM bytes (read + write) of one evaluation launch over its algorithmic bytes
# (16 d bytes of bounds in, 20 bytes of results out per region), from the ncu
# capture of setsum_kernel on 1,048,576 8-D C0 regions: 145,437,952 bytes
# against 134,217,728 + 20,971,520.
DRAM_OVER_ALGORITHMIC = 145437952 / (134217728 + 20971520)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--count", type=int, default=4096)
    p.add_argument("--eval-mode", default="sets", choices=sorted(EVAL_MODES))
    p.add_argument("--cpu-seconds", type=float, default=20.0)
    p.add_argument("--time-budget", type=float, default=1500.0,
                   help="seconds the whole run may take; legs after the timed steps shrink or are skipped to fit")
    p.add_argument("--max-regions", type=int, default=1 << 26)
    p.add_argument("--config", default="4", choices=["3", "4", "5", "eval", "single"],
                   help="4: batched workload (default, the metric's configuration); 5: served workload; "
                        "3: m-Cubes Gaussian; eval: one evaluation kernel on a synthetic region list; "
                        "single: one integral of the workload through the plain path")
    p.add_argument("--rate", type=float, default=2000.0, help="config 5: Poisson arrival rate (requests/s)")
    p.add_argument("--duration", type=float, default=60.0, help="config 5: arrival window (s)")
    p.add_argument("--budget-gb", type=float, default=120.0, help="config 5: device budget of the region pool")
    p.add_argument("--serve-seconds", type=float, default=0.0,
                   help="config 5: stop serving after this many seconds (0: arrival window + 60 s)")
    p.add_argument("--family", default="c0", help="config eval: integrand family name")
    p.add_argument("--ndim", type=int, default=8, help="config eval: dimension")
    p.add_argument("--regions", type=int, default=1 << 20, help="config eval: regions per launch")
    p.add_argument("--index", type=int, default=2069,
                   help="config single: workload integral (default 2069: 8-D C0, epsrel 4.6e-6, 1.3e7 regions)")
    return p.parse_args()


# ---------------------------------------------------------------------------
def _feval(d):
    return 1 + 8 * d + 2 * d * (d - 1) + 4 * d * (d - 1) + 4 * d * (d - 1) * (d - 2) // 3 + (1 << d)


def _first_split(d):
    """Regions of an integral's first list (the uniform split)."""
    return (4 if d < 5 else (2 if d <= 10 else 1)) ** d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def within(c, r):
    from gpuintegration_gb300 import workloads as W
    return r.status == 0 and W.within_tolerance(r.estimate, c.exact, c.epsrel)


def load_screen():
    return json.load(open(SCREEN))


def _oracle_checked(screen):
    """The screen's oracle re-check (tests/golden/make_config4_screen.py --oracle-check), in words."""
    oc = screen.get("oracle_check")
    if not oc:
        return "no candidate (not run)"
    return (f"{oc['accepted_agree']} of {oc['accepted_checked']} accepted candidates with <= {oc['max_regions']} "
            f"regions and {oc['rejected_agree']} of {oc['rejected_checked']} rejected candidates of dimension <= "
            f"{oc['max_rejected_dim']}")


# ---------------------------------------------------------------------------
# Roofline of region evaluation.  The kernels are bound by the FP64 pipe
# (GB300: 2 FP64 lanes per SM per clock, one pipe slot per FP64 instruction
# whether FMA, multiply or add), so their work is counted in FP64 operations
# per region of each kernel's algorithm, and the peak is this GPU's FP64
# instruction rate, measured by pg_probe_fp64_peak (an FMA loop; TFLOP/s / 2).
# The measured-peaks file holds HBM and bf16 figures only.  A libm call or a
# division counts the FP64 instructions it executes on this GPU, measured by
# ncu (smsp__sass_thread_inst_executed_op_fp64_pred_on per region, less the
# counted arithmetic: profiles/setsum_kernel_fp64_mix.md).  Multiplies that
# run on the integer pipe (pg::mul_rn_int) are not counted: the point-by-point
# kernel's products of the point values and the set-sum kernel's products of
# the fourth differences' point values.
LIBM_OPS = {"exp": 17.2, "div": 6.2, "cos": 22.0}
# ncu's FP64-pipe utilisation of setsum_kernel (sm__pipe_fp64_cycles_active over
# 152 SMs x elapsed cycles), from profiles/setsum_kernel_fp64_mix.md: the
# counter-side view of the same roofline.
NCU_FP64_PIPE_ACTIVE = {"cached_sibling_pairs_c0_8d": 0.699, "lone_regions_c0_8d": 0.833,
                        "source": "profiles/setsum_kernel_fp64_mix.md"}


def _hbm_frac(gbs):
    """Evaluation DRAM GB/s over the measured copy bandwidth (MEASURED_PEAKS.json), when that file is present."""
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        return None
    return gbs / peak


def _factor_ops(family):
    import gpuintegration_gb300 as pg
    return {pg.PRODUCT_PEAK: 2 + LIBM_OPS["div"],    # sub, fma, 1/()
            pg.GAUSSIAN: 4 + LIBM_OPS["exp"],        # sub, mul, mul, normalisation test, exp
            pg.C0: 2 + LIBM_OPS["exp"],              # sub, mul, exp
            pg.DISCONTINUOUS: 2 + LIBM_OPS["exp"],   # compare, mul, exp
            pg.PRODUCT: 0}.get(family, 0)


def setsum_ops(family, d, unit=True, paired=0.0, cached=0.0):
    """FP64 operations per region of setsum_kernel (PG_EVAL_SET_SUMS).  An evaluated axis
    costs 11 coordinates (a multiply and an FMA, one more off the unit cube), 11 factors and
    5 pair sums; a step of the set-sum recurrence 8 FMAs and 9 multiplies; a region's tail
    40 rule-sum FMAs and 5 multiplies, the fourth differences (5 d + 1; the products of
    their point values run on the integer pipe), 27 null-rule FMAs and 27 multiplies, and
    10 more (volume, error ladder, results).  A region alone evaluates d axes and d steps.  A sibling pair
    evaluates d + 1 axes (the second sibling's split axis only) and d + 1 steps (d - 1
    shared); a pair whose parent's terms are kept evaluates the split axis of each sibling
    and adds 2 sums for every other axis.  `paired`: the share of regions evaluated in
    pairs; `cached`: the share of pairs with their parent's terms."""
    axis = 11 * (2 if unit else 3) + 11 * _factor_ops(family) + 5
    step = 8 + 9
    tail = 45 + (5 * d + 1) + 54 + (d - 1) + 10
    alone = d * (axis + step) + tail
    pair = (d + 1) * axis + (d + 1) * step + 2 * tail
    pair_cached = 2 * axis + 2 * (d - 1) + (d + 1) * step + 2 * tail
    per_pair = (1.0 - cached) * pair + cached * pair_cached
    return (1.0 - paired) * alone + paired * per_pair / 2


def points_ops(family, d, unit=True):
    """FP64 operations of one region of eval_kernel (PG_EVAL_POINTS): 5 rule-sum FMAs per point,
    the pointwise integrand of the non-product families, the per-axis factors of the product
    families, and the per-region reduction trees (320 adds), null rules and tail."""
    import gpuintegration_gb300 as pg
    fe = _feval(d)
    per_point = 5
    if family == pg.OSCILLATORY:
        per_point += d + LIBM_OPS["cos"]
    elif family == pg.CORNER_PEAK:
        per_point += d + LIBM_OPS["div"] + 4
    return fe * per_point + 11 * d * ((1 if unit else 2) + _factor_ops(family)) + 320 + 27 + 6 * d


# ---------------------------------------------------------------------------
def run_served(args):
    """Served PAGANI (Poisson arrivals, continuous batching, HBM budget)."""
    import gpuintegration_gb300 as pg
    from gpuintegration_gb300 import workloads as W
    arrivals = W.poisson_arrivals(args.rate, args.duration)
    cases = W.config5_cases(len(arrivals))
    ctx = pg.Context(0)
    fs = (pg.PgIntegrand * len(cases))(*[c.integrand.to_c() for c in cases])
    eps = np.array([c.epsrel for c in cases])
    opt = pg.default_options(eval_mode=EVAL_MODES[args.eval_mode])
    clocks = ClockSampler(0)
    clocks.start()
    deadline = 1000.0 * (args.serve_seconds if args.serve_seconds > 0 else args.duration + 60.0)
    t0 = time.perf_counter()
    res, done = ctx.serve(fs, eps, 0.0, arrivals, budget_bytes=int(args.budget_gb * 1e9), deadline_ms=deadline,
                          options=opt)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    fin = done >= 0
    lat = (done - arrivals)[fin]
    arrived = int((arrivals <= wall * 1000.0).sum())
    conv = sum(1 for c, r, ok in zip(cases, res, fin) if ok and within(c, r))
    st = ctx.stats()
    line = {"metric": "served PAGANI: integrals/s and p50/p99 latency", "value": conv / wall, "unit": "integrals/s",
            "n_gpus": 1, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"Poisson arrivals {args.rate:g}/s for {args.duration:g} s, Genz dim 3..10, "
                                   f"epsrel log-U[1e-6,1e-3]", "requests": len(cases), "budget_gb": args.budget_gb,
                       "deadline_s": deadline / 1000.0, "eval_mode": args.eval_mode},
            "latency_ms_finished": {"p50": float(np.percentile(lat, 50)) if lat.size else None,
                                    "p99": float(np.percentile(lat, 99)) if lat.size else None,
                                    "max": float(lat.max()) if lat.size else None},
            "arrived": arrived, "finished": int(fin.sum()), "unfinished_at_deadline": int((~fin).sum()),
            "wall_s": wall, "converged_within_tolerance": conv,
            "status0": sum(1 for r, ok in zip(res, fin) if ok and r.status == 0),
            "gpu_launches": int(st.launches), "points_per_s": st.points_evaluated / wall, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_mcubes(args):
    """m-Cubes on the 6-D sigma = 0.01 Gaussian (2^24 calls x 20 iterations, fixed seed): time to
    solution by CUDA events on the library's stream (each run ends with its synchronisation), and
    whether two runs from the seed agree bit for bit."""
    import torch
    import gpuintegration_gb300 as pg
    from gpuintegration_gb300 import workloads as W
    ctx = pg.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device="cuda:0")
    f = W.config3_integrand()

    def run():
        return ctx.mcubes_integrate(f, 1e-4, 0.0, 2.0 ** 24, titer=20, itmax=20, skip=5, seed=2024)

    for _ in range(args.warmup):
        first = run()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        r = run()
    ev1.record(stream)
    torch.cuda.synchronize()
    el_wall = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    el = ev0.elapsed_time(ev1) / 1000.0 / args.steps
    key = lambda x: (x.estimate, x.errorest, x.chi_sq, x.iters, x.status)
    line = {"metric": "m-Cubes time to solution, 6-D Gaussian sigma 0.01", "value": el * 1000, "unit": "ms",
            "higher_is_better": False, "dtype": "f64", "data": "synthetic", "steps": args.steps,
            "wall_ms": el_wall * 1000, "clocks": clk,
            "estimate": r.estimate, "errorest": r.errorest, "sigma_from_1": (r.estimate - 1.0) / r.errorest,
            "iters": r.iters, "status": r.status, "samples_per_s": r.neval / el,
            "same_seed_bitwise": (key(first) == key(r)) if args.warmup else None}
    # CPU baseline: the oracle's m-Cubes restatement (one host thread) on a bounded sample of the same
    # integrand (ncall 2^20, 3 iterations), its sampling rate applied to this run's samples.
    from oracle import oracle as orc
    t0 = time.perf_counter()
    o, _ = orc.mcubes_integrate(f, 1e-4, 0.0, 2.0 ** 20, titer=3, itmax=3, skip=5, seed=2024)
    cpu_s = time.perf_counter() - t0
    rate = o.neval / cpu_s
    line["cpu_baseline"] = {"value": 1000.0 * r.neval / rate, "unit": "ms", "cores": 1, "kind": "port",
                            "samples_per_s": rate,
                            "sample": f"ncall 2^20 x 3 iterations ({o.neval} samples, {cpu_s:.1f} s), time to "
                                      f"solution extrapolated to this run's {r.neval} samples"}
    print(json.dumps(line), flush=True)


def run_eval(args):
    """One evaluation kernel on a synthetic list of dyadic regions (device buffers), CUDA-event timed."""
    import torch
    import gpuintegration_gb300 as pg
    fam = {v: k for k, v in pg.FAMILY_NAMES.items()}[args.family]
    d, n, mode = args.ndim, args.regions, EVAL_MODES[args.eval_mode]
    ctx = pg.Context(0)
    rng = np.random.default_rng(1)
    a = rng.random(d)
    a *= 12.0 / a.sum()
    f = pg.Integrand(fam, d, list(a), list(rng.random(d)))
    depth = rng.integers(0, 8, size=(d, n))
    length = 0.5 ** depth
    left = np.floor(rng.random((d, n)) / length) * length
    dev = torch.device("cuda:0")
    L, N = torch.from_numpy(left).to(dev), torch.from_numpy(length).to(dev)
    est = torch.empty(n, dtype=torch.float64, device=dev)
    err = torch.empty_like(est)
    bis = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=dev)
    fc = f.to_c()

    def launch():
        rc = ctx.lib.pg_evaluate_regions_device(ctx.h, ctypes.byref(fc), None, None, n, L.data_ptr(), N.data_ptr(),
                                                est.data_ptr(), err.data_ptr(), bis.data_ptr(), mode)
        if rc != 0:
            raise RuntimeError(ctx.lib.pg_last_error(ctx.h).decode())

    for _ in range(args.warmup):
        launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        launch()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ops = (setsum_ops if mode == 1 and fam in (pg.PRODUCT_PEAK, pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS, pg.PRODUCT)
           else points_ops)(fam, d) * n
    peak = ctx.probe_fp64_peak() / 2.0
    achieved = ops / (ms / 1000.0) / 1e12
    line = {"metric": "region evaluations/s", "value": n / (ms / 1000.0), "unit": "regions/s", "ms_per_launch": ms,
            "config": {"workload": f"{args.family} d={d}, {n} dyadic regions", "eval_mode": args.eval_mode},
            "rule_points_per_s": n * _feval(d) / (ms / 1000.0),
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "T FP64 ops/s",
                         "frac": achieved / peak, "fp64_ops_per_region": ops / n,
                         "peak_source": "pg_probe_fp64_peak (FP64 FMA instruction rate of this GPU)"}}
    print(json.dumps(line), flush=True)


def run_single(args):
    """One integral of the batched workload through pg_integrate, with the
    evaluation launches' CUDA-event time (the kernels as the iteration runs
    them: after the first iteration the set-sum kernel evaluates siblings in
    pairs)."""
    import gpuintegration_gb300 as pg
    from gpuintegration_gb300 import workloads as W
    c = W.config4_cases(args.index + 1)[args.index]
    ctx = pg.Context(0)
    opt = pg.default_options(eval_mode=EVAL_MODES[args.eval_mode])
    for _ in range(args.warmup):
        ctx.integrate(c.integrand, c.epsrel, 0.0, options=opt)
    ctx.reset_stats()
    ctx.set_profiling(True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = ctx.integrate(c.integrand, c.epsrel, 0.0, options=opt)
    wall = (time.perf_counter() - t0) / args.steps
    st = ctx.stats()
    f = c.integrand
    line = {"metric": "plain PAGANI, one integral", "config": {"workload": f"workload integral {args.index}: "
            f"{pg.FAMILY_NAMES[f.family]} d={f.ndim} epsrel {c.epsrel:.3g}", "eval_mode": args.eval_mode},
            "wall_ms": wall * 1000.0, "eval_ms": st.eval_ms / args.steps, "stage_ms": st.stage_ms / args.steps,
            "host_ms": st.host_ms / args.steps, "regions": st.regions_evaluated // args.steps,
            "ns_per_region_eval": st.eval_ms * 1e6 / max(st.regions_evaluated, 1),
            "estimate": r.estimate, "errorest": r.errorest, "status": r.status, "within": within(c, r),
            "iters": r.iters}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
CPU_SAMPLE_MAX_REGIONS = 200000


def cpu_sample(cases, screen, point_budget, seed=4242):
    """A fixed sample of the workload for the CPU oracle: integrals in a seeded
    random order, skipping any whose screened region count exceeds
    CPU_SAMPLE_MAX_REGIONS, until their evaluation count reaches point_budget."""
    order = np.random.default_rng(seed).permutation(len(cases))
    out, pts = [], 0
    for i in order:
        nreg = screen["nregions"][i]
        if nreg > CPU_SAMPLE_MAX_REGIONS:
            continue
        ne = screen["neval"][i]
        if pts + ne > point_budget and out:
            continue
        out.append(int(i))
        pts += ne
        if pts >= point_budget:
            break
    return out


def cpu_leg(cases, idx):
    """Runs the CPU oracle (point by point, every host thread) over cases[idx];
    returns evaluation points/s and the sample's size and time."""
    from oracle import oracle
    oracle.load()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    pts, conv = 0, 0
    for i in idx:
        c = cases[i]
        r, _ = oracle.integrate(c.integrand, c.epsrel, 0.0, nthreads=threads)
        pts += r.neval
        conv += 1 if within(c, r) else 0
    el = time.perf_counter() - t0
    return {"points_per_s": pts / el, "points": pts, "integrals": len(idx), "converged": conv, "seconds": el,
            "threads": threads}


def run_reference(args, cases, rank, world):
    """Reference arm: the CPU restatement of the reference's PAGANI on every host core, rank 0 only."""
    if rank != 0:
        return
    screen = load_screen()
    total_pts = float(sum(screen["neval"][:len(cases)]))
    # each step: the same fixed sample, a few seconds of CPU work on the GPU machine's host
    budget = max(1e8, 2e9 * args.cpu_seconds / 20.0)
    idx = cpu_sample(cases, screen, budget)
    vals = []
    for i in range(args.warmup + args.steps):
        s = cpu_leg(cases, idx)
        if i >= args.warmup:
            vals.append(s)
    pps = sum(v["points"] for v in vals) / sum(v["seconds"] for v in vals)
    value = len(cases) / (total_pts / pps)
    ms = 1000.0 * sum(v["seconds"] for v in vals) / len(vals)
    sample = (f"each step: the same {len(idx)} integrals of the workload ({vals[-1]['points']:.3g} rule points, "
              f"seeded random order, <= {CPU_SAMPLE_MAX_REGIONS} screened regions each); value = the workload's "
              f"integral count / (its {total_pts:.3g} rule points / the sample's points per second)")
    line = {"metric": METRIC, "value": value, "unit": "integrals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "count": len(cases), "l2": "n/a (CPU)", "eval_mode": "points"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "integrals/s", "cores": vals[-1]["threads"], "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "integrals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "converged_in_sample": vals[-1]["converged"],
            "note": "no CPU PAGANI in the reference (Cuhre via cubacpp needs libcuba, absent); the oracle port "
                    "restates the reference's CUDA iteration point by point on host threads"}
    print(json.dumps(line), flush=True)


def max_over_ranks(values, dist, device="cpu"):
    """Element-wise maximum of `values` over the ranks of the process group (the
    time of the slowest replica); the values themselves without a group."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


# ---------------------------------------------------------------------------
def roofline(ctx, cases, results, st, steps, mode):
    """Roofline of the dominant kernel (region evaluation, FP64 pipe)."""
    import gpuintegration_gb300 as pg
    sep = (pg.PRODUCT_PEAK, pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS, pg.PRODUCT)
    # Every region after an integral's first split is evaluated with its
    # sibling; the share of pairs with kept parent terms is the run's.
    cached = st.setsum_cached_pairs / max(st.setsum_pairs, 1)
    ops = 0.0
    for c, r in zip(cases, results):
        f = c.integrand
        regions = r.neval // _feval(f.ndim)
        if mode == 1 and f.family in sep:
            first = _first_split(f.ndim)
            paired = max(regions - first, 0) / max(regions, 1)
            per = setsum_ops(f.family, f.ndim, paired=paired, cached=cached)
        else:
            per = points_ops(f.family, f.ndim)
        ops += regions * per
    ops *= steps
    eval_s = st.eval_ms / 1000.0
    achieved = ops / eval_s / 1e12
    peak = ctx.probe_fp64_peak() / 2.0
    launches = max(st.eval_launches, 1)
    alg_bytes = st.eval_bytes / launches
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "T FP64 ops/s", "frac": achieved / peak,
            "traffic": alg_bytes * DRAM_OVER_ALGORITHMIC,
            "kernel": "setsum_kernel" if mode == 1 else "eval_kernel",
            "peak_source": "FP64 instruction rate of this GPU: pg_probe_fp64_peak's FMA loop (TFLOP/s / 2); "
                           "MEASURED_PEAKS.json has HBM and bf16 figures only",
            "fp64_ops_per_step": ops / steps,
            "op_model": "FP64 operations per region of the kernel's algorithm (libm calls and divisions at their "
                        "ncu-measured FP64 instruction counts); agrees with ncu's FP64 instruction count within "
                        "a few per cent",
            "algorithmic_bytes_per_launch": alg_bytes,
            "traffic_note": "algorithmic bytes x the DRAM/algorithmic ratio ncu measured on a 1M-region 8-D "
                            "setsum_kernel launch",
            "hbm_gbs_of_eval": st.eval_bytes / eval_s / 1e9,
            "hbm_frac_of_measured": _hbm_frac(st.eval_bytes / eval_s / 1e9),
            "ncu_fp64_pipe_active": NCU_FP64_PIPE_ACTIVE}


def iteration_summary(it, steps):
    """Evaluation time by the size of the iteration's region list."""
    out = {"per_step": len(it) / steps, "eval_ms_by_list_size": {}}
    edges = [0, 10 ** 4, 10 ** 5, 10 ** 6, 10 ** 7, 10 ** 9]
    for lo, hi in zip(edges[:-1], edges[1:]):
        sel = (it["regions"] >= lo) & (it["regions"] < hi)
        if not sel.any():
            continue
        ms = float(it["eval_ms"][sel].sum())
        reg = float(it["regions"][sel].sum())
        out["eval_ms_by_list_size"][f"[{lo:.0e},{hi:.0e})"] = {
            "iterations": int(sel.sum()) / steps, "eval_ms": ms / steps, "ns_per_region": 1e6 * ms / max(reg, 1.0)}
    return out


def run_batched(args, rank, world, local, t_begin):
    import torch
    import gpuintegration_gb300 as pg
    from gpuintegration_gb300 import workloads as W
    cases = W.config4_cases(args.count)
    mode = EVAL_MODES[args.eval_mode]
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ctx = pg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=f"cuda:{local}")
    n = len(cases)
    fs = (pg.PgIntegrand * n)(*[c.integrand.to_c() for c in cases])
    eps = np.array([c.epsrel for c in cases])
    opt = pg.default_options(max_regions=args.max_regions, eval_mode=mode)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")  # > 129 MB L2

    def step(completion=None):
        return ctx.batch_integrate(fs, eps, 0.0, options=opt, completion_ms=completion)

    for _ in range(args.warmup):
        step()
    ctx.reset_stats()
    ctx.set_profiling(True)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    wall, conv_counts, lat = [], [], []
    results = None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        comp = np.zeros(n)
        ev0[k].record(stream)
        t0 = time.perf_counter()
        results = step(comp)
        t1 = time.perf_counter()
        ev1[k].record(stream)
        wall.append(t1 - t0)
        lat.append(comp)
        conv_counts.append(sum(1 for c, r in zip(cases, results) if within(c, r)))
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    dev_ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
    st = ctx.stats()
    ctx.set_profiling(False)
    dev_s, wall_s = max_over_ranks([sum(dev_ms) / 1000.0, sum(wall)], dist, f"cuda:{local}")
    converged = sum(conv_counts)
    value = world * converged / dev_s
    e2e = world * converged / wall_s
    lat_all = np.concatenate(lat)
    screen = load_screen()
    line = {"metric": METRIC, "value": value, "unit": "integrals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "count": n, "pool_regions": args.max_regions,
                       "l2": "256 MB flush before every step", "seed": "config4_screen.json master 4096",
                       "eval_mode": args.eval_mode,
                       "screen": f"{len(screen['accepted'])} of the first {screen['accepted'][-1] + 1} candidates "
                                 f"converge within tolerance (unscreened pass rate "
                                 f"{len(screen['accepted']) / (screen['accepted'][-1] + 1):.3f}); the CPU oracle "
                                 f"repeats the decision on {_oracle_checked(screen)}"},
            "e2e": {"value": e2e, "unit": "integrals/s", "h2d_bytes_per_step": st.h2d_bytes // args.steps,
                    "d2h_bytes_per_step": st.d2h_bytes // args.steps},
            "gpu_launches": int(st.launches), "clocks": clk,
            "roofline": roofline(ctx, cases, results, st, args.steps, mode),
            "latency_ms": {"p50": float(np.percentile(lat_all, 50)), "p99": float(np.percentile(lat_all, 99))},
            "converged_per_step": conv_counts, "rule_points_per_s": st.points_evaluated / dev_s,
            "regions_per_step": st.regions_evaluated // args.steps,
            "step_breakdown_ms": {"evaluation": st.eval_ms / args.steps, "stages": st.stage_ms / args.steps,
                                  "host_decisions": st.host_ms / args.steps, "spill": st.spill_ms / args.steps,
                                  "admission": st.admit_ms / args.steps,
                                  "classifier_host": st.classify_ms / args.steps,
                                  "classifier_passes": st.classify_passes / args.steps},
            "setsum_region_share": st.setsum_regions / max(st.regions_evaluated, 1),
            "iterations": iteration_summary(ctx.iterations(), args.steps)}
    if rank == 0:
        step_s = wall_s / args.steps
        left = args.time_budget - (time.perf_counter() - t_begin)
        # Plain per-call path on the same GPU: every integral of the workload by
        # its own pg_integrate call, when it fits the budget; else a seeded
        # random sample, extrapolated to the workload by evaluation count.
        popt = pg.default_options(eval_mode=mode)
        tot_pts = float(sum(screen["neval"][:n]))
        if left > 3.0 * step_s + args.cpu_seconds + 60.0:
            t0 = time.perf_counter()
            pres = [ctx.integrate(c.integrand, c.epsrel, 0.0, options=popt) for c in cases]
            plain_s = time.perf_counter() - t0
            line["plain"] = {"sample": f"all {n} integrals, one pg_integrate call each (one pass)",
                             "plain_integrals_per_s": sum(1 for c, r in zip(cases, pres) if within(c, r)) / plain_s,
                             "plain_seconds": plain_s, "batched_seconds_per_step": step_s,
                             "batched_over_plain": plain_s / step_s}
        elif left > step_s + args.cpu_seconds + 30.0:
            idx = np.random.default_rng(7).permutation(n)
            t0 = time.perf_counter()
            pts, done = 0.0, 0
            for i in idx:
                if time.perf_counter() - t0 > 0.5 * step_s:
                    break
                c = cases[i]
                ctx.integrate(c.integrand, c.epsrel, 0.0, options=popt)
                pts += screen["neval"][i]
                done += 1
            plain_s = (time.perf_counter() - t0) * tot_pts / max(pts, 1.0)
            line["plain"] = {"sample": f"{done} integrals in a seeded random order, time extrapolated to the "
                                       f"workload by evaluation count",
                             "plain_seconds_estimated": plain_s, "batched_seconds_per_step": step_s,
                             "batched_over_plain": plain_s / step_s}
        else:
            line["plain"] = {"skipped": f"time budget ({args.time_budget:.0f} s) spent"}
        # CPU baseline: the oracle on all host cores, bounded sample, extrapolated by evaluation count.
        left = args.time_budget - (time.perf_counter() - t_begin)
        if left > args.cpu_seconds + 10.0:
            idx = cpu_sample(cases, screen, max(1e8, 2e9 * args.cpu_seconds / 20.0))
            cpu = cpu_leg(cases, idx)
            line["cpu_baseline"] = {"value": n / (tot_pts / cpu["points_per_s"]), "unit": "integrals/s",
                                    "cores": cpu["threads"], "kind": "port",
                                    "sample": f"{cpu['integrals']} integrals of the workload ({cpu['points']:.3g} rule "
                                              f"points, {cpu['seconds']:.1f} s, point by point), throughput "
                                              f"extrapolated to the whole step by evaluation count"}
        else:
            line["cpu_baseline"] = {"value": None, "skipped": "time budget spent"}
        line["wall_s_total"] = time.perf_counter() - t_begin
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def main():
    t_begin = time.perf_counter()
    args = parse()
    if args.config == "5" and args.impl == "gb300":
        return run_served(args)
    if args.config == "3" and args.impl == "gb300":
        return run_mcubes(args)
    if args.config == "eval":
        return run_eval(args)
    if args.config == "single":
        return run_single(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        from gpuintegration_gb300 import workloads as W
        run_reference(args, W.config4_cases(args.count) if rank == 0 else [], rank, world)
        return
    run_batched(args, rank, world, local, t_begin)


if __name__ == "__main__":
    main()
