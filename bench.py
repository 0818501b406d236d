#!/usr/bin/env python3
"""Benchmark of the GB300 PAGANI library on the batched Genz workload.

Workload (one step): the 4096 pre-screened mixed Genz integrals of the
batched configuration -- dim ~ U{2..8}, family ~ U{6 Genz families}, seeded
a_i/u_i scaled per family, epsrel log-uniform in [1e-7, 1e-4], FP64, unit
cube -- integrated together by pg_batch_integrate (one device region pool,
one evaluation launch per iteration over every live region).

Metric: converged integrals per second, where an integral counts when PAGANI
reports status 0 and the estimate lies within its epsrel of the analytic
value.  `value` is timed with CUDA events on the library's stream (the step's
integrand descriptors are a few MB; everything else is produced on the
device); `e2e` is the same metric by host wall clock around the C-ABI call,
including the host->device copy of the descriptors and the device->host copy
of the results.  p50/p99 are the per-integral completion latencies inside a
step.  The reference arm (--impl reference) times the CPU restatement of
PAGANI on all host cores on a bounded sample of the same workload.
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
# DRAM traffic of an evaluation launch over its algorithmic bytes, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of a batched launch.
DRAM_OVER_ALGORITHMIC = 1828488704 / 1800148656
WORKLOAD = "batched PAGANI: 4096 pre-screened mixed Genz integrals, dim 2..8, 6 families, epsrel log-U[1e-7,1e-4]"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--count", type=int, default=4096)
    p.add_argument("--plain-sample", type=int, default=256)
    p.add_argument("--cpu-seconds", type=float, default=20.0)
    p.add_argument("--max-regions", type=int, default=1 << 26)
    p.add_argument("--config", type=int, default=4, choices=[3, 4, 5],
                   help="4: batched workload (default, the metric's configuration); 5: served workload; "
                        "3: m-Cubes Gaussian")
    p.add_argument("--rate", type=float, default=2000.0, help="config 5: Poisson arrival rate (requests/s)")
    p.add_argument("--duration", type=float, default=60.0, help="config 5: arrival window (s)")
    p.add_argument("--budget-gb", type=float, default=120.0, help="config 5: device budget of the region pool")
    p.add_argument("--serve-seconds", type=float, default=0.0,
                   help="config 5: stop serving after this many seconds (0: arrival window + 60 s)")
    return p.parse_args()


def run_served(args):
    """Served PAGANI (Poisson arrivals, continuous batching, HBM budget)."""
    import gpuintegration_gb300 as pg
    from gpuintegration_gb300 import workloads as W
    arrivals = W.poisson_arrivals(args.rate, args.duration)
    cases = W.config5_cases(len(arrivals))
    ctx = pg.Context(0)
    fs = (pg.PgIntegrand * len(cases))(*[c.integrand.to_c() for c in cases])
    eps = np.array([c.epsrel for c in cases])
    clocks = ClockSampler(0)
    clocks.start()
    deadline = 1000.0 * (args.serve_seconds if args.serve_seconds > 0 else args.duration + 60.0)
    t0 = time.perf_counter()
    res, done = ctx.serve(fs, eps, 0.0, arrivals, budget_bytes=int(args.budget_gb * 1e9), deadline_ms=deadline)
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
                       "deadline_s": deadline / 1000.0},
            "latency_ms_finished": {"p50": float(np.percentile(lat, 50)) if lat.size else None,
                                    "p99": float(np.percentile(lat, 99)) if lat.size else None,
                                    "max": float(lat.max()) if lat.size else None},
            "arrived": arrived, "finished": int(fin.sum()), "unfinished_at_deadline": int((~fin).sum()),
            "wall_s": wall, "converged_within_tolerance": conv,
            "status0": sum(1 for r, ok in zip(res, fin) if ok and r.status == 0),
            "gpu_launches": int(st.launches), "points_per_s": st.points_evaluated / wall, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_mcubes(args):
    """m-Cubes on the 6-D sigma = 0.01 Gaussian (2^24 calls x 20 iterations, fixed seed)."""
    import gpuintegration_gb300 as pg
    from gpuintegration_gb300 import workloads as W
    ctx = pg.Context(0)
    f = W.config3_integrand()
    for _ in range(args.warmup):
        ctx.mcubes_integrate(f, 1e-4, 0.0, 2.0 ** 24, titer=20, itmax=20, skip=5, seed=2024)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = ctx.mcubes_integrate(f, 1e-4, 0.0, 2.0 ** 24, titer=20, itmax=20, skip=5, seed=2024)
    el = (time.perf_counter() - t0) / args.steps
    line = {"metric": "m-Cubes time to solution, 6-D Gaussian sigma 0.01", "value": el * 1000, "unit": "ms",
            "higher_is_better": False, "dtype": "f64", "data": "synthetic",
            "estimate": r.estimate, "errorest": r.errorest, "sigma_from_1": (r.estimate - 1.0) / r.errorest,
            "iters": r.iters, "status": r.status, "samples_per_s": r.neval / el}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def _feval(d):
    return 1 + 8 * d + 2 * d * (d - 1) + 4 * d * (d - 1) + 4 * d * (d - 1) * (d - 2) // 3 + (1 << d)


def ops_per_point(family, d):
    """Algorithmic FP64 operations (add, mul, FMA, compare, one per libm call)
    per evaluation point of the library's algorithm."""
    import gpuintegration_gb300 as pg
    if family in (pg.PRODUCT_PEAK, pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS, pg.PRODUCT):
        f = 1  # L * R from the half tries
    elif family == pg.OSCILLATORY:
        f = d + 1
    elif family == pg.CORNER_PEAK:
        e, muls = d + 1, 0
        while e:
            muls += (e & 1) + (1 if e > 1 else 0)
            e >>= 1
        f = d + muls + 1
    else:
        f = d + 1
    return f + 5  # five rule sums, one FMA each


def ops_per_region(family, d):
    import gpuintegration_gb300 as pg
    sep = family in (pg.PRODUCT_PEAK, pg.GAUSSIAN, pg.C0, pg.DISCONTINUOUS, pg.PRODUCT)
    factor = {pg.PRODUCT_PEAK: 3, pg.GAUSSIAN: 4, pg.C0: 3, pg.DISCONTINUOUS: 2, pg.PRODUCT: 0}.get(family, 0)
    m = d // 2  # half tries: depths 2..m of the left half, 2..d-m of the right half
    trie = (sum(_feval(k) for k in range(2, m + 1)) + sum(_feval(k) for k in range(2, d - m + 1))) if sep else 0
    return 11 * d * (2 + factor) + trie + 320 + (5 * d + 2) + 113 + d


def algorithmic_ops(cases, results):
    tot = 0.0
    for c, r in zip(cases, results):
        f = c.integrand
        regions = r.neval // _feval(f.ndim)
        tot += r.neval * ops_per_point(f.family, f.ndim) + regions * ops_per_region(f.family, f.ndim)
    return tot


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


# ---------------------------------------------------------------------------
CPU_SAMPLE_MAX_REGIONS = 200000


def cpu_leg(cases, seconds, totals=None):
    """Times the CPU oracle (all host threads) on the integrals of the workload,
    in workload order, whose screened region count is at most
    CPU_SAMPLE_MAX_REGIONS (so no single integral runs for minutes), until
    `seconds` have passed; returns evaluation points/s and the sample."""
    from oracle import oracle
    oracle.load()
    screen = json.load(open(os.path.join(ROOT, "tests", "golden", "config4_screen.json")))
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    pts, done, conv = 0, 0, 0
    for c, nreg in zip(cases, screen["nregions"]):
        if nreg > CPU_SAMPLE_MAX_REGIONS:
            continue
        r, _ = oracle.integrate(c.integrand, c.epsrel, 0.0, nthreads=threads)
        pts += r.neval
        done += 1
        conv += 1 if within(c, r) else 0
        if time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    return {"points_per_s": pts / el, "integrals": done, "converged": conv, "seconds": el, "threads": threads}


def run_reference(args, cases, rank, world):
    """Reference arm: the CPU restatement of PAGANI on every host core."""
    if rank != 0:
        return
    total_pts = None
    screen = json.load(open(os.path.join(ROOT, "tests", "golden", "config4_screen.json")))
    import gpuintegration_gb300 as pg
    lib = pg.load_library()
    # evaluation count of the whole workload, from the screen run (leaf regions x points, x2 for inner nodes)
    fe = [lib.pg_feval(c.integrand.ndim) for c in cases]
    total_pts = float(sum(2 * n * f for n, f in zip(screen["nregions"][:len(cases)], fe)))
    vals = []
    for i in range(args.warmup + args.steps):
        s = cpu_leg(cases, args.cpu_seconds / 2)
        if i >= args.warmup:
            vals.append(s)
    pps = sum(v["points_per_s"] for v in vals) / len(vals)
    value = len(cases) / (total_pts / pps)
    sample = f"first {vals[-1]['integrals']} integrals of the workload per step, extrapolated by evaluation count"
    line = {"metric": METRIC, "value": value, "unit": "integrals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * vals[-1]["seconds"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "count": len(cases), "l2": "n/a (CPU)"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "integrals/s", "cores": vals[-1]["threads"], "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "integrals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "no CPU PAGANI in the reference (Cuhre via cubacpp needs libcuba, absent); the oracle port "
                    "restates the reference's CUDA iteration on host threads"}
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
def main():
    args = parse()
    if args.config == 5 and args.impl == "gb300":
        return run_served(args)
    if args.config == 3 and args.impl == "gb300":
        return run_mcubes(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    from gpuintegration_gb300 import workloads as W
    cases = W.config4_cases(args.count)
    if args.impl == "reference":
        run_reference(args, cases, rank, world)
        return

    import torch
    import gpuintegration_gb300 as pg
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
    opt = pg.default_options(max_regions=args.max_regions)
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
    dev_s = sum(dev_ms) / 1000.0
    wall_s = sum(wall)
    dev_s, wall_s = max_over_ranks([dev_s, wall_s], dist, f"cuda:{local}")
    converged = sum(conv_counts)
    value = world * converged / dev_s
    e2e = world * converged / wall_s
    lat_all = np.concatenate(lat)
    # Roofline of the dominant kernel (region evaluation, FP64 pipe), in FP64
    # operations per second against the measured FP64 FMA instruction rate.
    alg = algorithmic_ops(cases, results) * args.steps
    achieved = alg / (st.eval_ms / 1000.0) / 1e12
    peak = ctx.probe_fp64_peak() / 2.0
    # DRAM bytes per evaluation launch: the launch's algorithmic bytes (region
    # bounds in, estimate/error/split axis out, owner index) times the ratio
    # ncu measured on one batched evaluation launch of this workload (14.27M
    # regions of the first 4096 integrals, iteration 8: 1.830 GB read+written
    # against 1.800 GB algorithmic).
    alg_bytes_per_launch = st.eval_bytes / max(st.eval_launches, 1)
    traffic = alg_bytes_per_launch * DRAM_OVER_ALGORITHMIC
    roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "FP64 Top/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": "eval_kernel",
            "peak_source": "measured FP64 FMA instruction rate of this GPU (pg_probe_fp64_peak, TFLOP/s / 2); "
                           "MEASURED_PEAKS.json has no FP64 figure",
            "algorithmic_ops_per_step": alg / args.steps,
            "algorithmic_bytes_per_launch": alg_bytes_per_launch,
            "eval_ms_per_step": st.eval_ms / args.steps, "stage_ms_per_step": st.stage_ms / args.steps,
            "host_decision_ms_per_step": st.host_ms / args.steps,
            "spill_ms_per_step": st.spill_ms / args.steps, "admit_ms_per_step": st.admit_ms / args.steps,
            "note": "the point loop's multiplies run on the integer pipe (bit-identical to the FP64 multiply); "
                    "achieved counts every algorithmic multiply as an FP64 operation",
            "stage_gbs": (st.stage_bytes / max(st.stage_ms, 1e-9)) / 1e6,
            "autotuned_launch": {"warps_per_block": list(st.tune_warps), "ctas_per_sm": list(st.tune_ctas_per_sm)}}
    line = {"metric": METRIC, "value": value, "unit": "integrals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "count": n, "pool_regions": args.max_regions,
                       "l2": "256 MB flush before every step", "seed": "config4_screen.json master 4096"},
            "e2e": {"value": e2e, "unit": "integrals/s", "h2d_bytes_per_step": st.h2d_bytes // args.steps,
                    "d2h_bytes_per_step": st.d2h_bytes // args.steps},
            "gpu_launches": int(st.launches), "clocks": clk, "roofline": roof,
            "latency_ms": {"p50": float(np.percentile(lat_all, 50)), "p99": float(np.percentile(lat_all, 99))},
            "converged_per_step": conv_counts, "points_per_s": st.points_evaluated / dev_s,
            "regions_per_step": st.regions_evaluated // args.steps}
    if rank == 0:
        # Plain per-call path on the same GPU, on a sample (batched on the same sample for the ratio).
        ns = min(args.plain_sample, n)
        sub = cases[:ns]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for c in sub:
            ctx.integrate(c.integrand, c.epsrel, 0.0)
        plain_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        ctx.batch_integrate([c.integrand for c in sub], [c.epsrel for c in sub], 0.0, options=opt)
        batch_s = time.perf_counter() - t0
        line["plain"] = {"sample": f"first {ns} integrals of the workload",
                         "plain_integrals_per_s": ns / plain_s, "batched_integrals_per_s": ns / batch_s,
                         "batched_over_plain": plain_s / batch_s}
        # Where batching pays: the light integrals (<= 20000 regions when screened), whose plain
        # runs are bound by per-iteration launches and synchronisation rather than by FP64 work.
        screen = json.load(open(os.path.join(ROOT, "tests", "golden", "config4_screen.json")))
        light = [c for c, nr in zip(cases, screen["nregions"]) if nr <= 20000][:1024]
        t0 = time.perf_counter()
        for c in light:
            ctx.integrate(c.integrand, c.epsrel, 0.0)
        pl = time.perf_counter() - t0
        t0 = time.perf_counter()
        ctx.batch_integrate([c.integrand for c in light], [c.epsrel for c in light], 0.0, options=opt)
        bl = time.perf_counter() - t0
        line["plain_light"] = {"sample": f"first {len(light)} integrals with <= 20000 screened regions",
                               "plain_integrals_per_s": len(light) / pl, "batched_integrals_per_s": len(light) / bl,
                               "batched_over_plain": pl / bl}
        # CPU baseline: the oracle on all host cores, bounded sample, extrapolated by evaluation count.
        cpu = cpu_leg(cases, args.cpu_seconds)
        total_pts = sum(r.neval for r in results)
        line["cpu_baseline"] = {"value": n / (total_pts / cpu["points_per_s"]), "unit": "integrals/s",
                                "cores": cpu["threads"], "kind": "port",
                                "sample": f"first {cpu['integrals']} integrals with <= {CPU_SAMPLE_MAX_REGIONS} regions "
                                          f"({cpu['seconds']:.1f} s), throughput extrapolated to the whole step "
                                          f"by evaluation count"}
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
