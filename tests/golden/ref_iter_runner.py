"""Runs the reference's PAGANI iteration on the GPU with the reference's own
device stages.  TEST INFRASTRUCTURE (generates tests/golden/ref_iter.npz).

Device work is the reference's compiled code, built from the reference sources
by oracle/ref/build_ref.sh and loaded through the CUDA driver API:
  region evaluation        INIT_REGION_POOL / SampleRegionBlock   (oracle/_ref/ref_phase1.cubin)
  two-level error + flags  quad::RefineError<double>              (oracle/_ref/ref_stages.cubin)
  filter                   alignRegions<double, D>                (ref_stages.cubin)
  split                    divideIntervalsGPU<double, D>          (ref_stages.cubin)
The host loop around them restates Workspace::integrate
(cuda/pagani/quad/GPUquad/Workspace.cuh:361-494): accuracy_reached
(PaganiUtils.cuh:387-394), compute_finished_estimates (PaganiUtils.cuh:368-385),
fix_error_budget_overflow (Workspace.cuh:121-146), the heuristic classifier's
trigger (Workspace.cuh:74-118, heuristic_classifier.cuh:89-145,349-360; the
cases used never reach it, and this runner refuses to run one that would), the
exclusive scan and active count of Sub_region_filter.cuh:61-82, and the
iteration cap of 700.  Sums use numpy's order; the reference's thrust::reduce
order is unspecified, so iteration totals may differ from a real run in the
last bits.
"""
import ctypes
import os

import numpy as np

from tests.golden.ref_phase1_runner import RefKernel

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
STAGES = os.path.join(ROOT, "oracle", "_ref", "ref_stages.cubin")


def _mem_required(n, d):
    # heuristic_classifier.cuh:96-133 (bytes of a full split of n regions)
    doubles = 2 * n + 2 * n + 2 * n * d + 2 * n * d + n + n + 2 * n * d + 2 * n * d + n + n + n * d + n * d
    ints = n + 2 * n + n
    return 8 * doubles + 4 * ints


class RefStages:
    def __init__(self, phase1: RefKernel):
        self.p1 = phase1
        self.torch = phase1.torch
        self.cu = phase1.cu
        self.mod = ctypes.c_void_p()
        data = open(STAGES, "rb").read()
        rc = self.cu.cuModuleLoadData(ctypes.byref(self.mod), ctypes.c_char_p(data))
        if rc != 0:
            raise RuntimeError(f"cuModuleLoadData(ref_stages) failed: {rc}")
        # The kernels are template instantiations: find them by (mangled) name.
        cnt = ctypes.c_uint()
        if self.cu.cuModuleGetFunctionCount(ctypes.byref(cnt), self.mod) != 0:
            raise RuntimeError("cuModuleGetFunctionCount failed")
        fns = (ctypes.c_void_p * cnt.value)()
        if self.cu.cuModuleEnumerateFunctions(fns, cnt, self.mod) != 0:
            raise RuntimeError("cuModuleEnumerateFunctions failed")
        self.byname = {}
        for f in fns:
            name = ctypes.c_char_p()
            if self.cu.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(f)) != 0:
                raise RuntimeError("cuFuncGetName failed")
            self.byname[name.value.decode()] = ctypes.c_void_p(f)

    def _fn(self, key):
        hits = [v for k, v in self.byname.items() if key in k]
        if len(hits) != 1:
            raise RuntimeError(f"kernel {key!r}: {len(hits)} matches")
        return hits[0]

    def _launch(self, fn, grid, block, vals):
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        rc = self.cu.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, None, params, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel: {rc}")
        self.torch.cuda.synchronize()

    def _dev(self, a, dt=None):
        torch = self.torch
        return torch.tensor(np.ascontiguousarray(a), dtype=dt or torch.float64, device="cuda")

    def refine_error(self, est, err, parent_est, epsrel, relerr=True):
        """quad::RefineError<double>: two-level errors and active flags (doubles)."""
        torch = self.torch
        n = est.size
        t_est, t_err, t_par = self._dev(est), self._dev(err), self._dev(parent_est)
        t_new = torch.zeros(n, dtype=torch.float64, device="cuda")
        t_act = torch.ones(n, dtype=torch.float64, device="cuda")
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        vals = [P(t_est), P(t_err), P(t_par), P(t_par), P(t_new), P(t_act), ctypes.c_size_t(n),
                ctypes.c_double(epsrel), ctypes.c_int(0 if relerr else 1)]
        self._launch(self._fn("RefineError"), (n + 63) // 64, 64, vals)
        return t_new.cpu().numpy(), t_act.cpu().numpy()

    def filter_split(self, d, left, length, active, est, err, bisect):
        """alignRegions + divideIntervalsGPU: the next list (children of the
        active regions, child c of kept region k at c*A + k) and the kept
        regions' estimates and errors (the next iteration's parents)."""
        torch = self.torch
        n = est.size
        scan = np.concatenate([[0.0], np.cumsum(active)[:-1]])  # thrust::exclusive_scan of the double flags
        A = int(scan[-1] + (1 if active[-1] == 1.0 else 0))
        if A == 0:
            return None
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        t_left, t_len = self._dev(left.reshape(-1)), self._dev(length.reshape(-1))
        t_act, t_est, t_err = self._dev(active), self._dev(est), self._dev(err)
        t_bis, t_scan = self._dev(bisect, torch.int32), self._dev(scan)
        p_est = torch.zeros(A, dtype=torch.float64, device="cuda")
        p_err = torch.zeros(A, dtype=torch.float64, device="cuda")
        n_left = torch.zeros(A * d, dtype=torch.float64, device="cuda")
        n_len = torch.zeros(A * d, dtype=torch.float64, device="cuda")
        n_bis = torch.zeros(A, dtype=torch.int32, device="cuda")
        vals = [P(t_left), P(t_len), P(t_act), P(t_est), P(t_err), P(p_est), P(p_err), P(t_bis), P(t_scan),
                P(n_left), P(n_len), P(n_bis), ctypes.c_size_t(n), ctypes.c_size_t(A), ctypes.c_int(1)]
        self._launch(self._fn(f"alignRegionsIdLi{d}E"), (n + 255) // 256, 256, vals)
        c_left = torch.zeros(2 * A * d, dtype=torch.float64, device="cuda")
        c_len = torch.zeros(2 * A * d, dtype=torch.float64, device="cuda")
        vals = [P(c_left), P(c_len), P(n_left), P(n_len), P(n_bis), ctypes.c_size_t(A), ctypes.c_int(2)]
        self._launch(self._fn(f"divideIntervalsGPUIdLi{d}E"), (A + 255) // 256, 256, vals)
        return (c_left.cpu().numpy().reshape(d, 2 * A), c_len.cpu().numpy().reshape(d, 2 * A),
                p_est.cpu().numpy(), p_err.cpu().numpy())


def reference_integrate(stages: RefStages, f, epsrel, epsabs, uniform_split, total_mem=16e9, max_iters=700):
    """Workspace<double, d>::integrate(f, epsrel, epsabs, unit cube) with the
    reference's device stages; returns (result dict, per-iteration records)."""
    d = f.ndim
    parts = 4 if d < 5 else (2 if d <= 10 else 1)
    left, length = uniform_split(d, parts)
    cum = {"estimate": 0.0, "errorest": 0.0, "nregions": 0, "iters": 0, "status": 1}
    parent = None
    recs = []
    for it in range(max_iters):
        n = left.shape[1]
        if n == 0:
            break
        est, err_raw, bis = stages.p1.evaluate(f, left, length)
        iter_est = float(np.sum(est))
        act = np.ones(n)
        err = err_raw
        if parent is not None:
            err, act = stages.refine_error(est, err_raw, parent, epsrel)
        act_refine = act.copy()
        iter_err = float(np.sum(err))
        rec = {"n": n, "est": est, "err_raw": err_raw, "bisect": bis, "err": err, "act_refine": act_refine,
               "iter_est": iter_est, "iter_err": iter_err}
        recs.append(rec)
        if (cum["errorest"] + iter_err) / abs(cum["estimate"] + iter_est) <= epsrel or \
                cum["errorest"] + iter_err <= epsabs:
            cum["estimate"] += iter_est
            cum["errorest"] += iter_err
            cum["status"] = 0
            cum["nregions"] += n
            rec["act"] = act
            rec["fixed"] = False
            return cum, recs
        fin_est = iter_est - float(np.dot(act, est))
        fin_err = iter_err - float(np.dot(act, err))
        fixed = cum["errorest"] + fin_err > abs(cum["estimate"] + iter_est) * epsrel
        if fixed:  # fix_error_budget_overflow
            act = np.ones(n)
            fin_est = fin_err = 0.0
        rec["act"] = act
        rec["fixed"] = fixed
        occ = _mem_required(n, d)
        free = total_mem - occ if total_mem > occ else 1
        if occ / free > 0.1:
            raise RuntimeError("the heuristic classifier would be consulted; pick a smaller case")
        cum["estimate"] += fin_est
        cum["errorest"] += fin_err
        nxt = stages.filter_split(d, left, length, act, est, err, bis)
        A = 0 if nxt is None else nxt[2].size
        cum["nregions"] += n - A
        cum["iters"] += 1
        if nxt is None:
            left = np.zeros((d, 0))
            break
        left, length, parent, _ = nxt
    cum["nregions"] += left.shape[1]
    return cum, recs
