"""Runs the reference's own region-evaluation kernel (oracle/_ref/ref_phase1.cubin,
built from the reference sources by oracle/ref/build_ref.sh) through the CUDA
driver API.  TEST INFRASTRUCTURE.

The kernel takes the reference's rule tables (tests/golden/rule_tables.json,
produced by the reference's Rule::Init) and a region list, and returns the
reference's per-region estimate, error and split axis for an integrand of the
library's families.
"""
import ctypes
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_phase1.cubin")
MAXD = 16


class IntegralDesc(ctypes.Structure):
    """Byte layout of the library's IntegralDesc (csrc/pg_integrands.cuh)."""
    _fields_ = [("family", ctypes.c_int32), ("d", ctypes.c_int32), ("unit", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("jac", ctypes.c_double), ("c", ctypes.c_double), ("s0", ctypes.c_double),
                ("glo", ctypes.c_double * MAXD), ("range", ctypes.c_double * MAXD), ("a", ctypes.c_double * MAXD),
                ("u", ctypes.c_double * MAXD), ("ia2", ctypes.c_double * MAXD)]


def make_desc(f, lows=None, highs=None):
    """Same values as the library's prepare_desc (IEEE double arithmetic)."""
    D = IntegralDesc()
    D.family, D.d = f.family, f.ndim
    D.c = float(f.c)
    u = list(f.u) + [0.0] * (MAXD - len(f.u))
    a = list(f.a) + [0.0] * (MAXD - len(f.a))
    D.s0 = 2.0 * 3.14159265358979323846 * float(u[0])
    if f.family == 10:  # FUN6 normalisation
        D.c = 12.0 / (7.0 - 6.0 * math.log(2.0) * math.log(2.0) + math.log(64.0))
    for k in range(MAXD):
        D.a[k], D.u[k] = a[k], u[k]
        D.ia2[k] = 1.0 / (a[k] * a[k]) if a[k] != 0.0 else math.inf
    jac, unit = 1.0, 1
    for k in range(f.ndim):
        lo = 0.0 if lows is None else float(lows[k])
        hi = 1.0 if highs is None else float(highs[k])
        D.glo[k], D.range[k] = lo, hi - lo
        jac = jac * D.range[k]
        if lo != 0.0 or D.range[k] != 1.0:
            unit = 0
    D.jac, D.unit = jac, unit
    return D


class RefKernel:
    def __init__(self):
        import torch
        self.torch = torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # makes the primary context current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        data = open(CUBIN, "rb").read()
        rc = self.cu.cuModuleLoadData(ctypes.byref(self.mod), ctypes.c_char_p(data))
        if rc != 0:
            raise RuntimeError(f"cuModuleLoadData failed: {rc}")
        self.fns = {}

    def fn(self, d):
        if d not in self.fns:
            f = ctypes.c_void_p()
            rc = self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, f"ref_phase1_d{d}".encode())
            if rc != 0:
                raise RuntimeError(f"cuModuleGetFunction d={d}: {rc}")
            self.fns[d] = f
        return self.fns[d]

    def evaluate(self, f, left, length, lows=None, highs=None):
        torch = self.torch
        d = f.ndim
        t = json.load(open(os.path.join(HERE, "rule_tables.json")))["tables"][str(d)]
        mags = [float.fromhex(v) for v in t["gen_mag"]]
        code = "0abcdeABCDE"
        gen = []
        for ch in t["gen_code"]:
            k = code.index(ch)
            gen.append(0.0 if k == 0 else (mags[k - 1] if k <= 5 else -mags[k - 6]))
        fe = t["feval"]
        gen = np.array(gen).reshape(fe, d)
        # gpuG: only the two entries the fourth difference reads (Sample.cuh:195-196)
        gpuG = np.zeros(9 * d)
        g1 = gen[1]  # point 1 = +G0 on axis 0
        g2 = gen[1 + 2 * d]  # first point of set 2 = +G1 on axis 0
        gpuG[d * 1] = g1[0]
        gpuG[d * 2] = g2[0]
        dev = "cuda"
        T = lambda a, dt=torch.float64: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
        n = left.shape[1]
        t_left, t_len = T(left.reshape(-1)), T(length.reshape(-1))
        t_est, t_err = torch.zeros(n, dtype=torch.float64, device=dev), torch.zeros(n, dtype=torch.float64, device=dev)
        t_bis = torch.zeros(n, dtype=torch.int32, device=dev)
        t_G = T(gpuG)
        t_w = T([float.fromhex(v) for v in t["w"]])
        t_s = T([float.fromhex(v) for v in t["scale"]])
        t_n = T([float.fromhex(v) for v in t["norm"]])
        t_gi = T(t["gindex"], torch.int32)
        t_lo = T(np.zeros(d) if lows is None else lows)
        t_hi = T(np.ones(d) if highs is None else highs)
        t_gen = T(gen.T.reshape(-1))  # [FEVAL * dim + p]
        desc = make_desc(f, lows, highs)
        t_desc = torch.tensor(np.frombuffer(bytes(desc), dtype=np.uint8).copy(), device=dev)
        ptrs = [t_desc, t_left, t_len]
        vals = [ctypes.c_void_p(x.data_ptr()) for x in ptrs] + [ctypes.c_size_t(n)] + \
               [ctypes.c_void_p(x.data_ptr()) for x in (t_est, t_err, t_bis, t_G, t_w, t_s, t_n, t_gi, t_lo, t_hi, t_gen)]
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
        torch.cuda.synchronize()
        rc = self.cu.cuLaunchKernel(self.fn(d), n, 1, 1, 64, 1, 1, 0, None, params, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel: {rc}")
        torch.cuda.synchronize()
        return t_est.cpu().numpy(), t_err.cpu().numpy(), t_bis.cpu().numpy()
