"""Runs the reference's GPU m-Cubes with the reference's own sampling kernels.
TEST INFRASTRUCTURE (generates the "gpu" part of tests/golden/mcubes_ref.json).

Device work is cuda_mcubes::vegas_kernel / vegas_kernelF with the reference's
Curand_generator, compiled from the reference sources
(oracle/_ref/ref_mcubes.cubin, oracle/ref/build_ref.sh) and loaded through the
CUDA driver API.  The host loop restates cuda_mcubes::vegas
(cuda/mcubes/vegasT.cuh:643-997): the geometry, the chunked launch
(GetChunkSize, Kernel_Params: vegas_utils.cuh:199-263), the adapting and
frozen iterations, the weighted mean, GetStatus (vegas_utils.cuh:237-248), the
smoothing of the bin sums and the rebinning (vegasT.cuh:616-637,873-910) with
damping exponent 1.5.  The reference seeds each iteration's kernel with
(milliseconds since the start + it) + it; here that is base_seed + 2 * it
with base_seed recorded.
"""
import ctypes
import math
import os

import numpy as np

from tests.golden.ref_phase1_runner import make_desc

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_mcubes.cubin")
NDMX, MXDIM_P1, ALPH = 500, 21, 1.5
NDMX_P1 = NDMX + 1


def _rebin(rc, nd, r, xin, xi, off):
    k = 0
    dr = xn = xo = 0.0
    for i in range(1, nd):
        while rc > dr:
            k += 1
            dr += r[k]
        if k > 1:
            xo = xi[off + k - 1]
        xn = xi[off + k]
        dr -= rc
        xin[i] = xn - (xn - xo) * dr / r[k]
    for i in range(1, nd):
        xi[off + i] = xin[i]
    xi[off + nd] = 1.0


def _chunk_size(ncall):
    if ncall < 1e6:
        return 4
    if ncall <= 1e7:
        return 32
    if ncall <= 8e9:
        return 2048
    return 4096


class RefMcubes:
    def __init__(self):
        import torch
        self.torch = torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        if self.cu.cuModuleLoadData(ctypes.byref(self.mod), ctypes.c_char_p(open(CUBIN, "rb").read())) != 0:
            raise RuntimeError("cuModuleLoadData(ref_mcubes) failed")
        cnt = ctypes.c_uint()
        self.cu.cuModuleGetFunctionCount(ctypes.byref(cnt), self.mod)
        fns = (ctypes.c_void_p * cnt.value)()
        self.cu.cuModuleEnumerateFunctions(fns, cnt, self.mod)
        self.byname = {}
        for f in fns:
            name = ctypes.c_char_p()
            self.cu.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(f))
            self.byname[name.value.decode()] = ctypes.c_void_p(f)

    def _fn(self, frozen, d):
        key = ("vegas_kernelFI" if frozen else "vegas_kernelI") + f"9RefMcubesILi{d}E"
        hits = [v for k, v in self.byname.items() if key in k]
        if len(hits) != 1:
            raise RuntimeError(f"{key}: {len(hits)} matches")
        return hits[0]

    def integrate(self, f, epsrel, epsabs, ncall, titer, itmax, skip, base_seed):
        torch = self.torch
        ndim = f.ndim
        dev = "cuda"
        regn = np.zeros(2 * MXDIM_P1)
        for j in range(1, ndim + 1):
            regn[j], regn[j + ndim] = 0.0, 1.0
        xi = np.zeros(MXDIM_P1 * NDMX_P1)
        for j in range(1, ndim + 1):
            xi[j * NDMX_P1 + 1] = 1.0
        si = swgt = schi = 0.0
        nd = NDMX
        ng = int(math.pow(ncall / 2.0 + 0.25, 1.0 / ndim))
        k = 1.0
        for _ in range(1, ndim):
            k *= ng
        sci, sc = 1.0 / k, k
        k *= ng
        ncubes = k
        npg = max(int(ncall / k), 2)
        calls = float(npg) * k
        dxg = 1.0 / ng
        ing = dxg
        dv2g = 1.0
        for _ in range(ndim):
            dv2g *= dxg
        dv2g = (calls * dv2g * calls * dv2g) / npg / npg / (npg - 1.0)
        xnd = float(nd)
        dxg *= xnd
        xjac = 1.0 / calls
        dx = np.zeros(MXDIM_P1)
        for j in range(1, ndim + 1):
            dx[j] = regn[j + ndim] - regn[j]
            xjac *= dx[j]
        r = np.ones(NDMX_P1)
        xin = np.zeros(NDMX_P1)
        for j in range(1, ndim + 1):
            _rebin(1 / xnd, nd, r, xin, xi, j * NDMX_P1)
        chunk = _chunk_size(ncall)
        total_threads = int(ncubes / chunk)
        extra = int(ncubes - total_threads * chunk)
        last_chunk = extra + chunk
        nblocks = (total_threads + 127) // 128
        T = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
        t_int = torch.tensor(np.frombuffer(bytes(make_desc(f)), dtype=np.uint8).copy(), device=dev)
        t_res = torch.zeros(2, dtype=torch.float64, device=dev)
        t_d = torch.zeros(NDMX_P1 * MXDIM_P1, dtype=torch.float64, device=dev)
        t_dx = T(dx)
        t_regn = T(regn[:2 * ndim + 1])
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        tgral = sd = chi2a = 0.0
        status, iters = 1, 0

        def launch(frozen, it, t_xi):
            vals = [P(t_int), ctypes.c_int(ng), ctypes.c_int(npg), ctypes.c_double(xjac), ctypes.c_double(dxg),
                    P(t_res), ctypes.c_double(xnd), P(t_xi), P(t_d), P(t_dx), P(t_regn), ctypes.c_int(int(ncubes)),
                    ctypes.c_int(it), ctypes.c_double(sc), ctypes.c_double(sci), ctypes.c_double(ing),
                    ctypes.c_int(chunk), ctypes.c_uint32(total_threads), ctypes.c_int(last_chunk),
                    ctypes.c_uint(base_seed + 2 * it)]
            if not frozen:
                vals += [ctypes.c_void_p(0), ctypes.c_void_p(0)]
            params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.pointer(v), ctypes.c_void_p) for v in vals])
            torch.cuda.synchronize()
            if self.cu.cuLaunchKernel(self._fn(frozen, ndim), nblocks, 1, 1, 128, 1, 1, 0, None, params, None) != 0:
                raise RuntimeError("cuLaunchKernel failed")
            torch.cuda.synchronize()

        def accumulate(it, ti, tsi):
            nonlocal si, schi, swgt, tgral, chi2a, sd, status
            wgt = 1.0 / tsi
            si += wgt * ti
            schi += wgt * ti * ti
            swgt += wgt
            tgral = si / swgt
            chi2a = (schi - si * tgral) / (float(it) - 0.9999)
            if chi2a < 0.0:
                chi2a = 0.0
            sd = math.sqrt(1.0 / swgt)
            ok = abs(sd / tgral) <= epsrel or sd <= epsabs
            status = 0 if (ok and it >= 5) else 1

        it = 1
        while it <= itmax and status == 1:
            t_d.zero_()
            t_res.zero_()
            t_xi = T(xi)
            launch(False, it, t_xi)
            d = t_d.cpu().numpy().copy()
            res = t_res.cpu().numpy()
            ti, tsi = res[0], res[1] * dv2g
            if it > skip:
                accumulate(it, ti, tsi)
            dt = np.zeros(MXDIM_P1)
            for j in range(1, ndim + 1):
                xo, xn = d[1 * MXDIM_P1 + j], d[2 * MXDIM_P1 + j]
                d[1 * MXDIM_P1 + j] = (xo + xn) / 2.0
                dt[j] = d[1 * MXDIM_P1 + j]
                for i in range(2, nd):
                    rc = xo + xn
                    xo = xn
                    xn = d[(i + 1) * MXDIM_P1 + j]
                    d[i * MXDIM_P1 + j] = (rc + xn) / 3.0
                    dt[j] += d[i * MXDIM_P1 + j]
                d[nd * MXDIM_P1 + j] = (xo + xn) / 2.0
                dt[j] += d[nd * MXDIM_P1 + j]
            for j in range(1, ndim + 1):
                if dt[j] > 0.0:
                    rc = 0.0
                    for i in range(1, nd + 1):
                        di = d[i * MXDIM_P1 + j]
                        r[i] = math.pow((1.0 - di / dt[j]) / (math.log(dt[j]) - (math.log(di) if di > 0 else -math.inf)),
                                        ALPH)
                        rc += r[i]
                    _rebin(rc / xnd, nd, r, xin, xi, j * NDMX_P1)
            it += 1
            iters += 1
        t_xi = T(xi)
        it = itmax + 1
        while it <= titer and status:
            t_res.zero_()
            launch(True, it, t_xi)
            res = t_res.cpu().numpy()
            accumulate(it, res[0], res[1] * dv2g)
            it += 1
            iters += 1
        return {"estimate": tgral, "errorest": sd, "chi_sq": chi2a, "status": status, "iters": iters}
