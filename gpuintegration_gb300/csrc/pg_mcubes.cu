// m-Cubes (stratified VEGAS) on the GB300.
//
// Restates cuda_mcubes::vegas (cuda/mcubes/vegasT.cuh:643-997) with its
// sampling kernels (vegasT.cuh:136-614):
//   * the same stratification: ng = floor((ncall/2 + 0.25)^(1/d)) intervals per
//     axis, ncubes = ng^d, npg = max(ncall/ncubes, 2) samples per cube, 500 bins
//     per axis, the same point map, weights and per-cube variance term;
//   * random numbers from Philox4x32-10 (Salmon et al., SC'11), keyed by the
//     seed with counter (cube, sample, axis pair, iteration), so a run is
//     reproducible from its seed (the reference seeds XORWOW from the clock,
//     vegasT.cuh:801-803);
//   * per-bin sums of f^2 in a shared-memory histogram per block, flushed once
//     per block, instead of one global atomic per sample and axis;
//   * a fixed grid of 1024 x 256 threads, each taking a contiguous run of cubes,
//     and block-tree sums: the estimate does not depend on the GPU's SM count;
//   * grid smoothing and rebinning on the host between iterations, damping
//     exponent alpha (1.5 in the reference's GPU code, vegas_utils.cuh:139).
#include "pg_mcubes.h"

#include "pg_mcubes_kernel.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace pg {

struct McubesState {
  Engine* eng = nullptr;
  DevBuf xi, bins, partial;
};

McubesState* mcubes_create(Engine* eng) {
  McubesState* st = new McubesState;
  st->eng = eng;
  return st;
}

void mcubes_destroy(McubesState* st) {
  if (!st) return;
  if (st->xi.p) cudaFree(st->xi.p);
  if (st->bins.p) cudaFree(st->bins.p);
  if (st->partial.p) cudaFree(st->partial.p);
  delete st;
}

namespace {

// Rebinning of one axis so every new bin holds the same share of r
// (vegasT.cuh:616-637).  xi[0..nd] with xi[0] = 0, r[1..nd].
void rebin(double rc, int nd, const double* r, double* xin, double* xi) {
  int k = 0;
  double dr = 0.0, xn = 0.0, xo = 0.0;
  for (int i = 1; i < nd; i++) {
    while (rc > dr) dr += r[++k];
    if (k > 1) xo = xi[k - 1];
    xn = xi[k];
    dr -= rc;
    xin[i] = xn - (xn - xo) * dr / r[k];
  }
  for (int i = 1; i < nd; i++) xi[i] = xin[i];
  xi[nd] = 1.0;
}

int status_of(double est, double err, int it, double epsrel, double epsabs) {
  // GetStatus (vegas_utils.cuh:237-248)
  const bool ok = std::fabs(err / est) <= epsrel || err <= epsabs;
  return (ok && it >= 5) ? 0 : 1;
}

}  // namespace

cudaError_t launch_family_mcubes(const pg_mcubes_args& a) {
  return a.maxd <= 8 ? launch_mcubes<8>(a, FamilyFn{}) : launch_mcubes<16>(a, FamilyFn{});
}

int mcubes_run(McubesState* st, const IntegralDesc& D, double epsrel, double epsabs, const pg_mcubes_options& opt,
               pg_result* out, std::string* why, const McubesLauncher& launcher) {
  Engine* E = st->eng;
  const int d = D.d;
  const int nd = opt.nbins > 1 ? opt.nbins : 500;
  if (opt.ncall < 2 || opt.titer < 1 || opt.itmax < 0) {
    if (why) *why = "m-Cubes needs ncall >= 2 and titer >= 1";
    return PG_BAD_ARG;
  }
  // Geometry (vegasT.cuh:704-735).
  const uint64_t ng = (uint64_t)std::pow(opt.ncall / 2.0 + 0.25, 1.0 / d);
  if (ng < 1) {
    if (why) *why = "ncall too small for this dimension";
    return PG_BAD_ARG;
  }
  double k = 1;
  for (int i = 1; i < d; ++i) k *= (double)ng;
  k *= (double)ng;
  const double ncubes = k;
  const int npg = (int)std::max(opt.ncall / k, 2.0);
  const double calls = (double)npg * k;
  double dxg = 1.0 / (double)ng;
  double dv2g = 1;
  for (int i = 1; i <= d; ++i) dv2g *= dxg;
  dv2g = (calls * dv2g * calls * dv2g) / npg / npg / (npg - 1.0);
  const double xnd = nd;
  dxg *= xnd;
  double xjac = 1.0 / calls;
  std::vector<double> regn(d), dx(d);
  for (int j = 0; j < d; ++j) {
    regn[j] = D.glo[j];
    dx[j] = D.range[j];
    xjac *= dx[j];
  }
  const int nb1 = nd + 1;
  std::vector<double> xi((size_t)d * nb1, 0.0), r(nb1, 1.0), xin(nb1, 0.0), dbin((size_t)d * nb1, 0.0), dt(d);
  for (int j = 0; j < d; ++j) {
    xi[(size_t)j * nb1 + 1] = 1.0;
    rebin(1.0 / xnd, nd, r.data(), xin.data(), &xi[(size_t)j * nb1]);
  }
  int rc;
  if ((rc = E->ensure(st->xi, xi.size() * 8)) != PG_OK || (rc = E->ensure(st->bins, xi.size() * 8)) != PG_OK ||
      (rc = E->ensure(st->partial, kMcBlocks * 2 * 8)) != PG_OK) {
    if (why) *why = E->last_error;
    return rc;
  }
  cudaStream_t s = E->stream();
  const size_t smem = 2 * (size_t)d * nb1 * 8;
  auto fail = [&](cudaError_t e, const char* what) {
    if (why) *why = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PG_OOM : PG_CUDA_ERROR;
  };
  if (smem > kMcMaxSmem) {
    if (why) *why = "too many bins for this dimension";
    return PG_BAD_ARG;
  }
  McArgs A;
  std::memset(&A, 0, sizeof A);
  A.desc = D;
  A.d = d;
  A.ng = (int)ng;
  A.npg = npg;
  A.nbins = nd;
  A.ncubes = (uint64_t)ncubes;
  A.dxg = dxg;
  A.xnd = xnd;
  A.xjac = xjac;
  for (int j = 0; j < d; ++j) {
    A.regn[j] = regn[j];
    A.dx[j] = dx[j];
  }
  A.key0 = (uint32_t)opt.seed;
  A.key1 = (uint32_t)(opt.seed >> 32);
  A.xi = (const double*)st->xi.p;
  A.bins = (double*)st->bins.p;
  A.partial = (double*)st->partial.p;
  std::vector<double> part(kMcBlocks * 2);
  double si = 0, swgt = 0, schi = 0, tgral = 0, sd = 0, chi2a = 0;
  int status = 1;
  uint64_t iters = 0;
  auto launch = [&](int it, int adapt) -> int {
    A.iter = (uint32_t)it;
    A.adapt = adapt;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(st->xi.p, xi.data(), xi.size() * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return fail(e, "grid upload");
    if (adapt && (e = cudaMemsetAsync(st->bins.p, 0, xi.size() * 8, s)) != cudaSuccess) return fail(e, "memset");
    pg_mcubes_args la;
    la.args = &A;
    la.smem = smem;
    la.stream = (void*)s;
    la.maxd = d;
    la.pad = 0;
    e = launcher(la);
    E->stats.launches++;
    E->stats.points_evaluated += (uint64_t)calls;
    if (e != cudaSuccess) return fail(e, "m-Cubes launch");
    if ((e = cudaMemcpyAsync(part.data(), st->partial.p, part.size() * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return fail(e, "readback");
    if (adapt &&
        (e = cudaMemcpyAsync(dbin.data(), st->bins.p, dbin.size() * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
      return fail(e, "readback");
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e, "m-Cubes iteration");
    return PG_OK;
  };
  auto totals = [&](double* ti, double* tsi) {
    double a = 0, b = 0;
    for (int bI = 0; bI < kMcBlocks; ++bI) {
      a += part[2 * bI];
      b += part[2 * bI + 1];
    }
    *ti = a;
    *tsi = b * dv2g;
  };
  // Adapting iterations (vegasT.cuh:784-911).
  for (int it = 1; it <= opt.itmax && status == 1; ++iters, ++it) {
    if ((rc = launch(it, 1)) != PG_OK) return rc;
    double ti, tsi;
    totals(&ti, &tsi);
    if (it > opt.skip) {
      const double wgt = 1.0 / tsi;
      si += wgt * ti;
      schi += wgt * ti * ti;
      swgt += wgt;
      tgral = si / swgt;
      chi2a = (schi - si * tgral) / (static_cast<double>(it) - 0.9999);
      if (chi2a < 0.0) chi2a = 0.0;
      sd = std::sqrt(1.0 / swgt);
      status = status_of(tgral, sd, it, epsrel, epsabs);
    }
    // Smooth the bin sums and rebin every axis (vegasT.cuh:873-910).
    for (int j = 0; j < d; ++j) {
      double* dj = &dbin[(size_t)j * nb1];
      double xo = dj[1], xn = dj[2];
      dj[1] = (xo + xn) / 2.0;
      dt[j] = dj[1];
      for (int i = 2; i < nd; ++i) {
        const double rcv = xo + xn;
        xo = xn;
        xn = dj[i + 1];
        dj[i] = (rcv + xn) / 3.0;
        dt[j] += dj[i];
      }
      dj[nd] = (xo + xn) / 2.0;
      dt[j] += dj[nd];
    }
    for (int j = 0; j < d; ++j) {
      if (dt[j] > 0.0) {
        const double* dj = &dbin[(size_t)j * nb1];
        double rsum = 0.0;
        for (int i = 1; i <= nd; ++i) {
          r[i] = std::pow((1.0 - dj[i] / dt[j]) / (std::log(dt[j]) - std::log(dj[i])), opt.alpha);
          rsum += r[i];
        }
        rebin(rsum / xnd, nd, r.data(), xin.data(), &xi[(size_t)j * nb1]);
      }
    }
  }
  // Frozen-grid iterations (vegasT.cuh:921-977).
  for (int it = opt.itmax + 1; it <= opt.titer && status; ++iters, ++it) {
    if ((rc = launch(it, 0)) != PG_OK) return rc;
    double ti, tsi;
    totals(&ti, &tsi);
    const double wgt = 1.0 / tsi;
    si += wgt * ti;
    schi += wgt * ti * ti;
    swgt += wgt;
    tgral = si / swgt;
    chi2a = (schi - si * tgral) / (it - 0.9999);
    if (chi2a < 0.0) chi2a = 0.0;
    sd = std::sqrt(1.0 / swgt);
    status = status_of(tgral, sd, it, epsrel, epsabs);
  }
  pg_result R;
  std::memset(&R, 0, sizeof R);
  R.estimate = tgral;
  R.errorest = sd;
  R.chi_sq = chi2a;
  R.neval = (uint64_t)calls * iters;
  R.nregions = (uint64_t)ncubes;
  R.iters = iters;
  R.status = status;
  R.last_phase = -1;
  *out = R;
  return PG_OK;
}

}  // namespace pg
