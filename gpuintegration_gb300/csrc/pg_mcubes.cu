// m-Cubes (stratified VEGAS) on the GB300.
//
// Restates cuda_mcubes::vegas (cuda/mcubes/vegasT.cuh:643-997) with its
// sampling kernels (vegasT.cuh:136-614):
//   * the same stratification: ng = floor((ncall/2 + 0.25)^(1/d)) intervals per
//     axis, ncubes = ng^d, npg = max(ncall/ncubes, 2) samples per cube, 500 bins
//     per axis, the same point map, weights and per-cube variance term;
//   * random numbers from Philox4x32-10 (Salmon et al., SC'11), keyed by the
//     seed with counter (cube, sample, axis pair, iteration) (the reference
//     seeds XORWOW from the clock, vegasT.cuh:801-803);
//   * per-bin sums of f^2 formed in a fixed order (mcubes_kernel, then
//     mcubes_bins_kernel over the blocks), and every other sum in a fixed
//     order too, so a run is reproducible bit for bit from its seed;
//   * a fixed grid of 1024 x 256 threads: the estimate does not depend on the
//     GPU's SM count;
//   * the weighted mean over iterations, the convergence test, the smoothing
//     of the bin sums and the rebinning with damping exponent alpha (1.5 in the
//     reference's GPU code, vegas_utils.cuh:139; vegasT.cuh:834-910) run on
//     the device (mcubes_update_kernel).  The host enqueues every iteration at
//     once; after convergence the remaining iterations' kernels return at once,
//     so a run needs one synchronisation instead of one per iteration.
#include "pg_mcubes.h"

#include "pg_mcubes_kernel.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace pg {

struct McubesState {
  Engine* eng = nullptr;
  DevBuf xi, bins, part_hist, partial, scratch, state;
};

McubesState* mcubes_create(Engine* eng) {
  McubesState* st = new McubesState;
  st->eng = eng;
  return st;
}

void mcubes_destroy(McubesState* st) {
  if (!st) return;
  DevBuf* bufs[] = {&st->xi, &st->bins, &st->part_hist, &st->partial, &st->scratch, &st->state};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  delete st;
}

namespace {

// Rebinning of one axis so every new bin holds the same share of r
// (vegasT.cuh:616-637; Lepage's VEGAS, J. Comput. Phys. 27 (1978) 192).
// xi[0..nd] with xi[0] = 0, r[1..nd].
__host__ __device__ void rebin(double rc, int nd, const double* r, double* xin, double* xi) {
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

// Sum of the blocks' histograms, bin by bin, in block order.
__global__ void mcubes_bins_kernel(const double* __restrict__ part_hist, int nbins_total, double* __restrict__ bins,
                                   const McState* __restrict__ state) {
  if (state->stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbins_total) return;
  double s = 0.0;
  for (int b = 0; b < kMcBlocks; ++b) s = s + part_hist[(size_t)b * nbins_total + i];
  bins[i] = s;
}

struct McUpdate {
  int it, adapt, skip, d, nd;
  double epsrel, epsabs, dv2g, xnd, alpha;
};

// One iteration's bookkeeping (vegasT.cuh:834-910): the iteration's estimate
// and variance from the block sums, the weighted mean, chi^2 and status, then
// (adapting iterations) per axis the smoothing of the bin sums and the
// rebinning.  One warp per axis.  `bins` is smoothed in place; scratch holds
// r and xin per axis.
__global__ void mcubes_update_kernel(McUpdate U, const double* __restrict__ partial, double* __restrict__ bins,
                                     double* __restrict__ xi, double* __restrict__ scratch, McState* state) {
  __shared__ int go;
  if (threadIdx.x == 0) go = state->stop == 0;
  __syncthreads();
  if (!go) return;
  const int nb1 = U.nd + 1;
  if (threadIdx.x == 0) {
    double ti = 0.0, tsi = 0.0;
    for (int b = 0; b < kMcBlocks; ++b) {
      ti = ti + partial[2 * b];
      tsi = tsi + partial[2 * b + 1];
    }
    tsi = tsi * U.dv2g;
    McState S = *state;
    if (!U.adapt || U.it > U.skip) {
      const double wgt = 1.0 / tsi;
      S.si = S.si + wgt * ti;
      S.schi = S.schi + wgt * ti * ti;
      S.swgt = S.swgt + wgt;
      S.tgral = S.si / S.swgt;
      S.chi2a = (S.schi - S.si * S.tgral) / (static_cast<double>(U.it) - 0.9999);
      if (S.chi2a < 0.0) S.chi2a = 0.0;
      S.sd = sqrt(1.0 / S.swgt);
      // GetStatus (vegas_utils.cuh:237-248)
      const bool ok = fabs(S.sd / S.tgral) <= U.epsrel || S.sd <= U.epsabs;
      S.status = (ok && U.it >= 5) ? 0 : 1;
    }
    S.iters += 1;
    S.stop = S.status == 0;
    *state = S;
  }
  if (!U.adapt) return;
  const int j = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (j >= U.d) return;
  double* dj = bins + (size_t)j * nb1;
  double* r = scratch + (size_t)j * 2 * nb1;
  double* xin = r + nb1;
  __shared__ double dt[kMaxDim];
  if (lane == 0) {
    double xo = dj[1], xn = dj[2];
    dj[1] = (xo + xn) / 2.0;
    double t = dj[1];
    for (int i = 2; i < U.nd; ++i) {
      const double rcv = xo + xn;
      xo = xn;
      xn = dj[i + 1];
      dj[i] = (rcv + xn) / 3.0;
      t = t + dj[i];
    }
    dj[U.nd] = (xo + xn) / 2.0;
    dt[j] = t + dj[U.nd];
  }
  __syncwarp();
  const double dtj = dt[j];
  if (!(dtj > 0.0)) return;  // no contribution on this axis: the grid stays
  for (int i = 1 + lane; i <= U.nd; i += 32) r[i] = pow((1.0 - dj[i] / dtj) / (log(dtj) - log(dj[i])), U.alpha);
  __syncwarp();
  if (lane == 0) {
    double rsum = 0.0;
    for (int i = 1; i <= U.nd; ++i) rsum = rsum + r[i];
    rebin(rsum / U.xnd, U.nd, r, xin, xi + (size_t)j * nb1);
  }
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
  if (nd > 65535) {
    if (why) *why = "at most 65535 bins per axis";
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
  std::vector<double> xi((size_t)d * nb1, 0.0), r(nb1, 1.0), xin(nb1, 0.0);
  for (int j = 0; j < d; ++j) {
    xi[(size_t)j * nb1 + 1] = 1.0;
    rebin(1.0 / xnd, nd, r.data(), xin.data(), &xi[(size_t)j * nb1]);
  }
  const size_t nbt = (size_t)d * nb1;
  const size_t smem = mcubes_smem_bytes(d, nd);
  if (smem > kMcMaxSmem) {
    if (why) *why = "too many bins for this dimension";
    return PG_BAD_ARG;
  }
  int rc;
  if ((rc = E->ensure(st->xi, nbt * 8)) != PG_OK || (rc = E->ensure(st->bins, nbt * 8)) != PG_OK ||
      (rc = E->ensure(st->part_hist, (size_t)kMcBlocks * nbt * 8)) != PG_OK ||
      (rc = E->ensure(st->partial, kMcBlocks * 2 * 8)) != PG_OK ||
      (rc = E->ensure(st->scratch, 2 * nbt * 8)) != PG_OK || (rc = E->ensure(st->state, sizeof(McState))) != PG_OK) {
    if (why) *why = E->last_error;
    return rc;
  }
  cudaStream_t s = E->stream();
  auto fail = [&](cudaError_t e, const char* what) {
    if (why) *why = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PG_OOM : PG_CUDA_ERROR;
  };
  McState S0;
  std::memset(&S0, 0, sizeof S0);
  S0.status = 1;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(st->state.p, &S0, sizeof S0, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(st->xi.p, xi.data(), nbt * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return fail(e, "m-Cubes setup");
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
  A.part_hist = (double*)st->part_hist.p;
  A.partial = (double*)st->partial.p;
  A.state = (const McState*)st->state.p;
  McUpdate U;
  U.skip = opt.skip;
  U.d = d;
  U.nd = nd;
  U.epsrel = epsrel;
  U.epsabs = epsabs;
  U.dv2g = dv2g;
  U.xnd = xnd;
  U.alpha = opt.alpha;
  // Every iteration is enqueued at once: the adapting iterations
  // (vegasT.cuh:784-911), then the frozen-grid ones (vegasT.cuh:921-977);
  // the kernels of iterations after convergence return at once.
  for (int it = 1; it <= opt.titer; ++it) {
    const int adapt = it <= opt.itmax;
    A.iter = (uint32_t)it;
    A.adapt = adapt;
    pg_mcubes_args la;
    la.args = &A;
    la.smem = smem;
    la.stream = (void*)s;
    la.maxd = d;
    la.pad = 0;
    if ((e = launcher(la)) != cudaSuccess) return fail(e, "m-Cubes launch");
    E->stats.launches++;
    if (adapt) {
      mcubes_bins_kernel<<<(unsigned)((nbt + 255) / 256), 256, 0, s>>>((const double*)st->part_hist.p, (int)nbt,
                                                                      (double*)st->bins.p, A.state);
      E->stats.launches++;
    }
    U.it = it;
    U.adapt = adapt;
    mcubes_update_kernel<<<1, 32 * d, 0, s>>>(U, (const double*)st->partial.p, (double*)st->bins.p,
                                              (double*)st->xi.p, (double*)st->scratch.p, (McState*)st->state.p);
    E->stats.launches++;
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "m-Cubes launch");
  }
  McState S;
  if ((e = cudaMemcpyAsync(&S, st->state.p, sizeof S, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(e, "m-Cubes run");
  E->stats.points_evaluated += (uint64_t)calls * S.iters;
  pg_result R;
  std::memset(&R, 0, sizeof R);
  R.estimate = S.tgral;
  R.errorest = S.sd;
  R.chi_sq = S.chi2a;
  R.neval = (uint64_t)calls * S.iters;
  R.nregions = (uint64_t)ncubes;
  R.iters = S.iters;
  R.status = S.status;
  R.last_phase = -1;
  *out = R;
  return PG_OK;
}

}  // namespace pg
