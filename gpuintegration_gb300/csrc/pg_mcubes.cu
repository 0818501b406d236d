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

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace pg {

constexpr int kMcThreads = 256;
constexpr int kMcBlocks = 1024;
constexpr double kTiny = 1.0e-30;  // vegas_utils.cuh:141

__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[1] = (uint32_t)p1;
    c[3] = (uint32_t)p0;
    c[0] = n0;
    c[2] = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// Uniform double in (0, 1] from 53 random bits.
__host__ __device__ inline double philox_unit(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)(m + 1) * 1.1102230246251565404236316680908203125e-16;  // 2^-53
}

struct McArgs {
  IntegralDesc desc;
  int d, ng, npg, nbins;
  uint64_t ncubes;
  double dxg, xnd, xjac;
  double regn[kMaxDim], dx[kMaxDim];
  uint32_t key0, key1, iter;
  int adapt;
  const double* xi;   // [d][nbins + 1], xi[j][0] = 0
  double* bins;       // [d][nbins + 1] sums of f^2 per bin (adapt)
  double* partial;    // [kMcBlocks][2]
};

template <int MAXD>
__global__ void __launch_bounds__(kMcThreads) mcubes_kernel(McArgs A) {
  extern __shared__ __align__(16) double mc_smem[];
  const int nb1 = A.nbins + 1;
  double* sxi = mc_smem;                 // d * nb1
  double* hist = mc_smem + A.d * nb1;    // d * nb1 (adapt)
  for (int i = threadIdx.x; i < A.d * nb1; i += blockDim.x) {
    sxi[i] = A.xi[i];
    if (A.adapt) hist[i] = 0.0;
  }
  __syncthreads();
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nthreads = (uint64_t)kMcBlocks * kMcThreads;
  const uint64_t per = (A.ncubes + nthreads - 1) / nthreads;
  const uint64_t c0 = tid * per, c1 = min(A.ncubes, c0 + per);
  double fbg = 0.0, f2bg = 0.0;
  for (uint64_t cube = c0; cube < c1; ++cube) {
    // kg: 1-based interval index per axis, axis 0 most significant (get_indx, vegasT.cuh:136-154)
    int kg[MAXD];
    uint64_t q = cube;
#pragma unroll
    for (int j = MAXD - 1; j >= 0; --j) {
      if (j < A.d) {
        kg[j] = 1 + (int)(q % (uint64_t)A.ng);
        q /= (uint64_t)A.ng;
      }
    }
    double fb = 0.0, f2b = 0.0;
    for (int k = 1; k <= A.npg; ++k) {
      double wgt = A.xjac;
      double x[MAXD];
      int ia[MAXD];
      uint32_t rnd[4] = {0, 0, 0, 0};
#pragma unroll
      for (int j = 0; j < MAXD; ++j) {
        if (j < A.d) {
          if ((j & 1) == 0) {
            rnd[0] = (uint32_t)cube;
            rnd[1] = (uint32_t)k | ((uint32_t)(cube >> 32) << 16);
            rnd[2] = (uint32_t)(j >> 1);
            rnd[3] = A.iter;
            philox4x32_10(rnd, A.key0, A.key1);
          }
          const double ran = (j & 1) ? philox_unit(rnd[2], rnd[3]) : philox_unit(rnd[0], rnd[1]);
          // Setup_Integrand_Eval (vegasT.cuh:173-212)
          const double xn = __fma_rn(__dsub_rn((double)kg[j], ran), A.dxg, 1.0);
          const int b = max(min((int)xn, A.nbins), 1);
          const double* xij = sxi + j * nb1;
          double xo, rc;
          if (b > 1) {
            xo = __dsub_rn(xij[b], xij[b - 1]);
            rc = __fma_rn(__dsub_rn(xn, (double)b), xo, xij[b - 1]);
          } else {
            xo = xij[b];
            rc = __dmul_rn(__dsub_rn(xn, (double)b), xo);
          }
          x[j] = __fma_rn(rc, A.dx[j], A.regn[j]);
          wgt = __dmul_rn(wgt, __dmul_rn(xo, A.xnd));
          ia[j] = b;
        }
      }
      const double f = __dmul_rn(wgt, family_eval<MAXD>(A.desc, x));
      const double f2 = __dmul_rn(f, f);
      fb = __dadd_rn(fb, f);
      f2b = __dadd_rn(f2b, f2);
      if (A.adapt) {
#pragma unroll
        for (int j = 0; j < MAXD; ++j)
          if (j < A.d) atomicAdd(&hist[j * nb1 + ia[j]], f2);
      }
    }
    // per-cube variance term (vegasT.cuh:336-343)
    f2b = sqrt(__dmul_rn(f2b, (double)A.npg));
    f2b = __dmul_rn(__dsub_rn(f2b, fb), __dadd_rn(f2b, fb));
    if (f2b <= 0.0) f2b = kTiny;
    fbg = __dadd_rn(fbg, fb);
    f2bg = __dadd_rn(f2bg, f2b);
  }
  // Block sums: shuffle-down trees, then the 8 warp results in order.
  __shared__ double red[2][8];
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    fbg = __dadd_rn(fbg, __shfl_down_sync(0xffffffffu, fbg, off));
    f2bg = __dadd_rn(f2bg, __shfl_down_sync(0xffffffffu, f2bg, off));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = fbg;
    red[1][warp] = f2bg;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < kMcThreads / 32; ++w) {
      s0 = __dadd_rn(s0, red[0][w]);
      s1 = __dadd_rn(s1, red[1][w]);
    }
    A.partial[2 * blockIdx.x] = s0;
    A.partial[2 * blockIdx.x + 1] = s1;
  }
  if (A.adapt) {
    for (int i = threadIdx.x; i < A.d * nb1; i += blockDim.x) {
      const double v = hist[i];
      if (v != 0.0) atomicAdd(&A.bins[i], v);
    }
  }
}

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

int mcubes_run(McubesState* st, const IntegralDesc& D, double epsrel, double epsabs, const pg_mcubes_options& opt,
               pg_result* out, std::string* why) {
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
  static bool attr8 = false, attr16 = false;
  cudaError_t ce;
  if (d <= 8 && !attr8) {
    if ((ce = cudaFuncSetAttribute(mcubes_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)) !=
        cudaSuccess)
      return fail(ce, "cudaFuncSetAttribute");
    attr8 = true;
  }
  if (d > 8 && !attr16) {
    if ((ce = cudaFuncSetAttribute(mcubes_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)) !=
        cudaSuccess)
      return fail(ce, "cudaFuncSetAttribute");
    attr16 = true;
  }
  if (smem > 200 * 1024) {
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
    if (d <= 8)
      mcubes_kernel<8><<<kMcBlocks, kMcThreads, smem, s>>>(A);
    else
      mcubes_kernel<16><<<kMcBlocks, kMcThreads, smem, s>>>(A);
    E->stats.launches++;
    E->stats.points_evaluated += (uint64_t)calls;
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "m-Cubes launch");
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
