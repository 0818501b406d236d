// m-Cubes sampling kernel (stratified VEGAS), shared by the library's
// integrand families and by the C++ layer's user integrands
// (include/pagani_gb300.cuh), which instantiate it in their own translation
// unit.  Restates the sampling of cuda_mcubes::vegas_kernel / vegas_kernelF
// (cuda/mcubes/vegasT.cuh:136-614):
//   * the same point map, weights and per-cube variance term;
//   * random numbers from Philox4x32-10 (Salmon et al., SC'11), keyed by the
//     seed with counter (cube, sample, axis pair, iteration);
//   * per-bin sums of f^2 accumulated in a fixed order, so a seed reproduces
//     a run bit for bit: the reference adds every sample to every axis's bin
//     with a global floating-point atomic (vegasT.cuh:304-307), whose order
//     varies from run to run.  Here each block samples in rounds, one sample
//     per thread; after a round warp w adds the round's samples to the bins
//     of axis w (and w + 8), 32 samples at a time: samples that fall into one
//     bin are summed by the lowest lane among them in lane order
//     (__match_any_sync), and that lane adds the sum to the block's
//     shared-memory histogram.  Blocks write their histograms to global
//     memory, and mcubes_bins_kernel sums them over the blocks in block order;
//   * a fixed grid of 1024 x 256 threads, each taking a contiguous run of
//     cubes, and block-tree sums, so the estimate does not depend on the SM count.
// Every floating-point operation is an explicit IEEE intrinsic.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pagani_gb300.h"
#include "pg_common.cuh"
#include "pg_integrands.cuh"

namespace pg {

constexpr int kMcThreads = 256;
constexpr int kMcBlocks = 1024;
constexpr double kTiny = 1.0e-30;  // vegas_utils.cuh:141

__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
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

// Exact conversions built from bit patterns on the integer pipe.  The
// sampling kernel is bound by GB300's FP64 pipe, which also executes the
// hardware's double<->integer conversions; these give the same values.

// v * 2^shift as a double, for 1 <= v <= 2^53 (exact: v has at most 53
// significant bits) and a result in the normal range.
__device__ __forceinline__ double exact_u53_scaled(uint64_t v, int shift) {
  const int lz = __clzll((long long)v);
  const uint64_t mant = ((v << lz) << 1) >> 12;  // the bits below the leading one
  return __longlong_as_double((long long)(((uint64_t)(1023 + 63 - lz + shift) << 52) | mant));
}

// max(min((int)x, nbins), 1) for a finite x (the bin of a sample), with the
// comparisons on the bit pattern and the integer part from the exponent and
// mantissa.
__device__ __forceinline__ int bin_index(double x, int nbins) {
  const long long bits = __double_as_longlong(x);
  if (bits < 0x3ff0000000000000ll) return 1;       // x < 1, negative x included
  if (bits >= 0x41e0000000000000ll) return nbins;  // x >= 2^31: (int)x saturates
  const int e = (int)(bits >> 52) - 1023;          // 0..30
  const int t = (int)(((((unsigned long long)bits << 12) >> 12) | (1ull << 52)) >> (52 - e));
  return max(min(t, nbins), 1);
}

// Uniform double in (0, 1] from 53 random bits: (m + 1) * 2^-53.
__host__ __device__ __forceinline__ double philox_unit(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
#ifdef __CUDA_ARCH__
  return exact_u53_scaled(m + 1, -53);
#else
  return (double)(m + 1) * 1.1102230246251565404236316680908203125e-16;  // 2^-53
#endif
}

// Device-side state of one m-Cubes run (the weighted mean over iterations,
// vegasT.cuh:834-852, and the stop flag of the iteration loop).
struct McState {
  double si, schi, swgt, tgral, sd, chi2a;
  int32_t status;  // 1 until the result meets the tolerance (GetStatus, vegas_utils.cuh:237-248)
  int32_t stop;    // nonzero: the loop has ended, later iterations' kernels return at once
  uint64_t iters;
};

struct McArgs {
  IntegralDesc desc;
  int d, ng, npg, nbins;
  uint64_t ncubes;
  double dxg, xnd, xjac;
  double regn[kMaxDim], dx[kMaxDim];
  uint32_t key0, key1, iter;
  int adapt;
  const double* xi;   // [d][nbins + 1], xi[j][0] = 0
  double* part_hist;  // [kMcBlocks][d * (nbins + 1)] per-block sums of f^2 per bin (adapt)
  double* partial;    // [kMcBlocks][2] per-block sums of f and of the per-cube variance terms
  const McState* state;
};

// Dynamic shared memory of mcubes_kernel: the grid, the block's histogram,
// and one round's f^2 and bins.
inline size_t mcubes_smem_bytes(int d, int nbins) {
  const size_t nb1 = (size_t)nbins + 1;
  return 2 * (size_t)d * nb1 * 8 + (size_t)kMcThreads * 8 + (size_t)d * kMcThreads * 2;
}

template <int MAXD, class Fn>
__global__ void __launch_bounds__(kMcThreads) mcubes_kernel(McArgs A, Fn fn) {
  if (A.state->stop) return;  // the run has converged
  extern __shared__ __align__(16) double mc_smem[];
  const int nb1 = A.nbins + 1;
  double* sxi = mc_smem;                   // d * nb1
  double* hist = sxi + A.d * nb1;          // d * nb1 (adapt)
  double* rf2 = hist + A.d * nb1;          // kMcThreads: this round's f^2
  uint16_t* rbin = reinterpret_cast<uint16_t*>(rf2 + kMcThreads);  // [d][kMcThreads]: bins (0: no sample)
  for (int i = threadIdx.x; i < A.d * nb1; i += blockDim.x) {
    sxi[i] = A.xi[i];
    hist[i] = 0.0;
  }
  __syncthreads();
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nthreads = (uint64_t)kMcBlocks * kMcThreads;
  const uint64_t per = (A.ncubes + nthreads - 1) / nthreads;
  const uint64_t c0 = tid * per, c1 = min(A.ncubes, c0 + per);
  const uint64_t mine = (c1 > c0 ? c1 - c0 : 0) * (uint64_t)A.npg;
  const uint64_t rounds = per * (uint64_t)A.npg;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double fbg = 0.0, f2bg = 0.0, fb = 0.0, f2b = 0.0;
  int kg[MAXD];
  for (uint64_t round = 0; round < rounds; ++round) {
    double f2 = 0.0;
    int ia[MAXD];
#pragma unroll
    for (int j = 0; j < MAXD; ++j) ia[j] = 0;
    if (round < mine) {
      const uint64_t cube = c0 + round / (uint64_t)A.npg;
      const int k = 1 + (int)(round % (uint64_t)A.npg);
      if (k == 1) {
        // kg: 1-based interval index per axis, axis 0 most significant (get_indx, vegasT.cuh:136-154)
        uint64_t q = cube;
#pragma unroll
        for (int j = MAXD - 1; j >= 0; --j) {
          if (j < A.d) {
            kg[j] = 1 + (int)(q % (uint64_t)A.ng);
            q /= (uint64_t)A.ng;
          }
        }
      }
      double wgt = A.xjac;
      double x[MAXD];
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
          const double xn = __fma_rn(__dsub_rn(exact_u53_scaled((uint64_t)kg[j], 0), ran), A.dxg, 1.0);
          const int b = bin_index(xn, A.nbins);
          const double* xij = sxi + j * nb1;
          double xo, rc;
          if (b > 1) {
            xo = __dsub_rn(xij[b], xij[b - 1]);
            rc = __fma_rn(__dsub_rn(xn, exact_u53_scaled((uint64_t)b, 0)), xo, xij[b - 1]);
          } else {
            xo = xij[b];
            rc = __dmul_rn(__dsub_rn(xn, 1.0), xo);
          }
          x[j] = __fma_rn(rc, A.dx[j], A.regn[j]);
          wgt = __dmul_rn(wgt, __dmul_rn(xo, A.xnd));
          ia[j] = b;
        }
      }
      const double f = __dmul_rn(wgt, fn.template eval<MAXD>(A.desc, x));
      f2 = __dmul_rn(f, f);
      fb = __dadd_rn(fb, f);
      f2b = __dadd_rn(f2b, f2);
      if (k == A.npg) {
        // per-cube variance term (vegasT.cuh:336-343)
        double v = sqrt(__dmul_rn(f2b, (double)A.npg));
        v = __dmul_rn(__dsub_rn(v, fb), __dadd_rn(v, fb));
        if (v <= 0.0) v = kTiny;
        fbg = __dadd_rn(fbg, fb);
        f2bg = __dadd_rn(f2bg, v);
        fb = f2b = 0.0;
      }
    }
    if (A.adapt) {
      rf2[threadIdx.x] = f2;
#pragma unroll
      for (int j = 0; j < MAXD; ++j)
        if (j < A.d) rbin[j * kMcThreads + threadIdx.x] = (uint16_t)ia[j];
      __syncthreads();
      for (int j = warp; j < A.d; j += kMcThreads / 32) {
        for (int i = 0; i < kMcThreads / 32; ++i) {
          const int t = i * 32 + lane;
          const int b = rbin[j * kMcThreads + t];
          const unsigned peers = __match_any_sync(0xffffffffu, b);
          if (b != 0 && lane == __ffs(peers) - 1) {
            double s = 0.0;
            for (unsigned m = peers; m; m &= m - 1) s = __dadd_rn(s, rf2[i * 32 + __ffs(m) - 1]);
            hist[j * nb1 + b] = __dadd_rn(hist[j * nb1 + b], s);
          }
          __syncwarp();
        }
      }
      __syncthreads();
    }
  }
  // Block sums: shuffle-down trees, then the 8 warp results in order.
  __shared__ double red[2][8];
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    fbg = __dadd_rn(fbg, __shfl_down_sync(0xffffffffu, fbg, off));
    f2bg = __dadd_rn(f2bg, __shfl_down_sync(0xffffffffu, f2bg, off));
  }
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
    double* out = A.part_hist + (size_t)blockIdx.x * (size_t)(A.d * nb1);
    for (int i = threadIdx.x; i < A.d * nb1; i += blockDim.x) out[i] = hist[i];
  }
}

// Shared memory the kernel may use.
constexpr size_t kMcMaxSmem = 200 * 1024;

// Host launch of one m-Cubes iteration for an integrand functor type Fn.
template <int MAXD, class Fn>
inline cudaError_t launch_mcubes(const pg_mcubes_args& a, const Fn& fn) {
  static std::atomic<unsigned long long> attr_done{0};
  const cudaError_t ae = ensure_dynamic_smem(mcubes_kernel<MAXD, Fn>, (int)kMcMaxSmem, attr_done);
  if (ae != cudaSuccess) return ae;
  mcubes_kernel<MAXD, Fn><<<kMcBlocks, kMcThreads, (size_t)a.smem, (cudaStream_t)a.stream>>>(
      *static_cast<const McArgs*>(a.args), fn);
  return cudaGetLastError();
}

}  // namespace pg
