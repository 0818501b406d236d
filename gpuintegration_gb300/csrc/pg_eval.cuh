// Region-evaluation kernel of the GB300 PAGANI iteration (FP64-pipe bound),
// shared by the library's integrand families and by the C++ layer's user
// integrands (include/pagani_gb300.cuh), which instantiate it in their own
// translation unit.  Every floating-point operation is an explicit IEEE
// intrinsic, so the results do not depend on the compiler's contraction
// setting (the library builds with --fmad=false, user code usually with the
// default --fmad=true).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pagani_gb300.h"
#include "pg_common.cuh"
#include "pg_integrands.cuh"

namespace pg {

// Rule tables for every ndim, in device memory; passed by value.
struct RuleDev {
  const uint64_t* code;             // packed points, concatenated over ndim
  const uint16_t* trie;             // prefix tries (pg_rule.h), concatenated over ndim <= kTrieMaxDim
  int32_t trie_off[kMaxNdim + 1];
  const double* w;                  // [(kMaxNdim + 1) * 45]
  const double* scale;
  const double* norm;
  int32_t code_off[kMaxNdim + 1];
  int32_t feval[kMaxNdim + 1];
  double A[kCodesPerDim];           // .5 + g for the 11 coordinate codes
  double B[kCodesPerDim];           // .5 - g
  double ratio;                     // (G1 / G0)^2 of the fourth difference (Sample.cuh:195-196)
};

// ---------------------------------------------------------------------------
// Region evaluation.  One warp per region; the 32 lanes stand in for the 64
// threads of the reference's block (Phases.cuh:365-404): lane l accumulates
// the points of virtual threads l and l+32 in two separate sets of sums, in
// ascending point order, with fused multiply-adds, and the sums are combined
// as the reference's block reduction does (Sample.cuh:49-83): a shuffle-down
// tree per 32-lane half, then (half0 + 0) + half1.  Each per-axis coordinate
// value a region can take (centre, +-G0..G4) is computed once per region.
// ---------------------------------------------------------------------------
// Trie buffers of the d <= 8 kernel: depth d-1 (at most feval(7) = 717 nodes)
// and depth d-2 (at most feval(6) = 453), alternating downwards.
constexpr int kTrieMaxDim = 8;
constexpr int kTrieBufA = 720, kTrieBufB = 456;

template <int MAXD>
struct EvalTrieSmem {
  double a[kTrieBufA];
  double b[kTrieBufB];
};
template <>
struct EvalTrieSmem<16> {};

template <int MAXD>
struct EvalWarpSmem {
  EvalTrieSmem<MAXD> trie;
  IntegralDesc desc;
  double tab[MAXD * kCodesPerDim];  // (tab and fac double as the reduction area of the d > 8 kernel)
  double fac[MAXD * kCodesPerDim];  // per-axis factors of separable integrands
  double fv[64];
  double lo[MAXD];
  double up[MAXD];
  double w[kNSets * kNRules];
  double scale[kNSets * kNRules];
  double norm[kNSets * kNRules];
};

template <int MAXD, int WARPS, class Fn>
static __global__ void __launch_bounds__(WARPS * 32)
    eval_kernel(const double* __restrict__ left, const double* __restrict__ length, uint64_t n, uint64_t stride,
                const uint32_t* __restrict__ owner, const IntegralDesc* __restrict__ descs, RuleDev rule, Fn fn,
                double* __restrict__ est, double* __restrict__ err, int32_t* __restrict__ bisect) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  EvalWarpSmem<MAXD>* all = reinterpret_cast<EvalWarpSmem<MAXD>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  EvalWarpSmem<MAXD>& S = all[warp];
  const unsigned full = 0xffffffffu;
  uint32_t cur = 0xffffffffu;
  int d = 0, feval = 0;
  const uint64_t* codes = nullptr;

  for (uint64_t r = (uint64_t)blockIdx.x * WARPS + warp; r < n; r += (uint64_t)gridDim.x * WARPS) {
    const uint32_t j = owner ? owner[r] : 0u;
    if (j != cur) {
      const double* src = reinterpret_cast<const double*>(&descs[j]);
      double* dst = reinterpret_cast<double*>(&S.desc);
      for (int q = lane; q < (int)(sizeof(IntegralDesc) / 8); q += 32) dst[q] = src[q];
      __syncwarp();
      d = S.desc.d;
      feval = rule.feval[d];
      codes = rule.code + rule.code_off[d];
      for (int q = lane; q < kNSets * kNRules; q += 32) {
        S.w[q] = rule.w[d * 45 + q];
        S.scale[q] = rule.scale[d * 45 + q];
        S.norm[q] = rule.norm[d * 45 + q];
      }
      cur = j;
      __syncwarp();
    }
    // Region bounds in unit-cube coordinates (Phases.cuh:329-336).
    if (lane < d) {
      const double lo = left[(uint64_t)lane * stride + r];
      S.lo[lane] = lo;
      S.up[lane] = __dadd_rn(lo, length[(uint64_t)lane * stride + r]);
    }
    __syncwarp();
    // Coordinate of every (axis, code): lo + ((.5+g)*lower + (.5-g)*upper)*range
    // (Sample.cuh:126-131), with the reference's contraction of the inner sum.
    for (int v = lane; v < d * kCodesPerDim; v += 32) {
      const int k = v / kCodesPerDim, c = v - k * kCodesPerDim;
      const double t = __fma_rn(rule.A[c], S.lo[k], __dmul_rn(rule.B[c], S.up[k]));
      S.tab[v] = S.desc.unit ? t : __fma_rn(t, S.desc.range[k], S.desc.glo[k]);
    }
    const bool sep = fn.separable(S.desc);
    if (sep)
      for (int v = lane; v < d * kCodesPerDim; v += 32) S.fac[v] = fn.factor(S.desc, v / kCodesPerDim, S.tab[v]);
    __syncwarp();
    // Product-form integrands with d <= 8: inner trie depths 2..d-1 (depth k
    // goes to buffer a when d-1-k is even, else b; depth 1 is the axis-0
    // factor row).  Depth d is formed point by point below.
    const double* leaf_src = S.fac;
    const uint16_t* leaf_tab = nullptr;
    if constexpr (MAXD <= kTrieMaxDim) {
      if (sep) {
        const uint16_t* tt = rule.trie + rule.trie_off[d];
        int off = 0;
        for (int k = 2; k <= d - 1; ++k) {
          const int m = rule.feval[k];
          const double* src = (k - 1 == 1) ? S.fac : (((d - 1 - (k - 1)) & 1) ? S.trie.b : S.trie.a);
          double* dst = ((d - 1 - k) & 1) ? S.trie.b : S.trie.a;
          const double* fk = S.fac + (k - 1) * kCodesPerDim;
          for (int i = lane; i < m; i += 32) {
            const uint32_t e = __ldg(&tt[off + i]);
            dst[i] = __dmul_rn(src[e & 0xfffu], fk[e >> 12]);
          }
          off += m;
          __syncwarp();
        }
        leaf_src = (d == 2) ? S.fac : S.trie.a;
        leaf_tab = tt + off;
      }
    }
    const double* leaf_fac = S.fac + (d - 1) * kCodesPerDim;
    const double jac = S.desc.jac;
    const bool scale = jac != 1.0;
    double sa0 = 0, sa1 = 0, sa2 = 0, sa3 = 0, sa4 = 0;
    double sb0 = 0, sb1 = 0, sb2 = 0, sb3 = 0, sb4 = 0;
    for (int base = 0; base < feval; base += 64) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int p = base + half * 32 + lane;
        if (p < feval) {
          const uint64_t code = __ldg(&codes[p]);
          double f;
          if (sep && leaf_tab) {
            const uint32_t e = __ldg(&leaf_tab[p]);
            f = __dmul_rn(leaf_src[e & 0xfffu], leaf_fac[e >> 12]);
          } else if (sep) {
            f = S.fac[(int)(code & 15u)];
#pragma unroll
            for (int k = 1; k < MAXD; ++k)
              if (k < d) f = __dmul_rn(f, S.fac[k * kCodesPerDim + (int)((code >> (4 * k)) & 15u)]);
          } else {
            double x[MAXD];
#pragma unroll
            for (int k = 0; k < MAXD; ++k)
              x[k] = (k < d) ? S.tab[k * kCodesPerDim + (int)((code >> (4 * k)) & 15u)] : 0.0;
            f = fn.template eval<MAXD>(S.desc, x);
          }
          if (scale) f = __dmul_rn(f, jac);
          if (base == 0) S.fv[p] = f;
          const double* w = &S.w[(int)(code >> 60) * kNRules];
          if (half == 0) {
            sa0 = __fma_rn(f, w[0], sa0);
            sa1 = __fma_rn(f, w[1], sa1);
            sa2 = __fma_rn(f, w[2], sa2);
            sa3 = __fma_rn(f, w[3], sa3);
            sa4 = __fma_rn(f, w[4], sa4);
          } else {
            sb0 = __fma_rn(f, w[0], sb0);
            sb1 = __fma_rn(f, w[1], sb1);
            sb2 = __fma_rn(f, w[2], sb2);
            sb3 = __fma_rn(f, w[3], sb3);
            sb4 = __fma_rn(f, w[4], sb4);
          }
        }
      }
    }
    // The reference's block sum (Sample.cuh:49-83) per rule: a shuffle-down
    // tree over each 32-lane half (offsets 16, 8, 4, 2, 1), then
    // (half0 + 0) + half1.  The same additions in the same pairs are done here
    // level by level on shared memory, packing the 10 trees' additions of a
    // level into as few warp instructions as possible.
    double* red;  // free by now: the trie buffer (d <= 8 kernel) or tab + fac (352 doubles)
    if constexpr (MAXD <= kTrieMaxDim)
      red = S.trie.a;
    else
      red = S.tab;
    __syncwarp();
    red[0 * 32 + lane] = sa0;
    red[1 * 32 + lane] = sa1;
    red[2 * 32 + lane] = sa2;
    red[3 * 32 + lane] = sa3;
    red[4 * 32 + lane] = sa4;
    red[5 * 32 + lane] = sb0;
    red[6 * 32 + lane] = sb1;
    red[7 * 32 + lane] = sb2;
    red[8 * 32 + lane] = sb3;
    red[9 * 32 + lane] = sb4;
    __syncwarp();
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      for (int t = lane; t < 10 * off; t += 32) {
        const int q = t / off, i = t - q * off;
        red[q * 32 + i] = __dadd_rn(red[q * 32 + i], red[q * 32 + i + off]);
      }
      __syncwarp();
    }
    if (lane < 5) red[320 + lane] = __dadd_rn(__dadd_rn(red[lane * 32], 0.0), red[(5 + lane) * 32]);
    __syncwarp();
    const double s0 = red[320], s1 = red[321], s2 = red[322], s3 = red[323], s4 = red[324];
    __syncwarp();

    // base + ratio*(fp+fm) - (fp2+fm2): the reference's compiled code fuses
    // the multiply of base (2*f0*(1-ratio)) for d <= 4 and the multiply
    // ratio*(fp+fm) for d >= 5 (pinned against the reference kernel's output).
    double key = -1.0;
    if (lane < d) {
      const double f02 = __dmul_rn(S.fv[0], 2.0), omr = __dsub_rn(1.0, rule.ratio);
      const double fp = S.fv[1 + 2 * lane], fm = S.fv[2 + 2 * lane];
      const double fp2 = S.fv[1 + 2 * lane + 2 * d], fm2 = S.fv[2 + 2 * lane + 2 * d];
      const double X = __dadd_rn(fp, fm);
      const double s = (d <= 4) ? __fma_rn(f02, omr, __dmul_rn(rule.ratio, X))
                                : __fma_rn(rule.ratio, X, __dmul_rn(f02, omr));
      const double fd = fabs(__dsub_rn(s, __dadd_rn(fp2, fm2)));
      if (fd > 0.0) key = fd;
    }
    double kmax = key;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) kmax = fmax(kmax, __shfl_xor_sync(full, kmax, off));
    int cand = (kmax > 0.0 && key == kmax) ? lane : 64;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) cand = min(cand, __shfl_xor_sync(full, cand, off));

    // Null-rule error (Sample.cuh:261-289): lanes 0..26 evaluate the 27
    // (rule, set) terms, lanes 0..2 take the maximum per rule.
    double term = 0.0;
    if (lane < 27) {
      const int q = 1 + lane / 9, s = lane - (q - 1) * 9;
      const double sq = (q == 1) ? s1 : (q == 2) ? s2 : s3;
      const double sq1 = (q == 1) ? s2 : (q == 2) ? s3 : s4;
      term = __dmul_rn(fabs(__fma_rn(S.scale[s * kNRules + q], sq, sq1)), S.norm[s * kNRules + q]);
    }
    double m = 0.0;
#pragma unroll
    for (int s = 0; s < 9; ++s) {
      const double o = __shfl_sync(full, term, (lane < 3 ? lane : 0) * 9 + s);
      m = fmax(m, o);
    }
    const double e1 = __shfl_sync(full, m, 0), e2 = __shfl_sync(full, m, 1), e3 = __shfl_sync(full, m, 2);
    // Region volume and widest axis (Phases.cuh:329-348): the side lengths in
    // parallel, the product in axis order (1.0 * r0 = r0), and the widest-axis
    // comparison on the bit patterns (side lengths are non-negative).
    if (lane < d) S.up[lane] = __dsub_rn(S.up[lane], S.lo[lane]);
    __syncwarp();
    if (lane == 0) {
      double vol = S.up[0];
      long long maxbits = __double_as_longlong(vol);
      int maxdim = 0;
      for (int k = 1; k < d; ++k) {
        const double rk = S.up[k];
        vol = __dmul_rn(vol, rk);
        const long long b = __double_as_longlong(rk);
        if (b > maxbits) {
          maxdim = k;
          maxbits = b;
        }
      }
      est[r] = __dmul_rn(vol, s0);
      const bool ladder = (__dmul_rn(5.0, e1) <= e2) && (__dmul_rn(5.0, e2) <= e3);
      err[r] = __dmul_rn(vol, ladder ? e1 : __dmul_rn(5.0, fmax(fmax(e1, e2), e3)));
      bisect[r] = (cand < 64) ? cand : maxdim;
    }
    __syncwarp();
  }
}


// ---------------------------------------------------------------------------
// Host launch of the evaluation kernel for an integrand functor type Fn: a
// grid-stride loop over the regions, at most ctas_per_sm blocks per SM.
// ---------------------------------------------------------------------------
template <int MAXD, int WARPS, class Fn>
inline cudaError_t launch_eval_shape(const pg_eval_args& a, const Fn& fn) {
  const size_t smem = sizeof(EvalWarpSmem<MAXD>) * WARPS;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(eval_kernel<MAXD, WARPS, Fn>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const uint64_t want = (a.n + WARPS - 1) / WARPS;
  const uint64_t cap = (uint64_t)(a.num_sms > 0 ? a.num_sms : 1) * (uint64_t)(a.ctas_per_sm > 0 ? a.ctas_per_sm : 32);
  const uint64_t g = want < cap ? want : cap;
  const unsigned grid = (unsigned)(g > 0 ? g : 1);
  eval_kernel<MAXD, WARPS, Fn><<<grid, WARPS * 32, smem, (cudaStream_t)a.stream>>>(
      a.left, a.length, a.n, a.stride, a.owner, static_cast<const IntegralDesc*>(a.descs),
      *static_cast<const RuleDev*>(a.rule), fn, a.est, a.err, a.bisect);
  return cudaGetLastError();
}

// Dispatch on the autotuned regions per block (4 or 8 warps).
template <int MAXD, class Fn>
inline cudaError_t launch_eval(const pg_eval_args& a, const Fn& fn) {
  return a.warps == 4 ? launch_eval_shape<MAXD, 4>(a, fn) : launch_eval_shape<MAXD, 8>(a, fn);
}

}  // namespace pg
