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
  const uint16_t* trie;             // inner entries of the half tries (split_trie in pg_rule.h),
  int32_t trie_off[kMaxNdim + 1];   // concatenated over ndim
  // Per point of every rule: left node | right node << 12 | generator set << 24.
  const uint32_t* leafset;
  int32_t leafset_off[kMaxNdim + 1];
  const double* w;                  // [(kMaxNdim + 1) * 45]
  const double* scale;
  const double* norm;
  int32_t code_off[kMaxNdim + 1];
  int32_t feval[kMaxNdim + 1];
  double A[kCodesPerDim];           // .5 + g for the 11 coordinate codes
  double B[kCodesPerDim];           // .5 - g
  double ratio;                     // (G1 / G0)^2 of the fourth difference (Sample.cuh:195-196)
  double omr;                       // 1 - ratio
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
// Half-trie buffers: per half, the nodes of even depths (2, 4, 6) share one
// buffer and those of odd depths (3, 5) the other.  A half has at most 4 axes
// in the d <= 8 kernel (depth-4 nodes: feval(4) = 153, depth 3: 77) and at
// most 6 in the d <= 12 kernel (feval(6) = 453, feval(5) = 273).  The area
// also holds the reduction trees (325 doubles).
constexpr int kWStride = 6;  // padded row of the 5 rule weights of a generator set

template <int MAXD>
struct HalfTrie {
  static constexpr int even = MAXD <= 8 ? 160 : 456;
  static constexpr int odd = MAXD <= 8 ? 80 : 280;
  static constexpr int total = 2 * (even + odd);
};

template <int MAXD>
struct EvalTrieSmem {
  double a[HalfTrie<MAXD>::total];  // left even | left odd | right even | right odd
};

template <int MAXD>
struct EvalWarpSmem {
  EvalTrieSmem<MAXD> trie;
  IntegralDesc desc;
  double tab[MAXD * kCodesPerDim];
  double fac[MAXD * kCodesPerDim];  // per-axis factors of separable integrands
  double fv[64];
  double lo[MAXD];
  double up[MAXD];
  alignas(16) double w[kNSets * kWStride];  // weights of set s at [s * kWStride, +5), 16-byte aligned rows
  double scale[kNSets * kNRules];
  double norm[kNSets * kNRules];
};

// Rule sums of one region: virtual thread l (lane l) in a*, virtual thread
// l + 32 in b*, rules 0..4.
struct RuleSums {
  double a0, a1, a2, a3, a4, b0, b1, b2, b3, b4;
};

// How a point's value is formed: from the half tries of per-axis factors
// (product-form integrands: one multiply L * R), or by evaluating the
// integrand on the point's coordinates.
constexpr int kPointsTrie = 0, kPointsEval = 2;

// The per-point loop of eval_kernel: lane l takes points l, l+64, ... into a*
// and l+32, l+96, ... into b*, in ascending order, with fused multiply-adds,
// as the reference's threads l and l+32 do (Sample.cuh:221-259).  f is
// multiplied by the box's Jacobian when SCALE (Sample.cuh:236).  The first 64
// values are kept in S.fv for the fourth differences.
template <int MAXD, int MODE, bool SCALE, class Fn>
__device__ __forceinline__ void point_sums(RuleSums& rs, EvalWarpSmem<MAXD>& S, const Fn& fn,
                                           const uint64_t* __restrict__ codes, int feval, int d, int lane,
                                           const uint32_t* __restrict__ leafset, const double* leaf_l,
                                           const double* leaf_r, double jac) {
  for (int base = 0; base < feval; base += 64) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int p = base + half * 32 + lane;
      if (p < feval) {
        double f;
        int set;
        if constexpr (MODE == kPointsTrie) {
          const uint32_t e = __ldg(&leafset[p]);
          f = mul_rn_int(leaf_l[e & 0xfffu], leaf_r[(e >> 12) & 0xfffu]);
          set = (int)(e >> 24);
        } else {
          const uint64_t code = __ldg(&codes[p]);
          set = (int)(code >> 60);
          double x[MAXD];
#pragma unroll
          for (int k = 0; k < MAXD; ++k)
            x[k] = (k < d) ? S.tab[k * kCodesPerDim + (int)((code >> (4 * k)) & 15u)] : 0.0;
          f = fn.template eval<MAXD>(S.desc, x);
        }
        if constexpr (SCALE) f = mul_rn_int(f, jac);
        if (base == 0) S.fv[p] = f;
        const double* wr = &S.w[set * kWStride];
        const double2 w01 = *reinterpret_cast<const double2*>(wr);
        const double2 w23 = *reinterpret_cast<const double2*>(wr + 2);
        const double w4 = wr[4];
        if (half == 0) {
          rs.a0 = __fma_rn(f, w01.x, rs.a0);
          rs.a1 = __fma_rn(f, w01.y, rs.a1);
          rs.a2 = __fma_rn(f, w23.x, rs.a2);
          rs.a3 = __fma_rn(f, w23.y, rs.a3);
          rs.a4 = __fma_rn(f, w4, rs.a4);
        } else {
          rs.b0 = __fma_rn(f, w01.x, rs.b0);
          rs.b1 = __fma_rn(f, w01.y, rs.b1);
          rs.b2 = __fma_rn(f, w23.x, rs.b2);
          rs.b3 = __fma_rn(f, w23.y, rs.b3);
          rs.b4 = __fma_rn(f, w4, rs.b4);
        }
      }
    }
  }
}

template <int MAXD, int WARPS, class Fn>
static __global__ void __launch_bounds__(WARPS * 32, 16 / WARPS)
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
        S.w[(q / kNRules) * kWStride + q % kNRules] = rule.w[d * 45 + q];
        S.scale[q] = rule.scale[d * 45 + q];
        S.norm[q] = rule.norm[d * 45 + q];
      }
      if (lane < kNSets) S.w[lane * kWStride + kNRules] = 0.0;
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
    // Product-form integrands: the half products L (axes 0..m-1) and R (axes
    // m..d-1), depth by depth, both halves' nodes of a depth in the same warp
    // instructions (depth 1 is the factor row of the half's first axis).  Each
    // point then takes one multiply, L * R.
    const double* leaf_l = S.fac;
    const double* leaf_r = S.fac;
    const uint32_t* leafset = nullptr;
    {
      if (sep) {
        constexpr int ev = HalfTrie<MAXD>::even, od = HalfTrie<MAXD>::odd;
        const uint16_t* tt = rule.trie + rule.trie_off[d];
        const int m = d / 2, mr = d - m;
        // depth k of the left half at trie.a + (k odd ? ev : 0), of the right
        // half at trie.a + ev + od + (k odd ? ev : 0)
        double* const ta = S.trie.a;
        int off = 0;
        for (int k = 2; k <= mr; ++k) {  // mr >= m
          const int nl = (k <= m) ? rule.feval[k] : 0, nr = rule.feval[k];
          const int cur = (k & 1) ? ev : 0, prev = (k & 1) ? 0 : ev;
          const double* srcl = (k == 2) ? S.fac : ta + prev;
          const double* srcr = (k == 2) ? S.fac + m * kCodesPerDim : ta + ev + od + prev;
          const double* fl = S.fac + (k - 1) * kCodesPerDim;
          const double* fr = S.fac + (m + k - 1) * kCodesPerDim;
          for (int i = lane; i < nl + nr; i += 32) {
            const uint32_t e = __ldg(&tt[off + i]);
            const bool left = i < nl;
            const double* src = left ? srcl : srcr;
            const double* fk = left ? fl : fr;
            double* dst = left ? ta + cur + i : ta + ev + od + cur + (i - nl);
            *dst = mul_rn_int(src[e & 0xfffu], fk[e >> 12]);
          }
          off += nl + nr;
          __syncwarp();
        }
        leaf_l = (m == 1) ? S.fac : ta + ((m & 1) ? ev : 0);
        leaf_r = (mr == 1) ? S.fac + m * kCodesPerDim : ta + ev + od + ((mr & 1) ? ev : 0);
        leafset = rule.leafset + rule.leafset_off[d];
      }
    }
    // The per-point loop, specialised on how f is formed and on whether the
    // box's Jacobian differs from 1 (both uniform over the region), so no
    // per-point instruction is spent on either decision.
    const double jac = S.desc.jac;
    RuleSums rs{0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int mode = (sep && leafset) ? kPointsTrie : kPointsEval;
    if (jac != 1.0) {
      if (mode == kPointsTrie)
        point_sums<MAXD, kPointsTrie, true>(rs, S, fn, codes, feval, d, lane, leafset, leaf_l, leaf_r, jac);
      else
        point_sums<MAXD, kPointsEval, true>(rs, S, fn, codes, feval, d, lane, leafset, leaf_l, leaf_r, jac);
    } else {
      if (mode == kPointsTrie)
        point_sums<MAXD, kPointsTrie, false>(rs, S, fn, codes, feval, d, lane, leafset, leaf_l, leaf_r, jac);
      else
        point_sums<MAXD, kPointsEval, false>(rs, S, fn, codes, feval, d, lane, leafset, leaf_l, leaf_r, jac);
    }
    // The reference's block sum (Sample.cuh:49-83) per rule: a shuffle-down
    // tree over each 32-lane half (offsets 16, 8, 4, 2, 1), then
    // (half0 + 0) + half1.  The same additions in the same pairs are done here
    // level by level on shared memory, packing the 10 trees' additions of a
    // level into as few warp instructions as possible.
    double* red = S.trie.a;  // free by now (at least 480 doubles; 325 used)
    __syncwarp();
    red[0 * 32 + lane] = rs.a0;
    red[1 * 32 + lane] = rs.a1;
    red[2 * 32 + lane] = rs.a2;
    red[3 * 32 + lane] = rs.a3;
    red[4 * 32 + lane] = rs.a4;
    red[5 * 32 + lane] = rs.b0;
    red[6 * 32 + lane] = rs.b1;
    red[7 * 32 + lane] = rs.b2;
    red[8 * 32 + lane] = rs.b3;
    red[9 * 32 + lane] = rs.b4;
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

    // Fourth difference per axis k: base + ratio*(fp+fm) - (fp2+fm2) with
    // base = 2*f0*(1-ratio) (Sample.cuh:190-215).  The reference's compiled
    // code fuses the base multiply for d <= 4 and the ratio multiply for
    // d >= 5 (pinned against the reference kernel's output).  The three sums
    // share one warp addition: lanes 0..d-1 form fp+fm, lanes d..2d-1 form
    // fp2+fm2 of axis lane-d, lane 31 forms f0+f0 = 2*f0.
    //
    // The split-axis search and the null-rule maxima below are maxima of
    // non-negative doubles, taken on their bit patterns (for non-negative
    // doubles the integer order is the numeric order) so they stay off the
    // FP64 pipe.  A bit pattern of 0 means "no candidate".
    double ua = 0.0, ub = 0.0;
    if (lane < d) {
      ua = S.fv[1 + 2 * lane];
      ub = S.fv[2 + 2 * lane];
    } else if (lane < 2 * d) {
      ua = S.fv[1 + 2 * (lane - d) + 2 * d];
      ub = S.fv[2 + 2 * (lane - d) + 2 * d];
    } else if (lane == 31) {
      ua = ub = S.fv[0];
    }
    const double sums = __dadd_rn(ua, ub);
    const double fsec = __shfl_sync(full, sums, (lane + d) & 31);  // fp2 + fm2 of this lane's axis
    const double f02 = __shfl_sync(full, sums, 31);
    unsigned long long key = 0;
    if (lane < d) {
      const double X = sums;
      const double s = (d <= 4) ? __fma_rn(f02, rule.omr, __dmul_rn(rule.ratio, X))
                                : __fma_rn(rule.ratio, X, __dmul_rn(f02, rule.omr));
      const unsigned long long fd = (unsigned long long)__double_as_longlong(fabs(__dsub_rn(s, fsec)));
      if (fd != 0ull && fd <= 0x7ff0000000000000ull) key = fd;  // fd > 0 (a NaN is no candidate)
    }
    unsigned long long kmax = key;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      const unsigned long long o = __shfl_xor_sync(full, kmax, off);
      kmax = o > kmax ? o : kmax;
    }
    const unsigned cmask = __ballot_sync(full, kmax != 0ull && key == kmax);
    const int cand = cmask ? __ffs(cmask) - 1 : 64;

    // Null-rule error (Sample.cuh:261-289): lanes 0..26 evaluate the 27
    // (rule, set) terms, lanes 0..2 take the maximum per rule.
    // The terms are >= 0 (the null-rule norms are >= 0); a NaN term is
    // ignored, as the reference's max() does.
    unsigned long long term = 0;
    if (lane < 27) {
      const int q = 1 + lane / 9, s = lane - (q - 1) * 9;
      const double sq = (q == 1) ? s1 : (q == 2) ? s2 : s3;
      const double sq1 = (q == 1) ? s2 : (q == 2) ? s3 : s4;
      const unsigned long long b = (unsigned long long)__double_as_longlong(
          __dmul_rn(fabs(__fma_rn(S.scale[s * kNRules + q], sq, sq1)), S.norm[s * kNRules + q]));
      term = (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull ? 0ull : b;
    }
    unsigned long long m = 0;
#pragma unroll
    for (int s = 0; s < 9; ++s) {
      const unsigned long long o = __shfl_sync(full, term, (lane < 3 ? lane : 0) * 9 + s);
      m = o > m ? o : m;
    }
    const unsigned long long m1 = __shfl_sync(full, m, 0), m2 = __shfl_sync(full, m, 1), m3 = __shfl_sync(full, m, 2);
    const double e1 = __longlong_as_double((long long)m1), e2 = __longlong_as_double((long long)m2),
                 e3 = __longlong_as_double((long long)m3);
    unsigned long long mmax = m1 > m2 ? m1 : m2;
    mmax = m3 > mmax ? m3 : mmax;
    const double emax = __longlong_as_double((long long)mmax);

    // Side lengths, widest axis and volume (Phases.cuh:329-348).  The volume
    // is the product of the side lengths in axis order.  When every side is a
    // power of two no larger than 1 (regions made by uniform splits and
    // bisections in unit coordinates always are) and the product stays
    // normal, every partial product is exact and the volume is 2^(sum of
    // exponents), formed on the integer pipe; otherwise lane 0 multiplies in
    // order.  The widest axis is the first one whose length exceeds all
    // earlier ones, starting from 0 (a negative or NaN length never wins),
    // compared on bit patterns.
    unsigned long long sb = 0, sk = 0;
    int expo = 0;
    bool pow2 = true;
    if (lane < d) {
      const double side = __dsub_rn(S.up[lane], S.lo[lane]);
      S.up[lane] = side;
      sb = (unsigned long long)__double_as_longlong(side);
      const int e = (int)((sb >> 52) & 0x7ffull);
      pow2 = (sb & 0x800fffffffffffffull) == 0ull && e >= 1 && e <= 1023;
      expo = e - 1023;
      sk = ((sb >> 63) || (sb & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) ? 0ull : sb;
    }
    const unsigned hi_max = __reduce_max_sync(full, (unsigned)(sk >> 32));
    const unsigned lo_max = __reduce_max_sync(full, (unsigned)(sk >> 32) == hi_max ? (unsigned)sk : 0u);
    const unsigned wmask = __ballot_sync(full, lane < d && (unsigned)(sk >> 32) == hi_max && (unsigned)sk == lo_max);
    const int maxdim = __ffs(wmask) - 1;
    const bool all_pow2 = __all_sync(full, pow2);
    const int esum = __reduce_add_sync(full, expo);
    double vol;
    if (all_pow2 && esum >= -1022) {
      vol = __longlong_as_double((long long)(esum + 1023) << 52);
    } else {
      __syncwarp();
      double v = 0.0;
      if (lane == 0) {
        v = S.up[0];
        for (int k = 1; k < d; ++k) v = __dmul_rn(v, S.up[k]);
      }
      vol = __shfl_sync(full, v, 0);
    }
    // One multiply for vol*s0 (lane 0) and 5*e1, 5*e2, 5*max (lanes 1..3), one
    // compare for the error ladder 5*e1 <= e2, 5*e2 <= e3 (lanes 1, 2), one
    // multiply for the error (Sample.cuh:284-289).
    const double pa = (lane == 0) ? vol : 5.0;
    const double pb = (lane == 0) ? s0 : (lane == 1) ? e1 : (lane == 2) ? e2 : emax;
    const double prod = __dmul_rn(pa, pb);
    const bool le = prod <= ((lane == 1) ? e2 : e3);
    const unsigned lmask = __ballot_sync(full, le);
    const bool ladder = ((lmask >> 1) & 3u) == 3u;
    const double five_max = __shfl_sync(full, prod, 3);
    if (lane == 0) {
      est[r] = prod;
      err[r] = __dmul_rn(vol, ladder ? e1 : five_max);
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
  static std::atomic<unsigned long long> attr_done{0};
  const cudaError_t ae = ensure_dynamic_smem(eval_kernel<MAXD, WARPS, Fn>, (int)smem, attr_done);
  if (ae != cudaSuccess) return ae;
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
