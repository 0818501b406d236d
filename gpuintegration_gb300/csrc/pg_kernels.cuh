// Device kernels of the GB300 PAGANI iteration.
//
//   eval_kernel          region evaluation: degree-9 rule, 4 null rules, split
//                        axis (FP64-pipe bound)
//   two_level_kernel     two-level error, rel-err classification and per-chunk
//                        compensated partial sums (HBM bound)
//   finalize_kernel      per-integral merge of the chunk partials and exclusive
//                        scan of the per-chunk active counts
//   compact_split_kernel stream compaction of the active regions fused with the
//                        bisection into the next region list (HBM bound)
//   threshold_kernel     threshold statistics for the memory-pressure classifier
//
// Region lists are SoA: coordinate `dim` of region i sits at [dim * stride + i].
// Several integrals can share one list; integral j owns the contiguous segment
// [start_j, start_j + n_j).  Reductions are per segment, in a fixed order, so an
// integral's results do not depend on what else shares the list.
#pragma once

#include <stdint.h>

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

// Segment of one integral in the current region list.
struct SegDesc {
  uint64_t start;      // first region
  uint64_t n;          // regions
  uint64_t par_start;  // first parent estimate (n/2 of them) when has_parent
  uint32_t chunk_start;
  uint32_t nchunks;
  int32_t has_parent;
  int32_t relerr;
  double epsrel;
};

struct ChunkRef {
  uint32_t integral;  // index into the SegDesc / Transition arrays
  uint32_t local;     // chunk index inside that integral's segment
};

// Per-chunk partial sums: estimate, two-level error, active*estimate,
// active*error, and the active count.
struct Partial {
  NS q[4];
  uint64_t count;
};

struct IterScalars {
  double iter_est;   // sum of estimates
  double iter_err;   // sum of (two-level) errors
  double act_est;    // sum of active * estimate
  double act_err;    // sum of active * error
  uint64_t active;   // active regions
  uint64_t pad;
};

// Where an integral's kept regions go in the next list.
struct Transition {
  uint64_t out_start;  // first child
  uint64_t A;          // kept regions (children: 2A)
  uint64_t par_out;    // first parent estimate written for the next iteration
  int32_t mode;        // 0 drop, 1 keep the flagged regions, 2 keep every region
  int32_t pad;
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

template <int MAXD, class Fn>
static __global__ void __launch_bounds__(kEvalWarps * 32)
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

  for (uint64_t r = (uint64_t)blockIdx.x * kEvalWarps + warp; r < n; r += (uint64_t)gridDim.x * kEvalWarps) {
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
// Two-level error and classification (Phases.cuh:219-268) fused with the
// per-chunk compensated partial sums of the quantities the iteration needs
// (PaganiUtils.cuh:368-385, thrust_utils.cuh:16-47).
// ---------------------------------------------------------------------------
static __global__ void __launch_bounds__(kRedThreads)
    two_level_kernel(const ChunkRef* __restrict__ chunks, const SegDesc* __restrict__ segs,
                     const double* __restrict__ est, const double* __restrict__ err,
                     const double* __restrict__ parent_est, double* __restrict__ err_out,
                     uint8_t* __restrict__ active, Partial* __restrict__ partials) {
  __shared__ NS scratch[8];
  __shared__ unsigned long long cnt_s;
  const ChunkRef cr = chunks[blockIdx.x];
  const SegDesc S = segs[cr.integral];
  NS a0 = ns_zero(), a1 = ns_zero(), a2 = ns_zero(), a3 = ns_zero();
  uint32_t cnt = 0;
  if (threadIdx.x == 0) cnt_s = 0;
  const uint64_t half = S.n / 2;
#pragma unroll
  for (int k = 0; k < kRedItems; ++k) {
    const uint64_t li = (uint64_t)cr.local * kChunk + (uint64_t)k * kRedThreads + threadIdx.x;
    if (li < S.n) {
      const uint64_t i = S.start + li;
      const double selfRes = est[i];
      double selfErr = err[i];
      uint8_t act = 1;
      if (S.has_parent) {
        const bool right = 2 * li >= S.n;
        const uint64_t sib = right ? li - half : li + half;
        const uint64_t par = right ? li - half : li;
        const double siblErr = err[S.start + sib], siblRes = est[S.start + sib];
        const double parRes = parent_est[S.par_start + par];
        double diff = __dsub_rn(__dadd_rn(siblRes, selfRes), parRes);
        diff = fabs(__dmul_rn(.25, diff));
        const double e2 = __dadd_rn(selfErr, siblErr);
        if (e2 > 0.0) {
          const double c = __dadd_rn(1.0, __ddiv_rn(__dmul_rn(2.0, diff), e2));
          selfErr = __dmul_rn(selfErr, c);
        }
        selfErr = __dadd_rn(selfErr, diff);
        const bool pass = S.relerr && (selfErr < fmax(__dmul_rn(S.epsrel, fabs(selfRes)), 1e-200));
        act = pass ? 0 : 1;
      }
      err_out[i] = selfErr;
      active[i] = act;
      const double fa = act ? 1.0 : 0.0;
      a0 = ns_merge(a0, NS{selfRes, 0.0});
      a1 = ns_merge(a1, NS{selfErr, 0.0});
      a2 = ns_merge(a2, NS{__dmul_rn(fa, selfRes), 0.0});
      a3 = ns_merge(a3, NS{__dmul_rn(fa, selfErr), 0.0});
      cnt += act;
    }
  }
  a0 = ns_block_tree(a0, scratch);
  a1 = ns_block_tree(a1, scratch);
  a2 = ns_block_tree(a2, scratch);
  a3 = ns_block_tree(a3, scratch);
  atomicAdd(&cnt_s, (unsigned long long)cnt);
  __syncthreads();
  if (threadIdx.x == 0) {
    Partial& P = partials[blockIdx.x];
    P.q[0] = a0;
    P.q[1] = a1;
    P.q[2] = a2;
    P.q[3] = a3;
    P.count = cnt_s;
  }
}

// Exclusive scan of 256 per-thread values over the block; returns the
// thread's exclusive prefix, *total gets the block total.
__device__ __forceinline__ uint64_t block_exclusive_scan(uint64_t v, uint64_t* scratch, uint64_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t inc = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint64_t o = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc += o;
  }
  if (lane == 31) scratch[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint64_t wv = (lane < (int)(blockDim.x >> 5)) ? scratch[lane] : 0;
    uint64_t winc = wv;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint64_t o = __shfl_up_sync(0xffffffffu, winc, off);
      if (lane >= off) winc += o;
    }
    if (lane < (int)(blockDim.x >> 5)) scratch[lane] = winc - wv;
    if (lane == (int)(blockDim.x >> 5) - 1) scratch[32] = winc;
  }
  __syncthreads();
  const uint64_t res = scratch[warp] + inc - v;
  *total = scratch[32];
  __syncthreads();
  return res;
}

// One block per integral: merge the integral's chunk partials (lane t takes
// chunks t, t+256, ... then the block tree) and scan the chunk counts.
static __global__ void __launch_bounds__(kRedThreads)
    finalize_kernel(const uint32_t* __restrict__ live, const SegDesc* __restrict__ segs,
                    const Partial* __restrict__ partials, uint64_t* __restrict__ chunk_off,
                    IterScalars* __restrict__ out) {
  __shared__ NS scratch[8];
  __shared__ uint64_t sc[33];
  const uint32_t j = live ? live[blockIdx.x] : blockIdx.x;
  const SegDesc S = segs[j];
  NS a[4] = {ns_zero(), ns_zero(), ns_zero(), ns_zero()};
  for (uint32_t b = threadIdx.x; b < S.nchunks; b += kRedThreads) {
    const Partial& P = partials[S.chunk_start + b];
#pragma unroll
    for (int q = 0; q < 4; ++q) a[q] = ns_merge(a[q], P.q[q]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) a[q] = ns_block_tree(a[q], scratch);
  // Scan of the chunk counts: thread t owns a contiguous run of chunks.
  const uint32_t per = (S.nchunks + kRedThreads - 1) / kRedThreads;
  const uint32_t b0 = threadIdx.x * per, b1 = min(S.nchunks, b0 + per);
  uint64_t local = 0;
  for (uint32_t b = b0; b < b1; ++b) local += partials[S.chunk_start + b].count;
  uint64_t total;
  uint64_t run = block_exclusive_scan(local, sc, &total);
  for (uint32_t b = b0; b < b1; ++b) {
    chunk_off[S.chunk_start + b] = run;
    run += partials[S.chunk_start + b].count;
  }
  if (threadIdx.x == 0) {
    IterScalars o;
    o.iter_est = ns_value(a[0]);
    o.iter_err = ns_value(a[1]);
    o.act_est = ns_value(a[2]);
    o.act_err = ns_value(a[3]);
    o.active = total;
    o.pad = 0;
    out[j] = o;
  }
}

// ---------------------------------------------------------------------------
// Compaction of the kept regions (Sub_region_filter.cuh:8-47) fused with their
// bisection (Sub_region_splitter.cuh:8-46).  Kept region k of integral j gives
// child 0 at out_start + k and child 1 at out_start + A + k; the parent
// estimate goes to par_out + k for the next two-level step.
// ---------------------------------------------------------------------------
template <int MAXD>
static __global__ void __launch_bounds__(kRedThreads)
    compact_split_kernel(const ChunkRef* __restrict__ chunks, const SegDesc* __restrict__ segs,
                         const Transition* __restrict__ trans, const uint64_t* __restrict__ chunk_off,
                         const IntegralDesc* __restrict__ descs, const uint8_t* __restrict__ active,
                         const double* __restrict__ left, const double* __restrict__ length, uint64_t stride,
                         const int32_t* __restrict__ bisect, const double* __restrict__ est,
                         double* __restrict__ out_left, double* __restrict__ out_length, uint64_t out_stride,
                         uint32_t* __restrict__ out_owner, double* __restrict__ parent_out, uint32_t chunk0) {
  __shared__ uint64_t sc[33];
  const uint32_t cidx = chunk0 + blockIdx.x;
  const ChunkRef cr = chunks[cidx];
  const Transition T = trans[cr.integral];
  if (T.mode == 0) return;
  const SegDesc S = segs[cr.integral];
  const int d = descs[cr.integral].d;
  const uint64_t first = (uint64_t)cr.local * kChunk + (uint64_t)threadIdx.x * kRedItems;
  uint8_t keep[kRedItems];
  uint64_t cnt = 0;
#pragma unroll
  for (int q = 0; q < kRedItems; ++q) {
    const uint64_t li = first + q;
    keep[q] = (li < S.n) ? ((T.mode == 2) ? 1 : active[S.start + li]) : 0;
    cnt += keep[q];
  }
  uint64_t total;
  uint64_t pos = block_exclusive_scan(cnt, sc, &total);
  pos += (T.mode == 2) ? (uint64_t)cr.local * kChunk : chunk_off[cidx];
#pragma unroll
  for (int q = 0; q < kRedItems; ++q) {
    if (!keep[q]) continue;
    const uint64_t i = S.start + first + q;
    const uint64_t k = pos++;
    const uint64_t c0 = T.out_start + k, c1 = T.out_start + T.A + k;
    const int bd = bisect[i];
#pragma unroll
    for (int dim = 0; dim < MAXD; ++dim) {
      if (dim < d) {
        const double l = left[(uint64_t)dim * stride + i];
        const double h = length[(uint64_t)dim * stride + i];
        if (dim == bd) {
          const double hh = __ddiv_rn(h, 2.0);
          out_left[(uint64_t)dim * out_stride + c0] = __dadd_rn(l, __dmul_rn(0.0, hh));
          out_left[(uint64_t)dim * out_stride + c1] = __dadd_rn(l, __dmul_rn(1.0, hh));
          out_length[(uint64_t)dim * out_stride + c0] = hh;
          out_length[(uint64_t)dim * out_stride + c1] = hh;
        } else {
          out_left[(uint64_t)dim * out_stride + c0] = l;
          out_left[(uint64_t)dim * out_stride + c1] = l;
          out_length[(uint64_t)dim * out_stride + c0] = h;
          out_length[(uint64_t)dim * out_stride + c1] = h;
        }
      }
    }
    if (out_owner) {
      out_owner[c0] = cr.integral;
      out_owner[c1] = cr.integral;
    }
    parent_out[T.par_out + k] = est[i];
  }
}

// ---------------------------------------------------------------------------
// Memory-pressure classifier support (heuristic_classifier.cuh:60-87,283-325):
// per chunk of one integral, count(err > thr), sum(err * flag), sum(est * flag)
// and (optionally) the new flags.  Partial.q[0] = err*flag, q[1] = est*flag,
// q[2] = min(err) in .s, max(err) in .c (when `minmax`).
// ---------------------------------------------------------------------------
static __global__ void __launch_bounds__(kRedThreads)
    threshold_kernel(const ChunkRef* __restrict__ chunks, const SegDesc* __restrict__ segs, uint32_t chunk0,
                     const double* __restrict__ est, const double* __restrict__ err, double thr, int write_flags,
                     int minmax, uint8_t* __restrict__ active, Partial* __restrict__ partials) {
  __shared__ NS scratch[8];
  __shared__ unsigned long long cnt_s;
  __shared__ double mm[2][8];
  const ChunkRef cr = chunks[chunk0 + blockIdx.x];
  const SegDesc S = segs[cr.integral];
  NS a0 = ns_zero(), a1 = ns_zero();
  uint32_t cnt = 0;
  double mn = INFINITY, mx = -INFINITY;
  if (threadIdx.x == 0) cnt_s = 0;
#pragma unroll
  for (int k = 0; k < kRedItems; ++k) {
    const uint64_t li = (uint64_t)cr.local * kChunk + (uint64_t)k * kRedThreads + threadIdx.x;
    if (li < S.n) {
      const uint64_t i = S.start + li;
      const double e = err[i];
      const uint8_t f = e > thr ? 1 : 0;
      const double ff = f ? 1.0 : 0.0;
      if (write_flags) active[i] = f;
      a0 = ns_merge(a0, NS{__dmul_rn(e, ff), 0.0});
      a1 = ns_merge(a1, NS{__dmul_rn(est[i], ff), 0.0});
      cnt += f;
      if (minmax && !isnan(e)) {
        mn = fmin(mn, e);
        mx = fmax(mx, e);
      }
    }
  }
  a0 = ns_block_tree(a0, scratch);
  a1 = ns_block_tree(a1, scratch);
  atomicAdd(&cnt_s, (unsigned long long)cnt);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, off));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  }
  if (lane == 0) {
    mm[0][warp] = mn;
    mm[1][warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 0; w < 8; ++w) {
      mn = fmin(mn, mm[0][w]);
      mx = fmax(mx, mm[1][w]);
    }
    Partial& P = partials[chunk0 + blockIdx.x];
    P.q[0] = a0;
    P.q[1] = a1;
    P.q[2] = NS{mn, mx};
    P.q[3] = ns_zero();
    P.count = cnt_s;
  }
}

// Merge of threshold partials of one integral (same order as finalize_kernel)
// plus min/max; chunk offsets of the flags when requested.
static __global__ void __launch_bounds__(kRedThreads)
    threshold_finalize_kernel(const SegDesc* __restrict__ segs, uint32_t integral, const Partial* __restrict__ partials,
                              uint64_t* __restrict__ chunk_off, int scan, double* __restrict__ out) {
  __shared__ NS scratch[8];
  __shared__ uint64_t sc[33];
  __shared__ double mm[2][8];
  __shared__ unsigned long long cnt_s;
  const SegDesc S = segs[integral];
  NS a0 = ns_zero(), a1 = ns_zero();
  double mn = INFINITY, mx = -INFINITY;
  if (threadIdx.x == 0) cnt_s = 0;
  __syncthreads();
  uint64_t cnt = 0;
  for (uint32_t b = threadIdx.x; b < S.nchunks; b += kRedThreads) {
    const Partial& P = partials[S.chunk_start + b];
    a0 = ns_merge(a0, P.q[0]);
    a1 = ns_merge(a1, P.q[1]);
    mn = fmin(mn, P.q[2].s);
    mx = fmax(mx, P.q[2].c);
    cnt += P.count;
  }
  a0 = ns_block_tree(a0, scratch);
  a1 = ns_block_tree(a1, scratch);
  atomicAdd(&cnt_s, (unsigned long long)cnt);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, off));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  }
  if (lane == 0) {
    mm[0][warp] = mn;
    mm[1][warp] = mx;
  }
  __syncthreads();
  if (scan) {
    const uint32_t per = (S.nchunks + kRedThreads - 1) / kRedThreads;
    const uint32_t b0 = threadIdx.x * per, b1 = min(S.nchunks, b0 + per);
    uint64_t local = 0;
    for (uint32_t b = b0; b < b1; ++b) local += partials[S.chunk_start + b].count;
    uint64_t total;
    uint64_t run = block_exclusive_scan(local, sc, &total);
    for (uint32_t b = b0; b < b1; ++b) {
      chunk_off[S.chunk_start + b] = run;
      run += partials[S.chunk_start + b].count;
    }
  }
  if (threadIdx.x == 0) {
    for (int w = 0; w < 8; ++w) {
      mn = fmin(mn, mm[0][w]);
      mx = fmax(mx, mm[1][w]);
    }
    out[0] = ns_value(a0);
    out[1] = ns_value(a1);
    out[2] = (double)cnt_s;
    out[3] = mn;
    out[4] = mx;
  }
}

// Uniform initial split (Sub_regions.cuh:11-36): region r has coordinate
// (r / p^dim) mod p along `dim`, times 1/p; integral j's regions start at
// seg_start.
static __global__ void uniform_split_kernel(double* __restrict__ left, double* __restrict__ length, uint64_t stride,
                                     uint32_t* __restrict__ owner, uint64_t seg_start, uint64_t nregions, int d,
                                     int parts, uint32_t integral) {
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nregions) return;
  const double len = __ddiv_rn(1.0, (double)parts);
  uint64_t q = r;
  for (int k = 0; k < d; ++k) {
    const uint64_t id = q % (uint64_t)parts;
    q /= (uint64_t)parts;
    left[(uint64_t)k * stride + seg_start + r] = __dmul_rn((double)id, len);
    length[(uint64_t)k * stride + seg_start + r] = len;
  }
  owner[seg_start + r] = integral;
}

// Plain blocked compensated sum of one array (test entry point).
static __global__ void __launch_bounds__(kRedThreads) sum_chunks_kernel(const double* __restrict__ x, uint64_t n,
                                                               NS* __restrict__ part) {
  __shared__ NS scratch[8];
  NS a = ns_zero();
#pragma unroll
  for (int k = 0; k < kRedItems; ++k) {
    const uint64_t i = (uint64_t)blockIdx.x * kChunk + (uint64_t)k * kRedThreads + threadIdx.x;
    if (i < n) a = ns_merge(a, NS{x[i], 0.0});
  }
  a = ns_block_tree(a, scratch);
  if (threadIdx.x == 0) part[blockIdx.x] = a;
}

static __global__ void __launch_bounds__(kRedThreads) sum_final_kernel(const NS* __restrict__ part, uint64_t nparts,
                                                              double* __restrict__ out) {
  __shared__ NS scratch[8];
  NS a = ns_zero();
  for (uint64_t b = threadIdx.x; b < nparts; b += kRedThreads) a = ns_merge(a, part[b]);
  a = ns_block_tree(a, scratch);
  if (threadIdx.x == 0) *out = ns_value(a);
}

}  // namespace pg

namespace pg {

// Initial uniform split of newly admitted integrals (Sub_regions.cuh:11-36,
// partition rule Workspace.cuh:379-387).  Slot s covers regions
// [starts[s], starts[s+1]) of the list and belongs to integral ids[s].
static __global__ void uniform_split_batch_kernel(double* __restrict__ left, double* __restrict__ length,
                                                  uint64_t stride, uint32_t* __restrict__ owner,
                                                  const uint64_t* __restrict__ starts, const uint32_t* __restrict__ ids,
                                                  const IntegralDesc* __restrict__ descs, uint32_t nslots) {
  const uint64_t r = starts[0] + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= starts[nslots]) return;
  uint32_t lo = 0, hi = nslots;  // largest s with starts[s] <= r
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (starts[mid] <= r) lo = mid; else hi = mid;
  }
  const uint32_t j = ids[lo];
  const int d = descs[j].d;
  const int parts = d < 5 ? 4 : (d <= 10 ? 2 : 1);
  const double len = __ddiv_rn(1.0, (double)parts);
  uint64_t q = r - starts[lo];
  for (int k = 0; k < d; ++k) {
    const uint64_t id = q % (uint64_t)parts;
    q /= (uint64_t)parts;
    left[(uint64_t)k * stride + r] = __dmul_rn((double)id, len);
    length[(uint64_t)k * stride + r] = len;
  }
  owner[r] = j;
}

static __global__ void fill_owner_kernel(uint32_t* __restrict__ owner, uint64_t start, uint64_t n, uint32_t j) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) owner[start + i] = j;
}

}  // namespace pg
