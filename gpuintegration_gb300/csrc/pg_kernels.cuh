// Device kernels of the GB300 PAGANI iteration.
//
//   eval_kernel          (pg_eval.cuh) region evaluation: degree-9 rule, 4 null rules, split
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
#include "pg_eval.cuh"
#include "pg_integrands.cuh"

namespace pg {

// Per-axis values of a region that the set-sum evaluation keeps for its
// children: the factor at the centre, at +-G0 and +-G1, and the sums p2..p4.
constexpr int kTermValues = 8;

// Term buffers are tiled by 32 consecutive positions: value `row` of position
// `pos` sits at ((pos / 32) * rows + row) * 32 + pos % 32, so a warp's values
// share one block of rows * 256 bytes (a plain row-major layout puts each row
// a list's length apart, and a warp touching a hundred rows spreads over a
// hundred pages).
__host__ __device__ __forceinline__ uint64_t term_at(uint64_t pos, int row, int rows) {
  return ((pos >> 5) * (uint64_t)rows + (uint64_t)row) * 32ull + (pos & 31ull);
}

// Bounds checks of the term lookups: the first index found outside its
// buffer is recorded (rec[0] = check code, rec[1] = index, rec[2] = bound,
// rec[3..6] = integral, segment start, regions, list position) and the access
// is skipped; the host reads the record after each iteration and fails the
// run.
__device__ __forceinline__ bool in_bounds(unsigned long long* rec, int code, uint64_t i, uint64_t bound,
                                          uint64_t a = 0, uint64_t b = 0, uint64_t c = 0, uint64_t e = 0) {
  if (i < bound) return true;
  if (rec && atomicCAS(rec, 0ull, (unsigned long long)code) == 0ull) {
    rec[1] = i;
    rec[2] = bound;
    rec[3] = a;
    rec[4] = b;
    rec[5] = c;
    rec[6] = e;
  }
  return false;
}

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
  int32_t has_cache;  // the parents' per-axis terms are kept (set-sum evaluation of sibling pairs)
  int32_t pad;
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
  int32_t cache;       // 1: record the kept regions' positions for their children's term lookups
};

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
      a0 = ns_add(a0, selfRes);
      a1 = ns_add(a1, selfErr);
      a2 = ns_add(a2, __dmul_rn(fa, selfRes));
      a3 = ns_add(a3, __dmul_rn(fa, selfErr));
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
//
// A chunk of 2048 regions is taken as 8 slices of 256, one region per thread
// and slice, so a warp's loads of the SoA rows and its stores of the children
// are consecutive addresses.  The kept regions' order is the list order:
// slice by slice, and inside a slice by a warp ballot and the 8 warps' counts.
// ---------------------------------------------------------------------------
template <int MAXD>
static __global__ void __launch_bounds__(kRedThreads, 3)
    compact_split_kernel(const ChunkRef* __restrict__ chunks, const SegDesc* __restrict__ segs,
                         const Transition* __restrict__ trans, const uint64_t* __restrict__ chunk_off,
                         const IntegralDesc* __restrict__ descs, const uint8_t* __restrict__ active,
                         const double* __restrict__ left, const double* __restrict__ length, uint64_t stride,
                         const int32_t* __restrict__ bisect, const double* __restrict__ est,
                         double* __restrict__ out_left, double* __restrict__ out_length, uint64_t out_stride,
                         uint32_t* __restrict__ out_owner, double* __restrict__ parent_out, uint32_t chunk0,
                         uint32_t* __restrict__ ppos_out, uint64_t ppos_n, unsigned long long* __restrict__ chk) {
  __shared__ uint32_t wcount[kRedThreads / 32];
  const uint32_t cidx = chunk0 + blockIdx.x;
  const ChunkRef cr = chunks[cidx];
  const Transition T = trans[cr.integral];
  if (T.mode == 0) return;
  const SegDesc S = segs[cr.integral];
  const int d = descs[cr.integral].d;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t chunk_first = (uint64_t)cr.local * kChunk;
  // kept regions of this integral before the chunk
  uint64_t run = (T.mode == 2) ? chunk_first : chunk_off[cidx];
#pragma unroll 1
  for (int k = 0; k < kRedItems; ++k) {
    const uint64_t li = chunk_first + (uint64_t)k * kRedThreads + threadIdx.x;
    const bool keep = li < S.n && (T.mode == 2 || active[S.start + li]);
    const unsigned mask = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wcount[warp] = __popc(mask);
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kRedThreads / 32; ++w) {
      const uint32_t c = wcount[w];
      before += (w < warp) ? c : 0u;
      total += c;
    }
    if (keep) {
      const uint64_t pos = run + before + __popc(mask & ((1u << lane) - 1u));
      const uint64_t i = S.start + li;
      const uint64_t c0 = T.out_start + pos, c1 = T.out_start + T.A + pos;
      const int bd = bisect[i];
      // every load of the region before any store: 2d loads in flight per thread
      double l[MAXD], h[MAXD];
#pragma unroll
      for (int dim = 0; dim < MAXD; ++dim) {
        if (dim < d) {
          l[dim] = left[(uint64_t)dim * stride + i];
          h[dim] = length[(uint64_t)dim * stride + i];
        }
      }
      const double e = est[i];
#pragma unroll
      for (int dim = 0; dim < MAXD; ++dim) {
        if (dim < d) {
          if (dim == bd) {
            const double hh = __ddiv_rn(h[dim], 2.0);
            out_left[(uint64_t)dim * out_stride + c0] = __dadd_rn(l[dim], __dmul_rn(0.0, hh));
            out_left[(uint64_t)dim * out_stride + c1] = __dadd_rn(l[dim], __dmul_rn(1.0, hh));
            out_length[(uint64_t)dim * out_stride + c0] = hh;
            out_length[(uint64_t)dim * out_stride + c1] = hh;
          } else {
            out_left[(uint64_t)dim * out_stride + c0] = l[dim];
            out_left[(uint64_t)dim * out_stride + c1] = l[dim];
            out_length[(uint64_t)dim * out_stride + c0] = h[dim];
            out_length[(uint64_t)dim * out_stride + c1] = h[dim];
          }
        }
      }
      if (out_owner) {
        out_owner[c0] = cr.integral;
        out_owner[c1] = cr.integral;
      }
      parent_out[T.par_out + pos] = e;
      // where the children find the region's per-axis terms: its position
      // in this list's term buffer
      if (ppos_out && T.cache && in_bounds(chk, 4, T.par_out + pos, ppos_n)) ppos_out[T.par_out + pos] = (uint32_t)i;
    }
    run += total;
    __syncthreads();  // wcount is rewritten by the next slice
  }
}

// ---------------------------------------------------------------------------
// Memory-pressure classifier support (heuristic_classifier.cuh:60-87,283-325):
// per chunk of one integral, count(err > thr), sum(err * flag), sum(est * flag)
// and (optionally) the new flags.  Partial.q[0] = err*flag, q[1] = est*flag,
// q[2] = min(err) in .s, max(err) in .c (when `minmax`).  Without SUMS the
// compensated sums are left out (zero): the min/max pass and the pass that
// writes the final flags read only counts and extremes, and the sums cost
// ~10 FP64 operations per region on the scarce FP64 pipe.
// ---------------------------------------------------------------------------
template <bool SUMS>
static __global__ void __launch_bounds__(kRedThreads)
    threshold_kernel(const ChunkRef* __restrict__ chunks, const SegDesc* __restrict__ segs, uint32_t chunk0,
                     const double* __restrict__ est, const double* __restrict__ err, double thr_arg,
                     const double* __restrict__ thr_dev, int write_flags, int minmax, uint8_t* __restrict__ active,
                     Partial* __restrict__ partials) {
  const double thr = thr_dev ? *thr_dev : thr_arg;  // a threshold chosen on the device, else the argument
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
      if (SUMS) {
        a0 = ns_add(a0, __dmul_rn(e, ff));
        a1 = ns_add(a1, __dmul_rn(est[i], ff));
      }
      cnt += f;
      if (minmax && !isnan(e)) {
        mn = fmin(mn, e);
        mx = fmax(mx, e);
      }
    }
  }
  if (SUMS) {
    a0 = ns_block_tree(a0, scratch);
    a1 = ns_block_tree(a1, scratch);
  }
  atomicAdd(&cnt_s, (unsigned long long)cnt);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (minmax) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    if (lane == 0) {
      mm[0][warp] = mn;
      mm[1][warp] = mx;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (minmax)
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

// Counts of one integral's errors above each of up to kMaxThresholds
// thresholds (the memory-pressure classifier's stopping test needs only the
// count): integer totals, added with atomics, so the order does not matter.
// The thresholds are non-negative, so for a non-negative error the comparison
// is one on bit patterns; a NaN or negative-signed error exceeds none of them,
// as in threshold_kernel.
constexpr int kMaxThresholds = 20;
struct ThresholdSet {
  unsigned long long bits[kMaxThresholds];
  int k;
};

static __global__ void __launch_bounds__(kRedThreads)
    threshold_count_kernel(const ChunkRef* __restrict__ chunks, const SegDesc* __restrict__ segs, uint32_t chunk0,
                           const double* __restrict__ err, ThresholdSet ts_arg, const ThresholdSet* __restrict__ ts_dev,
                           unsigned long long* __restrict__ counts) {
  __shared__ unsigned long long sc[kMaxThresholds];
  __shared__ ThresholdSet ts_s;  // the set built on the device, else the argument
  if (threadIdx.x < kMaxThresholds) {
    sc[threadIdx.x] = 0ull;
    ts_s.bits[threadIdx.x] = ts_dev ? ts_dev->bits[threadIdx.x] : ts_arg.bits[threadIdx.x];
  }
  if (threadIdx.x == 0) ts_s.k = ts_dev ? ts_dev->k : ts_arg.k;
  __syncthreads();
  const ThresholdSet& ts = ts_s;
  const ChunkRef cr = chunks[chunk0 + blockIdx.x];
  const SegDesc S = segs[cr.integral];
  uint32_t c[kMaxThresholds];
#pragma unroll
  for (int q = 0; q < kMaxThresholds; ++q) c[q] = 0;
#pragma unroll
  for (int k = 0; k < kRedItems; ++k) {
    const uint64_t li = (uint64_t)cr.local * kChunk + (uint64_t)k * kRedThreads + threadIdx.x;
    if (li < S.n) {
      const unsigned long long e = (unsigned long long)__double_as_longlong(err[S.start + li]);
      if (e <= 0x7ff0000000000000ull) {  // not NaN, sign bit clear
#pragma unroll
        for (int q = 0; q < kMaxThresholds; ++q) c[q] += (q < ts.k && e > ts.bits[q]) ? 1u : 0u;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kMaxThresholds; ++q) {
    const unsigned v = __reduce_add_sync(0xffffffffu, c[q]);
    if ((threadIdx.x & 31) == 0 && q < ts.k && v) atomicAdd(&sc[q], (unsigned long long)v);
  }
  __syncthreads();
  if (threadIdx.x < ts.k && sc[threadIdx.x]) atomicAdd(&counts[threadIdx.x], sc[threadIdx.x]);
}

// The classifier's raise sequence t_0 = thr0, t_(q+1) = t_q + |max - t_q| / 2
// (heuristic_classifier.cuh:380-395), max being the largest error of a
// min/max pass (mm[4]), built on the device so the counting pass can follow
// the min/max pass without a host round trip.  The host forms the same
// sequence with the same operations.
static __global__ void threshold_seq_kernel(const double* __restrict__ mm, double thr0, ThresholdSet* __restrict__ ts,
                                            double* __restrict__ seq) {
  if (threadIdx.x != 0) return;
  const double high = mm[4];
  double t = thr0;
  for (int q = 0; q < kMaxThresholds; ++q) {
    seq[q] = t;
    ts->bits[q] = (unsigned long long)__double_as_longlong(__dadd_rn(t, 0.0));  // +0 for a -0 threshold
    t = __dadd_rn(t, __dmul_rn(fabs(__dsub_rn(high, t)), 0.5));
  }
  ts->k = kMaxThresholds;
}

// Where the raise loop stops: the first threshold of the sequence that leaves
// at most the share `pct` of the n regions active, else the last
// (heuristic_classifier.cuh:380-395, with the reference's int conversions);
// its value goes to *sel for the pass at that threshold.
static __global__ void threshold_select_kernel(const unsigned long long* __restrict__ counts,
                                               const double* __restrict__ seq, uint64_t n, double pct,
                                               double* __restrict__ sel) {
  if (threadIdx.x != 0) return;
  int stop = -1;
  for (int q = 0; q < kMaxThresholds && stop < 0; ++q)
    if (__ddiv_rn((double)(int)counts[q], (double)(int)n) <= pct) stop = q;
  *sel = seq[stop >= 0 ? stop : kMaxThresholds - 1];
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

// Plain blocked compensated sum of one array (test entry point).
static __global__ void __launch_bounds__(kRedThreads) sum_chunks_kernel(const double* __restrict__ x, uint64_t n,
                                                               NS* __restrict__ part) {
  __shared__ NS scratch[8];
  NS a = ns_zero();
#pragma unroll
  for (int k = 0; k < kRedItems; ++k) {
    const uint64_t i = (uint64_t)blockIdx.x * kChunk + (uint64_t)k * kRedThreads + threadIdx.x;
    if (i < n) a = ns_add(a, x[i]);
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
  uint64_t total = 1;
  for (int k = 0; k < d; ++k) total *= (uint64_t)parts;
  if (q >= total) return;  // a gap held by another admitted integral
  for (int k = 0; k < d; ++k) {
    const uint64_t id = q % (uint64_t)parts;
    q /= (uint64_t)parts;
    left[(uint64_t)k * stride + r] = __dmul_rn((double)id, len);
    length[(uint64_t)k * stride + r] = len;
  }
  owner[r] = j;
}

// One spilled integral's way back into the list: its rows (left, length),
// parent estimates and owner.  src_* point at a pinned host slice the device
// reads directly (NVLink-C2C on Grace); block0 is its first block.
struct RestoreItem {
  const double* src_left;
  const double* src_len;
  const double* src_par;
  uint64_t src_stride;
  uint64_t start, par_start, n;
  uint64_t block0;
  uint32_t owner;
  int32_t d;
};

constexpr int kRestoreRegions = 1024;  // regions per block of restore_kernel

// Every integral restored in one admission, one kernel: block b serves the
// item with the largest block0 <= b, regions [1024 (b - block0), +1024).
static __global__ void __launch_bounds__(256)
    restore_kernel(const RestoreItem* __restrict__ items, uint32_t nitems, double* __restrict__ left,
                   double* __restrict__ length, uint64_t stride, uint32_t* __restrict__ owner,
                   double* __restrict__ parent) {
  uint32_t lo = 0, hi = nitems;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (items[mid].block0 <= blockIdx.x) lo = mid; else hi = mid;
  }
  const RestoreItem I = items[lo];
  const uint64_t base = (uint64_t)(blockIdx.x - I.block0) * kRestoreRegions;
  for (int q = 0; q < kRestoreRegions / 256; ++q) {
    const uint64_t k = base + (uint64_t)q * 256 + threadIdx.x;
    if (k >= I.n) break;
    for (int dim = 0; dim < I.d; ++dim) {
      left[(uint64_t)dim * stride + I.start + k] = I.src_left[(uint64_t)dim * I.src_stride + k];
      length[(uint64_t)dim * stride + I.start + k] = I.src_len[(uint64_t)dim * I.src_stride + k];
    }
    owner[I.start + k] = I.owner;
    if (k < I.n / 2) parent[I.par_start + k] = I.src_par[k];
  }
}

static __global__ void fill_owner_kernel(uint32_t* __restrict__ owner, uint64_t start, uint64_t n, uint32_t j) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) owner[start + i] = j;
}

}  // namespace pg
