// Region evaluation by generator-set sums, for product-form integrands
// (eval_mode 1).  FP64-pipe bound.
//
// The degree-9 rule's points fall into 9 generator sets (Rule.cuh:201-249):
// the centre, +-G_t on one axis (t = 0..3), +-G0 on two axes, +-G0 and +-G1
// on two axes, +-G0 on three axes, and +-G4 on every axis.  Each rule sum is
// sum_s w[s][r] * S_s with S_s the sum of f over set s (Sample.cuh:145-148
// accumulates f * w[set(p)][r] point by point).  When f is a product of
// per-axis factors, f(x) = prod_k h_k(x_k), every S_s is a symmetric sum of
// products that a recurrence over the axes forms exactly:
//
//   c = h_k(centre), p_t = h_k(+G_t) + h_k(-G_t)
//   t3 <- t3*c + b*p0          (three axes at +-G0)
//   g  <- g*c + a0*p1 + a1*p0   (one axis at +-G0, another at +-G1)
//   b  <- b*c + a0*p0          (two axes at +-G0)
//   a_t <- a_t*c + e0*p_t      (one axis at +-G_t, t = 0..3)
//   e0 <- e0*c                 (centre)
//   z  <- z*p4                 (every axis at +-G4)
//
// from e0 = z = 1 and the rest 0.  A region then costs its 11*d factors and
// ~20 operations per axis instead of FEVAL(d) point values (1105 at d = 8).
// The sums are those of the reference's rule, rounded differently; per-region
// estimates and errors agree with the point-by-point evaluation to ~1e-15 of
// the region's estimate.
//
// The recurrence is a product of per-axis terms, so the axes can be taken in
// any order.  Each region has a deferred axis s that enters last: the other
// axes in axis order, then s.  For a region whose sibling is evaluated with it
// (below) s is the axis the two differ on; otherwise s = d - 1, which is the
// plain axis order.
//
// Siblings: after the first iteration an integral's list holds the two
// children of its k-th kept region at k and n/2 + k, equal on every axis but
// the parent's split axis (Sub_region_splitter.cuh:8-46).  One thread
// evaluates both: the factors of the d - 1 shared axes once, the recurrence
// over them once, then each child's own factors of the split axis.  At d = 8
// that is 99 factor evaluations per pair instead of 176.
//
// The split axis needs f at the centre and at +-G0, +-G1 on each axis, and it
// must be the reference's decision exactly, so those 4d+1 values are formed
// exactly as the point-by-point evaluation forms them: the two half products
// L = h_0*...*h_{m-1}, R = h_m*...*h_{d-1} (m = d/2), each in axis order,
// then L*R (and *Jacobian for a general box).  The fourth differences, the
// null-rule error, the widest axis and the volume are the reference's
// (Sample.cuh:190-290, Phases.cuh:329-348) with the same operations as
// eval_kernel.
//
// Parent terms: a region's eight values per axis (c, h(+G0), h(-G0),
// h(+G1), h(-G1), p2, p3, p4; p0 and p1 are sums of the second to fifth) and
// its split axis (one more row) are written to `terms`, the list's term
// buffer, and stay there while the next list is evaluated; the compaction
// records each bisected region's position in that buffer (`ppos`, by parent
// index).  Both children of a region share its coordinates on every axis but
// the split one, so a pair whose parent's values are kept takes them from
// there and evaluates only the split axis's factors: 22 per pair instead of
// 99 at d = 8.  The values are those the children would compute, bit for bit.
//
// One thread per region or sibling pair: with a thread per region every FP64
// warp instruction carries 32 regions' work, and the SoA loads of the bounds
// and the stores of the results are coalesced across the warp.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_eval.cuh"
#include "pg_kernels.cuh"

namespace pg {

// Multiplies of the set-sum kernel, each site on the FP64 pipe (__dmul_rn) or
// on the integer pipe (pg::mul_rn_int), the same bits either way.  The kernel
// is FP64-bound, so the split balances the two pipes: measured on GB300, the
// fourth differences' point products (117 per 8-D region) on the integer pipe
// and the rest on the FP64 pipe is 11% faster on the batched workload than
// all on the FP64 pipe, which is itself 10-18% faster than all on the integer
// pipe on 8-D integrals.
#ifndef PG_SETSUM_MUL
#define PG_SETSUM_MUL __dmul_rn
#endif
#ifndef PG_SETSUM_MUL_FD
#define PG_SETSUM_MUL_FD mul_rn_int  // the fourth differences' point products
#endif
#ifndef PG_SETSUM_MUL_NULL
#define PG_SETSUM_MUL_NULL PG_SETSUM_MUL  // the null rules' scaled terms
#endif
#ifndef PG_SETSUM_MUL_STEP
#define PG_SETSUM_MUL_STEP PG_SETSUM_MUL  // the set-sum recurrence
#endif

constexpr int kSetSumThreads = 128;
#ifndef PG_SETSUM_MIN_BLOCKS
#define PG_SETSUM_MIN_BLOCKS 4  // resident blocks per SM the register allocation allows
#endif
constexpr int kFdValues = 5;  // per axis: factor at the centre, +G0, -G0, +G1, -G1

template <int MAXD>
struct SetSumSmem {
  double w[(MAXD + 1) * 45];
  double scale[(MAXD + 1) * 45];
  double norm[(MAXD + 1) * 45];
  double fd[kFdValues * (MAXD + 1) * kSetSumThreads];  // [(k * 5 + v) * threads + thread]; row MAXD: sibling's axis
};

// Inputs of one axis to the recurrence.
struct AxisTerm {
  double c, p0, p1, p2, p3, p4;
};

// The nine generator-set sums (sets 0..8).
struct SetSums {
  double e0, a0, a1, a2, a3, b, g, t3, z;
};

__device__ __forceinline__ void set_step(SetSums& S, const AxisTerm& A) {
  S.t3 = __fma_rn(S.b, A.p0, PG_SETSUM_MUL_STEP(S.t3, A.c));
  S.g = __fma_rn(S.a1, A.p0, __fma_rn(S.a0, A.p1, PG_SETSUM_MUL_STEP(S.g, A.c)));
  S.b = __fma_rn(S.a0, A.p0, PG_SETSUM_MUL_STEP(S.b, A.c));
  S.a0 = __fma_rn(S.e0, A.p0, PG_SETSUM_MUL_STEP(S.a0, A.c));
  S.a1 = __fma_rn(S.e0, A.p1, PG_SETSUM_MUL_STEP(S.a1, A.c));
  S.a2 = __fma_rn(S.e0, A.p2, PG_SETSUM_MUL_STEP(S.a2, A.c));
  S.a3 = __fma_rn(S.e0, A.p3, PG_SETSUM_MUL_STEP(S.a3, A.c));
  S.e0 = PG_SETSUM_MUL_STEP(S.e0, A.c);
  S.z = PG_SETSUM_MUL_STEP(S.z, A.p4);
}

// The 11 factor values of axis k over [lo, up] (coordinates as Sample.cuh:126-131
// forms them); writes the five the fourth differences read to fd[v * T].
__device__ __forceinline__ AxisTerm axis_term(const IntegralDesc& D, const RuleDev& rule, int k, double lo,
                                              double up, bool unit, double* fd, int T) {
  double h[kCodesPerDim];
#pragma unroll
  for (int c = 0; c < kCodesPerDim; ++c) {
    const double t = __fma_rn(rule.A[c], lo, PG_SETSUM_MUL(rule.B[c], up));
    h[c] = family_factor(D, k, unit ? t : __fma_rn(t, D.range[k], D.glo[k]));
  }
  fd[0 * T] = h[0];
  fd[1 * T] = h[1];
  fd[2 * T] = h[6];
  fd[3 * T] = h[2];
  fd[4 * T] = h[7];
  return AxisTerm{h[0], __dadd_rn(h[1], h[6]), __dadd_rn(h[2], h[7]), __dadd_rn(h[3], h[8]), __dadd_rn(h[4], h[9]),
                  __dadd_rn(h[5], h[10])};
}

// Writes one axis's terms (the five values at fd[v * T] and p2..p4) for the
// region at list position pos.
__device__ __forceinline__ void put_terms(double* __restrict__ terms, int rows, uint64_t pos, int k,
                                          const double* fd, int T, const AxisTerm& A) {
  double* t = terms + term_at(pos, k * kTermValues, rows);
#pragma unroll
  for (int v = 0; v < kFdValues; ++v) t[v * 32] = fd[v * T];
  t[5 * 32] = A.p2;
  t[6 * 32] = A.p3;
  t[7 * 32] = A.p4;
}

// One axis's terms of a parent at position ppos of the previous list's term
// buffer; the five values the fourth differences read go to fd[v * T].
__device__ __forceinline__ AxisTerm cached_term(const double* __restrict__ pterms, int rows, uint64_t ppos, int k,
                                                double* fd, int T) {
  const double* t = pterms + term_at(ppos, k * kTermValues, rows);
  double v[kTermValues];
#pragma unroll
  for (int q = 0; q < kTermValues; ++q) v[q] = t[q * 32];
#pragma unroll
  for (int q = 0; q < kFdValues; ++q) fd[q * T] = v[q];
  return AxisTerm{v[0], __dadd_rn(v[1], v[2]), __dadd_rn(v[3], v[4]), v[5], v[6], v[7]};
}

// Rule sums, split axis and null-rule error of one region from its set sums.
// Factor value v of axis k is fv[(k * 5 + v) * T], except on axis `sk`, whose
// values are at own[v * T].
template <int MAXD, bool SCALE>
__device__ __forceinline__ int region_result(const SetSumSmem<MAXD>& Sm, const RuleDev& rule, const SetSums& Q,
                                             int d, double jac, double vol, int maxdim, const double* fv, int sk,
                                             const double* own, double* est, double* err, int32_t* bisect) {
  constexpr int T = kSetSumThreads;
  // Jacobian scaling (a box other than the unit cube): compiled out of
  // launches whose integrals all have jac = 1, where a predicated multiply
  // would still run.
  const bool scale_jac = SCALE && jac != 1.0;
  const double* W = Sm.w + d * 45;
  double s5[kNRules];
#pragma unroll
  for (int q = 0; q < kNRules; ++q) {
    double v = PG_SETSUM_MUL(W[q], Q.e0);
    v = __fma_rn(W[5 + q], Q.a0, v);
    v = __fma_rn(W[10 + q], Q.a1, v);
    v = __fma_rn(W[15 + q], Q.a2, v);
    v = __fma_rn(W[20 + q], Q.a3, v);
    v = __fma_rn(W[25 + q], Q.b, v);
    v = __fma_rn(W[30 + q], Q.g, v);
    v = __fma_rn(W[35 + q], Q.t3, v);
    v = __fma_rn(W[40 + q], Q.z, v);
    s5[q] = scale_jac ? PG_SETSUM_MUL(v, jac) : v;
  }
  auto F = [&](int k, int v) -> double { return (k == sk) ? own[v * T] : fv[(k * kFdValues + v) * T]; };
  // Point values of the fourth differences, formed as the point-by-point
  // evaluation forms them: L * R from the two half products in axis order.
  const int m = d / 2;
  double Lc = F(0, 0), Rc = F(m, 0);
  for (int k = 1; k < m; ++k) Lc = PG_SETSUM_MUL_FD(Lc, F(k, 0));
  for (int k = m + 1; k < d; ++k) Rc = PG_SETSUM_MUL_FD(Rc, F(k, 0));
  double f0 = PG_SETSUM_MUL_FD(Lc, Rc);
  if (scale_jac) f0 = PG_SETSUM_MUL_FD(f0, jac);
  const double f02 = __dadd_rn(f0, f0);
  unsigned long long kmax = 0ull;
  int cand = -1;
  double pre = 1.0;  // product of the centre factors of the earlier axes of the current half
  for (int k = 0; k < d; ++k) {
    const bool lhalf = k < m;
    const int hbeg = lhalf ? 0 : m, hend = lhalf ? m : d;
    // The half product of each of the four points, the four chains side by side.
    double f[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) f[v] = (k == hbeg) ? F(k, 1 + v) : PG_SETSUM_MUL_FD(pre, F(k, 1 + v));
    for (int q = k + 1; q < hend; ++q) {
      const double cq = F(q, 0);
#pragma unroll
      for (int v = 0; v < 4; ++v) f[v] = PG_SETSUM_MUL_FD(f[v], cq);
    }
    const double other = lhalf ? Rc : Lc;  // the other half's centre product
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      f[v] = PG_SETSUM_MUL_FD(f[v], other);
      if (scale_jac) f[v] = PG_SETSUM_MUL_FD(f[v], jac);
    }
    const double ck = F(k, 0);
    pre = (k == hbeg) ? ck : PG_SETSUM_MUL_FD(pre, ck);
    if (k + 1 == m) pre = 1.0;
    // base + ratio*(fp+fm) - (fp2+fm2), base = 2*f0*(1-ratio): the
    // reference's compiled code fuses the base multiply for d <= 4 and the
    // ratio multiply for d >= 5 (Sample.cuh:190-215).
    const double X = __dadd_rn(f[0], f[1]);
    const double Y = __dadd_rn(f[2], f[3]);
    const double s = (d <= 4) ? __fma_rn(f02, rule.omr, __dmul_rn(rule.ratio, X))
                              : __fma_rn(rule.ratio, X, __dmul_rn(f02, rule.omr));
    const unsigned long long fd = (unsigned long long)__double_as_longlong(fabs(__dsub_rn(s, Y)));
    if (fd != 0ull && fd <= 0x7ff0000000000000ull && fd > kmax) {
      kmax = fd;
      cand = k;
    }
  }
  // Null-rule error (Sample.cuh:261-289): maxima of non-negative terms on
  // their bit patterns, a NaN term ignored.
  const double* SC = Sm.scale + d * 45;
  const double* NM = Sm.norm + d * 45;
  // (A maximum of bit patterns does not depend on the order of its terms; one
  // generator set at a time keeps few products live.)
  unsigned long long mq[3] = {0ull, 0ull, 0ull};
#pragma unroll 1
  for (int st = 0; st < kNSets; ++st) {
#pragma unroll
    for (int q = 1; q <= 3; ++q) {
      const unsigned long long bt = (unsigned long long)__double_as_longlong(
          PG_SETSUM_MUL_NULL(fabs(__fma_rn(SC[st * kNRules + q], s5[q], s5[q + 1])), NM[st * kNRules + q]));
      const unsigned long long term = (bt & 0x7fffffffffffffffull) > 0x7ff0000000000000ull ? 0ull : bt;
      mq[q - 1] = term > mq[q - 1] ? term : mq[q - 1];
    }
  }
  const double e1 = __longlong_as_double((long long)mq[0]), e2 = __longlong_as_double((long long)mq[1]),
               e3 = __longlong_as_double((long long)mq[2]);
  unsigned long long mmax = mq[0] > mq[1] ? mq[0] : mq[1];
  mmax = mq[2] > mmax ? mq[2] : mmax;
  const double emax = __longlong_as_double((long long)mmax);
  const bool ladder = PG_SETSUM_MUL(5.0, e1) <= e2 && PG_SETSUM_MUL(5.0, e2) <= e3;
  *est = PG_SETSUM_MUL(vol, s5[0]);
  *err = PG_SETSUM_MUL(vol, ladder ? e1 : PG_SETSUM_MUL(5.0, emax));
  const int axis = cand >= 0 ? cand : maxdim;
  *bisect = axis;
  return axis;
}

// Widest axis (first strictly widest; a negative or NaN side never wins) and
// the volume as the product of the sides in axis order (Phases.cuh:329-348).
__device__ __forceinline__ void side_step(int k, double side, double& vol, unsigned long long& widest, int& maxdim) {
  const unsigned long long sb = (unsigned long long)__double_as_longlong(side);
  const unsigned long long key = ((sb >> 63) || (sb & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) ? 0ull : sb;
  if (key > widest) {
    widest = key;
    maxdim = k;
  }
  vol = (k == 0) ? side : PG_SETSUM_MUL(vol, side);
}

// Regions [0, n) of a run that starts at list position `base`, one per
// thread, blocks in list order.  With `terms` (tiles of `terms_rows` rows,
// by list position) every region's terms are written; with `pterms` (the
// previous list's term buffer, same rows) and `ppos` (parent index -> its
// position there), pairs of segments flagged has_cache take their shared
// axes' terms from their parent.
// (A grid-stride loop over tens of millions of regions lets the blocks drift
// apart over the list, and the scattered loads
// of the SoA rows made each region up to 40% dearer.)  With `segs` (the
// integrals' segments of the list), a region in the first half of a segment
// that has a parent level is evaluated together with its sibling in the
// second half, and second-half regions are left to their sibling's thread;
// without, every region is evaluated alone.
template <int MAXD, bool SCALE>
static __global__ void __launch_bounds__(kSetSumThreads, PG_SETSUM_MIN_BLOCKS)
    setsum_kernel(const double* __restrict__ left, const double* __restrict__ length, uint64_t n, uint64_t stride,
                  const uint32_t* __restrict__ owner, const IntegralDesc* __restrict__ descs, RuleDev rule,
                  double* __restrict__ est, double* __restrict__ err, int32_t* __restrict__ bisect,
                  const SegDesc* __restrict__ segs, uint64_t base, const double* __restrict__ pterms,
                  const uint32_t* __restrict__ ppos, double* __restrict__ terms, int terms_rows, uint64_t terms_n,
                  uint64_t pterms_n, uint64_t ppos_n, unsigned long long* __restrict__ chk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SetSumSmem<MAXD>& Sm = *reinterpret_cast<SetSumSmem<MAXD>*>(smem_raw);
  constexpr int T = kSetSumThreads;
  const uint64_t r = (uint64_t)blockIdx.x * T + threadIdx.x;
  bool work = r < n;
  uint32_t j = 0;
  uint64_t rb = r;  // the sibling evaluated with r (r itself: none)
  bool cached = false;
  uint64_t pp = 0;  // the pair's parent's position in the previous list
  if (work) {
    j = owner ? owner[r] : 0u;
    if (segs) {
      const SegDesc& S = segs[j];
      const uint64_t local = base + r - S.start, half = S.n / 2;
      if (S.has_parent && (S.n & 1ull) == 0ull && half > 0) {
        if (local >= half) {
          work = false;  // evaluated with its sibling; its parent index would be past the segment's parents
        } else {
          rb = r + half;
          if (rb >= n) rb = r;  // a segment always lies inside one run; never read outside it
          cached = pterms && S.has_cache && rb != r &&
                   in_bounds(chk, 1, S.par_start + local, ppos_n, j, S.start, S.n, base + r);
          if (cached) {
            pp = ppos[S.par_start + local];
            cached = in_bounds(chk, 2, pp, pterms_n, j, S.start, S.n, base + r);
          }
        }
      }
    }
  }
  if (!__syncthreads_or(work)) return;
  for (int q = threadIdx.x; q < (MAXD + 1) * 45; q += kSetSumThreads) {
    Sm.w[q] = rule.w[q];
    Sm.scale[q] = rule.scale[q];
    Sm.norm[q] = rule.norm[q];
  }
  __syncthreads();
  double* const fv = Sm.fd + threadIdx.x;
  double* const fvb = Sm.fd + (MAXD * kFdValues) * T + threadIdx.x;
  if (!work) return;
  const bool pair = rb != r;
  if (terms && !(in_bounds(chk, 3, base + r, terms_n) && in_bounds(chk, 3, base + rb, terms_n))) terms = nullptr;
  const IntegralDesc& D = descs[j];
  const int d = D.d;
  const bool unit = D.unit != 0;
  // The deferred axis: the parent's split axis when its terms are kept, else
  // the one the siblings differ on, else the last.  (Siblings whose lower
  // bounds coincide, when half the parent's side is below the bound's
  // rounding, still differ from the parent on the split axis.)
  int s = d - 1;
  if (cached)
    s = min(max((int)pterms[term_at(pp, kTermValues * d, terms_rows)], 0), d - 1);
  else if (pair)
    for (int k = d - 1; k >= 0; --k)
      if (left[(uint64_t)k * stride + r] != left[(uint64_t)k * stride + rb]) s = k;
  SetSums Q{1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0};
  AxisTerm As{};
  double vol = 1.0, volb = 1.0;
  unsigned long long widest = 0ull, widestb = 0ull;
  int maxdim = 0, maxdimb = 0;
  // The sibling's own side and factors on the deferred axis.
  double sideb = 0.0;
  AxisTerm Bs{};
  if (pair) {
    const double lo = left[(uint64_t)s * stride + rb];
    const double up = __dadd_rn(lo, length[(uint64_t)s * stride + rb]);
    sideb = __dsub_rn(up, lo);
    Bs = axis_term(D, rule, s, lo, up, unit, fvb, T);
  }
  // With the parent's terms, the pair's own factors on the split axis come
  // first: every thread of the warp evaluates one axis here, whichever it is,
  // and the loop below only loads.  (Evaluated inside the loop at k == s, the
  // lanes' different split axes would make the warp run the factors at
  // nearly every k.)
  AxisTerm Ac{};
  if (cached) {
    const double lo = left[(uint64_t)s * stride + r];
    const double up = __dadd_rn(lo, length[(uint64_t)s * stride + r]);
    Ac = axis_term(D, rule, s, lo, up, unit, fv + (s * kFdValues) * T, T);
  }
  for (int k = 0; k < d; ++k) {
    const double lo = left[(uint64_t)k * stride + r];
    const double up = __dadd_rn(lo, length[(uint64_t)k * stride + r]);
    const double side = __dsub_rn(up, lo);
    side_step(k, side, vol, widest, maxdim);
    if (pair) side_step(k, k == s ? sideb : side, volb, widestb, maxdimb);
    double* const fk = fv + (k * kFdValues) * T;
    AxisTerm A;
    if (cached)
      A = (k == s) ? Ac : cached_term(pterms, terms_rows, pp, k, fk, T);
    else
      A = axis_term(D, rule, k, lo, up, unit, fk, T);
    if (terms) {
      put_terms(terms, terms_rows, base + r, k, fk, T, A);
      if (pair && k != s) put_terms(terms, terms_rows, base + rb, k, fk, T, A);
    }
    if (k == s)
      As = A;
    else
      set_step(Q, A);
  }
  if (pair && terms) put_terms(terms, terms_rows, base + rb, s, fvb, T, Bs);
  const double jac = D.jac;
  {
    SetSums R = Q;
    set_step(R, As);
    const int ax = region_result<MAXD, SCALE>(Sm, rule, R, d, jac, vol, maxdim, fv, -1, fv, &est[r], &err[r],
                                              &bisect[r]);
    if (terms) terms[term_at(base + r, kTermValues * d, terms_rows)] = (double)ax;
  }
  if (pair) {
    SetSums R = Q;
    set_step(R, Bs);
    const int ax = region_result<MAXD, SCALE>(Sm, rule, R, d, jac, volb, maxdimb, fv, s, fvb, &est[rb], &err[rb],
                                              &bisect[rb]);
    if (terms) terms[term_at(base + rb, kTermValues * d, terms_rows)] = (double)ax;
  }
}

// Launch of the set-sum kernel over a run of the region list whose integrals
// all have product-form families: one thread per region.  `segs` may be null
// (no sibling pairing); `base` is the run's first list position.
struct SetSumCache {
  const double* pterms = nullptr;  // the previous list's terms (the parents')
  const uint32_t* ppos = nullptr;  // parent index -> the parent's position in the previous list
  double* terms = nullptr;         // this list's terms: row k * 8 + v, then the split axis, tiles by position
  int terms_rows = 0;              // rows per tile (8 * the list's largest dimension + 1)
  uint64_t terms_n = 0, pterms_n = 0, ppos_n = 0;  // positions in terms and pterms, parents in ppos
  unsigned long long* chk = nullptr;               // bounds record
  bool scale = true;               // some integral of the run has a box other than the unit cube
};

template <int MAXD, bool SCALE>
inline cudaError_t launch_setsum_shape(const pg_eval_args& a, const SegDesc* segs, uint64_t base,
                                       const SetSumCache& c) {
  const size_t smem = sizeof(SetSumSmem<MAXD>);
  static std::atomic<unsigned long long> attr_done{0};
  const cudaError_t ae = ensure_dynamic_smem(setsum_kernel<MAXD, SCALE>, (int)smem, attr_done);
  if (ae != cudaSuccess) return ae;
  if (a.n == 0) return cudaSuccess;
  const uint64_t g = (a.n + kSetSumThreads - 1) / kSetSumThreads;
  if (g > 0x7fffffffull) return cudaErrorInvalidValue;
  setsum_kernel<MAXD, SCALE><<<(unsigned)g, kSetSumThreads, smem, (cudaStream_t)a.stream>>>(
      a.left, a.length, a.n, a.stride, a.owner, static_cast<const IntegralDesc*>(a.descs),
      *static_cast<const RuleDev*>(a.rule), a.est, a.err, a.bisect, segs, base, c.pterms, c.ppos, c.terms,
      c.terms_rows, c.terms_n, c.pterms_n, c.ppos_n, c.chk);
  return cudaGetLastError();
}

inline cudaError_t launch_setsum(const pg_eval_args& a, const SegDesc* segs, uint64_t base,
                                 const SetSumCache& c = SetSumCache()) {
  if (a.maxd <= 8)
    return c.scale ? launch_setsum_shape<8, true>(a, segs, base, c) : launch_setsum_shape<8, false>(a, segs, base, c);
  return c.scale ? launch_setsum_shape<kMaxNdim, true>(a, segs, base, c)
                 : launch_setsum_shape<kMaxNdim, false>(a, segs, base, c);
}

}  // namespace pg
