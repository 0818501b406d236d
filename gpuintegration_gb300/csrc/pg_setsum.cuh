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
// The split axis needs f at the centre and at +-G0, +-G1 on each axis, and it
// must be the reference's decision exactly, so those 4d+1 values are formed
// exactly as the point-by-point evaluation forms them: the two half products
// L = h_0*...*h_{m-1}, R = h_m*...*h_{d-1} (m = d/2), each in axis order,
// then L*R (and *Jacobian for a general box).  The fourth differences, the
// null-rule error, the widest axis and the volume are the reference's
// (Sample.cuh:190-290, Phases.cuh:329-348) with the same operations as
// eval_kernel.
//
// One thread per region: a region's recurrence is sequential over the axes,
// and with a thread per region every FP64 warp instruction carries 32
// regions' work.  Loads of the SoA bounds and stores of the results are
// coalesced across the warp.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_eval.cuh"

namespace pg {

constexpr int kSetSumThreads = 128;
constexpr int kFdValues = 5;  // per axis: factor at the centre, +G0, -G0, +G1, -G1

template <int MAXD>
struct SetSumSmem {
  double w[(MAXD + 1) * 45];
  double scale[(MAXD + 1) * 45];
  double norm[(MAXD + 1) * 45];
  double fd[kFdValues * MAXD * kSetSumThreads];  // [(k * 5 + v) * threads + thread]
};

template <int MAXD>
static __global__ void __launch_bounds__(kSetSumThreads, 4)
    setsum_kernel(const double* __restrict__ left, const double* __restrict__ length, uint64_t n, uint64_t stride,
                  const uint32_t* __restrict__ owner, const IntegralDesc* __restrict__ descs, RuleDev rule,
                  double* __restrict__ est, double* __restrict__ err, int32_t* __restrict__ bisect) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SetSumSmem<MAXD>& S = *reinterpret_cast<SetSumSmem<MAXD>*>(smem_raw);
  for (int q = threadIdx.x; q < (MAXD + 1) * 45; q += kSetSumThreads) {
    S.w[q] = rule.w[q];
    S.scale[q] = rule.scale[q];
    S.norm[q] = rule.norm[q];
  }
  __syncthreads();
  double* const fv = S.fd + threadIdx.x;
  constexpr int T = kSetSumThreads;

  for (uint64_t r = (uint64_t)blockIdx.x * T + threadIdx.x; r < n; r += (uint64_t)gridDim.x * T) {
    const uint32_t j = owner ? owner[r] : 0u;
    const IntegralDesc& D = descs[j];
    const int d = D.d;
    const bool unit = D.unit != 0;
    double e0 = 1.0, a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0, b = 0.0, g = 0.0, t3 = 0.0, z = 1.0;
    double vol = 1.0;
    unsigned long long widest = 0ull;
    int maxdim = 0;
    for (int k = 0; k < d; ++k) {
      const double lo = left[(uint64_t)k * stride + r];
      const double up = __dadd_rn(lo, length[(uint64_t)k * stride + r]);
      // Side length, widest axis (first strictly widest, a negative or NaN
      // side never wins) and the volume as the product of the sides in axis
      // order (Phases.cuh:329-348).
      const double side = __dsub_rn(up, lo);
      const unsigned long long sb = (unsigned long long)__double_as_longlong(side);
      const unsigned long long sk = ((sb >> 63) || (sb & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) ? 0ull : sb;
      if (sk > widest) {
        widest = sk;
        maxdim = k;
      }
      vol = (k == 0) ? side : mul_rn_int(vol, side);
      // The axis's 11 coordinates (Sample.cuh:126-131) and factors.
      double h[kCodesPerDim];
#pragma unroll
      for (int c = 0; c < kCodesPerDim; ++c) {
        const double t = __fma_rn(rule.A[c], lo, mul_rn_int(rule.B[c], up));
        h[c] = family_factor(D, k, unit ? t : __fma_rn(t, D.range[k], D.glo[k]));
      }
      fv[(k * kFdValues + 0) * T] = h[0];
      fv[(k * kFdValues + 1) * T] = h[1];
      fv[(k * kFdValues + 2) * T] = h[6];
      fv[(k * kFdValues + 3) * T] = h[2];
      fv[(k * kFdValues + 4) * T] = h[7];
      const double c = h[0];
      const double p0 = __dadd_rn(h[1], h[6]), p1 = __dadd_rn(h[2], h[7]), p2 = __dadd_rn(h[3], h[8]),
                   p3 = __dadd_rn(h[4], h[9]), p4 = __dadd_rn(h[5], h[10]);
      t3 = __fma_rn(b, p0, mul_rn_int(t3, c));
      g = __fma_rn(a1, p0, __fma_rn(a0, p1, mul_rn_int(g, c)));
      b = __fma_rn(a0, p0, mul_rn_int(b, c));
      a0 = __fma_rn(e0, p0, mul_rn_int(a0, c));
      a1 = __fma_rn(e0, p1, mul_rn_int(a1, c));
      a2 = __fma_rn(e0, p2, mul_rn_int(a2, c));
      a3 = __fma_rn(e0, p3, mul_rn_int(a3, c));
      e0 = mul_rn_int(e0, c);
      z = mul_rn_int(z, p4);
    }
    const double jac = D.jac;
    const bool scale_jac = jac != 1.0;

    // Rule sums: sum_s w[s][r] * S_s, times the box's Jacobian.
    const double* W = S.w + d * 45;
    double s5[kNRules];
#pragma unroll
    for (int q = 0; q < kNRules; ++q) {
      double v = mul_rn_int(W[q], e0);
      v = __fma_rn(W[5 + q], a0, v);
      v = __fma_rn(W[10 + q], a1, v);
      v = __fma_rn(W[15 + q], a2, v);
      v = __fma_rn(W[20 + q], a3, v);
      v = __fma_rn(W[25 + q], b, v);
      v = __fma_rn(W[30 + q], g, v);
      v = __fma_rn(W[35 + q], t3, v);
      v = __fma_rn(W[40 + q], z, v);
      s5[q] = scale_jac ? mul_rn_int(v, jac) : v;
    }

    // Point values of the fourth differences, formed as the point-by-point
    // evaluation forms them: L * R from the two half products in axis order.
    const int m = d / 2;
    double Lc = fv[0], Rc = fv[(m * kFdValues) * T];
    for (int k = 1; k < m; ++k) Lc = mul_rn_int(Lc, fv[(k * kFdValues) * T]);
    for (int k = m + 1; k < d; ++k) Rc = mul_rn_int(Rc, fv[(k * kFdValues) * T]);
    double f0 = mul_rn_int(Lc, Rc);
    if (scale_jac) f0 = mul_rn_int(f0, jac);
    const double f02 = __dadd_rn(f0, f0);
    unsigned long long kmax = 0ull;
    int cand = -1;
    double pre = 1.0;  // product of the centre factors of the earlier axes of the current half
    for (int k = 0; k < d; ++k) {
      const bool lhalf = k < m;
      const int hbeg = lhalf ? 0 : m, hend = lhalf ? m : d;
      double f[4];
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const double hv = fv[(k * kFdValues + 1 + v) * T];
        double P = (k == hbeg) ? hv : mul_rn_int(pre, hv);
        for (int q = k + 1; q < hend; ++q) P = mul_rn_int(P, fv[(q * kFdValues) * T]);
        double fp = lhalf ? mul_rn_int(P, Rc) : mul_rn_int(Lc, P);
        f[v] = scale_jac ? mul_rn_int(fp, jac) : fp;
      }
      const double ck = fv[(k * kFdValues) * T];
      pre = (k == hbeg) ? ck : mul_rn_int(pre, ck);
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
    const double* SC = S.scale + d * 45;
    const double* NM = S.norm + d * 45;
    unsigned long long mq[3] = {0ull, 0ull, 0ull};
#pragma unroll
    for (int q = 1; q <= 3; ++q) {
      unsigned long long mx = 0ull;
#pragma unroll
      for (int st = 0; st < kNSets; ++st) {
        const unsigned long long bt = (unsigned long long)__double_as_longlong(
            mul_rn_int(fabs(__fma_rn(SC[st * kNRules + q], s5[q], s5[q + 1])), NM[st * kNRules + q]));
        const unsigned long long term = (bt & 0x7fffffffffffffffull) > 0x7ff0000000000000ull ? 0ull : bt;
        mx = term > mx ? term : mx;
      }
      mq[q - 1] = mx;
    }
    const double e1 = __longlong_as_double((long long)mq[0]), e2 = __longlong_as_double((long long)mq[1]),
                 e3 = __longlong_as_double((long long)mq[2]);
    unsigned long long mmax = mq[0] > mq[1] ? mq[0] : mq[1];
    mmax = mq[2] > mmax ? mq[2] : mmax;
    const double emax = __longlong_as_double((long long)mmax);
    const bool ladder = mul_rn_int(5.0, e1) <= e2 && mul_rn_int(5.0, e2) <= e3;
    est[r] = mul_rn_int(vol, s5[0]);
    err[r] = mul_rn_int(vol, ladder ? e1 : mul_rn_int(5.0, emax));
    bisect[r] = cand >= 0 ? cand : maxdim;
  }
}

// Launch of the set-sum kernel over a region list whose integrals all have
// product-form families: a grid-stride loop with at most 8 blocks per SM.
template <int MAXD>
inline cudaError_t launch_setsum_shape(const pg_eval_args& a) {
  const size_t smem = sizeof(SetSumSmem<MAXD>);
  static std::atomic<unsigned long long> attr_done{0};
  const cudaError_t ae = ensure_dynamic_smem(setsum_kernel<MAXD>, (int)smem, attr_done);
  if (ae != cudaSuccess) return ae;
  const uint64_t want = (a.n + kSetSumThreads - 1) / kSetSumThreads;
  const uint64_t cap = (uint64_t)(a.num_sms > 0 ? a.num_sms : 1) * 8ull;
  const uint64_t g = want < cap ? want : cap;
  setsum_kernel<MAXD><<<(unsigned)(g > 0 ? g : 1), kSetSumThreads, smem, (cudaStream_t)a.stream>>>(
      a.left, a.length, a.n, a.stride, a.owner, static_cast<const IntegralDesc*>(a.descs),
      *static_cast<const RuleDev*>(a.rule), a.est, a.err, a.bisect);
  return cudaGetLastError();
}

inline cudaError_t launch_setsum(const pg_eval_args& a) {
  return a.maxd <= 8 ? launch_setsum_shape<8>(a) : launch_setsum_shape<kMaxNdim>(a);
}

}  // namespace pg
