// Integrand families of the C ABI, evaluated on the device.
//
// A device functor cannot cross a C ABI, so C callers name an integrand by
// family and parameters (pg_integrand).  Every family is written with explicit
// IEEE operations (__dadd_rn, __fma_rn, ...) in a fixed order so that the CPU
// oracle, which spells out the same operations, reproduces the values
// exactly for the families built from +, -, *, / alone.
#pragma once

#include <stdint.h>

#include "pg_common.cuh"

namespace pg {

enum Family : int32_t {
  FAM_CONSTANT = 0,
  FAM_OSCILLATORY = 1,
  FAM_PRODUCT_PEAK = 2,
  FAM_CORNER_PEAK = 3,
  FAM_GAUSSIAN = 4,
  FAM_C0 = 5,
  FAM_DISCONTINUOUS = 6,
  FAM_PRODUCT = 7,
  FAM_NAN = 8,
  FAM_BOX = 9,
  FAM_FUN6 = 10,
  FAM_GAUSSIAN_SUM = 11,  // exp of the sum of squares; s0 holds c^d (or 1)
  FAM_COUNT = 12,
  FAM_USER = 64  // a caller's functor (C++ layer); never accepted from a pg_integrand
};

// Everything a kernel needs to know about one integral: its integrand, the
// integration box and derived constants.  Prepared on the host once per call.
struct IntegralDesc {
  int32_t family;
  int32_t d;
  int32_t unit;  // 1 when the box is [0,1]^d: the final x = lo + t*range is then exactly t
  int32_t pad;
  double jac;    // product of the box's side lengths (Phases.cuh:329-348)
  double c;
  double s0;
  double glo[kMaxDim];
  double range[kMaxDim];
  double a[kMaxDim];
  double u[kMaxDim];
  double ia2[kMaxDim];  // 1 / a_i^2 (product peak)
};

__device__ __forceinline__ double ipow_dev(double s, int e) {
  double r = 1.0, b = s;
  while (e) {
    if (e & 1) r = __dmul_rn(r, b);
    e >>= 1;
    if (e) b = __dmul_rn(b, b);
  }
  return r;
}

// Families that are products of per-axis factors h_k(x_k).  The product is
// taken in two halves, f = L * R, L = h_0 * h_1 * ... * h_{m-1} and
// R = h_m * ... * h_{d-1} (m = d / 2), each half in axis order.  A region's
// points take only 11 coordinate values per axis, so the evaluation kernel
// computes each factor once per region, the distinct half products once per
// region (prefix tries of the two halves), and each point's value with one
// multiply (same operations, same order, same value as this definition).
__host__ __device__ __forceinline__ int product_split(int d) { return d / 2; }
__host__ __device__ __forceinline__ bool family_separable(int family) {
  return family == FAM_PRODUCT_PEAK || family == FAM_GAUSSIAN || family == FAM_C0 || family == FAM_DISCONTINUOUS ||
         family == FAM_PRODUCT;
}

__device__ __forceinline__ double family_factor(const IntegralDesc& D, int k, double x) {
  switch (D.family) {
    case FAM_PRODUCT_PEAK: {
      const double t = __dsub_rn(x, D.u[k]);
      return __ddiv_rn(1.0, __fma_rn(t, t, D.ia2[k]));
    }
    case FAM_GAUSSIAN: {
      const double q = __dmul_rn(D.a[k], __dsub_rn(x, D.u[k]));
      const double v = exp(-__dmul_rn(q, q));
      return D.c != 0.0 ? __dmul_rn(v, D.c) : v;  // c: per-axis normalisation (0 = none)
    }
    case FAM_C0:
      return exp(-__dmul_rn(D.a[k], fabs(__dsub_rn(x, D.u[k]))));
    case FAM_DISCONTINUOUS:
      return (x > D.u[k]) ? 0.0 : exp(__dmul_rn(D.a[k], x));
    case FAM_PRODUCT:
      return x;
  }
  return 1.0;
}

// L * R of the product-form families (factors, or the coordinates themselves
// for PRODUCT).
template <int MAXD>
__device__ __forceinline__ double split_product(const IntegralDesc& D, const double* x, bool factors) {
  const int d = D.d, m = product_split(d);  // 1 <= m < d
  double L = factors ? family_factor(D, 0, x[0]) : x[0];
  double R = 0.0;
#pragma unroll
  for (int i = 1; i < MAXD; ++i) {  // static indices keep x in registers
    if (i >= d) break;
    const double h = factors ? family_factor(D, i, x[i]) : x[i];
    if (i < m) L = __dmul_rn(L, h);
    else if (i == m) R = h;
    else R = __dmul_rn(R, h);
  }
  return __dmul_rn(L, R);
}

template <int MAXD>
__device__ __forceinline__ double family_eval(const IntegralDesc& D, const double* x) {
  const int d = D.d;
  switch (D.family) {
    case FAM_CONSTANT:
      return D.c;
    case FAM_OSCILLATORY: {
      double s = D.s0;
#pragma unroll
      for (int i = 0; i < MAXD; ++i)
        if (i < d) s = __fma_rn(D.a[i], x[i], s);
      return cos(s);
    }
    case FAM_PRODUCT_PEAK:
      return split_product<MAXD>(D, x, true);
    case FAM_CORNER_PEAK: {
      double s = 1.0;
#pragma unroll
      for (int i = 0; i < MAXD; ++i)
        if (i < d) s = __fma_rn(D.a[i], x[i], s);
      return __ddiv_rn(1.0, ipow_dev(s, d + 1));
    }
    case FAM_GAUSSIAN:
    case FAM_C0:
    case FAM_DISCONTINUOUS:
      return split_product<MAXD>(D, x, true);
    case FAM_PRODUCT:
      return split_product<MAXD>(D, x, false);
    case FAM_GAUSSIAN_SUM: {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < MAXD; ++i) {
        if (i < d) {
          const double q = __dmul_rn(D.a[i], __dsub_rn(x[i], D.u[i]));
          s = __fma_rn(q, q, s);
        }
      }
      return __dmul_rn(exp(-s), D.s0);
    }
    case FAM_NAN:
      return __longlong_as_double(0x7ff8000000000000LL);
    case FAM_BOX: {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < MAXD; ++i)
        if (i < d) s = __fma_rn(x[i], x[i], s);
      return pow(s, __dmul_rn(0.5, D.c));
    }
    case FAM_FUN6: {
      if (MAXD < 6) return 0.0;
      const double t = __dmul_rn(__dmul_rn(pow(x[2], x[4]), x[3]), x[4]);
      const double q = __dadd_rn(__dadd_rn(__dmul_rn(x[0], x[1]), __ddiv_rn(t, __dadd_rn(1.0, x[0]))),
                                 __dmul_rn(x[5], x[5]));
      return __dmul_rn(D.c, q);
    }
  }
  return 0.0;
}

// Functor adapter used by the kernels for the C ABI families.
struct FamilyFn {
  template <int MAXD>
  __device__ __forceinline__ double eval(const IntegralDesc& D, const double* x) const {
    return family_eval<MAXD>(D, x);
  }
  __device__ __forceinline__ bool separable(const IntegralDesc& D) const { return family_separable(D.family); }
  __device__ __forceinline__ double factor(const IntegralDesc& D, int k, double x) const {
    return family_factor(D, k, x);
  }
};

}  // namespace pg
