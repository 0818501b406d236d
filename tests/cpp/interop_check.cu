// Compile-only check: include/pagani_gb300.cuh together with headers that
// declare the reference's numint::integration_result and quad::Volume under
// the reference's include guards (as its integrand-side headers such as
// common/cuda/Interp1D.cuh do through cuda/pagani/quad/quad.h), in either
// order.  REFERENCE_FIRST selects the order.
#include <cstddef>

#define DECLARE_REFERENCE_TYPES                                                     \
  namespace numint {                                                                \
  struct integration_result {                                                       \
    double estimate = 0.;                                                           \
    double errorest = 0.;                                                           \
    size_t neval = 0;                                                               \
    size_t nregions = 0;                                                            \
    size_t nFinishedRegions = 0;                                                    \
    int status = -1;                                                                \
    int lastPhase = -1;                                                             \
    double chi_sq = 0.;                                                             \
    size_t iters = 0;                                                               \
  };                                                                                \
  }                                                                                 \
  namespace quad {                                                                  \
  template <typename T, int NDIM>                                                   \
  struct Volume {                                                                   \
    T lows[NDIM] = {0.0};                                                           \
    T highs[NDIM];                                                                  \
    Volume() {                                                                      \
      for (T& x : highs) x = 1.0;                                                   \
    }                                                                               \
  };                                                                                \
  }

#if REFERENCE_FIRST
#define GPUINTEGRATION_COMMON_INTEGRATION_RESULT_H
#define CUDACUHRE_QUAD_GPUQUAD_VOLUME_CUH
DECLARE_REFERENCE_TYPES
#include "pagani_gb300.cuh"
#else
#include "pagani_gb300.cuh"
#ifndef GPUINTEGRATION_COMMON_INTEGRATION_RESULT_H
#error "the C++ layer must define the reference's result include guard"
#endif
#ifndef CUDACUHRE_QUAD_GPUQUAD_VOLUME_CUH
#error "the C++ layer must define the reference's Volume include guard"
#endif
#endif

struct Product2 {
  __device__ double operator()(double x, double y) const { return x * y; }
};

int run() {
  Workspace<double, 2> ws;
  quad::Volume<double, 2> vol;
  numint::integration_result r = ws.integrate(Product2{}, 1e-6, 0.0, vol);
  numint::integration_result m = cuda_mcubes::integrate<Product2, 2>(Product2{}, 1e-3, 0.0, 1e5, &vol);
  return r.status + m.status;
}
