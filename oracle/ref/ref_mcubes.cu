// The reference's own m-Cubes sampling kernels, compiled from the reference
// sources for sm_103a into a cubin (oracle/_ref/ref_mcubes.cubin) by
// oracle/ref/build_ref.sh.  TEST INFRASTRUCTURE: tests/golden/ref_mcubes_runner.py
// runs them in the reference's iteration loop to produce golden results.
//
// Explicit instantiations, unchanged, of cuda_mcubes::vegas_kernel (adapting
// iterations, vegasT.cuh:396-485) and vegas_kernelF (frozen grid,
// vegasT.cuh:487-614) with the reference's Curand_generator, for an
// integrand that evaluates the library's families (the same code the library
// evaluates) at d = 3, 4, 6.
#include "cuda/mcubes/vegasT.cuh"
#include "gpuintegration_gb300/csrc/pg_integrands.cuh"

template <int NDIM>
struct RefMcubes {
  pg::IntegralDesc D;
  template <class... Ts>
  __device__ double operator()(Ts... xs) const {
    const double x[NDIM] = {xs...};
    return pg::family_eval<(NDIM <= 8 ? 8 : 16)>(D, x);
  }
};

#define REF_MCUBES(D)                                                                                              \
  template __global__ void cuda_mcubes::vegas_kernel<RefMcubes<D>, D, false, Curand_generator>(                   \
      RefMcubes<D>*, int, int, double, double, double*, double, double*, double*, double*, double*, int, int,     \
      double, double, double, int, uint32_t, int, unsigned int, double*, FuncEval<D>*);                           \
  template __global__ void cuda_mcubes::vegas_kernelF<RefMcubes<D>, D, Curand_generator>(                         \
      RefMcubes<D>*, int, int, double, double, double*, double, double*, double*, double*, double*, int, int,     \
      double, double, double, int, uint32_t, int, unsigned int);

REF_MCUBES(3)
REF_MCUBES(4)
REF_MCUBES(6)
