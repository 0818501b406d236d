// The reference's own region-evaluation code, compiled from the reference
// sources for sm_103a into a cubin (oracle/_ref/ref_phase1.cubin) by
// oracle/ref/build_ref.sh.  TEST INFRASTRUCTURE: it produces the golden
// per-region values the library is checked against.
//
// Each ref_phase1_d<D> kernel is the body of INTEGRATE_GPU_PHASE1
// (cuda/pagani/quad/GPUquad/Phases.cuh:365-404): one 64-thread block per
// region calls the reference's INIT_REGION_POOL / SampleRegionBlock unchanged
// and writes the estimate, error and split axis.  The integrand is the
// library's family functor (the same code the library evaluates), called the
// way the reference calls integrands (gpu::apply with ndim scalars).  The
// rule tables come from the reference's Rule::Init via the golden file, so no
// host code of the reference is needed where the cubin runs.
#include "cuda/pagani/quad/GPUquad/Phases.cuh"
#include "gpuintegration_gb300/csrc/pg_integrands.cuh"

template <int NDIM>
struct RefFamily {
  pg::IntegralDesc D;
  template <class... Ts>
  __device__ double operator()(Ts... xs) const {
    const double x[NDIM] = {xs...};
    return pg::family_eval<(NDIM <= 8 ? 8 : 16)>(D, x);
  }
};

template <int NDIM>
__device__ void ref_phase1_body(const RefFamily<NDIM>* f, double* left, double* len, size_t n, double* est,
                                double* err, int* bis, double* gpuG, double* wt, double* scale, double* norm,
                                int* gindex, double* lows, double* highs, double* generators) {
  Structures<double> cm;
  cm.gpuG = gpuG;
  cm.cRuleWt = wt;
  cm.GPUScale = scale;
  cm.GPUNorm = norm;
  cm.gpuGenPermGIndex = gindex;
  __shared__ Region<NDIM> sRegionPool[1];
  __shared__ GlobalBounds sBound[NDIM];
  quad::Func_Evals<NDIM> fevals;
  quad::INIT_REGION_POOL<RefFamily<NDIM>, double, NDIM, 64, 0>(const_cast<RefFamily<NDIM>*>(f), left, len, n, cm,
                                                               sRegionPool, sBound, lows, highs, generators, fevals);
  if (threadIdx.x == 0) {
    bis[blockIdx.x] = sRegionPool[0].result.bisectdim;
    est[blockIdx.x] = sRegionPool[0].result.avg;
    err[blockIdx.x] = sRegionPool[0].result.err;
  }
}

#define REF_PHASE1(D)                                                                                       \
  extern "C" __global__ void ref_phase1_d##D(const RefFamily<D>* f, double* left, double* len, size_t n,    \
                                             double* est, double* err, int* bis, double* gpuG, double* wt,   \
                                             double* scale, double* norm, int* gindex, double* lows,        \
                                             double* highs, double* generators) {                           \
    ref_phase1_body<D>(f, left, len, n, est, err, bis, gpuG, wt, scale, norm, gindex, lows, highs, generators); \
  }

REF_PHASE1(2)
REF_PHASE1(3)
REF_PHASE1(4)
REF_PHASE1(5)
REF_PHASE1(6)
REF_PHASE1(7)
REF_PHASE1(8)
REF_PHASE1(9)
REF_PHASE1(10)
