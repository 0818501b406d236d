// The reference's own iteration-stage kernels, compiled from the reference
// sources for sm_103a into a cubin (oracle/_ref/ref_stages.cubin) by
// oracle/ref/build_ref.sh.  TEST INFRASTRUCTURE: with ref_phase1.cubin they
// run the reference's PAGANI iteration on the GPU to produce golden
// per-iteration data (tests/golden/make_ref_iter_golden.py).
//
// Explicit instantiations, unchanged, of:
//   quad::RefineError<double>            two-level error and rel-err classification
//                                        (cuda/pagani/quad/GPUquad/Phases.cuh:219-268)
//   alignRegions<double, D>               compaction of the active regions
//                                        (cuda/pagani/quad/GPUquad/Sub_region_filter.cuh:8-47)
//   divideIntervalsGPU<double, D>         bisection into the children
//                                        (cuda/pagani/quad/GPUquad/Sub_region_splitter.cuh:8-46)
// for D = 2..10.  The host side finds them by name through the driver API.
#include "cuda/pagani/quad/GPUquad/Phases.cuh"
#include "cuda/pagani/quad/GPUquad/Sub_region_filter.cuh"
#include "cuda/pagani/quad/GPUquad/Sub_region_splitter.cuh"

template __global__ void quad::RefineError<double>(double*, double*, double*, double*, double*, double*, size_t,
                                                   double, int);

#define REF_STAGES(D)                                                                                             \
  template __global__ void alignRegions<double, D>(double*, double*, double*, double*, double*, double*, double*, \
                                                   int*, double*, double*, double*, int*, size_t, size_t, int);   \
  template __global__ void divideIntervalsGPU<double, D>(double*, double*, double*, double*, int*, size_t, int);

REF_STAGES(2)
REF_STAGES(3)
REF_STAGES(4)
REF_STAGES(5)
REF_STAGES(6)
REF_STAGES(7)
REF_STAGES(8)
REF_STAGES(9)
REF_STAGES(10)
