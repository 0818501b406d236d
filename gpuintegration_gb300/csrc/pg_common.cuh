// Common device/host helpers of the GB300 PAGANI library.
//
// The library is compiled with --fmad=false: every fused multiply-add in device
// code is written out with __fma_rn, so the rounding of each expression is
// fixed by the source and does not depend on compiler contraction choices.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>

namespace pg {

constexpr int kNRules = 5;  // basic rule + 4 null rules (cuda/pagani/quad/quad.h:65)
constexpr int kNSets = 9;   // generator sets of the degree-9 rule (Rule.cuh:404-405)
constexpr int kMaxDim = 16;
constexpr int kMaxNdim = 12;        // largest ndim the library instantiates tables for
constexpr int kCodesPerDim = 11;    // 0, +G0..+G4, -G0..-G4
constexpr int kEvalWarps = 8;       // warps (regions in flight) per evaluation CTA

// Deterministic reduction geometry: chunk of 2048 elements, 256 threads x 8
// items, item k of thread t is element chunk*2048 + k*256 + t.
constexpr int kRedThreads = 256;
constexpr int kRedItems = 8;
constexpr int kChunk = kRedThreads * kRedItems;

// Neumaier-compensated pair (sum, correction).
struct NS {
  double s, c;
};

__host__ __device__ inline NS ns_zero() { return NS{0.0, 0.0}; }

// merge(a, b): t = a.s + b.s; the rounding error of that addition goes into
// the correction term; value = s + c.
__device__ __forceinline__ NS ns_merge(NS a, NS b) {
  const double t = __dadd_rn(a.s, b.s);
  const double e = (fabs(a.s) >= fabs(b.s)) ? __dadd_rn(__dadd_rn(a.s, -t), b.s) : __dadd_rn(__dadd_rn(b.s, -t), a.s);
  return NS{t, __dadd_rn(__dadd_rn(a.c, b.c), e)};
}

__device__ __forceinline__ NS ns_shfl_down(NS v, int off) {
  return NS{__shfl_down_sync(0xffffffffu, v.s, off), __shfl_down_sync(0xffffffffu, v.c, off)};
}

// Tree over the 256 threads of a block: shuffle-down offsets 16..1 inside each
// warp, then offsets 4,2,1 over the 8 warp results.  Result valid in thread 0.
// `scratch` needs 8 NS per quantity.
__device__ __forceinline__ NS ns_block_tree(NS v, NS* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    const NS o = ns_shfl_down(v, off);
    if (lane < off) v = ns_merge(v, o);
  }
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < 8) ? scratch[lane] : ns_zero();
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1) {
      const NS o = ns_shfl_down(v, off);
      if (lane < off) v = ns_merge(v, o);
    }
  }
  __syncthreads();
  return v;
}

__device__ __forceinline__ double ns_value(NS v) { return __dadd_rn(v.s, v.c); }

}  // namespace pg
