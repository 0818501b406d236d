// Common device/host helpers of the GB300 PAGANI library.
//
// The library is compiled with --fmad=false: every fused multiply-add in device
// code is written out with __fma_rn, so the rounding of each expression is
// fixed by the source and does not depend on compiler contraction choices.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cmath>
#include <string>

namespace pg {

constexpr int kNRules = 5;  // basic rule + 4 null rules (cuda/pagani/quad/quad.h:65)
constexpr int kNSets = 9;   // generator sets of the degree-9 rule (Rule.cuh:404-405)
constexpr int kMaxDim = 16;
constexpr int kMaxNdim = 12;        // largest ndim the library instantiates tables for
constexpr int kCodesPerDim = 11;    // 0, +G0..+G4, -G0..-G4

// Deterministic reduction geometry: chunk of 2048 elements, 256 threads x 8
// items, item k of thread t is element chunk*2048 + k*256 + t.
constexpr int kRedThreads = 256;
constexpr int kRedItems = 8;
constexpr int kChunk = kRedThreads * kRedItems;

// Opts `kernel` into `bytes` of dynamic shared memory on the current device,
// once per device (bit d of `done`); safe from several host threads.
template <class Kernel>
inline cudaError_t ensure_dynamic_smem(Kernel kernel, int bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_release);
  return e;
}

// ---------------------------------------------------------------------------
// Double-precision multiply on the integer pipe.  GB300 executes FP64 at 2
// lanes per SM per clock, which bounds region evaluation, while its integer
// units run 32x wider.  mul_rn_int(a, b) returns exactly __dmul_rn(a, b)
// (IEEE 754 binary64 product, round to nearest, ties to even): normal
// operands with a normal product are multiplied in integer arithmetic (the
// 106-bit product of the significands, normalised and rounded), a zero times
// a finite value gives the signed zero, and every other case (subnormals,
// infinities, NaNs, overflow, underflow) takes the FP64 multiply.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ unsigned long long mul_hi_u64(unsigned long long a, unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
#endif
}

// Fast-path product; *ok is false when the operands need the FP64 multiply.
__host__ __device__ __forceinline__ unsigned long long mul_rn_bits(unsigned long long A, unsigned long long B,
                                                                   bool* ok) {
  const unsigned long long sign = (A ^ B) & 0x8000000000000000ull;
  const unsigned ea = (unsigned)(A >> 52) & 0x7ffu, eb = (unsigned)(B >> 52) & 0x7ffu;
  const unsigned long long fa = A & 0x000fffffffffffffull, fb = B & 0x000fffffffffffffull;
  const bool za = ea == 0 && fa == 0, zb = eb == 0 && fb == 0;
  if ((za && eb != 0x7ffu) || (zb && ea != 0x7ffu)) {  // 0 * finite (either order)
    *ok = true;
    return sign;
  }
  int e = (int)ea + (int)eb - 1023;  // biased exponent of a product significand in [1, 2)
  if (ea - 1u >= 2046u || eb - 1u >= 2046u || e < 1 || e > 2046) {
    *ok = false;
    return 0;
  }
  const unsigned long long ma = fa | 0x0010000000000000ull, mb = fb | 0x0010000000000000ull;
  const unsigned long long lo = ma * mb, hi = mul_hi_u64(ma, mb);  // P = hi * 2^64 + lo in [2^104, 2^106)
  unsigned long long m, rest, half;
  if (hi >> 41) {  // P >= 2^105
    m = (hi << 11) | (lo >> 53);
    rest = lo & 0x001fffffffffffffull;
    half = 0x0010000000000000ull;
    e += 1;
  } else {
    m = (hi << 12) | (lo >> 52);
    rest = lo & 0x000fffffffffffffull;
    half = 0x0008000000000000ull;
  }
  if (rest > half || (rest == half && (m & 1ull))) ++m;
  if (m >> 53) {  // rounded up to 2^53
    m >>= 1;
    e += 1;
  }
  if (e > 2046) {
    *ok = false;
    return 0;
  }
  *ok = true;
  return sign | ((unsigned long long)e << 52) | (m & 0x000fffffffffffffull);
}

__device__ __forceinline__ double mul_rn_int(double a, double b) {
  bool ok;
  const unsigned long long r =
      mul_rn_bits((unsigned long long)__double_as_longlong(a), (unsigned long long)__double_as_longlong(b), &ok);
  return ok ? __longlong_as_double((long long)r) : __dmul_rn(a, b);
}

// Neumaier-compensated pair (sum, correction).
struct NS {
  double s, c;
};

__host__ __device__ inline NS ns_zero() { return NS{0.0, 0.0}; }

// |a| >= |b| on the integer pipe: for doubles that are not NaN, the order of
// the bit patterns with the sign bit cleared is the order of the magnitudes.
// (With a NaN operand the sum is NaN whichever operand is taken as larger.)
__device__ __forceinline__ bool mag_ge(double a, double b) {
  const unsigned long long m = 0x7fffffffffffffffull;
  return ((unsigned long long)__double_as_longlong(a) & m) >= ((unsigned long long)__double_as_longlong(b) & m);
}

// merge(a, b): t = a.s + b.s; the rounding error of that addition goes into
// the correction term; value = s + c.
// The larger-magnitude operand is selected first (compared on the integer
// pipe), so the error term costs two FP64 additions rather than both
// branches' four.
__device__ __forceinline__ NS ns_merge(NS a, NS b) {
  const double t = __dadd_rn(a.s, b.s);
  const bool ge = mag_ge(a.s, b.s);
  const double big = ge ? a.s : b.s, small = ge ? b.s : a.s;
  const double e = __dadd_rn(__dadd_rn(big, -t), small);
  return NS{t, __dadd_rn(__dadd_rn(a.c, b.c), e)};
}

// ns_merge(a, NS{x, 0.0}) with one addition fewer, bit for bit: a correction
// term is never -0.0 (it starts at +0.0, and an exact zero sum rounds to
// +0.0), so a.c + 0.0 is a.c.
__device__ __forceinline__ NS ns_add(NS a, double x) {
  const double t = __dadd_rn(a.s, x);
  const bool ge = mag_ge(a.s, x);
  const double big = ge ? a.s : x, small = ge ? x : a.s;
  const double e = __dadd_rn(__dadd_rn(big, -t), small);
  return NS{t, __dadd_rn(a.c, e)};
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
