// Device check of pg::mul_rn_int (the integer-pipe double multiply of the
// evaluation kernel) against the FP64 multiply __dmul_rn, bit for bit, on
// random bit patterns, on products with few significand bits (exact products
// and ties), and across the exponent range (overflow, underflow, subnormals,
// zeros, infinities, NaNs).  Prints the mismatch count; exit status 1 on any.
#include <cstdio>
#include <cstdint>

#include "../../gpuintegration_gb300/csrc/pg_common.cuh"

__device__ __forceinline__ uint64_t mix(uint64_t x) {  // splitmix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void check(uint64_t n, uint64_t seed, unsigned long long* bad, unsigned long long* fast) {
  unsigned long long b = 0, f = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t r1 = mix(seed ^ (2 * i)), r2 = mix(seed ^ (2 * i + 1));
    double a, c;
    switch (i % 3) {
      case 0:  // any bit patterns
        a = __longlong_as_double((long long)r1);
        c = __longlong_as_double((long long)r2);
        break;
      case 1: {  // few significand bits: exact products and halfway cases
        const int k1 = 1 + (int)(r1 % 53), k2 = 1 + (int)(r2 % 53);
        const double m1 = (double)((r1 >> (64 - k1)) | 1ull), m2 = (double)((r2 >> (64 - k2)) | 1ull);
        a = scalbn(m1, (int)((r1 >> 8) % 121) - 60 - k1);
        c = scalbn(m2, (int)((r2 >> 8) % 121) - 60 - k2);
        if (r1 & 1) a = -a;
        break;
      }
      default: {  // the whole exponent range
        a = scalbn(1.0 + (double)(r1 >> 12) * 0x1p-52, (int)(r1 % 2100) - 1075);
        c = scalbn(1.0 + (double)(r2 >> 12) * 0x1p-52, (int)(r2 % 2100) - 1075);
        if ((r2 >> 7) % 7 == 0) c = 0.0;
        if ((r2 >> 11) % 97 == 0) c = __longlong_as_double(0x7ff0000000000000ll);
        break;
      }
    }
    bool ok;
    const unsigned long long got =
        pg::mul_rn_bits((unsigned long long)__double_as_longlong(a), (unsigned long long)__double_as_longlong(c), &ok);
    const unsigned long long want = (unsigned long long)__double_as_longlong(__dmul_rn(a, c));
    if (ok) {
      ++f;
      if (got != want) ++b;
    }
    // the full function (fast path or FP64 fallback) must match too, NaNs as NaNs
    const double full = pg::mul_rn_int(a, c), ref = __dmul_rn(a, c);
    if (!(full != full && ref != ref) && __double_as_longlong(full) != __double_as_longlong(ref)) ++b;
  }
  atomicAdd(bad, b);
  atomicAdd(fast, f);
}

int main() {
  unsigned long long *d, h[2] = {0, 0};
  cudaMalloc(&d, 16);
  cudaMemset(d, 0, 16);
  const uint64_t n = 1ull << 30;
  check<<<152 * 16, 256>>>(n, 0x5EEDull, d, d + 1);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    std::printf("FAIL cuda error\n");
    return 2;
  }
  cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
  std::printf("%s products %llu integer-path %llu mismatches %llu\n", h[0] ? "FAIL" : "PASS",
              (unsigned long long)n, h[1], h[0]);
  return h[0] ? 1 : 0;
}
