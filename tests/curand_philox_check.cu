// Prints cuRAND's Philox4x32-10 block function for the counters/keys given on
// the command line (4 + 2 hex words per case), one output line per case.  Used
// by tests/test_gpu_mcubes.py to check the library's own Philox against cuRAND.
#include <cstdio>
#include <cstdlib>
#include <curand_kernel.h>

__global__ void k(const uint4* c, const uint2* key, uint4* out, int n) {
  int i = threadIdx.x;
  if (i < n) out[i] = curand_Philox4x32_10(c[i], key[i]);
}

int main(int argc, char** argv) {
  const int n = (argc - 1) / 6;
  uint4 hc[64];
  uint2 hk[64];
  for (int i = 0; i < n; ++i) {
    hc[i] = make_uint4(strtoul(argv[1 + 6 * i], 0, 16), strtoul(argv[2 + 6 * i], 0, 16),
                       strtoul(argv[3 + 6 * i], 0, 16), strtoul(argv[4 + 6 * i], 0, 16));
    hk[i] = make_uint2(strtoul(argv[5 + 6 * i], 0, 16), strtoul(argv[6 + 6 * i], 0, 16));
  }
  uint4 *dc, *dout;
  uint2* dk;
  cudaMalloc(&dc, sizeof hc);
  cudaMalloc(&dk, sizeof hk);
  cudaMalloc(&dout, sizeof hc);
  cudaMemcpy(dc, hc, sizeof hc, cudaMemcpyHostToDevice);
  cudaMemcpy(dk, hk, sizeof hk, cudaMemcpyHostToDevice);
  k<<<1, 64>>>(dc, dk, dout, n);
  uint4 ho[64];
  cudaMemcpy(ho, dout, sizeof ho, cudaMemcpyDeviceToHost);
  for (int i = 0; i < n; ++i) printf("%08x %08x %08x %08x\n", ho[i].x, ho[i].y, ho[i].z, ho[i].w);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
