// pg_reduce_sum_noalloc: the compensated FP64 sum of a device array, for
// callers that must not allocate device memory.
//
// pg_reduce_sum needs a context, and a context owns a growing device pool.
// Some callers cannot have that: a host program whose device memory is
// entirely reserved by another allocator (a framework's caching allocator,
// a preallocated arena) so that a cudaMalloc of ours would fail or fragment
// it, or a latency-critical loop that cannot afford cudaMalloc's implicit
// device synchronisation.  This entry point takes the caller's device input
// and output and keeps its only scratch -- one Neumaier partial per
// 2048-element chunk -- in a fixed-size array that is part of this library's
// device image.  It calls no cudaMalloc, cudaFree or allocating library
// routine.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/pagani_gb300.h"
#include "pg_kernels.cuh"

namespace {

constexpr uint64_t kMaxChunks = PG_REDUCE_NOALLOC_MAX_N / pg::kChunk;
static_assert(PG_REDUCE_NOALLOC_MAX_N % pg::kChunk == 0, "limit must be whole chunks");

// Scratch of every call on a device (2 MB per device that loads the library,
// held until the process exits).  Each call overwrites the partials it reads,
// so nothing has to be cleared between calls.
static __device__ __align__(256) pg::NS g_partials[kMaxChunks];

// Device address of g_partials, looked up once per device.  In host code the
// name g_partials is only a host-side stand-in, never a device address.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
pg::NS* g_addr[kMaxDevices] = {};

int scratch_for_current_device(pg::NS** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PG_CUDA_ERROR;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_partials);
    if (e != cudaSuccess || !p) return PG_CUDA_ERROR;
    g_addr[dev] = static_cast<pg::NS*>(p);
  }
  *out = g_addr[dev];
  return PG_OK;
}

}  // namespace

extern "C" int pg_reduce_sum_noalloc(const double* d_x, uint64_t n, double* d_out, void* stream) {
  if (!d_out || (n && !d_x)) return PG_BAD_ARG;
  if (n > PG_REDUCE_NOALLOC_MAX_N) return PG_BAD_ARG;
  pg::NS* scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch);
  if (rc != PG_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const uint64_t nch = (n + pg::kChunk - 1) / pg::kChunk;
  if (nch) pg::sum_chunks_kernel<<<(unsigned)nch, pg::kRedThreads, 0, s>>>(d_x, n, scratch);
  pg::sum_final_kernel<<<1, pg::kRedThreads, 0, s>>>(scratch, nch, d_out);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_CUDA_ERROR;
}
