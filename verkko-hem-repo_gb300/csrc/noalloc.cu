// glgpu_dot_noalloc: a deterministic FP64 dot product of two device vectors that
// allocates nothing.
//
// It exists for callers that cannot call cudaMalloc at the point where they need a
// norm: code that runs while a stream is being captured into a CUDA graph, code that
// must not take the allocator's locks or cause implicit device synchronisation in a
// tight loop, and host frameworks that own all device memory themselves and hand
// this library only the buffers they allocated.  Such callers pass their input
// vectors and a one-double device output; the partial sums that the two-pass
// reduction needs live in a fixed array of this file instead of in a context.
//
// Limits and sharing:
//  - at most kNoAllocMaxSegments segments of kNoAllocSegLen scalars, i.e. n <= 16,777,216;
//    larger n is rejected with GLGPU_ERR_ARG;
//  - the scratch array is one per device for the whole process and keeps the last
//    call's contents; every call overwrites exactly the partials it then reads, so
//    nothing has to start at zero, but calls whose work overlaps on the GPU (different
//    streams, or different host threads without ordering) race on it and must be
//    serialised by the caller;
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call before any
//    stream capture begins.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "glgpu.h"
#include "glgpu_internal.h"

namespace glgpu
{
namespace
{
constexpr int kNoAllocSegLen = 1024;
constexpr int kNoAllocMaxSegments = 16384;
constexpr int kNoAllocThreads = 256;
constexpr int kMaxDevices = 64;

// partial sums of the two-pass reduction: the only scratch this entry point uses
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxSegments];

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kMaxDevices] = {};

__global__ void __launch_bounds__(kNoAllocThreads) k_noalloc_partial(const double *__restrict__ x,
                                                                     const double *__restrict__ y, int64_t n,
                                                                     double *__restrict__ partial)
{
  __shared__ double sh[kNoAllocThreads / 32];
  const int64_t b = static_cast<int64_t>(blockIdx.x) * kNoAllocSegLen;
  const int64_t e = (b + kNoAllocSegLen < n) ? b + kNoAllocSegLen : n;
  double acc = 0.0;
  for (int64_t i = b + threadIdx.x; i < e; i += kNoAllocThreads) acc += x[i] * y[i];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0)
    {
      double s = 0.0;
      for (int w = 0; w < kNoAllocThreads / 32; ++w) s += sh[w];
      partial[blockIdx.x] = s;
    }
}

// one CTA: lanes take partials in a fixed order, then a fixed shuffle/shared tree
__global__ void __launch_bounds__(kNoAllocThreads) k_noalloc_final(const double *__restrict__ partial, int nseg,
                                                                   double *__restrict__ out)
{
  __shared__ double sh[kNoAllocThreads / 32];
  double acc = 0.0;
  for (int s = threadIdx.x; s < nseg; s += kNoAllocThreads) acc += partial[s];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0)
    {
      double s = 0.0;
      for (int w = 0; w < kNoAllocThreads / 32; ++w) s += sh[w];
      *out = s;
    }
}

// device address of the scratch array for the current device (looked up once)
glgpu_status scratch_for_current_device(double **ptr)
{
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(GLGPU_ERR_CUDA, std::string("glgpu_dot_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(GLGPU_ERR_ARG, "glgpu_dot_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev])
    {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess || !p)
        return set_error(GLGPU_ERR_CUDA,
                         std::string("glgpu_dot_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
  *ptr = g_noalloc_ptr[dev];
  return GLGPU_OK;
}
} // namespace
} // namespace glgpu

using namespace glgpu;

extern "C" glgpu_status glgpu_dot_noalloc(const double *x, const double *y, int64_t n, double *result, void *stream)
{
  if (!x || !y || !result) return set_error(GLGPU_ERR_ARG, "glgpu_dot_noalloc: NULL device pointer");
  if (n < 0) return set_error(GLGPU_ERR_ARG, "glgpu_dot_noalloc: negative length");
  const int64_t max_n = static_cast<int64_t>(kNoAllocMaxSegments) * kNoAllocSegLen;
  if (n > max_n)
    return set_error(GLGPU_ERR_ARG, "glgpu_dot_noalloc: n = " + std::to_string(n) + " exceeds the maximum " +
                                        std::to_string(max_n) + " (fixed scratch of " +
                                        std::to_string(kNoAllocMaxSegments) + " partial sums)");
  double *scratch = nullptr;
  glgpu_status s = scratch_for_current_device(&scratch);
  if (s != GLGPU_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nseg = static_cast<int>((n + kNoAllocSegLen - 1) / kNoAllocSegLen);
  if (nseg > 0) k_noalloc_partial<<<nseg, kNoAllocThreads, 0, st>>>(x, y, n, scratch);
  k_noalloc_final<<<1, kNoAllocThreads, 0, st>>>(scratch, nseg, result);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GLGPU_ERR_CUDA, std::string("glgpu_dot_noalloc: launch: ") + cudaGetErrorString(e));
  return GLGPU_OK;
}
