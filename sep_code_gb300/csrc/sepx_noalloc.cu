// sepx_noalloc.cu -- the FP64 dot product of two device float vectors with its
// scratch in a fixed, statically sized device array instead of memory the
// library allocates.
//
// For callers that cannot let a library allocate device memory: services that
// reserve their whole device-memory budget at start-up and forbid any later
// cudaMalloc, or host applications whose own pool owns every device
// allocation.  They pass the inputs and the output; this file never calls
// cudaMalloc, cudaFree or any allocating routine.
//
// Limits and sharing (also stated in include/sepx.h):
//  * at most kNoAllocMaxElems elements per call (256 KB of FP64 partials: one
//    per block of kChunk elements); larger calls are rejected with an error;
//  * every GPU that loads the library holds the 256 KB array until exit;
//  * all calls share the array, which keeps the last call's partials; a call
//    writes every partial it reads before reading it, so nothing has to start
//    at zero; calls that overlap on the GPU (different streams, or different
//    host threads) race on it and must be serialised by the caller;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/sepx.h"
#include "sepx_common.h"

namespace sepx {
namespace {

constexpr int kChunk = 8192;                  // elements per block
constexpr int kThreadsNA = 256;
constexpr long long kMaxBlocks = 32768;       // 32768 partials x 8 B = 256 KB
constexpr long long kNoAllocMaxElems = kMaxBlocks * kChunk;   // 268,435,456
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_dot_scratch[kMaxBlocks];

// The array's device address, looked up once per device.  Entries are
// atomic: two host threads making the first call on one device at the same
// time both look it up and store the same value.  The address belongs to the
// device's primary context: after cudaDeviceReset, or from another context
// on the same device, it is not valid (stated in include/sepx.h).
std::atomic<double *> g_scratch_addr[kMaxDevices] = {};

__device__ __forceinline__ double block_sum_na(double v) {
  __shared__ double red[kThreadsNA / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  v = 0.0;
  if (w == 0) {
    v = (l < kThreadsNA / 32) ? red[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// block b sums a[i]*b[i] over its chunk [b*kChunk, (b+1)*kChunk) into partials[b]
__global__ void __launch_bounds__(kThreadsNA)
    noalloc_dot_partial(const float *__restrict__ a, const float *__restrict__ b, long long n,
                        double *__restrict__ partials) {
  const long long base = (long long)blockIdx.x * kChunk;
  const long long end = (base + kChunk < n) ? base + kChunk : n;
  double acc = 0.0;
  for (long long i = base + threadIdx.x; i < end; i += kThreadsNA)
    acc += (double)a[i] * (b ? (double)b[i] : 1.0);
  acc = block_sum_na(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kThreadsNA)
    noalloc_dot_final(const double *__restrict__ partials, int nb, double *__restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < nb; i += kThreadsNA) acc += partials[i];
  acc = block_sum_na(acc);
  if (threadIdx.x == 0) *out = acc;
}

}  // namespace
}  // namespace sepx

using namespace sepx;

extern "C" int sepx_dot_f32_noalloc(const float *a, const float *b, long long n, double *d_result,
                                    void *stream) {
  if (n < 0 || !d_result || (n > 0 && !a))
    return set_error("sepx_dot_f32_noalloc: invalid arguments");
  if (n > kNoAllocMaxElems)
    return set_error("sepx_dot_f32_noalloc: n=%lld exceeds the fixed scratch limit of %lld elements",
                     n, kNoAllocMaxElems);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error("sepx_dot_f32_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error("sepx_dot_f32_noalloc: device %d out of range", dev);
  double *scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!scratch) {   // once per device, with that device current
    e = cudaGetSymbolAddress((void **)&scratch, g_dot_scratch);
    if (e != cudaSuccess || !scratch)
      return set_error("sepx_dot_f32_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_scratch_addr[dev].store(scratch, std::memory_order_release);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = (int)((n + kChunk - 1) / kChunk);
  if (nb > 0) noalloc_dot_partial<<<nb, kThreadsNA, 0, st>>>(a, b, n, scratch);
  noalloc_dot_final<<<1, kThreadsNA, 0, st>>>(scratch, nb, d_result);
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_error("sepx_dot_f32_noalloc: launch: %s", cudaGetErrorString(e));
  return 0;
}

extern "C" long long sepx_dot_f32_noalloc_max_elems(void) { return kNoAllocMaxElems; }
