// sepx_blas.cu -- BLAS-1 on device-resident float vectors for the operator
// and solver layer (my_vector / hypercube_float, Born/hypercube_float.cpp:
// 123-223): products accumulated in FP64 like the reference's dot / sum, the
// rest in FP32 with the reference's double scale factors.
//
// Reductions are deterministic: a fixed grid writes one FP64 partial per block
// into scratch and a single block sums the partials in a fixed order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sepx_blas.h"

namespace sepx {

constexpr int kDotBlocks = 4 * 152;   // 4 CTAs per SM on a 152-SM GB300
constexpr int kDotThreads = 256;

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[kDotThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  v = 0.0;
  if (w == 0) {
    v = (l < kDotThreads / 32) ? red[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// partials[b] = sum over the grid-stride elements of block b of a[i]*b[i]
// (b == nullptr: sum of a[i])
__global__ void __launch_bounds__(kDotThreads)
    dot_partial_kernel(const float *__restrict__ a, const float *__restrict__ b, long long n,
                       double *__restrict__ partials) {
  double acc = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    acc += (double)a[i] * (b ? (double)b[i] : 1.0);
  acc = block_sum(acc);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kDotThreads)
    sum_partials_kernel(const double *__restrict__ partials, int np, double *__restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc += partials[i];
  acc = block_sum(acc);
  if (threadIdx.x == 0) *out = acc;
}

__global__ void fill_kernel(float *x, long long n, float v) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) x[i] = v;
}

// y = y*a + x*b  (hypercube_float::scale_add(a, x, b): vals = vals*a + b*x,
// Born/hypercube_float.cpp:437-443; evaluated in double as the reference does)
__global__ void scale_add_kernel(float *y, const float *x, long long n, double a, double b) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = (float)((double)y[i] * a + b * (double)x[i]);
}

// y = x1*a + x2*b  (the four-argument scale_add, :368-378)
__global__ void scale_add2_kernel(float *y, const float *x1, const float *x2, long long n, double a,
                                  double b) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = (float)((double)x1[i] * a + (double)x2[i] * b);
}

__global__ void scale_kernel(float *y, long long n, double a) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = (float)((double)y[i] * a);
}

__global__ void add_kernel(float *y, const float *x, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = y[i] + x[i];
}

__global__ void mult_kernel(float *y, const float *x, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    y[i] = y[i] * x[i];
}

// uniform(-0.5, 0.5) from a counter hash (splitmix64) of (seed, index)
__global__ void random_kernel(float *y, long long n, unsigned long long seed) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    y[i] = (float)((double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5);
  }
}

static int grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 2048 ? (g < 1 ? 1 : g) : 2048);
}

cudaError_t vec_dot(const float *a, const float *b, long long n, double *partials, double *d_out,
                    cudaStream_t st) {
  dot_partial_kernel<<<kDotBlocks, kDotThreads, 0, st>>>(a, b, n, partials);
  sum_partials_kernel<<<1, kDotThreads, 0, st>>>(partials, kDotBlocks, d_out);
  return cudaGetLastError();
}

int vec_dot_scratch_doubles() { return kDotBlocks; }

cudaError_t vec_fill(float *x, long long n, float v, cudaStream_t st) {
  fill_kernel<<<grid_for(n), 256, 0, st>>>(x, n, v);
  return cudaGetLastError();
}
cudaError_t vec_scale(float *y, long long n, double a, cudaStream_t st) {
  scale_kernel<<<grid_for(n), 256, 0, st>>>(y, n, a);
  return cudaGetLastError();
}
cudaError_t vec_scale_add(float *y, const float *x, long long n, double a, double b, cudaStream_t st) {
  scale_add_kernel<<<grid_for(n), 256, 0, st>>>(y, x, n, a, b);
  return cudaGetLastError();
}
cudaError_t vec_scale_add2(float *y, const float *x1, const float *x2, long long n, double a, double b,
                           cudaStream_t st) {
  scale_add2_kernel<<<grid_for(n), 256, 0, st>>>(y, x1, x2, n, a, b);
  return cudaGetLastError();
}
cudaError_t vec_add(float *y, const float *x, long long n, cudaStream_t st) {
  add_kernel<<<grid_for(n), 256, 0, st>>>(y, x, n);
  return cudaGetLastError();
}
cudaError_t vec_mult(float *y, const float *x, long long n, cudaStream_t st) {
  mult_kernel<<<grid_for(n), 256, 0, st>>>(y, x, n);
  return cudaGetLastError();
}
cudaError_t vec_random(float *y, long long n, unsigned long long seed, cudaStream_t st) {
  random_kernel<<<grid_for(n), 256, 0, st>>>(y, n, seed);
  return cudaGetLastError();
}

}  // namespace sepx
