#include <algorithm>
#include <cstdint>
// sepx_aux.cu -- small kernels around the fused propagation step: per-step
// source injection values, the adjoint's injection into the current source
// field, trace layout transposes, and helpers for the trace/image operators.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sepx_aux.h"

namespace sepx {

// inj[j][i] = dir * sum_k sinc_s[j%jt][k] * src[i][j/jt + k]
// (new_src_inject_kernel, Born/gpu_funcs_3d.cu:64-75, evaluated for every step
// once before the time loop).
__global__ void inj_values_kernel(const float *__restrict__ src, int ntrace, int npts,
                                  const float *__restrict__ sinc, int nsinc, int jt, int nsteps,
                                  int j0, float dir, float *__restrict__ out) {
  const long long n = (long long)nsteps * npts;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / npts) + j0, i = (int)(t % npts);
    const int id = j / jt, ii = j - id * jt;
    const float *row = sinc + (long long)ii * nsinc;
    const float *tr = src + (long long)ntrace * i + id;
    float acc = __fmul_rn(row[0], tr[0]);
#pragma unroll
    for (int k = 1; k < 8; k++) acc = __fmaf_rn(row[k], tr[k], acc);
    out[(long long)(j - j0) * npts + i] = __fmul_rn(dir, acc);
  }
}

// p[off[i]] += inj[i], points in ascending order (one thread: duplicates add up
// in the same order as the CPU restatement).
__global__ void point_add_kernel(float *p, const long long *__restrict__ off,
                                 const float *__restrict__ inj, int npts) {
  if (threadIdx.x == 0 && blockIdx.x == 0)
    for (int i = 0; i < npts; i++) p[off[i]] = __fadd_rn(p[off[i]], inj[i]);
}

// out[c][r] = in[r][c] for an (rows x cols) block of a row-major matrix with
// row strides lda / ldb; 32x32 tiles through shared memory.
__global__ void transpose_kernel(const float *__restrict__ in, long long lda, float *__restrict__ out,
                                 long long ldb, int rows, int cols) {
  __shared__ float tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[k][threadIdx.x] = in[(long long)r * lda + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[(long long)c * ldb + r] = tile[threadIdx.x][k];
  }
}

cudaError_t launch_inj_values(const float *src, int ntrace, int npts, const float *sinc, int nsinc,
                              int jt, int nsteps, int j0, float dir, float *out, cudaStream_t st) {
  const long long n = (long long)nsteps * npts;
  if (n <= 0) return cudaSuccess;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  inj_values_kernel<<<blocks, 256, 0, st>>>(src, ntrace, npts, sinc, nsinc, jt, nsteps, j0, dir, out);
  return cudaGetLastError();
}

// One thread per grid: its points in order (several points may share a cell).
__global__ void point_add_multi_kernel(const PointAddSets sets) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= sets.n) return;
  const PointAddSet &s = sets.s[g];
  for (int i = 0; i < s.npts; i++) s.p[s.off[i]] = __fadd_rn(s.p[s.off[i]], s.inj[i]);
}

cudaError_t launch_point_add_multi(const PointAddSets &sets, cudaStream_t st) {
  if (sets.n <= 0) return cudaSuccess;
  point_add_multi_kernel<<<1, 32, 0, st>>>(sets);
  return cudaGetLastError();
}

cudaError_t launch_point_add(float *p, const long long *off, const float *inj, int npts,
                             cudaStream_t st) {
  if (npts <= 0) return cudaSuccess;
  point_add_kernel<<<1, 32, 0, st>>>(p, off, inj, npts);
  return cudaGetLastError();
}

// rows of `width` floats from one row pitch to another (a dense host-layout
// volume into the pitched device layout and back); 16-byte accesses where
// both pitches and both bases allow them
__global__ void repitch_kernel(const float *__restrict__ src, long long spitch, float *__restrict__ dst,
                               long long dpitch, int width, long long rows, int vec4) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (vec4) {
    const int w4 = width >> 2;
    const long long n = rows * w4;
    const bool narrow = n < (1LL << 31);   // 32-bit division (uniform per launch)
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
      const long long r = narrow ? (long long)((uint32_t)i / (uint32_t)w4) : i / w4, c = i - r * w4;
      const float4 v = __ldcs(reinterpret_cast<const float4 *>(src + r * spitch) + c);
      __stcs(reinterpret_cast<float4 *>(dst + r * dpitch) + c, v);
    }
  } else {
    const long long n = rows * width;
    const bool narrow = n < (1LL << 31);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
      const long long r = narrow ? (long long)((uint32_t)i / (uint32_t)width) : i / width, c = i - r * width;
      dst[r * dpitch + c] = __ldcs(src + r * spitch + c);
    }
  }
}

cudaError_t launch_repitch(const float *src, long long spitch, float *dst, long long dpitch,
                           int width, long long rows, cudaStream_t st) {
  if (width <= 0 || rows <= 0) return cudaSuccess;
  const int vec4 = (width % 4 == 0 && spitch % 4 == 0 && dpitch % 4 == 0 &&
                    reinterpret_cast<uintptr_t>(src) % 16 == 0 && reinterpret_cast<uintptr_t>(dst) % 16 == 0);
  const long long work = rows * (vec4 ? width / 4 : width);
  const long long blocks = std::min<long long>((work + 255) / 256, 152LL * 16);
  repitch_kernel<<<(unsigned)std::max<long long>(blocks, 1), 256, 0, st>>>(src, spitch, dst, dpitch, width,
                                                                           rows, vec4);
  return cudaGetLastError();
}

cudaError_t launch_transpose(const float *in, long long lda, float *out, long long ldb, int rows,
                             int cols, cudaStream_t st) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(in, lda, out, ldb, rows, cols);
  return cudaGetLastError();
}

}  // namespace sepx
