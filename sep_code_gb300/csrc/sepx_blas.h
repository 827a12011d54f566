// sepx_blas.h -- launchers of the BLAS-1 kernels (sepx_blas.cu).
#pragma once
#include <cuda_runtime.h>

namespace sepx {

// FP64 dot product of two float vectors (b == nullptr: sum of a), written to
// the device double *d_out; `partials` is scratch of vec_dot_scratch_doubles().
cudaError_t vec_dot(const float *a, const float *b, long long n, double *partials, double *d_out,
                    cudaStream_t st);
int vec_dot_scratch_doubles();
cudaError_t vec_fill(float *x, long long n, float v, cudaStream_t st);
cudaError_t vec_scale(float *y, long long n, double a, cudaStream_t st);
cudaError_t vec_scale_add(float *y, const float *x, long long n, double a, double b, cudaStream_t st);
cudaError_t vec_scale_add2(float *y, const float *x1, const float *x2, long long n, double a,
                           double b, cudaStream_t st);
cudaError_t vec_add(float *y, const float *x, long long n, cudaStream_t st);
cudaError_t vec_mult(float *y, const float *x, long long n, cudaStream_t st);
cudaError_t vec_random(float *y, long long n, unsigned long long seed, cudaStream_t st);

}  // namespace sepx
