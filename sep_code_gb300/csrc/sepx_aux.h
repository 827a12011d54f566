// sepx_aux.h -- launchers of the small kernels in sepx_aux.cu.
#pragma once
#include <cuda_runtime.h>

#include "sepx_prop.h"

namespace sepx {

cudaError_t launch_prop_step(int mode, const PropParams &P, cudaStream_t st);
size_t prop_smem_bytes(int mode);

cudaError_t launch_inj_values(const float *src, int ntrace, int npts, const float *sinc, int nsinc,
                              int jt, int nsteps, int j0, float dir, float *out, cudaStream_t st);
cudaError_t launch_point_add(float *p, const long long *off, const float *inj, int npts,
                             cudaStream_t st);
cudaError_t launch_transpose(const float *in, long long lda, float *out, long long ldb, int rows,
                             int cols, cudaStream_t st);

}  // namespace sepx
