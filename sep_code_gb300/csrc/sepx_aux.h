// sepx_aux.h -- launchers of the small kernels in sepx_aux.cu.
#pragma once
#include <cuda_runtime.h>

#include "sepx_prop.h"

namespace sepx {

cudaError_t launch_prop_step(int mode, const PropParams &P, cudaStream_t st);
size_t prop_smem_bytes(int mode);
// two-row tile (kSrcProp, kBornFwd, kRtmAdj): 32 x 32 cells per CTA
cudaError_t launch_prop_step2(int mode, const PropParams &P, const Rows2Maps &H, cudaStream_t st);
bool prop_step2_supported(int mode);
// persistent multi-grid launches (sepx_prop.cu): stages 3 or 4
bool batch_supported(int mode, int stages);
cudaError_t launch_prop_batch(int mode, int stages, const PropParams *params, const int4 *items,
                              int nitems, const BatchStep &step, int grid, cudaStream_t st);
int prop_batch_occupancy(int mode, int stages);   // resident CTAs per SM
cudaError_t launch_prop_multi(int mode, int stages, const MultiParams &mp, cudaStream_t st);

cudaError_t launch_inj_values(const float *src, int ntrace, int npts, const float *sinc, int nsinc,
                              int jt, int nsteps, int j0, float dir, float *out, cudaStream_t st);
cudaError_t launch_point_add(float *p, const long long *off, const float *inj, int npts,
                             cudaStream_t st);
// point adds of up to kMaxMulti grids in one launch
struct PointAddSet {
  float *p;
  const long long *off;
  const float *inj;
  int npts;
};
struct PointAddSets {
  PointAddSet s[kMaxMulti];
  int n;
};
cudaError_t launch_point_add_multi(const PointAddSets &sets, cudaStream_t st);
cudaError_t launch_transpose(const float *in, long long lda, float *out, long long ldb, int rows,
                             int cols, cudaStream_t st);
// rows of `width` floats from row pitch spitch to row pitch dpitch (floats)
cudaError_t launch_repitch(const float *src, long long spitch, float *dst, long long dpitch,
                           int width, long long rows, cudaStream_t st);

cudaError_t launch_img_from_model(const float *model, int m1, int m2, int m3, int f1, int f2, int f3,
                                  float *img, int n1, int n2, int n3, int pitch, cudaStream_t st);
cudaError_t launch_model_from_img(float *model, int m1, int m2, int m3, int f1, int f2, int f3,
                                  const float *img, int n1, int n2, int n3, int pitch,
                                  cudaStream_t st);
cudaError_t launch_data_from_traces(const float *trc, int nrec, int rnx, int nt, float dt,
                                    float *data, cudaStream_t st);
cudaError_t launch_traces_from_data(const float *data, int nrec, int rnx, int nt, int ntrace,
                                    float dt, float *trc, cudaStream_t st);
cudaError_t launch_window_add(float *img, int n1, int n2, int n3, const float *sub, int s1, int s2,
                              int s3, int f1, int f2, int f3, cudaStream_t st);
cudaError_t launch_window_extract(const float *img, const float *mute, int n1, int n2, int n3,
                                  float *sub, int s1, int s2, int s3, int f1, int f2, int f3,
                                  cudaStream_t st);
cudaError_t launch_tmute(const float *in, float *out, int add, float t0, float vmute, int n1,
                         float o1, float d1, int n2, float o2, float d2, long long nrep,
                         cudaStream_t st);

}  // namespace sepx
