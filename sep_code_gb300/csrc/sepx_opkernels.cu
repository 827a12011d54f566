// sepx_opkernels.cu -- the per-shot glue of rtm_zero_op on the device: the
// reference does these on the host between the C-ABI calls
// (Born/rtm_zero_op_3d.cpp:139-166, :248-274); each kernel reproduces the
// float operations of the reference's loops element by element.
#include <cuda_runtime.h>

#include "sepx_aux.h"

namespace sepx {

// img_pad = laplac::forward(extract_sub(model))  (Born/image_rtm_3d.cpp:52-90,
// Born/laplac_3d.cpp:46-96 with a unit mute): e(z) = model[z+f] (0 outside),
// d(0) = -e(0), d(z) = e(z-1) - e(z) for 0 < z < n3-1, d(n3-1) = e(n3-2).
__global__ void img_from_model_kernel(const float *__restrict__ model, int m1, int m2, int m3,
                                      int f1, int f2, int f3, float *__restrict__ img, int n1,
                                      int n2, int n3, int pitch) {
  const long long total = (long long)n1 * n2 * n3;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(t % n1), y = (int)((t / n1) % n2), z = (int)(t / ((long long)n1 * n2));
    const int mx = x + f1, my = y + f2;
    auto e = [&](int zz) -> float {
      const int mz = zz + f3;
      if (mx < 0 || mx >= m1 || my < 0 || my >= m2 || mz < 0 || mz >= m3) return 0.f;
      return model[mx + (long long)m1 * (my + (long long)m2 * mz)];
    };
    float d;
    if (z == n3 - 1) d = e(z - 1);
    else if (z == 0) d = -e(0);
    else d = __fsub_rn(e(z - 1), e(z));
    img[x + (long long)pitch * (y + (long long)n2 * z)] = d;
  }
}

// model += add_image(laplac::adjoint(img_pad)): m(z) = d(z+1) - d(z) for
// z < n3-1, 0 at z = n3-1, added into the model cell z+f.
__global__ void model_from_img_kernel(float *__restrict__ model, int m1, int m2, int m3, int f1,
                                      int f2, int f3, const float *__restrict__ img, int n1, int n2,
                                      int n3, int pitch) {
  const long long total = (long long)m1 * m2 * m3;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int mx = (int)(t % m1), my = (int)((t / m1) % m2), mz = (int)(t / ((long long)m1 * m2));
    const int x = mx - f1, y = my - f2, z = mz - f3;
    if (x < 0 || x >= n1 || y < 0 || y >= n2 || z < 0 || z >= n3) continue;
    const long long i = x + (long long)pitch * (y + (long long)n2 * z);
    const float v = (z < n3 - 1) ? __fsub_rn(img[i + (long long)pitch * n2], img[i]) : 0.f;
    model[t] = __fadd_rn(model[t], v);
  }
}

// data[r][t] += deriv::forward(map_data::forward(traces)) for one shot
// (Born/map_data_3d.cpp:58-76, Born/deriv_3d.cpp:25-46): m_r(t) = trc[t+4][r];
// d(0) = spill - a (- a again on the first trace of each y row), with spill
// the previous trace's last sample / dt; d(1) = a - b (a + a - b on the first
// trace of a row); d(t) = m(t-1)/dt - m(t)/dt.  nt >= 2.
__global__ void data_from_traces_kernel(const float *__restrict__ trc, int nrec, int rnx, int nt,
                                        float dt, float *__restrict__ data) {
  const long long total = (long long)nrec * nt;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(k / nt), t = (int)(k % nt);
    const bool first = (r % rnx) == 0;
    auto m = [&](int rr, int tt) { return __fdiv_rn(trc[(long long)(tt + 4) * nrec + rr], dt); };
    float v;
    if (t == 0) {
      const float spill = (r > 0) ? m(r - 1, nt - 1) : 0.f;
      const float a = m(r, 0);
      v = __fsub_rn(spill, a);
      if (first) v = __fsub_rn(v, a);
    } else if (t == 1) {
      const float a = m(r, 0), b = m(r, 1);
      v = first ? __fsub_rn(__fadd_rn(a, a), b) : __fsub_rn(a, b);
    } else {
      v = __fsub_rn(m(r, t - 1), m(r, t));
    }
    data[k] = __fadd_rn(data[k], v);
  }
}

// trc[t+4][r] = deriv::adjoint(data)[r][t] (map_data::adjoint): g(t) =
// (d(t+1) - d(t))/dt with d(nt) = the next trace's first sample (0 after the
// last); the first trace of each y row gets g(0) twice.  Other samples: 0.
__global__ void traces_from_data_kernel(const float *__restrict__ data, int nrec, int rnx, int nt,
                                        int ntrace, float dt, float *__restrict__ trc) {
  const long long total = (long long)nrec * ntrace;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(k / nrec), r = (int)(k % nrec);   // time-major output index
    const int t = s - 4;
    float v = 0.f;
    if (t >= 0 && t < nt) {
      const long long o = (long long)r * nt;
      const float cur = data[o + t];
      const float nxt = (t + 1 < nt) ? data[o + t + 1] : ((r + 1 < nrec) ? data[o + nt] : 0.f);
      const float g = __fdiv_rn(__fsub_rn(nxt, cur), dt);
      v = (t == 0 && (r % rnx) == 0) ? __fadd_rn(g, g) : g;
    }
    trc[k] = v;
  }
}

static int grid_of(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 4096 ? (g < 1 ? 1 : g) : 4096);
}

cudaError_t launch_img_from_model(const float *model, int m1, int m2, int m3, int f1, int f2, int f3,
                                  float *img, int n1, int n2, int n3, int pitch, cudaStream_t st) {
  img_from_model_kernel<<<grid_of((long long)n1 * n2 * n3), 256, 0, st>>>(model, m1, m2, m3, f1, f2,
                                                                          f3, img, n1, n2, n3, pitch);
  return cudaGetLastError();
}

cudaError_t launch_model_from_img(float *model, int m1, int m2, int m3, int f1, int f2, int f3,
                                  const float *img, int n1, int n2, int n3, int pitch,
                                  cudaStream_t st) {
  model_from_img_kernel<<<grid_of((long long)m1 * m2 * m3), 256, 0, st>>>(model, m1, m2, m3, f1, f2,
                                                                          f3, img, n1, n2, n3, pitch);
  return cudaGetLastError();
}

cudaError_t launch_data_from_traces(const float *trc, int nrec, int rnx, int nt, float dt,
                                    float *data, cudaStream_t st) {
  data_from_traces_kernel<<<grid_of((long long)nrec * nt), 256, 0, st>>>(trc, nrec, rnx, nt, dt, data);
  return cudaGetLastError();
}

cudaError_t launch_traces_from_data(const float *data, int nrec, int rnx, int nt, int ntrace,
                                    float dt, float *trc, cudaStream_t st) {
  traces_from_data_kernel<<<grid_of((long long)nrec * ntrace), 256, 0, st>>>(data, nrec, rnx, nt,
                                                                             ntrace, dt, trc);
  return cudaGetLastError();
}

}  // namespace sepx
