// sepx_opkernels.cu -- the per-shot glue of rtm_zero_op on the device: the
// reference does these on the host between the C-ABI calls
// (Born/rtm_zero_op_3d.cpp:139-166, :248-274); each kernel reproduces the
// float operations of the reference's loops element by element.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "sepx_aux.h"

namespace sepx {

// q = k / d, r = k % d with 32-bit division when the walk is shorter than 2^31
// (uniform per launch); 64-bit divisions otherwise.  Index arithmetic only.
__device__ __forceinline__ long long divmod(long long k, int d, bool narrow, int &rem) {
  if (narrow) {
    const uint32_t q = (uint32_t)k / (uint32_t)d;
    rem = (int)((uint32_t)k - q * (uint32_t)d);
    return q;
  }
  const long long q = k / d;
  rem = (int)(k - q * d);
  return q;
}

// img_pad = laplac::forward(extract_sub(model))  (Born/image_rtm_3d.cpp:52-90,
// Born/laplac_3d.cpp:46-96 with a unit mute): e(z) = model[z+f] (0 outside),
// d(0) = -e(0), d(z) = e(z-1) - e(z) for 0 < z < n3-1, d(n3-1) = e(n3-2).
__global__ void img_from_model_kernel(const float *__restrict__ model, int m1, int m2, int m3,
                                      int f1, int f2, int f3, float *__restrict__ img, int n1,
                                      int n2, int n3, int pitch) {
  const long long total = (long long)n1 * n2 * n3;
  const bool narrow = total < (1LL << 31);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int x, y;
    const int z = (int)divmod(divmod(t, n1, narrow, x), n2, narrow, y);
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
  const bool narrow = total < (1LL << 31);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int mx, my;
    const int mz = (int)divmod(divmod(t, m1, narrow, mx), m2, narrow, my);
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
  const bool narrow = total < (1LL << 31);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    int t;
    const int r = (int)divmod(k, nt, narrow, t);
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
  const bool narrow = total < (1LL << 31);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    int r;
    const int s = (int)divmod(k, nrec, narrow, r);   // time-major output index
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

// ---- data / image vectors kept on the device (the reference keeps them in
// out-of-core files and loops over them on the host) ----

// image_rtm_3d::add_image (Born/image_rtm_3d.cpp:24-49): img[j + f] += sub[j]
// for every sub cell whose shifted position lies inside img.  One block row
// per (i2, i3) row of sub, consecutive threads along axis 1.
__global__ void window_add_kernel(float *__restrict__ img, int n1, int n2, int n3,
                                  const float *__restrict__ sub, int s1, int s2, int s3, int f1,
                                  int f2, int f3) {
  const long long rows = (long long)s2 * s3;
  for (long long r = blockIdx.y; r < rows; r += gridDim.y) {
    const int i2 = (int)(r % s2), i3 = (int)(r / s2);
    const int j2 = i2 + f2, j3 = i3 + f3;
    if (j2 < 0 || j2 >= n2 || j3 < 0 || j3 >= n3) continue;   // uniform for the block
    float *orow = img + (long long)n1 * (j2 + (long long)n2 * j3);
    const float *irow = sub + (long long)s1 * r;
    for (int i1 = blockIdx.x * blockDim.x + threadIdx.x; i1 < s1; i1 += gridDim.x * blockDim.x) {
      const int j1 = i1 + f1;
      if (j1 >= 0 && j1 < n1) orow[j1] = __fadd_rn(orow[j1], irow[i1]);
    }
  }
}

// image_rtm_3d::extract_sub (Born/image_rtm_3d.cpp:52-90): sub[j] =
// img[j + f] * mute[j + f] (mute may be NULL: a unit mute), 0 where the
// shifted position lies outside img.
__global__ void window_extract_kernel(const float *__restrict__ img, const float *__restrict__ mute,
                                      int n1, int n2, int n3, float *__restrict__ sub, int s1,
                                      int s2, int s3, int f1, int f2, int f3) {
  const long long rows = (long long)s2 * s3;
  for (long long r = blockIdx.y; r < rows; r += gridDim.y) {
    const int i2 = (int)(r % s2), i3 = (int)(r / s2);
    const int j2 = i2 + f2, j3 = i3 + f3;
    const bool row_in = j2 >= 0 && j2 < n2 && j3 >= 0 && j3 < n3;
    const long long ro = (long long)n1 * (j2 + (long long)n2 * j3);
    float *orow = sub + (long long)s1 * r;
    for (int i1 = blockIdx.x * blockDim.x + threadIdx.x; i1 < s1; i1 += gridDim.x * blockDim.x) {
      const int j1 = i1 + f1;
      float v = 0.f;
      if (row_in && j1 >= 0 && j1 < n1) {
        v = img[ro + j1];
        if (mute) v = __fmul_rn(v, mute[ro + j1]);
      }
      orow[i1] = v;
    }
  }
}

// tmute (Born/tmute.cpp:4-76): out[rep][i2][i1] (+)= in[...] for i1 >= the
// first unmuted sample (int)((t_0 + (o2 + d2 i2) / vmute - o1) / d1) of
// trace i2, computed in single precision exactly as the reference does; a
// start before the first sample is taken as 0.  Without `add` the samples
// before the start are zeroed.
__global__ void tmute_kernel(const float *__restrict__ in, float *__restrict__ out, int add,
                             float t0, float vmute, int n1, float o1, float d1, int n2, float o2,
                             float d2, long long nrep) {
  const long long rows = (long long)n2 * nrep;
  for (long long r = blockIdx.y; r < rows; r += gridDim.y) {
    const int i2 = (int)(r % n2);
    const float tr = __fadd_rn(t0, __fdiv_rn(__fadd_rn(o2, __fmul_rn(d2, (float)i2)), vmute));
    const float sf = __fdiv_rn(__fsub_rn(tr, o1), d1);
    const int start = (sf >= (float)n1) ? n1 : max(0, __float2int_rz(sf));
    const float *irow = in + (long long)n1 * r;
    float *orow = out + (long long)n1 * r;
    for (int i1 = blockIdx.x * blockDim.x + threadIdx.x; i1 < n1; i1 += gridDim.x * blockDim.x) {
      float v = add ? orow[i1] : 0.f;
      if (i1 >= start) v = __fadd_rn(v, irow[i1]);
      orow[i1] = v;
    }
  }
}

// The same three operations four columns at a time (16-byte loads and
// stores), for rows whose lengths and offsets are multiples of 4 floats and
// whose buffers are 16-byte aligned: a float4 group then lies wholly inside
// or wholly outside the image.
__device__ __forceinline__ float4 add4(float4 a, float4 b) {
  return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}

__global__ void window_add4_kernel(float *__restrict__ img, int n1, int n2, int n3,
                                   const float *__restrict__ sub, int s1, int s2, int s3, int f1,
                                   int f2, int f3) {
  const long long rows = (long long)s2 * s3;
  const int q1 = s1 >> 2;
  for (long long r = (long long)blockIdx.y * blockDim.y + threadIdx.y; r < rows;
       r += (long long)gridDim.y * blockDim.y) {
    const int i2 = (int)(r % s2), i3 = (int)(r / s2);
    const int j2 = i2 + f2, j3 = i3 + f3;
    if (j2 < 0 || j2 >= n2 || j3 < 0 || j3 >= n3) continue;   // uniform for the block row
    float4 *orow = reinterpret_cast<float4 *>(img + (long long)n1 * (j2 + (long long)n2 * j3));
    const float4 *irow = reinterpret_cast<const float4 *>(sub + (long long)s1 * r);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < q1; k += gridDim.x * blockDim.x) {
      const int j1 = 4 * k + f1;
      if (j1 >= 0 && j1 < n1) orow[j1 >> 2] = add4(orow[j1 >> 2], irow[k]);
    }
  }
}

__global__ void window_extract4_kernel(const float *__restrict__ img, const float *__restrict__ mute,
                                       int n1, int n2, int n3, float *__restrict__ sub, int s1,
                                       int s2, int s3, int f1, int f2, int f3) {
  const long long rows = (long long)s2 * s3;
  const int q1 = s1 >> 2;
  for (long long r = (long long)blockIdx.y * blockDim.y + threadIdx.y; r < rows;
       r += (long long)gridDim.y * blockDim.y) {
    const int i2 = (int)(r % s2), i3 = (int)(r / s2);
    const int j2 = i2 + f2, j3 = i3 + f3;
    const bool row_in = j2 >= 0 && j2 < n2 && j3 >= 0 && j3 < n3;
    const long long ro = (long long)n1 * (j2 + (long long)n2 * j3);
    float4 *orow = reinterpret_cast<float4 *>(sub + (long long)s1 * r);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < q1; k += gridDim.x * blockDim.x) {
      const int j1 = 4 * k + f1;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row_in && j1 >= 0 && j1 < n1) {
        v = *reinterpret_cast<const float4 *>(img + ro + j1);
        if (mute) {
          const float4 m = *reinterpret_cast<const float4 *>(mute + ro + j1);
          v = make_float4(__fmul_rn(v.x, m.x), __fmul_rn(v.y, m.y), __fmul_rn(v.z, m.z),
                          __fmul_rn(v.w, m.w));
        }
      }
      orow[k] = v;
    }
  }
}

__global__ void tmute4_kernel(const float *__restrict__ in, float *__restrict__ out, int add,
                              float t0, float vmute, int n1, float o1, float d1, int n2, float o2,
                              float d2, long long nrep) {
  const long long rows = (long long)n2 * nrep;
  const int q1 = n1 >> 2;
  for (long long r = (long long)blockIdx.y * blockDim.y + threadIdx.y; r < rows;
       r += (long long)gridDim.y * blockDim.y) {
    const int i2 = (int)(r % n2);
    const float tr = __fadd_rn(t0, __fdiv_rn(__fadd_rn(o2, __fmul_rn(d2, (float)i2)), vmute));
    const float sf = __fdiv_rn(__fsub_rn(tr, o1), d1);
    const int start = (sf >= (float)n1) ? n1 : max(0, __float2int_rz(sf));
    const float4 *irow = reinterpret_cast<const float4 *>(in + (long long)n1 * r);
    float4 *orow = reinterpret_cast<float4 *>(out + (long long)n1 * r);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < q1; k += gridDim.x * blockDim.x) {
      const int i1 = 4 * k;
      float4 v = add ? orow[k] : make_float4(0.f, 0.f, 0.f, 0.f);
      if (i1 + 3 >= start) {   // some column of the group passes
        const float4 x = irow[k];
        if (i1 >= start) v.x = __fadd_rn(v.x, x.x);
        if (i1 + 1 >= start) v.y = __fadd_rn(v.y, x.y);
        if (i1 + 2 >= start) v.z = __fadd_rn(v.z, x.z);
        if (i1 + 3 >= start) v.w = __fadd_rn(v.w, x.w);
      }
      orow[k] = v;
    }
  }
}

static bool al16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// 2-D blocks for the 16-byte kernels: x covers a row of q float4 (whole
// warps, at most 256 threads), y takes as many rows as fill 256 threads
struct RowsLaunch {
  dim3 grid, block;
};
static RowsLaunch rows_launch4(int q, long long rows) {
  int bx = ((std::max(q, 1) + 31) / 32) * 32;
  if (bx > 256) bx = 256;
  const int by = 256 / bx;
  const int gx = std::min((q + bx - 1) / bx, 8);
  long long gy = (rows + by - 1) / by;
  if (gy > 2432) gy = 2432;
  RowsLaunch L;
  L.grid = dim3(std::max(gx, 1), (unsigned)std::max<long long>(gy, 1));
  L.block = dim3(bx, by);
  return L;
}

static dim3 rows_grid(int n1, long long rows) {
  // about 16 resident rows of 256 threads per SM on 152 SMs, x covering a row
  const int gx = (n1 + 255) / 256 < 8 ? (n1 + 255) / 256 : 8;
  long long gy = rows < 2432 ? rows : 2432;
  return dim3(gx < 1 ? 1 : gx, (unsigned)(gy < 1 ? 1 : gy));
}

cudaError_t launch_window_add(float *img, int n1, int n2, int n3, const float *sub, int s1, int s2,
                              int s3, int f1, int f2, int f3, cudaStream_t st) {
  if (n1 % 4 == 0 && s1 % 4 == 0 && f1 % 4 == 0 && al16(img) && al16(sub)) {
    const RowsLaunch L = rows_launch4(s1 / 4, (long long)s2 * s3);
    window_add4_kernel<<<L.grid, L.block, 0, st>>>(img, n1, n2, n3, sub, s1, s2, s3, f1, f2, f3);
  } else {
    window_add_kernel<<<rows_grid(s1, (long long)s2 * s3), 256, 0, st>>>(img, n1, n2, n3, sub, s1, s2,
                                                                         s3, f1, f2, f3);
  }
  return cudaGetLastError();
}

cudaError_t launch_window_extract(const float *img, const float *mute, int n1, int n2, int n3,
                                  float *sub, int s1, int s2, int s3, int f1, int f2, int f3,
                                  cudaStream_t st) {
  if (n1 % 4 == 0 && s1 % 4 == 0 && f1 % 4 == 0 && al16(img) && al16(sub) && (!mute || al16(mute))) {
    const RowsLaunch L = rows_launch4(s1 / 4, (long long)s2 * s3);
    window_extract4_kernel<<<L.grid, L.block, 0, st>>>(img, mute, n1, n2, n3, sub, s1, s2, s3, f1, f2,
                                                       f3);
  } else {
    window_extract_kernel<<<rows_grid(s1, (long long)s2 * s3), 256, 0, st>>>(img, mute, n1, n2, n3, sub,
                                                                             s1, s2, s3, f1, f2, f3);
  }
  return cudaGetLastError();
}

cudaError_t launch_tmute(const float *in, float *out, int add, float t0, float vmute, int n1,
                         float o1, float d1, int n2, float o2, float d2, long long nrep,
                         cudaStream_t st) {
  if (n1 % 4 == 0 && al16(in) && al16(out)) {
    const RowsLaunch L = rows_launch4(n1 / 4, (long long)n2 * nrep);
    tmute4_kernel<<<L.grid, L.block, 0, st>>>(in, out, add, t0, vmute, n1, o1, d1, n2, o2, d2, nrep);
  } else {
    tmute_kernel<<<rows_grid(n1, (long long)n2 * nrep), 256, 0, st>>>(in, out, add, t0, vmute, n1, o1,
                                                                      d1, n2, o2, d2, nrep);
  }
  return cudaGetLastError();
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
