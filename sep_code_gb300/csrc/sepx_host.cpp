// sepx_host.cpp -- host-side set-up math of the Born/RTM operator: sinc
// interpolation tables, the random-boundary velocity, the padded grid, the
// source stencil, the receiver map and the stability time step.  These are the
// per-shot preparations rtm_zero_op makes before it calls the C ABI; each
// follows the reference statement by statement because the time loops depend
// on the exact float values.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/sepx_host.h"

namespace {

// ---- 8-tap least-squares sinc (Born/sinc_bob.cpp:4-114; Hale 1983) ----
void toep(int m, const float *r, float *f, const float *g, float *a) {
  double c, e, v, w, bot;
  a[0] = 1.0f;
  v = r[0];
  f[0] = g[0] / r[0];
  for (int j = 1; j < m; j++) {
    e = 0.0;
    a[j] = 0.0f;
    f[j] = 0.0f;
    for (int i = 0; i < j; i++) e += a[i] * r[j - i];
    c = e / v;
    v -= e * c;
    const int jh = j / 2;
    for (int i = 0; i <= jh; i++) {
      bot = a[j - i] - c * a[i];
      a[i] = (float)(a[i] - c * a[j - i]);
      a[j - i] = (float)bot;
    }
    w = 0;
    for (int i = 0; i < j; i++) w += f[i] * r[j - i];
    c = (g[j] - w) / v;
    for (int i = 0; i <= j; i++) f[i] = (float)(f[i] + c * a[j - i]);
  }
}

void mksinc(float *sinc, int lsinc, float d, float *space) {
  const float pi = 3.141592654f;
  const float pi2 = pi * 2;
  const float snyq = 0.5f;
  const float snat = (float)(snyq * (0.066 + 0.265 * std::log((double)lsinc)));
  const float s0 = 0.0f;
  const float ds = (snat - s0) / (float)(lsinc * 2 - 1);
  const float eta = (float)(lsinc / 2 - 1.0 + d);
  float *b = space, *c = b + lsinc, *work = c + lsinc;
  for (int j = 0; j < lsinc; j++) {
    float s;
    for (s = s0, b[j] = c[j] = 0.0f; s <= snat; s += ds) {
      b[j] = b[j] + std::cos(pi2 * s * (float)j);          // float overload
      c[j] = c[j] + std::cos(pi2 * s * (eta - (float)j));
    }
  }
  toep(lsinc, b, sinc, c, work);
}

// ---- glibc random(): r[i] = r[i-3] + r[i-31], Park-Miller seeded, 310 discarded ----
struct GlibcRand {
  int32_t s[31];
  int f = 3, r = 0;
  explicit GlibcRand(unsigned int seed) {
    if (seed == 0) seed = 1;
    s[0] = (int32_t)seed;
    int64_t word = (int32_t)seed;
    for (int i = 1; i < 31; i++) {
      const int64_t hi = word / 127773, lo = word % 127773;
      word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      s[i] = (int32_t)word;
    }
    for (int i = 0; i < 310; i++) next();
  }
  int32_t next() {
    s[f] = (int32_t)((uint32_t)s[f] + (uint32_t)s[r]);
    const int32_t out = (int32_t)((uint32_t)s[f] >> 1);
    if (++f >= 31) f = 0;
    if (++r >= 31) r = 0;
    return out;
  }
};

inline float ramp2(int i, int n, int nr) {
  if (i < nr) return (float)((nr - i) * (nr - i)) / (float)(nr * nr);
  if (i >= n - nr) return (float)((i - (n - nr - 1)) * (i - (n - nr - 1))) / (float)(nr * nr);
  return 0.f;
}

}  // namespace

extern "C" {

void sepx_host_sinc_table(int ntab, int nsinc, float *out) {
  const float dtab = 1.0f / (float)ntab;
  float t = 0.0f;
  std::vector<float> junk((size_t)nsinc * 3);
  for (int it = 0; it < ntab; it++, t += dtab) mksinc(out + (size_t)it * nsinc, nsinc, t, junk.data());
}

int sepx_host_glibc_rand_sequence(unsigned int seed, int n, int *out) {
  GlibcRand g(seed);
  for (int i = 0; i < n; i++) out[i] = g.next();
  return 0;
}

// vel_fd_3d::rand_subspace (Born/vel_fd_3d.cpp:26-88)
void sepx_host_rand_subspace(int irand, int nrand1, int nrand2, int nrand3, float dt,
                             const float *model, int m1, int m2, int m3, float mo1, float mo2,
                             float mo3, float md1, float md2, float md3, int s1, int s2, int s3,
                             float so1, float so2, float so3, float sd1, float sd2, float sd3,
                             float *out) {
  double mx = model[0];
  const long long nm = (long long)m1 * m2 * m3;
  for (long long i = 1; i < nm; i++) mx = std::max(mx, (double)model[i]);
  const float vmax = (float)mx;
  GlibcRand rng((unsigned int)irand);
  long long i = 0;
  std::vector<int> ixv(s1);
  for (int ix = 0; ix < s1; ix++)
    ixv[ix] = std::max(0, std::min(m1 - 1, (int)((so1 + sd1 * (float)ix - mo1) / md1)));
  for (int iz = 0; iz < s3; iz++) {
    const int iz_v = std::max(0, std::min(m3 - 1, (int)((so3 + sd3 * (float)iz - mo3) / md3)));
    const float dz2 = ramp2(iz, s3, nrand3);
    for (int iy = 0; iy < s2; iy++) {
      const int iy_v = std::max(0, std::min(m2 - 1, (int)((so2 + sd2 * (float)iy - mo2) / md2)));
      const float dy2 = ramp2(iy, s2, nrand2);
      const float *mrow = model + (long long)iy_v * m1 + (long long)iz_v * m1 * m2;
      for (int ix = 0; ix < s1; ix++, i++) {
        const float val = mrow[ixv[ix]];
        float dx2 = ramp2(ix, s1, nrand1);
        if (dx2 < 0. || dx2 > 1) dx2 = 1;
        const float dist = std::sqrt(dx2 + dy2 + dz2);
        bool found = dist < .0001;
        float dev = 0.f;
        while (!found && nrand2 != 0) {
          const float rnd =
              (float)((double)((float)rng.next() / (float)2147483647) - .5 - .49 * dist);
          dev = (float)((double)rnd * 1.3 * dist * val);
          const float sv = dev + val;
          if ((double)std::fabs(sv) < vmax * 1.03 * (1. - std::min(1., (double)dist) * .4) &&
              sv > 0.0001)
            found = true;
        }
        const float s = val + dev;
        out[i] = s * s * dt * dt;
      }
    }
  }
}

// source_func::set_compute_size (Born/source_func_3d.cpp:37-64)
void sepx_host_compute_size(int m1, int m2, int m3, int nbt, int nb, int nby, int fat, int *n1,
                            int *n2, int *n3) {
  const int nbound = nb + fat, nbound_y = nby + fat;
  int ny = m2 + 2 * nbound_y, nx = m1 + 2 * nbound, nz = m3 + 2 * nbound;
  nz += nbt + nb + 2 * fat;
  int rx = nx % 16, ry = ny % 16, rz = nz % 16;
  if (ry) ry = 16 - ry;
  if (rz) rz = 16 - rz;
  if (rx) rx = 16 - rx;
  *n1 = nx + rx;
  *n2 = ny + ry;
  *n3 = nz + rz;
}

// source_func constructor: time derivative of the wavelet (:4-19)
void sepx_host_wavelet_deriv(const float *w, int n, float dt, float *out) {
  out[n - 1] = 0;
  for (int it = 0; it < n - 1; it++) out[it] = (w[it + 1] - w[it]) / dt;
}

// source_func::get_source_func (:100-133): 3x3 Gaussian-weighted points on the
// plane iz-1, wavelet samples at offset +4 of traces of length nts.
void sepx_host_source_func(const float *wav, int nwav, float sx, float sy, float sz, int n1, int n2,
                           float o1, float o2, float o3, float d1, float d2, float d3, int nts,
                           int *locs, float *vals) {
  const float fz = (sz - o3) / d3, fy = (sy - o2) / d2, fx = (sx - o1) / d1;
  const int iy = (int)fy, ix = (int)fx, iz = (int)fz;
  int i = 0;
  std::fill(vals, vals + (size_t)nts * 9, 0.f);
  for (int i3 = iz - 1; i3 <= iz - 1; i3++) {
    const float zn = fz - (float)i3;
    for (int i2 = iy - 1; i2 <= iy + 1; i2++) {
      const float yn = fy - (float)i2;
      for (int i1 = ix - 1; i1 <= ix + 1; i1++, i++) {
        const float xn = fx - (float)i1;
        locs[i] = i1 + i2 * n1 + i3 * n1 * n2;
        const float scale = std::exp(-zn * zn - xn * xn - yn * yn);
        for (int it = 0; it < nwav && it + 4 < nts; it++) vals[(size_t)nts * i + it + 4] = scale * wav[it];
      }
    }
  }
}

// fd_prop::calc_stability (Born/fd_prop_3d.cpp:7-26)
float sepx_host_calc_stability(float vmax, float dmin, float data_dt, int n_data, int *nt) {
  const float d = (float)(.5 * dmin / vmax);
  const float dt = data_dt / std::ceil(data_dt / d);
  *nt = (n_data - 1) * (int)(data_dt / dt) + 1;
  return dt;
}

// data_rtm_3d::get_source_func geometry + map_data constructor
// (Born/data_rtm_3d.cpp:115-140, Born/map_data_3d.cpp:4-35)
void sepx_host_receiver_map(int rnx, int rny, float ro2, float rd2, float ro3, float rd3,
                            float rec_depth, int n1, int n2, float o1, float o2, float o3, float d1,
                            float d2, float d3, int *locs) {
  int i = 0;
  for (int i3 = 0; i3 < rny; i3++)
    for (int i2 = 0; i2 < rnx; i2++, i++) {
      const float s_z = (rec_depth - o3) / d3;
      const float s_x = (ro2 + rd2 * (float)i2 - o1) / d1;
      const float s_y = (ro3 + rd3 * (float)i3 - o2) / d2;
      const int ix = (int)s_x, iz = (int)s_z + 4, iy = (int)s_y;
      locs[i] = ix + iy * n1 + iz * n1 * n2;
    }
}

}  // extern "C"
