/*
 * sepx_oracle.c -- CPU restatement of SEP_Code's acoustic Born/RTM path.
 * TEST INFRASTRUCTURE ONLY: the parity oracle and the timed CPU baseline.
 * Build: oracle/build_oracle.py (C11, -O3 -fopenmp -ffp-contract=off).
 */
#include "sepx_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* FD coefficients: Born/wave_fkernel.3d8o.cu:26-27 (C_C00, get_coeffs),
 * evaluated in double and stored as float as create_gpu_space does
 * (Born/gpu_funcs_3d.cu:783). */
static double c00(double d) { return 8.0 / (5.0 * d * d); }

static void fd_coeffs_d(double d1, double d2, double d3, double o[13]) {
  o[0] = -1025.0 / 576.0 * (c00(d1) + c00(d2) + c00(d3));
  o[1] = c00(d1); o[2] = c00(d2); o[3] = c00(d3);
  o[4] = -c00(d1) / 8.0; o[5] = -c00(d2) / 8.0; o[6] = -c00(d3) / 8.0;
  o[7] = c00(d1) / 63.0; o[8] = c00(d2) / 63.0; o[9] = c00(d3) / 63.0;
  o[10] = -c00(d1) / 896.0; o[11] = -c00(d2) / 896.0; o[12] = -c00(d3) / 896.0;
}

void orc_fd_coeffs(float d1, float d2, float d3, float out[13]) {
  double o[13];
  fd_coeffs_d((double)d1, (double)d2, (double)d3, o);
  for (int k = 0; k < 13; k++) out[k] = (float)o[k];
}

/* Sponge factor by edge distance: damp_kernel computes
 * expf(-bc_b*(bc_a-edge)) in float and multiplies only when it is < 1
 * (Born/wave_fkernel.3d8o.cu:201-205).  The exponential is taken in double and
 * rounded once so that the same table serves the CPU and GPU paths. */
void orc_damp_table_f32(float bc_a, float bc_b, int ntab, float *tab) {
  for (int e = 0; e < ntab; e++) {
    float arg = -bc_b * (bc_a - (float)e);
    float t = (float)exp((double)arg);
    tab[e] = (t < 1.0f) ? t : 1.0f;
  }
}

void orc_damp_table_f64(float bc_a, float bc_b, int ntab, double *tab) {
  for (int e = 0; e < ntab; e++) {
    double t = exp(-(double)bc_b * ((double)bc_a - (double)e));
    tab[e] = (t < 1.0) ? t : 1.0;
  }
}

/* ------------------------------------------------------------------------ */
/* Least-squares tapered sinc (Born/sinc_bob.cpp:4-114, after Hale 1983):
 * mksinc builds a Toeplitz system from cosine sums, toep solves it with the
 * Levinson recursion in double.  Types follow the reference statement by
 * statement (float work arrays, double recursion scalars). */
static void toep(int m, const float *r, float *f, const float *g, float *a) {
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
    int jh = j / 2;
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

static void mksinc(float *sinc, int lsinc, float d, float *space) {
  float pi = 3.141592654f;
  float pi2 = pi * 2;
  float snyq = 0.5f;
  float snat = (float)(snyq * (0.066 + 0.265 * log((double)lsinc)));
  float s0 = 0.0f;
  float ds = (snat - s0) / (float)(lsinc * 2 - 1);
  float eta = (float)(lsinc / 2 - 1.0 + d);
  float *b = space, *c = b + lsinc, *work = c + lsinc;
  for (int j = 0; j < lsinc; j++) {
    float s;
    for (s = s0, b[j] = c[j] = 0.0f; s <= snat; s += ds) {
      /* cos() of a float argument resolves to the float overload in C++ */
      b[j] = b[j] + cosf(pi2 * s * (float)j);
      c[j] = c[j] + cosf(pi2 * s * (eta - (float)j));
    }
  }
  toep(lsinc, b, sinc, c, work);
}

void orc_sinc_table(int ntab, int nsinc, float *out) {
  float dtab = 1.0f / (float)ntab;
  float t = 0.0f;
  float *junk = (float *)malloc(sizeof(float) * (size_t)nsinc * 3);
  for (int it = 0; it < ntab; it++, t += dtab) mksinc(out + (long)it * nsinc, nsinc, t, junk);
  free(junk);
}

/* ------------------------------------------------------------------------ */
/* glibc random(): the additive lagged-Fibonacci generator r[i] = r[i-3] +
 * r[i-31] (mod 2^32), seeded by the Park-Miller LCG (16807 mod 2^31-1) with
 * 310 outputs discarded; output = r >> 1.  This is the published TYPE_3
 * algorithm that srand()/rand() use; the reference draws its random boundary
 * from it (Born/vel_fd_3d.cpp:231, :277). */
static int32_t g_state[31];
static int g_f = 3, g_r = 0;

static int32_t glibc_next(void) {
  g_state[g_f] = (int32_t)((uint32_t)g_state[g_f] + (uint32_t)g_state[g_r]);
  int32_t result = (int32_t)((uint32_t)g_state[g_f] >> 1);
  if (++g_f >= 31) g_f = 0;
  if (++g_r >= 31) g_r = 0;
  return result;
}

void orc_glibc_srand(unsigned int seed) {
  if (seed == 0) seed = 1;
  g_state[0] = (int32_t)seed;
  int64_t word = (int32_t)seed;
  for (int i = 1; i < 31; i++) {
    int64_t hi = word / 127773, lo = word % 127773;
    word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    g_state[i] = (int32_t)word;
  }
  g_f = 3;
  g_r = 0;
  for (int i = 0; i < 310; i++) (void)glibc_next();
}

int orc_glibc_rand(void) { return glibc_next(); }

/* ------------------------------------------------------------------------ */
/* vel_fd_3d::rand_subspace (Born/vel_fd_3d.cpp:26-88): nearest-neighbour
 * resample of the model onto the padded grid, random velocity in the boundary
 * (quadratic ramp, rejection loop on rand()), output v^2 dt^2. */
#define RS_MIN(a, b) (((a) < (b)) ? (a) : (b))
#define RS_MAX(a, b) (((a) > (b)) ? (a) : (b))

void orc_rand_subspace(int irand, int nrand1, int nrand2, int nrand3, float dt,
                       const float *model, int m1, int m2, int m3,
                       float mo1, float mo2, float mo3, float md1, float md2, float md3,
                       int s1, int s2, int s3, float so1, float so2, float so3,
                       float sd1, float sd2, float sd3, float *out) {
  double mx = model[0];
  long nm = (long)m1 * m2 * m3;
  for (long i = 1; i < nm; i++)
    if (model[i] > mx) mx = model[i];
  float vmax = (float)mx;
  orc_glibc_srand((unsigned int)irand);
  float dy2, dx2, dz2, rnd;
  long i = 0;
  for (int iz = 0; iz < s3; iz++) {
    int iz_v = RS_MAX(0, RS_MIN(m3 - 1, (int)((so3 + sd3 * (float)iz - mo3) / md3)));
    if (iz < nrand3)
      dz2 = (float)((nrand3 - iz) * (nrand3 - iz)) / (float)(nrand3 * nrand3);
    else if (iz >= s3 - nrand3)
      dz2 = (float)((iz - (s3 - nrand3 - 1)) * (iz - (s3 - nrand3 - 1))) / (float)(nrand3 * nrand3);
    else
      dz2 = 0;
    for (int iy = 0; iy < s2; iy++) {
      int iy_v = RS_MAX(0, RS_MIN(m2 - 1, (int)((so2 + sd2 * (float)iy - mo2) / md2)));
      if (iy < nrand2)
        dy2 = (float)((nrand2 - iy) * (nrand2 - iy)) / (float)(nrand2 * nrand2);
      else if (iy >= s2 - nrand2)
        dy2 = (float)((iy - (s2 - nrand2 - 1)) * (iy - (s2 - nrand2 - 1))) / (float)(nrand2 * nrand2);
      else
        dy2 = 0;
      for (int ix = 0; ix < s1; ix++, i++) {
        int ix_v = RS_MAX(0, RS_MIN(m1 - 1, (int)((so1 + sd1 * (float)ix - mo1) / md1)));
        float val = model[ix_v + (long)iy_v * m1 + (long)iz_v * m1 * m2];
        if (ix < nrand1)
          dx2 = (float)((nrand1 - ix) * (nrand1 - ix)) / (float)(nrand1 * nrand1);
        else if (ix >= s1 - nrand1)
          dx2 = (float)((ix - (s1 - nrand1 - 1)) * (ix - (s1 - nrand1 - 1))) / (float)(nrand1 * nrand1);
        else
          dx2 = 0;
        if (dx2 < 0. || dx2 > 1) dx2 = 1;
        float dist = sqrtf(dx2 + dy2 + dz2);
        int found = 0;
        float dev;
        if (dist < .0001) found = 1;
        dev = 0.f;
        while (!found && nrand2 != 0) {
          rnd = (float)((double)((float)glibc_next() / (float)2147483647) - .5 - .49 * dist);
          dev = (float)((double)rnd * 1.3 * dist * val);
          float sv = dev + val;
          if ((double)fabsf(sv) < vmax * 1.03 * (1. - RS_MIN(1., (double)dist) * .4) &&
              sv > 0.0001)
            found = 1;
        }
        float s = val + dev;
        out[i] = s * s * dt * dt;
      }
    }
  }
}

/* source_func::set_compute_size (Born/source_func_3d.cpp:37-64): pad by
 * nb+fat on each lateral side, z by 2(nb+fat)+nbt+nb+2fat, round up to 16. */
void orc_compute_size(int m1, int m2, int m3, int nbt, int nb, int nby, int fat, int *n1,
                      int *n2, int *n3) {
  int nbound = nb + fat, nbound_y = nby + fat;
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

/* wavelet time derivative of the source_func constructor (:4-19) */
void orc_wavelet_deriv(const float *w, int n, float dt, float *out) {
  out[n - 1] = 0;
  for (int it = 0; it < n - 1; it++) out[it] = (w[it + 1] - w[it]) / dt;
}

/* source_func::get_source_func (:100-133): 3x3 Gaussian-weighted points on the
 * plane iz-1, wavelet samples placed at offset +4 of traces of length nts. */
void orc_source_func(const float *wav, int nwav, float sx, float sy, float sz, int n1, int n2,
                     float o1, float o2, float o3, float d1, float d2, float d3, int nts,
                     int *locs, float *vals) {
  float fz = (sz - o3) / d3, fy = (sy - o2) / d2, fx = (sx - o1) / d1;
  int iy = (int)fy, ix = (int)fx, iz = (int)fz;
  int i = 0;
  for (int it = 0; it < nts * 9; it++) vals[it] = 0;
  for (int i3 = iz - 1; i3 <= iz - 1; i3++) {
    float zn = fz - (float)i3;
    for (int i2 = iy - 1; i2 <= iy + 1; i2++) {
      float yn = fy - (float)i2;
      for (int i1 = ix - 1; i1 <= ix + 1; i1++, i++) {
        float xn = fx - (float)i1;
        locs[i] = i1 + i2 * n1 + i3 * n1 * n2;
        float scale = expf(-zn * zn - xn * xn - yn * yn);
        for (int it = 0; it < nwav && it + 4 < nts; it++) vals[(long)nts * i + it + 4] = scale * wav[it];
      }
    }
  }
}

/* fd_prop::calc_stability (Born/fd_prop_3d.cpp:7-26) */
float orc_calc_stability(float vmax, float dmin, float data_dt, int n_data, int *nt) {
  float d = (float)(.5 * dmin / vmax);
  float dt = data_dt / ceilf(data_dt / d);
  *nt = (n_data - 1) * (int)(data_dt / dt) + 1;
  return dt;
}

/* receiver geometry: data_rtm_3d::get_source_func (Born/data_rtm_3d.cpp:115-140)
 * then the map_data constructor (Born/map_data_3d.cpp:4-35): iz = (int)s_z + 4 */
void orc_receiver_map(int rnx, int rny, float ro2, float rd2, float ro3, float rd3, float rec_depth,
                      int n1, int n2, float o1, float o2, float o3, float d1, float d2, float d3,
                      int *locs) {
  int i = 0;
  for (int i3 = 0; i3 < rny; i3++)
    for (int i2 = 0; i2 < rnx; i2++, i++) {
      float s_z = (rec_depth - o3) / d3;
      float s_x = (ro2 + rd2 * (float)i2 - o1) / d1;
      float s_y = (ro3 + rd3 * (float)i3 - o2) / d2;
      int ix = (int)s_x, iz = (int)s_z + 4, iy = (int)s_y;
      locs[i] = ix + iy * n1 + iz * n1 * n2;
    }
}

/* deriv (Born/deriv_3d.cpp:4-46): first difference along time divided by dt.
 * The reference writes / reads one sample past the last trace; that access is
 * dropped / read as zero here. */
void orc_deriv_forward(int add, int nt, int n2, int n3, float dt, const float *m, float *d) {
  long n12 = (long)nt * n2, tot = n12 * n3;
  if (!add) memset(d, 0, sizeof(float) * tot);
  for (int i3 = 0; i3 < n3; i3++) {
    d[1 + i3 * n12] += m[i3 * n12] / dt;
    d[i3 * n12] -= m[i3 * n12] / dt;
    for (int i2 = 0; i2 < n2; i2++) {
      long o = (long)i2 * nt + i3 * n12;
      d[1 + o] += m[o] / dt;
      d[o] -= m[o] / dt;
      for (int i1 = 1; i1 < nt; i1++) {
        d[i1 + o] -= m[o + i1] / dt;
        if (i1 + 1 + o < tot) d[i1 + 1 + o] += m[o + i1] / dt;
      }
    }
  }
}

void orc_deriv_adjoint(int add, int nt, int n2, int n3, float dt, float *m, const float *d) {
  long n12 = (long)nt * n2, tot = n12 * n3;
  if (!add) memset(m, 0, sizeof(float) * tot);
  for (int i3 = 0; i3 < n3; i3++) {
    m[i3 * n12] += (d[i3 * n12 + 1] - d[i3 * n12]) / dt;
    for (int i2 = 0; i2 < n2; i2++) {
      long o = (long)i2 * nt + i3 * n12;
      m[o] += (d[o + 1] - d[o]) / dt;
      for (int i1 = 1; i1 < nt; i1++) {
        float nxt = (i1 + 1 + o < tot) ? d[i1 + 1 + o] : 0.0f;
        m[o + i1] += (nxt - d[i1 + o]) / dt;
      }
    }
  }
}

/* laplac (Born/laplac_3d.cpp:46-96): a first difference along axis 3 */
void orc_laplac_forward(int add, int n1, int n2, int n3, const float *m, float *d) {
  long n12 = (long)n1 * n2;
  if (!add) memset(d, 0, sizeof(float) * n12 * n3);
  for (int i3 = 0; i3 < n3 - 1; i3++)
    for (long j = 0; j < n12; j++) {
      long i = i3 * n12 + j;
      d[i + n12] += m[i];
      d[i] -= m[i];
    }
}

void orc_laplac_adjoint(int add, int n1, int n2, int n3, float *m, const float *d) {
  long n12 = (long)n1 * n2;
  if (!add) memset(m, 0, sizeof(float) * n12 * n3);
  for (int i3 = 0; i3 < n3 - 1; i3++)
    for (long j = 0; j < n12; j++) {
      long i = i3 * n12 + j;
      m[i] += d[i + n12] - d[i];
    }
}

/* map_data (Born/map_data_3d.cpp:37-76): traces of length ntb (the padded
 * propagation record) to the data cube of length nt, shifted by 4 samples */
void orc_map_data_forward(int add, int ntb, int nt, int n2, int n3, const float *m, float *d) {
  if (!add) memset(d, 0, sizeof(float) * (long)nt * n2 * n3);
  for (int i3 = 0; i3 < n3; i3++)
    for (int i2 = 0; i2 < n2; i2++)
      for (int it = 0; it < nt; it++)
        d[it + (long)i2 * nt + (long)i3 * nt * n2] += m[(long)ntb * i2 + it + 4 + (long)i3 * ntb * n2];
}

void orc_map_data_adjoint(int add, int ntb, int nt, int n2, int n3, float *m, const float *d) {
  if (!add) memset(m, 0, sizeof(float) * (long)ntb * n2 * n3);
  for (int i3 = 0; i3 < n3; i3++)
    for (int i2 = 0; i2 < n2; i2++)
      for (int it = 0; it < nt; it++)
        m[(long)ntb * i2 + it + 4 + (long)i3 * ntb * n2] += d[it + (long)i2 * nt + (long)i3 * nt * n2];
}

/* ------------------------------------------------------------------------ */
/* Snapshot quantisation of the product's linearised operator (test mirror):
 * blocks of 32 x 16 cells of each plane of the updated interior, tiles
 * anchored at x = y = 4; scale = 2^(e-15) with max|u| < 2^e (frexp), values
 * u/scale rounded to BF16 or FP16 (round to nearest even) and multiplied
 * back.  prec 0 keeps the values. */
static float bf16_round(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;   /* inf / nan */
  uint32_t lsb = (u >> 16) & 1u;
  u += 0x7fffu + lsb;
  u &= 0xffff0000u;
  float r;
  memcpy(&r, &u, 4);
  return r;
}

static float f16_round(float x) {
  /* nearest-even binary16 value of x, returned as float (|x| < 2^15 here) */
  const float a = fabsf(x);
  if (a == 0.0f || a != a) return x;
  int e;
  frexpf(a, &e);                          /* a in [2^(e-1), 2^e) */
  int q = e - 1 - 10;                     /* spacing exponent of 11-bit significands */
  if (q < -24) q = -24;                   /* subnormal spacing 2^-24 */
  const float step = ldexpf(1.0f, q);
  const float r = nearbyintf(a / step) * step;   /* a/step exact: power-of-two division */
  return x < 0 ? -r : r;
}

static void snap_quantise_blocks(const orc_grid *g, void *vol, int prec, int is_double) {
  if (prec == 0) return;
  const int n1 = g->n1, n2 = g->n2, n3 = g->n3;
  const long n12 = (long)n1 * n2;
  const int xe = 4 + 16 * ((n1 - 8) / 16), ye = 4 + 16 * ((n2 - 8) / 16), ze = n3 - 8;
#pragma omp parallel for schedule(static)
  for (int z = 4; z < ze; z++)
    for (int y0 = 4; y0 < ye; y0 += 16)
      for (int x0 = 4; x0 < xe; x0 += 32) {
        const int x1 = x0 + 32 < xe ? x0 + 32 : xe;
        float mx = 0.f;
        for (int y = y0; y < y0 + 16; y++)
          for (int x = x0; x < x1; x++) {
            const long i = z * n12 + (long)y * n1 + x;
            const float v = is_double ? (float)((double *)vol)[i] : ((float *)vol)[i];
            if (fabsf(v) > mx) mx = fabsf(v);
          }
        float sc = 1.f, inv = 1.f;
        if (mx > 0.f) {
          int e;
          frexpf(mx, &e);
          if (e < -100) e = -100;
          sc = ldexpf(1.0f, e - 15);
          inv = ldexpf(1.0f, 15 - e);
        }
        for (int y = y0; y < y0 + 16; y++)
          for (int x = x0; x < x1; x++) {
            const long i = z * n12 + (long)y * n1 + x;
            float v = is_double ? (float)((double *)vol)[i] : ((float *)vol)[i];
            float w = v * inv;
            w = (prec == 1) ? bf16_round(w) : f16_round(w);
            w = w * sc;
            if (is_double) ((double *)vol)[i] = w; else ((float *)vol)[i] = w;
          }
      }
}

static void snap_quantise_f32(const orc_ctx *b, float *vol, int prec) {
  snap_quantise_blocks(&b->g, vol, prec, 0);
}
static void snap_quantise_f64(const orc_ctx *b, double *vol, int prec) {
  snap_quantise_blocks(&b->g, vol, prec, 1);
}

/* ------------------------------------------------------------------------ */
/* precision-generic kernels and loops */
#define REAL float
#define FMA fmaf
#define SFX(name) name##_f32
#define CTX orc_ctx
#define BASE(c) (c)
#define DTAB(c) ((c)->damp_tab)
#define SINC_S(c) ((c)->sinc_s)
#define SINC_D(c) ((c)->sinc_d)
#define SRC_VALS(c) ((c)->src_vals)
#define COEF(c, k) ((c)->coeffs[k])
#include "sepx_oracle_loops.inc"
#undef REAL
#undef FMA
#undef SFX
#undef CTX
#undef BASE
#undef DTAB
#undef SINC_S
#undef SINC_D
#undef SRC_VALS
#undef COEF

/* FP64 context: the oracle context plus double coefficients */
typedef struct {
  const orc_ctx64 *c;
  double coef[13];
} ctx64_full;

#define REAL double
#define FMA fma
#define SFX(name) name##_f64
#define CTX ctx64_full
#define BASE(x) (&(x)->c->base)
#define DTAB(x) ((x)->c->damp_tab)
#define SINC_S(x) ((x)->c->sinc_s)
#define SINC_D(x) ((x)->c->sinc_d)
#define SRC_VALS(x) ((x)->c->src_vals)
#define COEF(x, k) ((x)->coef[k])
#include "sepx_oracle_loops.inc"
#undef REAL
#undef FMA
#undef SFX
#undef CTX
#undef BASE
#undef DTAB
#undef SINC_S
#undef SINC_D
#undef SRC_VALS
#undef COEF

void orc_wave_step_f32(const orc_ctx *c, int vel_inside, float *p0, const float *p1,
                       const float *vel) {
  if (vel_inside)
    wave_adj_f32(c, p0, p1, vel);
  else
    wave_plain_f32(c, p0, p1, vel);
}

void orc_damp_f32(const orc_ctx *c, float *p0, float *p1) { damp_f32(c, p0, p1); }

int orc_source_prop_f32(const orc_ctx *c, const float *vel, float *p0_out, float *p1_out, int jt,
                        int npts, int nt) {
  return source_prop_impl_f32(c, vel, p0_out, p1_out, jt, npts, nt);
}

int orc_rtm_forward_f32(const orc_ctx *c, const float *vel, int jt, const float *img, float *dat,
                        int npts_src, int nt) {
  return rtm_forward_impl_f32(c, vel, jt, img, dat, npts_src, nt);
}

int orc_rtm_adjoint_f32(const orc_ctx *c, const float *vel, int jt, const float *p0_s,
                        const float *p1_s, float *img, const float *dat, int npts_src, int nt) {
  return rtm_adjoint_impl_f32(c, vel, jt, p0_s, p1_s, img, dat, npts_src, nt);
}

/* FP64 twin: get_coeffs evaluated in double from the grid spacings */
static void fill64(const orc_ctx64 *c, ctx64_full *f) {
  f->c = c;
  fd_coeffs_d(c->d1, c->d2, c->d3, f->coef);
}

int orc_lin_source_f32(const orc_ctx *c, const float *vel, int jt, int npts, int nt, int js,
                       int prec, float *snaps) {
  return lin_source_impl_f32(c, vel, jt, npts, nt, js, prec, snaps);
}
int orc_lin_forward_f32(const orc_ctx *c, const float *vel, int jt, int npts, int nt, int js,
                        int prec, const float *m, float *dat) {
  return lin_forward_impl_f32(c, vel, jt, npts, nt, js, prec, m, dat);
}
int orc_lin_adjoint_f32(const orc_ctx *c, const float *vel, int jt, int nt, int js,
                        const float *snaps, const float *dat, float *img) {
  return lin_adjoint_impl_f32(c, vel, jt, nt, js, snaps, dat, img);
}
int orc_lin_adjoint_ckpt_f32(const orc_ctx *c, const float *vel, int jt, int npts, int nt, int js,
                             int prec, int seg, const float *dat, float *img) {
  return lin_adjoint_ckpt_impl_f32(c, vel, jt, npts, nt, js, prec, seg, dat, img);
}
int orc_lin_adjoint_ckpt_f64(const orc_ctx64 *c, const double *vel, int jt, int npts, int nt,
                             int js, int seg, const double *dat, double *img) {
  ctx64_full f;
  fill64(c, &f);
  return lin_adjoint_ckpt_impl_f64(&f, vel, jt, npts, nt, js, 0, seg, dat, img);
}
int orc_lin_source_f64(const orc_ctx64 *c, const double *vel, int jt, int npts, int nt, int js,
                       double *snaps) {
  ctx64_full f;
  fill64(c, &f);
  return lin_source_impl_f64(&f, vel, jt, npts, nt, js, 0, snaps);
}
int orc_lin_forward_f64(const orc_ctx64 *c, const double *vel, int jt, int npts, int nt, int js,
                        const double *m, double *dat) {
  ctx64_full f;
  fill64(c, &f);
  return lin_forward_impl_f64(&f, vel, jt, npts, nt, js, 0, m, dat);
}
int orc_lin_adjoint_f64(const orc_ctx64 *c, const double *vel, int jt, int nt, int js,
                        const double *snaps, const double *dat, double *img) {
  ctx64_full f;
  fill64(c, &f);
  return lin_adjoint_impl_f64(&f, vel, jt, nt, js, snaps, dat, img);
}

int orc_source_prop_f64(const orc_ctx64 *c, const double *vel, double *p0_out, double *p1_out,
                        int jt, int npts, int nt) {
  ctx64_full f;
  fill64(c, &f);
  return source_prop_impl_f64(&f, vel, p0_out, p1_out, jt, npts, nt);
}

int orc_rtm_forward_f64(const orc_ctx64 *c, const double *vel, int jt, const double *img,
                        double *dat, int npts_src, int nt) {
  ctx64_full f;
  fill64(c, &f);
  return rtm_forward_impl_f64(&f, vel, jt, img, dat, npts_src, nt);
}

int orc_rtm_adjoint_f64(const orc_ctx64 *c, const double *vel, int jt, const double *p0_s,
                        const double *p1_s, double *img, const double *dat, int npts_src, int nt) {
  ctx64_full f;
  fill64(c, &f);
  return rtm_adjoint_impl_f64(&f, vel, jt, p0_s, p1_s, img, dat, npts_src, nt);
}
