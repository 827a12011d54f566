// sepx_gpu_funcs.cu -- the device state and the three time loops behind the
// reference-named C ABI (include/sepx.h; Born/gpu_funcs_3d.h / .cu).
//
// Layout in HBM: every volume is stored with a row pitch rounded up to 32
// floats and its logical origin 28 floats into a 256-byte aligned allocation,
// so x = 4 (the first updated column) starts a 128-byte line; each volume owns
// two TMA descriptors (halo box and centre box).  Traces are held time-major
// ([ntrace][nrec]) so that injection / extraction touch contiguous receivers;
// the reference's trace-major host layout is restored on the way out.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <memory>
#include <cmath>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sepx.h"
#include "../../include/sepx_batch.h"
#include "sepx_aux.h"
#include "sepx_blas.h"
#include "sepx_common.h"
#include "sepx_device.cuh"
#include "sepx_prop.h"

namespace sepx {
namespace {

constexpr int kLead = 28;   // logical origin offset (floats) inside an allocation

struct Volume {
  float *base = nullptr;
  float *origin = nullptr;
  CUtensorMap tm_h, tm_c;
  CUtensorMap tm_h2;   // 40 x 40 halo box of the two-row tile
};

struct PointMapDev {
  int npts = -1;              // points the maps were built for (-1: none)
  int *plane_slot = nullptr;  // [n3]
  int *map = nullptr;         // [nslot][n2][n1]
  int *next = nullptr;        // [npts]
  long long *off = nullptr;   // [npts] pitched offsets from the origin
  int nslot = 0;
  std::vector<int> built;     // the points the maps were built from
};

struct Ctx {
  bool have_device = false;
  cudaStream_t stream = nullptr;
  int *d_err = nullptr;
  PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  int zchunk_override = 0;
  // modes (bit per PropMode) that run the two-row tile (32 x 32 cells per
  // CTA): none by default -- on GB300 at 560 x 560 x 496 it measured slower
  // than the one-row tile for every mode (2 CTAs per SM instead of 4)
  int rows2_mask = 0;
  int num_sms = 152;
  // grid
  bool have_grid = false;
  int n1 = 0, n2 = 0, n3 = 0, pitch = 0;
  long long plane = 0;
  size_t alloc_floats = 0;
  float d[3] = {0, 0, 0}, bc_a = 0, bc_b = 0, bc_b_y = 0;
  float coef[13];
  float *d_damp = nullptr;
  int ntab = 0;
  PropGeom geom;
  Volume vel, img, F[4], SL[2], X;   // X: increment of the linearised pair
  bool vel_set = false;
  int sl_p0 = 0, sl_p1 = 1;   // which SL volume holds the older / newest field
  bool sl_valid = false;
  // sinc tables
  int nsinc = 8, ns = 0, nd = 0;
  float *d_sinc_s = nullptr, *d_sinc_d = nullptr;
  int ntrace = 0;             // ntrace_gpu: the last transfer wins
  // sources
  int npts_s = 0, src_ntrace = 0;
  std::vector<int> src_loc;
  float *d_src_vals = nullptr;
  size_t src_cap = 0;
  PointMapDev srcmap;
  // receivers
  int rec_nx = 0, rec_ny = 0, rec_ntrace = 0;
  std::vector<int> rec_loc;
  float *d_trc = nullptr;     // time-major [ntrace][nrec]
  size_t trc_cap = 0;
  PointMapDev recmap;
  // scratch
  float *d_inj = nullptr;
  size_t inj_cap = 0;
  float *d_stage = nullptr;
  size_t stage_cap = 0;
  double *d_dot = nullptr;    // dot-product partials + result
  size_t dot_cap = 0;
  // compressed source snapshots of the linearised pair
  unsigned char *d_snap = nullptr;
  size_t snap_cap = 0;
  float *d_snap_scale = nullptr;
  size_t snap_scale_cap = 0;
  int snap_js = 0, snap_prec = -1, snap_nt = -1;
};

// The current context.  One shot lives in one context; a batch of shots
// (sepx_batch_*) holds one context per shot and switches between them.
Ctx g_default;
Ctx *g_cur = &g_default;
#define G (*g_cur)
std::string g_err;          // the last error message, whichever context raised it
long long g_launches = 0;   // kernels launched through this library

int fail(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return -1;
}

#define CK(expr)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail("%s failed at %s:%d: %s", #expr, __FILE__, __LINE__, cudaGetErrorString(e_)); \
  } while (0)

#define CKL(expr)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    g_launches++;                                                                        \
    if (e_ != cudaSuccess)                                                               \
      return fail("kernel launch %s failed: %s", #expr, cudaGetErrorString(e_));         \
  } while (0)

#define RET(x)            \
  do {                    \
    int r_ = (x);         \
    if (r_) return r_;    \
  } while (0)

// a buffer the call reads or writes: NULL is reported, never dereferenced
int need_buf(const void *p, const char *what) {
  return p ? 0 : fail("%s: NULL buffer", what);
}
// n elements at p (host or device): n >= 0, and p given when n > 0
int need_span(const void *p, long long n, const char *what) {
  if (n < 0) return fail("%s: negative length %lld", what, n);
  return n > 0 ? need_buf(p, what) : 0;
}

template <class T>
int ensure(T **p, size_t *cap, size_t n) {
  if (*cap >= n && *p) return 0;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  CK(cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(T)));
  *cap = n;
  return 0;
}

void free_pointmap(PointMapDev &m) {
  cudaFree(m.plane_slot); cudaFree(m.map); cudaFree(m.next); cudaFree(m.off);
  m = PointMapDev();
}

void free_volume(Volume &v) {
  if (v.base) cudaFree(v.base);
  v.base = v.origin = nullptr;
}

void free_grid() {
  free_volume(G.vel); free_volume(G.img);
  for (auto &v : G.F) free_volume(v);
  for (auto &v : G.SL) free_volume(v);
  free_volume(G.X);
  cudaFree(G.d_damp); G.d_damp = nullptr;
  free_pointmap(G.srcmap); free_pointmap(G.recmap);
  G.have_grid = G.vel_set = G.sl_valid = false;
}

int need_device() {
  if (G.have_device) return 0;
  return fail("setup_cuda must be called first");
}

int need_grid() {
  RET(need_device());
  if (G.have_grid) return 0;
  return fail("create_gpu_space must be called first");
}

int encode_map(CUtensorMap *m, float *origin, int bx, int by) {
  cuuint64_t dims[3] = {(cuuint64_t)G.n1, (cuuint64_t)G.n2, (cuuint64_t)G.n3};
  cuuint64_t strides[2] = {(cuuint64_t)G.pitch * 4, (cuuint64_t)G.plane * 4};
  cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = G.encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, origin, dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail("cuTensorMapEncodeTiled failed (%d)", (int)r);
  return 0;
}

int alloc_volume(Volume &v) {
  CK(cudaMalloc((void **)&v.base, G.alloc_floats * sizeof(float)));
  CK(cudaMemsetAsync(v.base, 0, G.alloc_floats * sizeof(float), G.stream));
  v.origin = v.base + kLead;
  RET(encode_map(&v.tm_h, v.origin, kHX, kHY));
  RET(encode_map(&v.tm_c, v.origin, kTX, kTY));
  RET(encode_map(&v.tm_h2, v.origin, kHX, kHY2));
  return 0;
}

int zero_volume(Volume &v) {
  CK(cudaMemsetAsync(v.base, 0, G.alloc_floats * sizeof(float), G.stream));
  return 0;
}

// Host volumes are dense (n1 floats per row), device volumes pitched.  A
// pitched copy (cudaMemcpy2D) moves rows of n1 floats one by one and runs far
// below the link's rate on GB300 (24-50 GB/s for 2240-byte rows against
// 191-208 GB/s for flat copies), so whole planes go over as flat copies
// through the staging buffer and a kernel re-pitches them on the device.
int h2d_volume(Volume &v, const float *host) {
  const size_t plane = (size_t)G.n1 * G.n2;
  const size_t nz = std::max<size_t>(1, ((size_t)64 << 20) / (plane * 4));
  RET(ensure(&G.d_stage, &G.stage_cap, std::min<size_t>(nz, G.n3) * plane));
  for (size_t z0 = 0; z0 < (size_t)G.n3; z0 += nz) {
    const size_t k = std::min(nz, (size_t)G.n3 - z0);
    CK(cudaMemcpyAsync(G.d_stage, host + z0 * plane, k * plane * 4, cudaMemcpyHostToDevice, G.stream));
    CKL(launch_repitch(G.d_stage, G.n1, v.origin + z0 * G.plane, G.pitch, G.n1, (long long)k * G.n2,
                       G.stream));
  }
  return 0;
}

int d2h_volume(float *host, const Volume &v) {
  const size_t plane = (size_t)G.n1 * G.n2;
  const size_t nz = std::max<size_t>(1, ((size_t)64 << 20) / (plane * 4));
  RET(ensure(&G.d_stage, &G.stage_cap, std::min<size_t>(nz, G.n3) * plane));
  for (size_t z0 = 0; z0 < (size_t)G.n3; z0 += nz) {
    const size_t k = std::min(nz, (size_t)G.n3 - z0);
    CKL(launch_repitch(v.origin + z0 * G.plane, G.pitch, G.d_stage, G.n1, G.n1, (long long)k * G.n2,
                       G.stream));
    CK(cudaMemcpyAsync(host + z0 * plane, G.d_stage, k * plane * 4, cudaMemcpyDeviceToHost, G.stream));
  }
  return 0;
}

int d2d_volume(Volume &dst, const Volume &src) {
  CK(cudaMemcpyAsync(dst.base, src.base, G.alloc_floats * sizeof(float), cudaMemcpyDeviceToDevice,
                     G.stream));
  return 0;
}

int check_dims(int n1, int n2, int n3) {
  if (n1 != G.n1 || n2 != G.n2 || n3 != G.n3)
    return fail("grid %dx%dx%d does not match create_gpu_space (%dx%dx%d)", n1, n2, n3, G.n1,
                G.n2, G.n3);
  return 0;
}

bool inside_interior(int loc, int *x, int *y, int *z) {
  if (loc < 0 || (long long)loc >= (long long)G.n1 * G.n2 * G.n3) return false;
  *x = loc % G.n1;
  *y = (loc / G.n1) % G.n2;
  *z = loc / (G.n1 * G.n2);
  const PropGeom &g = G.geom;
  return *x >= g.xb && *x < g.xe && *y >= g.yb && *y < g.ye && *z >= g.zb && *z < g.ze;
}

// Plane-indexed point maps: the kernel checks one slot per z plane and chains
// points that share a cell in ascending id order.
int build_pointmap(PointMapDev &m, const std::vector<int> &loc, int npts, const char *what) {
  // the same points again (a shot's receivers transferred once per loop):
  // the maps on the device are still right
  if (m.npts == npts && m.plane_slot && (int)m.built.size() == npts &&
      std::equal(m.built.begin(), m.built.end(), loc.begin()))
    return 0;
  free_pointmap(m);
  std::vector<int> slot(G.n3, -1), next(std::max(npts, 1), -1);
  std::vector<long long> off(std::max(npts, 1), 0);
  std::vector<int> planes;
  std::vector<int> xs(npts), ys(npts), zs(npts);
  for (int i = 0; i < npts; i++) {
    if (!inside_interior(loc[i], &xs[i], &ys[i], &zs[i]))
      return fail("%s point %d (cell %d) lies outside the propagated interior", what, i, loc[i]);
    if (slot[zs[i]] < 0) {
      slot[zs[i]] = (int)planes.size();
      planes.push_back(zs[i]);
    }
    off[i] = xs[i] + (long long)G.pitch * ys[i] + G.plane * zs[i];
  }
  const long long n12 = (long long)G.n1 * G.n2;
  std::vector<int> map(std::max<size_t>(1, planes.size() * n12), -1);
  for (int i = npts - 1; i >= 0; i--) {   // descending so that chains run ascending
    long long c = (long long)slot[zs[i]] * n12 + (long long)ys[i] * G.n1 + xs[i];
    next[i] = map[c];
    map[c] = i;
  }
  m.nslot = (int)planes.size();
  m.npts = npts;
  CK(cudaMalloc((void **)&m.plane_slot, sizeof(int) * G.n3));
  CK(cudaMalloc((void **)&m.map, sizeof(int) * map.size()));
  CK(cudaMalloc((void **)&m.next, sizeof(int) * next.size()));
  CK(cudaMalloc((void **)&m.off, sizeof(long long) * off.size()));
  CK(cudaMemcpyAsync(m.plane_slot, slot.data(), sizeof(int) * G.n3, cudaMemcpyHostToDevice, G.stream));
  CK(cudaMemcpyAsync(m.map, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice, G.stream));
  CK(cudaMemcpyAsync(m.next, next.data(), sizeof(int) * next.size(), cudaMemcpyHostToDevice, G.stream));
  CK(cudaMemcpyAsync(m.off, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, G.stream));
  CK(cudaStreamSynchronize(G.stream));   // host vectors go out of scope
  m.built.assign(loc.begin(), loc.begin() + npts);
  return 0;
}

// Planes per CTA along z.  Longer chunks amortise the 8-plane warm-up of the
// z-queues; shorter ones balance the waves.  Measured on GB300 at 560x560x496:
// source_prop and the Born forward are best near 80 planes, the RTM adjoint
// near 32.  Small grids shorten the chunk until there are two waves of
// 3 CTAs per SM.
int auto_zchunk(int mode) {
  if (G.zchunk_override > 0) return G.zchunk_override;
  const PropGeom &g = G.geom;
  const long long tiles = (long long)((g.xe - g.xb + kTX - 1) / kTX) * ((g.ye - g.yb + kTY - 1) / kTY);
  const int depth = std::max(1, g.ze - g.zb);
  int zc = (mode == kRtmAdj || mode == kRtmAdj1 || mode == kLinAdj) ? 32 : 80;
  while (zc > 16 && tiles * ((depth + zc - 1) / zc) < 2LL * 3 * G.num_sms) zc /= 2;
  return std::max(1, std::min(zc, depth));
}

// The same for the two-row tile (32 x 32 cells, 2 CTAs per SM): the chunk
// count of the target length, planes spread evenly over the chunks.
int auto_zchunk2(int mode) {
  if (G.zchunk_override > 0) return G.zchunk_override;
  const PropGeom &g = G.geom;
  const long long tiles = (long long)((g.xe - g.xb + kTX - 1) / kTX) * ((g.ye - g.yb + kTY2 - 1) / kTY2);
  const int depth = std::max(1, g.ze - g.zb);
  int zc = (mode == kRtmAdj) ? 32 : 80;
  while (zc > 16 && tiles * ((depth + zc - 1) / zc) < 2LL * 2 * G.num_sms) zc /= 2;
  const int nch = (depth + zc - 1) / zc;
  return std::max(1, std::min((depth + nch - 1) / nch, depth));
}

// One fused step with the mode's z-chunk; modes in rows2_mask take the
// two-row tile when the 40 x 40 halo maps are given.
cudaError_t launch_step(int mode, const PropParams &P0, const Rows2Maps *H = nullptr) {
  PropParams P = P0;
  if (H && ((G.rows2_mask >> mode) & 1) && prop_step2_supported(mode)) {
    P.g.zchunk = auto_zchunk2(mode);
    return launch_prop_step2(mode, P, *H, G.stream);
  }
  P.g.zchunk = auto_zchunk(mode);
  return launch_prop_step(mode, P, G.stream);
}

PropParams base_params() {
  PropParams P;
  memset(&P, 0, sizeof(P));
  P.g = G.geom;
  memcpy(P.coef, G.coef, sizeof(G.coef));
  P.damp_tab = G.d_damp;
  P.ntab = G.ntab;
  P.vel = G.vel.origin;
  P.tm_vel_h = G.vel.tm_h;
  P.tm_vel_c = G.vel.tm_c;
  P.tm_img_c = G.img.tm_c;
  P.img = G.img.origin;
  P.err = G.d_err;
  return P;
}

void set_field(PropParams &P, int f, const Volume &cur, const Volume &prev) {
  P.tm_cur_h[f] = cur.tm_h;
  P.tm_cur_c[f] = cur.tm_c;
  P.tm_prev_c[f] = prev.tm_c;
  P.cur[f] = cur.origin;
  P.out[f] = prev.origin;
}

int check_device_error() {
  int h = 0;
  CK(cudaMemcpyAsync(&h, G.d_err, sizeof(int), cudaMemcpyDeviceToHost, G.stream));
  CK(cudaStreamSynchronize(G.stream));
  if (h) {
    CK(cudaMemsetAsync(G.d_err, 0, sizeof(int), G.stream));
    return fail("a propagation kernel gave up waiting on its copy pipeline (code %d)", h);
  }
  return 0;
}

int prep_inj(int npts, int jt, int nsteps, int j0, float dir) {
  if (npts <= 0) return 0;
  if (npts > G.npts_s) return fail("npts (%d) exceeds the transferred source points (%d)", npts, G.npts_s);
  if (jt > G.ns) return fail("time ratio jt=%d needs %d source sinc rows, %d transferred", jt, jt, G.ns);
  const int last = j0 + nsteps - 1;
  if (last >= 0 && last / jt + 7 >= G.src_ntrace)
    return fail("source traces too short: step %d reads sample %d of %d", last, last / jt + 7,
                G.src_ntrace);
  RET(ensure(&G.d_inj, &G.inj_cap, (size_t)std::max(nsteps, 1) * npts));
  CKL(launch_inj_values(G.d_src_vals, G.src_ntrace, npts, G.d_sinc_s, G.nsinc, jt, nsteps, j0, dir,
                        G.d_inj, G.stream));
  if (G.srcmap.npts != npts) {
    std::vector<int> loc(G.src_loc.begin(), G.src_loc.begin() + npts);
    RET(build_pointmap(G.srcmap, loc, npts, "source"));
  }
  return 0;
}

int prep_receivers(int jt, int nt) {
  if (G.recmap.npts < 0) return fail("transfer_receiver_func must be called first");
  if (jt > G.nd) return fail("time ratio jt=%d needs %d receiver sinc rows, %d transferred", jt, jt, G.nd);
  if (nt > 0 && (nt - 1) / jt + 7 >= G.rec_ntrace)
    return fail("receiver traces too short: %d samples for %d steps", G.rec_ntrace, nt);
  return 0;
}

// ------------------------------------------------------------------ loops
int loop_source_prop(int jt, int npts, int nt) {
  RET(need_grid());
  if (!G.vel_set) return fail("transfer_vel_func1 must be called first");
  if (jt < 1 || nt < 0) return fail("invalid jt=%d / nt=%d", jt, nt);
  RET(prep_inj(npts, jt, nt + 1, 0, 1.0f));
  Volume *A = &G.SL[0], *B = &G.SL[1];
  RET(zero_volume(*A));
  RET(zero_volume(*B));
  PropParams P = base_params();
  Rows2Maps H;
  H.vel_h = G.vel.tm_h2;
  P.src.plane_slot = G.srcmap.plane_slot;
  P.src.map = G.srcmap.map;
  P.src.next = G.srcmap.next;
  for (int it = 0; it <= nt; it++) {
    set_field(P, 0, *B, *A);
    H.cur_h[0] = B->tm_h2;
    P.inj_s = G.d_inj + (size_t)it * std::max(npts, 0);
    if (npts <= 0) P.src.plane_slot = nullptr;
    CKL(launch_step(kSrcProp, P, &H));
    std::swap(A, B);
  }
  G.sl_p0 = (A == &G.SL[0]) ? 0 : 1;
  G.sl_p1 = 1 - G.sl_p0;
  G.sl_valid = true;
  return 0;
}

int loop_rtm_forward(int jt, int npts_src, int nt) {
  RET(need_grid());
  if (!G.vel_set) return fail("transfer_vel_func1 must be called first");
  if (jt < 1 || nt < 0) return fail("invalid jt=%d / nt=%d", jt, nt);
  RET(prep_receivers(jt, nt));
  RET(prep_inj(npts_src, jt, nt, 0, 1.0f));
  Volume *D0 = &G.F[0], *D1 = &G.F[1], *S0 = &G.F[2], *S1 = &G.F[3];
  for (auto *v : {D0, D1, S0, S1}) RET(zero_volume(*v));
  PropParams P = base_params();
  P.src.plane_slot = npts_src > 0 ? G.srcmap.plane_slot : nullptr;
  P.src.map = G.srcmap.map;
  P.src.next = G.srcmap.next;
  P.rec.plane_slot = G.recmap.plane_slot;
  P.rec.map = G.recmap.map;
  P.rec.next = G.recmap.next;
  P.trc = G.d_trc;
  P.nrec = G.rec_nx * G.rec_ny;
  Rows2Maps H;
  H.vel_h = G.vel.tm_h2;
  for (int it = 0; it < nt; it++) {
    const int id = it / jt, ii = it - id * jt;
    set_field(P, 0, *D1, *D0);
    set_field(P, 1, *S1, *S0);
    H.cur_h[0] = D1->tm_h2;
    H.cur_h[1] = S1->tm_h2;
    P.inj_s = G.d_inj + (size_t)it * std::max(npts_src, 0);
    P.do_scatter = (it % jt == 0);
    P.trc_id = id;
    P.sinc_row = G.d_sinc_d + (size_t)ii * G.nsinc;
    CKL(launch_step(kBornFwd, P, &H));
    std::swap(D0, D1);
    std::swap(S0, S1);
  }
  return 0;
}

// S0 / S1 hold the source wavefields (p0_s, p1_s) on entry (G.F[2], G.F[3]).
int loop_rtm_adjoint(int jt, int npts, int nt) {
  RET(need_grid());
  if (!G.vel_set) return fail("transfer_vel_func1 must be called first");
  if (jt < 1 || nt < 0) return fail("invalid jt=%d / nt=%d", jt, nt);
  RET(prep_receivers(jt, nt));
  if (nt > 1) RET(prep_inj(npts, jt, nt - 1, 1, -1.0f));
  Volume *D0 = &G.F[0], *D1 = &G.F[1], *S0 = &G.F[2], *S1 = &G.F[3];
  RET(zero_volume(*D0));
  RET(zero_volume(*D1));
  RET(zero_volume(G.img));
  PropParams P = base_params();
  P.rec.plane_slot = G.recmap.plane_slot;
  P.rec.map = G.recmap.map;
  P.rec.next = G.recmap.next;
  P.trc = G.d_trc;
  P.nrec = G.rec_nx * G.rec_ny;
  Rows2Maps H;
  H.vel_h = G.vel.tm_h2;
  for (int it = nt - 1; it >= 0; it--) {
    const int id = it / jt, ii = it - id * jt;
    P.trc_id = id;
    P.sinc_row = G.d_sinc_d + (size_t)ii * G.nsinc;
    P.do_image = (ii == 0);
    set_field(P, 0, *D1, *D0);
    if (it == nt - 1) {
      P.tm_aux_c = S0->tm_c;
      CKL(launch_step(kRtmAdj1, P));
    } else {
      set_field(P, 1, *S1, *S0);
      H.cur_h[0] = D1->tm_h2;
      H.cur_h[1] = S1->tm_h2;
      CKL(launch_step(kRtmAdj, P, &H));
      if (npts > 0)
        CKL(launch_point_add(S1->origin, G.srcmap.off, G.d_inj + (size_t)it * npts, npts, G.stream));
      std::swap(S0, S1);
    }
    std::swap(D0, D1);
  }
  return 0;
}

// ---------------------------------------------------------- linearised Born pair
long long snap_blocks_per_step() {
  const PropGeom &g = G.geom;
  const long long ntx = (g.xe - g.xb + kTX - 1) / kTX, nty = (g.ye - g.yb) / kTY;
  return ntx * nty * std::max(0, g.ze - g.zb);
}

int ensure_snapshots(int nt, int js, int prec) {
  if (js < 1) return fail("snapshot interval must be >= 1");
  if (prec < kSnapF32 || prec > kSnapF16) return fail("unknown snapshot precision %d", prec);
  const long long nsnap = (nt + js - 1) / js;
  const long long blocks = snap_blocks_per_step() * std::max(1LL, nsnap);
  const size_t bytes = (size_t)blocks * kCenterFloats * (prec == kSnapF32 ? 4 : 2);
  RET(ensure(&G.d_snap, &G.snap_cap, bytes));
  RET(ensure(&G.d_snap_scale, &G.snap_scale_cap, (size_t)blocks));
  return 0;
}

PropParams lin_params(int js, int prec) {
  PropParams P = base_params();
  P.snap = G.d_snap;
  P.snap_scale = G.d_snap_scale;
  P.snap_prec = prec;
  (void)js;
  return P;
}

// source wavefield u_t, t = 0..nt-1, stored every js steps
int loop_lin_source(int jt, int npts, int nt, int js, int prec) {
  RET(need_grid());
  if (!G.vel_set) return fail("transfer_vel_func1 must be called first");
  if (jt < 1 || nt < 0) return fail("invalid jt=%d / nt=%d", jt, nt);
  RET(ensure_snapshots(nt, js, prec));
  RET(prep_inj(npts, jt, nt, 0, 1.0f));
  Volume *A = &G.F[2], *B = &G.F[3];
  RET(zero_volume(*A));
  RET(zero_volume(*B));
  PropParams P = lin_params(js, prec);
  P.src.plane_slot = npts > 0 ? G.srcmap.plane_slot : nullptr;
  P.src.map = G.srcmap.map;
  P.src.next = G.srcmap.next;
  for (int it = 0; it < nt; it++) {
    set_field(P, 0, *B, *A);
    P.inj_s = G.d_inj + (size_t)it * std::max(npts, 0);
    P.do_snap = (it % js == 0);
    P.snap_index = it / js;
    CKL(launch_step(kLinSrc, P));
    std::swap(A, B);
  }
  G.snap_js = js;
  G.snap_prec = prec;
  G.snap_nt = nt;
  return 0;
}

// traces += R v_t with v from the model in the image buffer (increment form:
// positions ping-pong between F[0] / F[1], the increment X is updated in place)
int loop_lin_forward(int jt, int npts, int nt, int js, int prec) {
  RET(need_grid());
  if (!G.vel_set) return fail("transfer_vel_func1 must be called first");
  if (jt < 1 || nt < 0) return fail("invalid jt=%d / nt=%d", jt, nt);
  RET(prep_receivers(jt, nt));
  RET(prep_inj(npts, jt, nt, 0, 1.0f));
  if (prec < kSnapF32 || prec > kSnapF16 || js < 1) return fail("invalid snapshot settings");
  Volume *V0 = &G.F[0], *V1 = &G.F[1], *S0 = &G.F[2], *S1 = &G.F[3], *X = &G.X;
  for (auto *v : {V0, V1, S0, S1, X}) RET(zero_volume(*v));
  PropParams P = lin_params(js, prec);
  P.src.plane_slot = npts > 0 ? G.srcmap.plane_slot : nullptr;
  P.src.map = G.srcmap.map;
  P.src.next = G.srcmap.next;
  P.rec.plane_slot = G.recmap.plane_slot;
  P.rec.map = G.recmap.map;
  P.rec.next = G.recmap.next;
  P.trc = G.d_trc;
  P.nrec = G.rec_nx * G.rec_ny;
  for (int it = 0; it < nt; it++) {
    const int id = it / jt, ii = it - id * jt;
    set_field(P, 0, *V1, *X);   // current position, increment
    P.out[0] = V0->origin;      // new position
    P.out2 = X->origin;         // new increment (in place)
    set_field(P, 1, *S1, *S0);
    P.inj_s = G.d_inj + (size_t)it * std::max(npts, 0);
    P.do_snap = P.do_scatter = (it % js == 0);
    P.snap_index = it / js;
    P.trc_id = id;
    P.sinc_row = G.d_sinc_d + (size_t)ii * G.nsinc;
    CKL(launch_step(kLinFwd, P));
    std::swap(V0, V1);
    std::swap(S0, S1);
  }
  return 0;
}

// image := sum_t c u^_t b_t from the traces: the exact transpose of
// loop_lin_forward (B ping-pongs between F[0] / F[1], a is updated in F[2])
int loop_lin_adjoint(int jt, int nt, int js, int prec) {
  RET(need_grid());
  if (!G.vel_set) return fail("transfer_vel_func1 must be called first");
  if (jt < 1 || nt < 0) return fail("invalid jt=%d / nt=%d", jt, nt);
  if (G.snap_nt != nt || G.snap_js != js || G.snap_prec != prec)
    return fail("no source snapshots for nt=%d js=%d prec=%d: run the source pass first", nt, js, prec);
  RET(prep_receivers(jt, nt));
  Volume *B0 = &G.F[0], *B1 = &G.F[1], *A = &G.F[2];
  RET(zero_volume(*B0));
  RET(zero_volume(*B1));
  RET(zero_volume(*A));
  RET(zero_volume(G.img));
  PropParams P = lin_params(js, prec);
  P.rec.plane_slot = G.recmap.plane_slot;
  P.rec.map = G.recmap.map;
  P.rec.next = G.recmap.next;
  P.trc = G.d_trc;
  P.nrec = G.rec_nx * G.rec_ny;
  for (int it = nt - 1; it >= 0; it--) {
    const int id = it / jt, ii = it - id * jt;
    set_field(P, 0, *B1, *A);   // B_{t+1}, a_{t+1}
    P.out[0] = B0->origin;      // B_t
    P.out2 = A->origin;         // a_t (in place)
    P.do_snap = P.do_image = (it % js == 0);
    P.snap_index = it / js;
    P.trc_id = id;
    P.sinc_row = G.d_sinc_d + (size_t)ii * G.nsinc;
    CKL(launch_step(kLinAdj, P));
    std::swap(B0, B1);
  }
  return 0;
}

// traces: host trace-major [nrec][nt] <-> device time-major [nt][nrec]
int traces_h2d(const float *vals, int nrec, int nt) {
  const size_t chunk = std::max<size_t>(1, (size_t)(64u << 20) / std::max(nt, 1));
  RET(ensure(&G.d_stage, &G.stage_cap, std::min<size_t>(chunk, nrec) * nt));
  for (size_t r0 = 0; r0 < (size_t)nrec; r0 += chunk) {
    const int rows = (int)std::min(chunk, (size_t)nrec - r0);
    CK(cudaMemcpyAsync(G.d_stage, vals + r0 * nt, sizeof(float) * rows * nt, cudaMemcpyHostToDevice,
                       G.stream));
    CKL(launch_transpose(G.d_stage, nt, G.d_trc + r0, nrec, rows, nt, G.stream));
  }
  return 0;
}

int traces_d2h(float *vals, int nrec, int nt) {
  const size_t chunk = std::max<size_t>(1, (size_t)(64u << 20) / std::max(nt, 1));
  RET(ensure(&G.d_stage, &G.stage_cap, std::min<size_t>(chunk, nrec) * nt));
  for (size_t r0 = 0; r0 < (size_t)nrec; r0 += chunk) {
    const int rows = (int)std::min(chunk, (size_t)nrec - r0);
    CKL(launch_transpose(G.d_trc + r0, nrec, G.d_stage, nt, nt, rows, G.stream));
    CK(cudaMemcpyAsync(vals + r0 * nt, G.d_stage, sizeof(float) * rows * nt, cudaMemcpyDeviceToHost,
                       G.stream));
  }
  return 0;
}

}  // namespace

int set_error(const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return -1;
}

}  // namespace sepx

using namespace sepx;

extern "C" {

// ------------------------------------------------------------ set-up
int sepx_setup_cuda(int ngpus) {
  if (ngpus != 1)
    return fail("ngpus=%d: this implementation runs the whole model on one GPU (ngpus must be 1)",
                ngpus);
  if (G.have_device) return 0;
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev));
  if (ndev < 1) return fail("no CUDA device");
  CK(cudaSetDevice(0));
  CK(cudaDeviceGetAttribute(&G.num_sms, cudaDevAttrMultiProcessorCount, 0));
  CK(cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking));
  CK(cudaMalloc((void **)&G.d_err, sizeof(int)));
  CK(cudaMemsetAsync(G.d_err, 0, sizeof(int), G.stream));
  cudaDriverEntryPointQueryResult q;
  void *fn = nullptr;
  CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  if (!fn || q != cudaDriverEntryPointSuccess) return fail("cuTensorMapEncodeTiled is unavailable");
  G.encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  G.have_device = true;
  return 0;
}

int sepx_create_gpu_space(float d1, float d2, float d3, float bc_a, float bc_b, float bc_b_y,
                          int n1, int n2, int n3) {
  RET(need_device());
  if (n1 < 16 || n2 < 16 || n3 < 16) return fail("grid %dx%dx%d is smaller than 16 cells", n1, n2, n3);
  if (!(d1 > 0 && d2 > 0 && d3 > 0)) return fail("grid spacing must be positive");
  const bool same = G.have_grid && n1 == G.n1 && n2 == G.n2 && n3 == G.n3;
  if (!same) free_grid();
  G.n1 = n1; G.n2 = n2; G.n3 = n3;
  G.pitch = (n1 + 31) / 32 * 32;
  G.plane = (long long)G.pitch * n2;
  G.alloc_floats = (size_t)kLead + (size_t)G.plane * n3 + 32;
  G.d[0] = d1; G.d[1] = d2; G.d[2] = d3;
  G.bc_a = bc_a; G.bc_b = bc_b; G.bc_b_y = bc_b_y;
  // get_coeffs in double (Born/wave_fkernel.3d8o.cu:26-27), stored as float
  auto c00 = [](double d) { return 8.0 / (5.0 * d * d); };
  const double a = d1, b = d2, c = d3;
  const double cd[13] = {-1025.0 / 576.0 * (c00(a) + c00(b) + c00(c)), c00(a), c00(b), c00(c),
                         -c00(a) / 8.0, -c00(b) / 8.0, -c00(c) / 8.0, c00(a) / 63.0, c00(b) / 63.0,
                         c00(c) / 63.0, -c00(a) / 896.0, -c00(b) / 896.0, -c00(c) / 896.0};
  for (int k = 0; k < 13; k++) G.coef[k] = (float)cd[k];
  // sponge factor by edge distance: expf(-bc_b*(bc_a-edge)) when < 1
  int ntab_all = std::max(n1, std::max(n2, n3)) / 2 + 1;
  std::vector<float> tab(ntab_all);
  G.ntab = 0;   // entries past the last factor < 1 are 1: the kernels stop there
  for (int e = 0; e < ntab_all; e++) {
    const float arg = -bc_b * (bc_a - (float)e);
    const float t = (float)std::exp((double)arg);
    tab[e] = (t < 1.0f) ? t : 1.0f;
    if (tab[e] < 1.0f) G.ntab = e + 1;
  }
  PropGeom &g = G.geom;
  g.n1 = n1; g.n2 = n2; g.n3 = n3; g.pitch = G.pitch; g.plane = G.plane;
  g.xb = 4; g.xe = 4 + 16 * ((n1 - 8) / 16);
  g.yb = 4; g.ye = 4 + 16 * ((n2 - 8) / 16);
  g.zb = 4; g.ze = n3 - 8;
  g.xg = 16 * ((n1 - 8) / 16);
  g.yg = 16 * ((n2 - 8) / 16);
  g.zchunk = 0;
  if (!same) {
    RET(alloc_volume(G.vel));
    RET(alloc_volume(G.img));
    for (auto &v : G.F) RET(alloc_volume(v));
    for (auto &v : G.SL) RET(alloc_volume(v));
    RET(alloc_volume(G.X));
  }
  cudaFree(G.d_damp);
  G.d_damp = nullptr;
  CK(cudaMalloc((void **)&G.d_damp, sizeof(float) * std::max(G.ntab, 1)));
  if (G.ntab > 0)
    CK(cudaMemcpyAsync(G.d_damp, tab.data(), sizeof(float) * G.ntab, cudaMemcpyHostToDevice, G.stream));
  CK(cudaStreamSynchronize(G.stream));
  G.have_grid = true;
  // geometry changed: point maps are rebuilt on the next transfer
  if (!same) { G.srcmap.npts = -1; G.recmap.npts = -1; }
  return 0;
}

static int upload_sinc(int nsinc, int n, float **tables, float **dst, int *nrows) {
  RET(need_device());
  if (nsinc < 8) return fail("sinc tables need at least 8 taps (got %d)", nsinc);
  if (n < 1) return fail("empty sinc table");
  RET(need_buf(tables, "sinc tables"));
  for (int i = 0; i < n; i++) RET(need_buf(tables[i], "sinc table row"));
  std::vector<float> flat((size_t)nsinc * n);
  for (int i = 0; i < n; i++) memcpy(&flat[(size_t)i * nsinc], tables[i], sizeof(float) * nsinc);
  cudaFree(*dst);
  *dst = nullptr;
  CK(cudaMalloc((void **)dst, sizeof(float) * flat.size()));
  CK(cudaMemcpy(*dst, flat.data(), sizeof(float) * flat.size(), cudaMemcpyHostToDevice));
  *nrows = n;
  G.nsinc = nsinc;
  return 0;
}

int sepx_transfer_sinc_table_s(int nsinc, int ns, float **tables) {
  return upload_sinc(nsinc, ns, tables, &G.d_sinc_s, &G.ns);
}

int sepx_transfer_sinc_table_d(int nsinc, int nd, float **tables) {
  return upload_sinc(nsinc, nd, tables, &G.d_sinc_d, &G.nd);
}

int sepx_transfer_source_func(int npts, int nt, const int *locs, const float *vals) {
  if (npts < 0 || nt < 1) return fail("invalid source shape %d x %d", npts, nt);
  RET(need_span(locs, npts, "transfer_source_func locs"));
  RET(need_span(vals, npts, "transfer_source_func vals"));
  RET(need_grid());
  G.src_loc.assign(locs, locs + npts);
  G.npts_s = npts;
  G.src_ntrace = nt;
  G.ntrace = nt;
  RET(ensure(&G.d_src_vals, &G.src_cap, (size_t)std::max(npts, 1) * nt));
  if (npts > 0)
    CK(cudaMemcpyAsync(G.d_src_vals, vals, sizeof(float) * (size_t)npts * nt, cudaMemcpyHostToDevice,
                       G.stream));
  RET(build_pointmap(G.srcmap, G.src_loc, npts, "source"));
  // the caller's buffer is read when the call returns (the reference copies
  // synchronously)
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}

int sepx_transfer_receiver_func(int nx, int ny, int nt, const int *locs, const float *vals) {
  if (nx < 0 || ny < 0 || nt < 1) return fail("invalid receiver shape %d x %d x %d", nx, ny, nt);
  if ((long long)nx * ny > INT_MAX) return fail("too many receivers: %d x %d", nx, ny);
  const int nrec = nx * ny;
  RET(need_span(locs, nrec, "transfer_receiver_func locs"));
  RET(need_span(vals, nrec, "transfer_receiver_func vals"));
  RET(need_grid());
  G.rec_nx = nx;
  G.rec_ny = ny;
  G.rec_ntrace = nt;
  G.ntrace = nt;
  G.rec_loc.assign(locs, locs + nrec);
  RET(ensure(&G.d_trc, &G.trc_cap, (size_t)std::max(nrec, 1) * nt));
  if (nrec > 0) RET(traces_h2d(vals, nrec, nt));
  // the reference's 2-D receiver launch reaches receivers i < n1*n2 only
  const int nact = (int)std::min<long long>(nrec, (long long)G.n1 * G.n2);
  RET(build_pointmap(G.recmap, G.rec_loc, nact, "receiver"));
  // the caller's traces are read when the call returns (the reference copies
  // synchronously)
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}

int sepx_set_receivers(int nx, int ny, int nt, const int *locs) {
  if (nx < 0 || ny < 0 || nt < 1) return fail("invalid receiver shape %d x %d x %d", nx, ny, nt);
  if ((long long)nx * ny > INT_MAX) return fail("too many receivers: %d x %d", nx, ny);
  const int nrec = nx * ny;
  RET(need_span(locs, nrec, "set_receivers locs"));
  RET(need_grid());
  G.rec_nx = nx;
  G.rec_ny = ny;
  G.rec_ntrace = nt;
  G.ntrace = nt;
  G.rec_loc.assign(locs, locs + nrec);
  RET(ensure(&G.d_trc, &G.trc_cap, (size_t)std::max(nrec, 1) * nt));
  CK(cudaMemsetAsync(G.d_trc, 0, sizeof(float) * (size_t)std::max(nrec, 1) * nt, G.stream));
  const int nact = (int)std::min<long long>(nrec, (long long)G.n1 * G.n2);
  RET(build_pointmap(G.recmap, G.rec_loc, nact, "receiver"));
  // the caller's traces are read when the call returns (the reference copies
  // synchronously)
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}

int sepx_transfer_vel_func1(int nx, int ny, int nz, const float *vel) {
  RET(need_buf(vel, "transfer_vel_func1 vel"));
  RET(need_grid());
  RET(check_dims(nx, ny, nz));
  RET(h2d_volume(G.vel, vel));
  CK(cudaStreamSynchronize(G.stream));
  G.vel_set = true;
  return 0;
}

int sepx_transfer_vel_func2(int nx, int ny, int nz, const float *vel) {
  RET(need_grid());
  RET(check_dims(nx, ny, nz));
  (void)vel;
  return 0;
}

// ------------------------------------------------------------ host-buffer loops
int sepx_source_prop(int n1, int n2, int n3, bool damp, bool get_last, float *p0, float *p1, int jt,
                     int npts, int nt) {
  (void)damp;
  if (get_last) {
    RET(need_buf(p0, "source_prop p0"));
    RET(need_buf(p1, "source_prop p1"));
  }
  RET(need_grid());
  RET(check_dims(n1, n2, n3));
  RET(loop_source_prop(jt, npts, nt));
  if (get_last) {
    RET(d2h_volume(p0, G.SL[G.sl_p0]));
    RET(d2h_volume(p1, G.SL[G.sl_p1]));
  }
  CK(cudaStreamSynchronize(G.stream));
  return check_device_error();
}

int sepx_rtm_forward(int n1, int n2, int n3, int jt, const float *img, float *dat, int npts_src,
                     int nt, int nt_big, int nx, int ny) {
  RET(need_buf(img, "rtm_forward img"));
  RET(need_span(dat, (long long)nx * ny, "rtm_forward dat"));
  RET(need_grid());
  RET(check_dims(n1, n2, n3));
  if (nx != G.rec_nx || ny != G.rec_ny)
    return fail("receiver grid %dx%d does not match the transferred %dx%d", nx, ny, G.rec_nx, G.rec_ny);
  if (nt_big != G.rec_ntrace)
    return fail("nt_big=%d does not match the transferred trace length %d", nt_big, G.rec_ntrace);
  RET(h2d_volume(G.img, img));
  RET(loop_rtm_forward(jt, npts_src, nt));
  RET(traces_d2h(dat, nx * ny, nt_big));
  CK(cudaStreamSynchronize(G.stream));
  return check_device_error();
}

int sepx_rtm_adjoint(int n1, int n2, int n3, int jt, const float *p0_s, const float *p1_s,
                     float *img, int npts, int nt) {
  RET(need_buf(p0_s, "rtm_adjoint p0_s"));
  RET(need_buf(p1_s, "rtm_adjoint p1_s"));
  RET(need_buf(img, "rtm_adjoint img"));
  RET(need_grid());
  RET(check_dims(n1, n2, n3));
  RET(h2d_volume(G.F[2], p0_s));
  RET(h2d_volume(G.F[3], p1_s));
  RET(loop_rtm_adjoint(jt, npts, nt));
  RET(d2h_volume(img, G.img));
  CK(cudaStreamSynchronize(G.stream));
  return check_device_error();
}

// ------------------------------------------------------------ resident loops
int sepx_source_prop_resident(int jt, int npts, int nt) { return loop_source_prop(jt, npts, nt); }

int sepx_rtm_forward_resident(int jt, int npts_src, int nt) {
  return loop_rtm_forward(jt, npts_src, nt);
}

int sepx_rtm_adjoint_resident(int jt, int npts, int nt, int use_source_last) {
  RET(need_grid());
  if (use_source_last) {
    // rtm_zero_op::adjoint reads the two stored fields back swapped: the
    // newest becomes p0_s (Born/rtm_zero_op_3d.cpp:254-262)
    if (!G.sl_valid) return fail("no source wavefields: run sepx_source_prop_resident first");
    RET(d2d_volume(G.F[2], G.SL[G.sl_p1]));
    RET(d2d_volume(G.F[3], G.SL[G.sl_p0]));
  }
  return loop_rtm_adjoint(jt, npts, nt);
}

int sepx_lin_source_pass(int jt, int npts, int nt, int js, int prec) {
  return loop_lin_source(jt, npts, nt, js, prec);
}

int sepx_lin_forward_resident(int jt, int npts, int nt, int js, int prec) {
  return loop_lin_forward(jt, npts, nt, js, prec);
}

int sepx_lin_adjoint_resident(int jt, int nt, int js, int prec) {
  return loop_lin_adjoint(jt, nt, js, prec);
}

long long sepx_snapshot_bytes(int nt, int js, int prec) {
  if (!G.have_grid || js < 1) return -1;
  const long long nsnap = (nt + js - 1) / js;
  return snap_blocks_per_step() * std::max(1LL, nsnap) * kCenterFloats * (prec == kSnapF32 ? 4 : 2) +
         snap_blocks_per_step() * std::max(1LL, nsnap) * 4;
}

int sepx_set_image(const float *img) {
  RET(need_buf(img, "set_image"));
  RET(need_grid());
  RET(h2d_volume(G.img, img));
  return 0;
}

int sepx_get_image(float *img) {
  RET(need_buf(img, "get_image"));
  RET(need_grid());
  RET(d2h_volume(img, G.img));
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}

int sepx_set_source_fields(const float *p0, const float *p1) {
  RET(need_buf(p0, "set_source_fields p0"));
  RET(need_buf(p1, "set_source_fields p1"));
  RET(need_grid());
  RET(h2d_volume(G.F[2], p0));
  RET(h2d_volume(G.F[3], p1));
  return 0;
}

int sepx_get_source_fields(float *p0, float *p1) {
  RET(need_buf(p0, "get_source_fields p0"));
  RET(need_buf(p1, "get_source_fields p1"));
  RET(need_grid());
  if (!G.sl_valid) return fail("no source wavefields");
  RET(d2h_volume(p0, G.SL[G.sl_p0]));
  RET(d2h_volume(p1, G.SL[G.sl_p1]));
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}

int sepx_set_traces(const float *vals) {
  RET(need_grid());
  const int nrec = G.rec_nx * G.rec_ny;
  RET(need_span(vals, nrec, "set_traces"));
  if (nrec > 0) RET(traces_h2d(vals, nrec, G.rec_ntrace));
  return 0;
}

int sepx_get_traces(float *vals) {
  RET(need_grid());
  const int nrec = G.rec_nx * G.rec_ny;
  RET(need_span(vals, nrec, "get_traces"));
  if (nrec > 0) RET(traces_d2h(vals, nrec, G.rec_ntrace));
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}

int sepx_zero_traces(void) {
  RET(need_grid());
  if (G.d_trc && G.trc_cap) CK(cudaMemsetAsync(G.d_trc, 0, G.trc_cap * sizeof(float), G.stream));
  return 0;
}

int sepx_dot_f32(const float *a, const float *b, long long n, double *result) {
  RET(need_buf(result, "sepx_dot_f32 result"));
  RET(need_span(a, n, "sepx_dot_f32 a"));   // b == NULL: the sum of a
  RET(need_device());
  const int np = vec_dot_scratch_doubles();
  RET(ensure(&G.d_dot, &G.dot_cap, (size_t)np + 1));
  CKL(vec_dot(a, b, n, G.d_dot, G.d_dot + np, G.stream));
  CK(cudaMemcpyAsync(result, G.d_dot + np, sizeof(double), cudaMemcpyDeviceToHost, G.stream));
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}

// ------------------------------------------------------------ operator glue
int sepx_op_image_to_padded(const float *model, int m1, int m2, int m3, int f1, int f2, int f3) {
  RET(need_buf(model, "op_image_to_padded model"));
  RET(need_grid());
  CKL(launch_img_from_model(model, m1, m2, m3, f1, f2, f3, G.img.origin, G.n1, G.n2, G.n3, G.pitch,
                            G.stream));
  return 0;
}

int sepx_op_padded_to_image(float *model, int m1, int m2, int m3, int f1, int f2, int f3) {
  RET(need_buf(model, "op_padded_to_image model"));
  RET(need_grid());
  CKL(launch_model_from_img(model, m1, m2, m3, f1, f2, f3, G.img.origin, G.n1, G.n2, G.n3, G.pitch,
                            G.stream));
  return 0;
}

int sepx_op_traces_to_data(float *data, int nt, float dt) {
  RET(need_buf(data, "op_traces_to_data data"));
  RET(need_grid());
  const int nrec = G.rec_nx * G.rec_ny;
  if (nt < 2 || nt + 4 > G.rec_ntrace) return fail("data length %d does not fit traces of %d", nt, G.rec_ntrace);
  CKL(launch_data_from_traces(G.d_trc, nrec, G.rec_nx, nt, dt, data, G.stream));
  return 0;
}

int sepx_op_data_to_traces(const float *data, int nt, float dt) {
  RET(need_buf(data, "op_data_to_traces data"));
  RET(need_grid());
  const int nrec = G.rec_nx * G.rec_ny;
  if (nt < 2 || nt + 4 > G.rec_ntrace) return fail("data length %d does not fit traces of %d", nt, G.rec_ntrace);
  CKL(launch_traces_from_data(data, nrec, G.rec_nx, nt, G.rec_ntrace, dt, G.d_trc, G.stream));
  return 0;
}

// ------------------------------------------------------------ data / image vectors
int sepx_image_add_window(float *img, int n1, int n2, int n3, int f1, int f2, int f3,
                          const float *sub, int s1, int s2, int s3) {
  RET(need_device());
  if (!img || !sub) return fail("image_add_window: NULL buffer");
  if (n1 < 1 || n2 < 1 || n3 < 1 || s1 < 0 || s2 < 0 || s3 < 0)
    return fail("image_add_window: invalid sizes");
  if ((long long)s1 * s2 * s3 == 0) return 0;
  CKL(launch_window_add(img, n1, n2, n3, sub, s1, s2, s3, f1, f2, f3, G.stream));
  return 0;
}

int sepx_image_extract_window(const float *img, const float *mute, int n1, int n2, int n3, int f1,
                              int f2, int f3, float *sub, int s1, int s2, int s3) {
  RET(need_device());
  if (!img || !sub) return fail("image_extract_window: NULL buffer");
  if (n1 < 1 || n2 < 1 || n3 < 1 || s1 < 0 || s2 < 0 || s3 < 0)
    return fail("image_extract_window: invalid sizes");
  if ((long long)s1 * s2 * s3 == 0) return 0;
  CKL(launch_window_extract(img, mute, n1, n2, n3, sub, s1, s2, s3, f1, f2, f3, G.stream));
  return 0;
}

int sepx_tmute(int adj, int add, float t0, float vmute, int n1, float o1, float d1, int n2, float o2,
               float d2, long long nrep, float *model, float *data) {
  RET(need_device());
  if (!model || !data) return fail("tmute: NULL buffer");
  if (n1 < 1 || n2 < 1 || nrep < 0) return fail("tmute: invalid sizes");
  if (!(vmute != 0.f) || !(d1 != 0.f)) return fail("tmute: vmute and d1 must be non-zero");
  if (nrep == 0) return 0;
  if (adj)
    CKL(launch_tmute(data, model, add, t0, vmute, n1, o1, d1, n2, o2, d2, nrep, G.stream));
  else
    CKL(launch_tmute(model, data, add, t0, vmute, n1, o1, d1, n2, o2, d2, nrep, G.stream));
  return 0;
}

// ------------------------------------------------------------ device vectors (BLAS-1)
int sepx_vec_alloc(float **p, long long n) {
  RET(need_buf(p, "vec_alloc"));
  if (n < 0) return fail("vec_alloc: negative length %lld", n);
  RET(need_device());
  CK(cudaMalloc((void **)p, sizeof(float) * (size_t)std::max(n, 1LL)));
  return 0;
}
int sepx_vec_free(float *p) {
  if (p) cudaFree(p);
  return 0;
}
int sepx_vec_upload(float *d, const float *h, long long n) {
  RET(need_span(d, n, "vec_upload d"));
  RET(need_span(h, n, "vec_upload h"));
  RET(need_device());
  CK(cudaMemcpyAsync(d, h, sizeof(float) * n, cudaMemcpyHostToDevice, G.stream));
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}
int sepx_vec_download(float *h, const float *d, long long n) {
  RET(need_span(h, n, "vec_download h"));
  RET(need_span(d, n, "vec_download d"));
  RET(need_device());
  CK(cudaMemcpyAsync(h, d, sizeof(float) * n, cudaMemcpyDeviceToHost, G.stream));
  CK(cudaStreamSynchronize(G.stream));
  return 0;
}
int sepx_vec_copy(float *dst, const float *src, long long n) {
  RET(need_span(dst, n, "vec_copy dst"));
  RET(need_span(src, n, "vec_copy src"));
  RET(need_device());
  CK(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, G.stream));
  return 0;
}
int sepx_vec_fill(float *x, long long n, float v) {
  RET(need_span(x, n, "vec_fill x"));
  RET(need_device());
  CKL(vec_fill(x, n, v, G.stream));
  return 0;
}
int sepx_vec_scale(float *y, long long n, double a) {
  RET(need_span(y, n, "vec_scale y"));
  RET(need_device());
  CKL(vec_scale(y, n, a, G.stream));
  return 0;
}
int sepx_vec_scale_add(float *y, const float *x, long long n, double a, double b) {
  RET(need_span(y, n, "vec_scale_add y"));
  RET(need_span(x, n, "vec_scale_add x"));
  RET(need_device());
  CKL(vec_scale_add(y, x, n, a, b, G.stream));
  return 0;
}
int sepx_vec_scale_add2(float *y, const float *x1, const float *x2, long long n, double a, double b) {
  RET(need_span(y, n, "vec_scale_add2 y"));
  RET(need_span(x1, n, "vec_scale_add2 x1"));
  RET(need_span(x2, n, "vec_scale_add2 x2"));
  RET(need_device());
  CKL(vec_scale_add2(y, x1, x2, n, a, b, G.stream));
  return 0;
}
int sepx_vec_add(float *y, const float *x, long long n) {
  RET(need_span(y, n, "vec_add y"));
  RET(need_span(x, n, "vec_add x"));
  RET(need_device());
  CKL(vec_add(y, x, n, G.stream));
  return 0;
}
int sepx_vec_mult(float *y, const float *x, long long n) {
  RET(need_span(y, n, "vec_mult y"));
  RET(need_span(x, n, "vec_mult x"));
  RET(need_device());
  CKL(vec_mult(y, x, n, G.stream));
  return 0;
}
int sepx_vec_random(float *y, long long n, unsigned long long seed) {
  RET(need_span(y, n, "vec_random y"));
  RET(need_device());
  CKL(vec_random(y, n, seed, G.stream));
  return 0;
}

void *sepx_get_stream(void) { return G.have_device ? (void *)G.stream : nullptr; }

int sepx_synchronize(void) {
  RET(need_device());
  CK(cudaStreamSynchronize(G.stream));
  return check_device_error();
}

const char *sepx_last_error(void) { return g_err.c_str(); }

int sepx_device_error(void) {
  if (!G.have_device) return 0;
  int h = 0;
  if (cudaMemcpy(&h, G.d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  cudaMemset(G.d_err, 0, sizeof(int));
  return h;
}

long long sepx_kernel_launches(void) { return g_launches; }

int sepx_set_zchunk(int planes) {
  if (planes < 0) return fail("zchunk must be >= 0");
  G.zchunk_override = planes;
  return 0;
}

int sepx_set_tile_rows(int mode, int rows) {
  if (mode < 0 || mode > kLinAdj) return fail("unknown propagation mode %d", mode);
  if (rows != 1 && rows != 2) return fail("rows per thread must be 1 or 2 (got %d)", rows);
  if (rows == 2 && !prop_step2_supported(mode))
    return fail("mode %d has no two-row tile (only source_prop, Born forward and RTM adjoint steps)", mode);
  if (rows == 2)
    G.rows2_mask |= 1 << mode;
  else
    G.rows2_mask &= ~(1 << mode);
  return 0;
}

int sepx_reset(void) {
  free_grid();
  cudaFree(G.d_sinc_s); cudaFree(G.d_sinc_d); cudaFree(G.d_src_vals); cudaFree(G.d_trc);
  cudaFree(G.d_inj); cudaFree(G.d_stage);
  G.d_sinc_s = G.d_sinc_d = G.d_src_vals = G.d_trc = G.d_inj = G.d_stage = nullptr;
  G.src_cap = G.trc_cap = G.inj_cap = G.stage_cap = 0;
  G.ns = G.nd = G.npts_s = 0;
  return 0;
}

// ------------------------------------------------------------ reference-named ABI
static void report(int rc, const char *who) {
  if (rc) fprintf(stderr, "sepx: %s: %s\n", who, g_err.c_str());
}

void setup_cuda(int ngpus, int argc, char **argv) {
  (void)argc; (void)argv;
  report(sepx_setup_cuda(ngpus), "setup_cuda");
}
void create_gpu_space(float d1, float d2, float d3, float bc_a, float bc_b, float bc_b_y, int nx,
                      int ny, int nz) {
  report(sepx_create_gpu_space(d1, d2, d3, bc_a, bc_b, bc_b_y, nx, ny, nz), "create_gpu_space");
}
void transfer_sinc_table_s(int nsinc, int ns, float **tables) {
  report(sepx_transfer_sinc_table_s(nsinc, ns, tables), "transfer_sinc_table_s");
}
void transfer_sinc_table_d(int nsinc, int ns, float **tabled) {
  report(sepx_transfer_sinc_table_d(nsinc, ns, tabled), "transfer_sinc_table_d");
}
void transfer_source_func(int npts, int nt, int *locs, float *vals) {
  report(sepx_transfer_source_func(npts, nt, locs, vals), "transfer_source_func");
}
void transfer_receiver_func(int nx, int ny, int nt, int *locs, float *vals) {
  report(sepx_transfer_receiver_func(nx, ny, nt, locs, vals), "transfer_receiver_func");
}
void transfer_vel_func1(int nx, int ny, int nz, float *vel) {
  report(sepx_transfer_vel_func1(nx, ny, nz, vel), "transfer_vel_func1");
}
void transfer_vel_func2(int nx, int ny, int nz, float *vel) {
  report(sepx_transfer_vel_func2(nx, ny, nz, vel), "transfer_vel_func2");
}
void source_prop(int n1, int n2, int n3, bool damp, bool get_last, float *p0, float *p1, int jt,
                 int npts, int nt) {
  report(sepx_source_prop(n1, n2, n3, damp, get_last, p0, p1, jt, npts, nt), "source_prop");
}
void rtm_forward(int n1, int n2, int n3, int jt, float *img, float *dat, int npts_src, int nt,
                 int nt_big, int nx, int ny) {
  report(sepx_rtm_forward(n1, n2, n3, jt, img, dat, npts_src, nt, nt_big, nx, ny), "rtm_forward");
}
void rtm_adjoint(int n1, int n2, int n3, int j, float *p0_s_cpu, float *p1_s_cpu, float *img,
                 int npts, int nt) {
  report(sepx_rtm_adjoint(n1, n2, n3, j, p0_s_cpu, p1_s_cpu, img, npts, nt), "rtm_adjoint");
}

}  // extern "C"

// Batches of shots: one context per shot, one persistent launch per step.
#include "sepx_batch.inc"
