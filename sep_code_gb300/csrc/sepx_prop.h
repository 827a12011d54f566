// sepx_prop.h -- parameter block shared by the host driver and the fused
// propagation kernels (sepx_prop.cu).
#pragma once
#include <cuda.h>
#include <stdint.h>

namespace sepx {

// Tile of one CTA: 32 x 16 cells in (x, y), streaming along z.
constexpr int kTX = 32;
constexpr int kTY = 16;
constexpr int kHalo = 4;                                   // stencil radius
constexpr int kHX = kTX + 2 * kHalo;                       // 40
constexpr int kHY = kTY + 2 * kHalo;                       // 24
constexpr int kCenterFloats = kTX * kTY;                   // 512 (2 KB)
constexpr int kHaloFloats = kHX * kHY;                     // 960 (3840 B)
constexpr int kConsumerThreads = 128;                      // 4 cells (one float4) each
constexpr int kThreads = kConsumerThreads + 32;            // + one TMA producer warp

// Propagation step kinds (one kernel instantiation each):
//  kSrcProp  source_prop step: source field, vel outside the Laplacian, no
//            sponge, source injected into the new field
//  kBornFwd  rtm_forward step: scattered field (vel inside the Laplacian,
//            sponge twice) + source field (sponge once), source injection,
//            Born scattering, receiver extraction
//  kRtmAdj   rtm_adjoint step: receiver field (sponge once) + source field
//            rebuilt backwards (no sponge), receiver injection, imaging
//  kRtmAdj1  first rtm_adjoint step: receiver field only, imaging against the
//            given last source wavefield
//  kLinSrc   source pass of the linearised Born pair: as kSrcProp, and on
//            snapshot steps the new field is stored compressed
//  kLinFwd   linearised Born forward in increment form: dv_t = T (L(V v_{t-1})
//            + dv_{t-1}) + c u^_t m, v_t = T v_{t-1} + dv_t (u^ = the stored
//            snapshot value, recomputed bit-identically from the source field
//            carried along), receiver extraction from v_t
//  kLinAdj   its exact transpose: a_t = T a_{t+1} + V L(B_{t+1}) + R' d_t,
//            b_t = B_{t+1} + a_t, image += c u^_t b_t, B_t = T b_t
enum PropMode : int {
  kSrcProp = 0, kBornFwd = 1, kRtmAdj = 2, kRtmAdj1 = 3, kLinSrc = 4, kLinFwd = 5, kLinAdj = 6
};

// snapshot storage of the source wavefield
enum SnapPrec : int { kSnapF32 = 0, kSnapBF16 = 1, kSnapF16 = 2 };

// Cells that carry sources or receivers, indexed by z plane so the kernel
// tests a single flag per plane.
struct PointMap {
  const int *plane_slot;   // [n3]: -1, or the slot of this plane's map
  const int *map;          // [nslot][n2][n1]: first point id at the cell, or -1
  const int *next;         // [npts]: next point id at the same cell, or -1
};

struct PropGeom {
  int n1, n2, n3;          // padded grid (the reference's sizes)
  int pitch;               // row pitch in floats (multiple of 32)
  long long plane;         // pitch * n2
  int xb, xe, yb, ye, zb, ze;   // updated interior [b, e)
  int xg, yg;              // sponge / imaging region: x < xg, y < yg
  int zchunk;              // planes per CTA along z
};

struct alignas(64) PropParams {
  CUtensorMap tm_cur_h[2];    // current field, (kHX x kHY) halo box
  CUtensorMap tm_cur_c[2];    // current field, (kTX x kTY) box (z-queue feed)
  CUtensorMap tm_prev_c[2];   // previous field (overwritten by the new one)
  CUtensorMap tm_vel_h;       // v^2 dt^2, halo box
  CUtensorMap tm_vel_c;       // v^2 dt^2, centre box
  CUtensorMap tm_img_c;       // image / reflectivity
  CUtensorMap tm_aux_c;       // kRtmAdj1: the source wavefield used for imaging
  PropGeom g;
  float coef[13];
  const float *damp_tab;      // sponge factor by edge distance
  int ntab;
  const float *cur[2];        // logical-origin pointers (z-queue warm-up loads)
  const float *vel;
  float *out[2];              // new fields (the previous-field buffers)
  float *out2;                // kLinFwd / kLinAdj: the increment (dv / a), updated in place
  float *img;                 // image written back (kRtmAdj, kRtmAdj1)
  PointMap src;               // source points
  const float *inj_s;         // per-step injection values, row of this step
  PointMap rec;               // receiver points
  float *trc;                 // time-major receiver traces [ntrace][nrec]
  int nrec;
  int trc_id;                 // first coarse sample touched this step (it/jt)
  const float *sinc_row;      // 8 receiver interpolation taps of this step
  int do_scatter;             // Born scattering this step (it % jt == 0)
  int do_image;               // imaging this step (it % jt == 0)
  // snapshots (kLin*): block (32 x 16 cells of one plane) b of snapshot k is
  // at element ((k*nzi + z-zb)*ntiles + b)*512; one float scale per block
  int do_snap;                // store (kLinSrc) / use (kLinFwd, kLinAdj) this step
  int snap_prec;              // SnapPrec
  long long snap_index;       // k
  void *snap;                 // storage
  float *snap_scale;          // per-block scale (power of two)
  int *err;                   // device error word
  int inj_stride;             // batched launches: injection values per step (points)
};

// Tensor maps of the two-row tile (32 x 32 cells per CTA, two rows per
// consumer thread): 40 x 40 halo boxes of the current fields and of
// v^2 dt^2.  Centre boxes of that tile are two 32 x 16 boxes of the
// ordinary maps.
constexpr int kTY2 = 2 * kTY;                 // 32
constexpr int kHY2 = kTY2 + 2 * kHalo;        // 40
constexpr int kCenter2 = kTX * kTY2;          // 1024 floats
constexpr int kHalo2 = kHX * kHY2;            // 1600 floats
struct alignas(64) Rows2Maps {
  CUtensorMap cur_h[2];
  CUtensorMap vel_h;
};

// Parameter sets of up to kMaxMulti grids (shots) advanced by one launch:
// CTA b is tile b of the concatenated tile lists (tile_base: prefix sums;
// tiles of a grid numbered x fastest, then y, then z-chunk).  Held in the
// kernel's parameter space (at most 32 KB), like the single-grid launch.
constexpr int kMaxMulti = 18;
struct MultiParams {
  PropParams p[kMaxMulti];
  int tile_base[kMaxMulti + 1];
  int ntx[kMaxMulti];
  int nty[kMaxMulti];
  int nshot;
};

// Values of one time step shared by every parameter set of a batched launch:
// inj_s advances by inj_row rows, sinc_row by sinc_ii rows of 8 taps.
struct BatchStep {
  int inj_row;
  int trc_id;
  int sinc_ii;
  int do_scatter;
  int do_image;
  int pset;      // parameter set pstride*shot + pset (the fields' ping-pong)
  int pstride;
};

}  // namespace sepx
