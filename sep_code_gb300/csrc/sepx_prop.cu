// sepx_prop.cu -- fused 8th-order acoustic propagation steps for sm_103a.
//
// One launch advances one or two wavefields by one time step over the updated
// interior of the padded grid and applies, in the same pass, everything the
// reference does to those cells in that step with separate launches
// (Born/gpu_funcs_3d.cu:398-471 and :600-675): sponge damping, source and
// receiver injection, Born scattering, zero-lag imaging and receiver
// extraction.  Per cell it moves the compulsory bytes only (read previous,
// current and v^2dt^2 once, write the new field once); halo cells come from
// shared memory / L2.
//
// Structure of one CTA (tile of 32 x 16 cells, a chunk of z planes):
//  * warp 4, lane 0 is the producer: for every plane it issues TMA box loads
//    (cp.async.bulk.tensor) of the current field with a 4-cell halo, the
//    previous field, v^2dt^2, the image and the current field 4 planes ahead,
//    into a ring of STAGES shared-memory stages guarded by mbarriers;
//  * warps 0-3 consume: each thread owns 4 consecutive x cells (one float4),
//    keeps a 9-deep register queue of the current field along z and reads the
//    x/y neighbours from the staged halo tile;
//  * the sponge is applied when a value is written (the reference damps the
//    current and previous fields in place before each step; multiplying the
//    new field once per sponge pass at write time and the previous field the
//    same number of extra times reproduces its sequence of float multiplies
//    without touching halo cells).
//
// Arithmetic follows the oracle's contract term for term (explicit
// __fmaf_rn / __fmul_rn / __fadd_rn, no contraction freedom), so a step is
// bit-identical to the CPU restatement.
#include <cuda.h>
#include <algorithm>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "sepx_device.cuh"
#include "sepx_prop.h"
#include "sepx_tc.cuh"

// Resident CTAs per SM the register budget targets, and ring depths, of the
// two heaviest modes (compile-time tuning knobs; the defaults measured best
// on GB300 at 560x560x496: the Born forward with its z-queues in tensor
// memory, 96 registers and a 2-stage ring runs 4 CTAs per SM).
#ifndef SEPX_FWD_MINB
#define SEPX_FWD_MINB 4
#endif
#ifndef SEPX_ADJ_MINB
#define SEPX_ADJ_MINB 3
#endif
// 1: the z-queues of the Born forward live in tensor memory (tcgen05.ld/st)
// instead of registers
#ifndef SEPX_TMEMQ
#define SEPX_TMEMQ 1
#endif
// 1: the RTM adjoint's z-queues in tensor memory as well
#ifndef SEPX_TMEMQ_ADJ
#define SEPX_TMEMQ_ADJ 0
#endif
// the source propagation: z-queue in tensor memory, CTAs per SM, ring depth
#ifndef SEPX_TMEMQ_SP
#define SEPX_TMEMQ_SP 0
#endif
#ifndef SEPX_SP_MINB
#define SEPX_SP_MINB 4
#endif
#ifndef SEPX_SP_STAGES
#define SEPX_SP_STAGES 4
#endif
// the linearised forward: z-queues in tensor memory, CTAs per SM, ring depth
// (tensor memory frees the registers for 3 CTAs per SM: the forward pass of
// the linearised pair on 256^3 x 1500 steps 0.393 -> 0.386 s)
#ifndef SEPX_TMEMQ_LIN
#define SEPX_TMEMQ_LIN 1
#endif
#ifndef SEPX_LINFWD_MINB
#define SEPX_LINFWD_MINB 3
#endif
#ifndef SEPX_LINFWD_STAGES
#define SEPX_LINFWD_STAGES 3
#endif
#ifndef SEPX_FWD_STAGES
#define SEPX_FWD_STAGES 2
#endif
#ifndef SEPX_ADJ_STAGES
#define SEPX_ADJ_STAGES 3
#endif

namespace sepx {

template <int MODE>
struct Mode {
  static constexpr bool LIN = (MODE == kLinSrc || MODE == kLinFwd || MODE == kLinAdj);
  static constexpr int NF = (MODE == kBornFwd || MODE == kRtmAdj || MODE == kLinFwd) ? 2 : 1;
  static constexpr bool F0_VEL_INSIDE = (MODE == kBornFwd || MODE == kLinFwd);  // wave_kernel_adj
  static constexpr bool VEL_HALO = F0_VEL_INSIDE;
  static constexpr bool HAS_IMG = (MODE != kSrcProp && MODE != kLinSrc);
  static constexpr bool HAS_AUX = (MODE == kRtmAdj1);
  // sponge passes per step: KW* multiplies at write time, KP* extra multiplies
  // of the previous field; PRE0: field 0 is damped once before the epilogue
  // (kLinFwd: v = T (L(Vv) + 2v - T v_prev) + scattering)
  // INC0: field 0 is in increment form (kLinFwd, kLinAdj): the previous-field
  // slot carries the increment and the sponge is applied by the epilogue
  static constexpr bool INC0 = (MODE == kLinFwd || MODE == kLinAdj);
  static constexpr int KW0 = (MODE == kBornFwd) ? 2
                             : ((MODE == kSrcProp || MODE == kLinSrc || INC0) ? 0 : 1);
  static constexpr int KP0 = KW0;
  static constexpr bool PRE0 = false;
  static constexpr int KW1 = (MODE == kBornFwd) ? 1 : 0;
  static constexpr bool NEED_T = (KW0 > 0 || KP0 > 0 || KW1 > 0 || PRE0 || INC0);
  static constexpr bool SRC_INJ = (MODE == kSrcProp || MODE == kBornFwd || MODE == kLinSrc ||
                                   MODE == kLinFwd);
  static constexpr int SRC_FIELD = (MODE == kSrcProp || MODE == kLinSrc) ? 0 : 1;
  static constexpr bool REC_EXTRACT = (MODE == kBornFwd || MODE == kLinFwd);
  static constexpr bool REC_INJECT = (MODE == kRtmAdj || MODE == kRtmAdj1 || MODE == kLinAdj);
  // stage layout (floats)
  static constexpr int FEED = 0;
  static constexpr int FEEDV = FEED + NF * kCenterFloats;
  static constexpr int HALO = FEEDV + (VEL_HALO ? kCenterFloats : 0);
  static constexpr int VELT = HALO + NF * kHaloFloats;
  static constexpr int PREV = VELT + (VEL_HALO ? kHaloFloats : kCenterFloats);
  static constexpr int IMG = PREV + NF * kCenterFloats;
  static constexpr int AUX = IMG + (HAS_IMG ? kCenterFloats : 0);
  static constexpr int STAGE = AUX + (HAS_AUX ? kCenterFloats : 0);
  static constexpr uint32_t BYTES_NOIMG =
      4u * (NF * kCenterFloats + (VEL_HALO ? kCenterFloats : 0) + NF * kHaloFloats +
            (VEL_HALO ? kHaloFloats : kCenterFloats) + NF * kCenterFloats +
            (HAS_AUX ? kCenterFloats : 0));
  static constexpr uint32_t BYTES_IMG = BYTES_NOIMG + (HAS_IMG ? 4u * kCenterFloats : 0u);
  // TQ: the z-queues of the current fields live in tensor memory: per field
  // 16 slots of 4 columns (planes w and w+8 of a ring of 8, so the 8 planes
  // z-4 .. z+3 of every step are 32 consecutive columns); the z+4 feed is
  // read from shared memory and written to both copies of its slot
  static constexpr bool TQ = (SEPX_TMEMQ && MODE == kBornFwd) || (SEPX_TMEMQ_ADJ && MODE == kRtmAdj) ||
                              (SEPX_TMEMQ_LIN && MODE == kLinFwd) || (SEPX_TMEMQ_SP && MODE == kSrcProp);
  static constexpr uint32_t TQ_COLS = NF == 2 ? 128u : 64u;
  // resident blocks per SM the register budget is sized for
  static constexpr int MINB = (MODE == kSrcProp)  ? SEPX_SP_MINB
                              : (MODE == kBornFwd) ? SEPX_FWD_MINB
                              : (MODE == kRtmAdj)  ? SEPX_ADJ_MINB
                              : (MODE == kLinFwd)  ? SEPX_LINFWD_MINB
                                                   : 3;
};

// ---- compressed snapshots: power-of-two max-abs scale per 32x16 block-plane ----
// sc = 2^(e-15) with blockmax < 2^e, so |u/sc| < 2^15: the scaling is exact and
// FP16 keeps small values normal down to 2^-29 of the block maximum.
__device__ __forceinline__ float snap_scale_of(float bmax, int prec) {
  if (prec == kSnapF32 || !(bmax > 0.f)) return 1.0f;
  int e;
  frexpf(bmax, &e);
  e = max(e, -100);
  return ldexpf(1.0f, e - 15);
}

__device__ __forceinline__ unsigned short snap_q(float u, float inv, int prec) {
  const float x = __fmul_rn(u, inv);
  if (prec == kSnapBF16) return __bfloat16_as_ushort(__float2bfloat16_rn(x));
  return __half_as_ushort(__float2half_rn(x));
}

__device__ __forceinline__ float snap_dq(unsigned short q, float sc, int prec) {
  const float x = (prec == kSnapBF16) ? __bfloat162float(__ushort_as_bfloat16(q))
                                      : __half2float(__ushort_as_half(q));
  return __fmul_rn(x, sc);
}

// max over the 128 consumer threads (named barrier 1); every consumer calls it
__device__ __forceinline__ float consumer_max(float m, float *red, int warp, int lane) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) red[warp] = m;
  asm volatile("bar.sync 1, 128;" ::: "memory");
  const float r = fmaxf(fmaxf(red[0], red[1]), fmaxf(red[2], red[3]));
  asm volatile("bar.sync 1, 128;" ::: "memory");
  return r;
}

// Sponge factor of damp_kernel (Born/wave_fkernel.3d8o.cu:183-210), one GPU:
// cells with x < xg, y < yg and edge = distance to the nearest face minus 4
// >= 0 take tab[edge]; 1 elsewhere.
// Sponge from the z-invariant part exy = min over the x/y faces of the
// distance minus 4, clamped to 254, four columns packed one byte each; 255
// marks a cell outside the sponge region x < xg, y < yg (factor 1 at every
// z).  Inside, e = min(exy, z-4, n3-4-z).  The table (entries < 1 only,
// ntab <= kTabSmem, so a clamped 254 never indexes it) sits in shared memory;
// a longer table takes the per-cell path from global memory.
constexpr int kTabSmem = 254;

__device__ __forceinline__ int sponge_exy(const PropGeom &g, int x, int y) {
  if (x >= g.xg || y >= g.yg) return 255;
  const int e = min(min(x - 4, g.n1 - 4 - x), min(y - 4, g.n2 - 4 - y));
  return min(e, 254);   // e >= 0 here: x, y lie in the interior
}

__device__ __forceinline__ float sponge_full(const PropParams &P, int x, int y, int z) {
  const PropGeom &g = P.g;
  if (x >= g.xg || y >= g.yg) return 1.0f;
  int e = x - 4; e = min(e, z - 4); e = min(e, g.n2 - 4 - y); e = min(e, g.n1 - 4 - x);
  e = min(e, g.n3 - 4 - z); e = min(e, y - 4);
  if (e < 0 || e >= P.ntab) return 1.0f;
  return __ldg(P.damp_tab + e);
}

template <int K>
__device__ __forceinline__ float damp_k(float v, float t) {
#pragma unroll
  for (int k = 0; k < K; k++) v = __fmul_rn(v, t);
  return v;
}

// z-pair sums of a queue (plane z-4+j in qz[j]): zs[k-1] = qz[4+k] + qz[4-k]
__device__ __forceinline__ void zpairs(const float4 (&qz)[9], float4 (&zs)[4]) {
#pragma unroll
  for (int k = 1; k <= 4; k++)
    zs[k - 1] = make_float4(__fadd_rn(qz[4 + k].x, qz[4 - k].x), __fadd_rn(qz[4 + k].y, qz[4 - k].y),
                            __fadd_rn(qz[4 + k].z, qz[4 - k].z), __fadd_rn(qz[4 + k].w, qz[4 - k].w));
}

// z-pair k of column c: from the 9-plane queue, summed where it is used, or
// from the pair sums
__device__ __forceinline__ float zterm(const float4 (&qz)[9], int k, int c) {
  return __fadd_rn(comp(qz[4 + k], c), comp(qz[4 - k], c));
}
__device__ __forceinline__ float zterm(const float4 (&zs)[4], int k, int c) {
  return comp(zs[k - 1], c);
}

// Laplacian part of wave_kernel (vel outside): s = c0 p + sum_k pairs.
// xw: x-4 .. x+7 of the row, ym/yp: rows y-k / y+k, zq: the z-queue (plane
// z-4+j in zq[j]) or its pair sums.
template <int NZ>
__device__ __forceinline__ void lap_plain(const float *coef, const float (&xw)[12],
                                          const float4 (&ym)[4], const float4 (&yp)[4],
                                          const float4 (&zq)[NZ], float (&s)[4]) {
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float p = xw[4 + c];
    float acc = __fmul_rn(coef[0], p);
#pragma unroll
    for (int k = 1; k <= 4; k++) {
      acc = __fmaf_rn(coef[3 * k - 2], __fadd_rn(xw[4 + c + k], xw[4 + c - k]), acc);
      acc = __fmaf_rn(coef[3 * k - 1], __fadd_rn(comp(yp[k - 1], c), comp(ym[k - 1], c)), acc);
      acc = __fmaf_rn(coef[3 * k], zterm(zq, k, c), acc);
    }
    s[c] = acc;
  }
}

// Laplacian of (v p), wave_kernel_adj (vel inside): centre (c0 p) v, pairs of
// rounded products; zq: z-queue of the products p v, or its pair sums.
template <int NZ>
__device__ __forceinline__ void lap_velin(const float *coef, const float (&xw)[12],
                                          const float (&vw)[12], const float4 (&ym)[4],
                                          const float4 (&yp)[4], const float4 (&vym)[4],
                                          const float4 (&vyp)[4], const float4 (&zq)[NZ],
                                          float (&s)[4]) {
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float acc = __fmul_rn(__fmul_rn(coef[0], xw[4 + c]), vw[4 + c]);
#pragma unroll
    for (int k = 1; k <= 4; k++) {
      float px = __fadd_rn(__fmul_rn(xw[4 + c + k], vw[4 + c + k]),
                           __fmul_rn(xw[4 + c - k], vw[4 + c - k]));
      acc = __fmaf_rn(coef[3 * k - 2], px, acc);
      float py = __fadd_rn(__fmul_rn(comp(yp[k - 1], c), comp(vyp[k - 1], c)),
                           __fmul_rn(comp(ym[k - 1], c), comp(vym[k - 1], c)));
      acc = __fmaf_rn(coef[3 * k - 1], py, acc);
      acc = __fmaf_rn(coef[3 * k], zterm(zq, k, c), acc);
    }
    s[c] = acc;
  }
}

__device__ __forceinline__ void load_window(const float *h, float (&w)[12], float4 (&ym)[4],
                                            float4 (&yp)[4]) {
  float4 a = lds4(h), b = lds4(h + 4), c = lds4(h + 8);
  w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w;
  w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
  w[8] = c.x; w[9] = c.y; w[10] = c.z; w[11] = c.w;
#pragma unroll
  for (int k = 1; k <= 4; k++) {
    ym[k - 1] = lds4(h + 4 - k * kHX);
    yp[k - 1] = lds4(h + 4 + k * kHX);
  }
}

__device__ __forceinline__ float4 mul4(float4 a, float4 b) {
  return make_float4(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z),
                     __fmul_rn(a.w, b.w));
}

// Shared-memory carve of one CTA: [STAGES stages][full bars][empty bars]
// [4-float block max][sponge table] from a 128-byte aligned base.
template <int MODE, int STAGES>
__device__ __forceinline__ float *smem_base(unsigned char *raw) {
  return reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(raw) + 127) &
                                   ~static_cast<uintptr_t>(127));
}
template <int MODE, int STAGES>
__host__ __device__ constexpr size_t smem_carve_bytes() {
  return (size_t)STAGES * Mode<MODE>::STAGE * 4 + 2 * STAGES * 8 + 16 + 4 * kTabSmem;
}

// One tile (32 x 16 cells, z-chunk bz) of one fused step.  P holds the
// parameters the step reads; T the tensor maps (param or global memory: TMA
// cannot read them from shared memory).  Leaves the CTA with no copy in
// flight and its barriers invalidated, so that the next tile may start.
template <int MODE, int STAGES>
__device__ __forceinline__ void run_tile(const PropParams &P, const PropParams &T, int bx, int by,
                                         int bz, float *smem, uint32_t tq_base) {
  using M = Mode<MODE>;
  constexpr int NF = M::NF;
  unsigned long long *bar_full = reinterpret_cast<unsigned long long *>(smem + STAGES * M::STAGE);
  unsigned long long *bar_empty = bar_full + STAGES;
  float *red = reinterpret_cast<float *>(bar_empty + STAGES);   // 4 floats: block max
  float *tab_s = red + 4;                                       // kTabSmem floats: sponge

  const PropGeom &g = P.g;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int x0 = g.xb + kTX * bx;
  const int y0 = g.yb + kTY * by;
  const int za = g.zb + g.zchunk * bz;
  const int niter = min(g.zchunk, g.ze - za);
  if (niter <= 0) return;   // uniform for the CTA

  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), kConsumerThreads / 32);
    }
    mbar_fence_init();
  }
  __syncthreads();

  const bool load_img =
      M::HAS_IMG && ((MODE == kBornFwd || MODE == kLinFwd) ? P.do_scatter : P.do_image);
  const uint32_t stage_bytes = load_img ? M::BYTES_IMG : M::BYTES_NOIMG;
  int issued = 0;

  if (warp == kConsumerThreads / 32) {
    // ---------------- producer ----------------
    if (lane == 0) {
      for (int f = 0; f < NF; f++) {
        prefetch_tmap(&T.tm_cur_h[f]);
        prefetch_tmap(&T.tm_cur_c[f]);
        prefetch_tmap(&T.tm_prev_c[f]);
      }
      for (int i = 0; i < niter; i++) {
        const int s = i % STAGES;
        if (i >= STAGES) {
          if (!mbar_wait_bounded(smem_u32(&bar_empty[s]), ((i / STAGES) - 1) & 1, P.err,
                                 kErrEmptyWait))
            break;
        }
        const uint32_t fb = smem_u32(&bar_full[s]);
        mbar_arrive_expect_tx(fb, stage_bytes);
        float *st = smem + s * M::STAGE;
        const int z = za + i;
        for (int f = 0; f < NF; f++)
          tma_load_3d(smem_u32(st + M::FEED + f * kCenterFloats), &T.tm_cur_c[f], x0, y0, z + 4, fb);
        if (M::VEL_HALO) tma_load_3d(smem_u32(st + M::FEEDV), &T.tm_vel_c, x0, y0, z + 4, fb);
        for (int f = 0; f < NF; f++)
          tma_load_3d(smem_u32(st + M::HALO + f * kHaloFloats), &T.tm_cur_h[f], x0 - kHalo,
                      y0 - kHalo, z, fb);
        if (M::VEL_HALO)
          tma_load_3d(smem_u32(st + M::VELT), &T.tm_vel_h, x0 - kHalo, y0 - kHalo, z, fb);
        else
          tma_load_3d(smem_u32(st + M::VELT), &T.tm_vel_c, x0, y0, z, fb);
        for (int f = 0; f < NF; f++)
          tma_load_3d(smem_u32(st + M::PREV + f * kCenterFloats), &T.tm_prev_c[f], x0, y0, z, fb);
        if (load_img) tma_load_3d(smem_u32(st + M::IMG), &T.tm_img_c, x0, y0, z, fb);
        if (M::HAS_AUX) tma_load_3d(smem_u32(st + M::AUX), &T.tm_aux_c, x0, y0, z, fb);
        issued = i + 1;
      }
    }
  } else {
    // ---------------- consumers ----------------
    const int row = tid >> 3, xq = tid & 7;
    const int x = x0 + 4 * xq, y = y0 + row;
    const bool active = (x < g.xe);
    const long long rowoff = (long long)x + (long long)g.pitch * y;
    uint32_t exy4 = 0;   // packed z-invariant sponge distances of the 4 columns
    if (M::NEED_T) {
      if (P.ntab <= kTabSmem)
        for (int e = tid; e < P.ntab; e += kConsumerThreads) tab_s[e] = __ldg(P.damp_tab + e);
#pragma unroll
      for (int c = 0; c < 4; c++) exy4 |= (uint32_t)sponge_exy(g, x + c, y) << (8 * c);
      asm volatile("bar.sync 1, 128;" ::: "memory");
    }
    // per-plane point-map slots, fetched one plane ahead
    auto src_slot = [&](int zz) { return (M::SRC_INJ && P.src.plane_slot) ? __ldg(P.src.plane_slot + zz) : -1; };
    auto rec_slot = [&](int zz) {
      return ((M::REC_INJECT || M::REC_EXTRACT) && P.rec.plane_slot) ? __ldg(P.rec.plane_slot + zz) : -1;
    };
    int src_next = src_slot(za), rec_next = rec_slot(za);
    float4 q[NF][9];
    // M::TQ: this warp's lanes of the z-queues in tensor memory (allocated by
    // the kernel once, for every tile it runs)
    const uint32_t tq = tq_base + ((uint32_t)(warp * 32) << 16);
    // warm-up: planes za-4 .. za+3 of the current field(s) along z
    if (active || M::TQ) {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const long long off = rowoff + g.plane * (za - 4 + j);
#pragma unroll
        for (int f = 0; f < NF; f++) {
          float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
          if (active) {
            p = ldg4(P.cur[f] + off);
            if (f == 0 && M::F0_VEL_INSIDE) p = mul4(p, ldg4(P.vel + off));
          }
          if (M::TQ) {
            tc::tmem_st4x2_sync(tq + f * 64 + 4 * j, tq + f * 64 + 4 * (j + 8), p);
          } else {
            q[f][j] = p;
          }
        }
      }
    }
    const int hoff = (kHalo + row) * kHX + 4 * xq;   // halo tile: column of x-4
    const int coff = row * kTX + 4 * xq;             // centre tile
    for (int i = 0; i < niter; i++) {
      const int s = i % STAGES;
      const bool ok = mbar_wait_bounded(smem_u32(&bar_full[s]), (i / STAGES) & 1, P.err, kErrFullWait);
      float4 zs[NF][4];   // M::TQ: z-pair sums of each field's queue
      if constexpr (M::TQ) {
        // tensor-memory operations are warp-wide: leave the loop together
        if (!__all_sync(0xffffffffu, ok)) break;
        // field by field: its 8 planes z-4 .. z+3 (the previous plane's feed
        // is in place: its stores were waited for) and the z+4 feed, folded
        // into the four pair sums at once; then the feed replaces plane z-4
        // (slot i & 7 and its copy).  One field's ring at a time is held in
        // registers.
        const float *sf = smem + s * M::STAGE;
#pragma unroll
        for (int f = 0; f < NF; f++) {
          float4 qf[9];
          tc::tmem_ld32_q8(tq + f * 64 + 4 * (i & 7), qf);
          float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
          if (active) {
            p = lds4(sf + M::FEED + f * kCenterFloats + coff);
            if (f == 0 && M::F0_VEL_INSIDE) p = mul4(p, lds4(sf + M::FEEDV + coff));
          }
          qf[8] = p;
          zpairs(qf, zs[f]);
          tc::tmem_st4x2_sync(tq + f * 64 + 4 * (i & 7), tq + f * 64 + 4 * ((i & 7) + 8), p);
        }
      } else {
        if (!ok) break;
      }
      const float *st = smem + s * M::STAGE;
      const int z = za + i;
      const int src_sl = src_next, rec_sl = rec_next;
      if (i + 1 < niter) {
        src_next = src_slot(z + 1);
        rec_next = rec_slot(z + 1);
      }
      float res[NF][4];
      float4 prevv[NF], velc, imgv = make_float4(0.f, 0.f, 0.f, 0.f), auxv, cur0;
      float vwc[4];
      if (active) {
        // z-queue feed: plane z+4
        if constexpr (!M::TQ) {
#pragma unroll
          for (int f = 0; f < NF; f++) {
            float4 p = lds4(st + M::FEED + f * kCenterFloats + coff);
            if (f == 0 && M::F0_VEL_INSIDE) p = mul4(p, lds4(st + M::FEEDV + coff));
            q[f][8] = p;
          }
        }
        float vw[12];
        float4 vym[4], vyp[4];
        if (M::VEL_HALO) {
          load_window(st + M::VELT + hoff, vw, vym, vyp);
          velc = make_float4(vw[4], vw[5], vw[6], vw[7]);
        } else {
          velc = lds4(st + M::VELT + coff);
        }
        vwc[0] = velc.x; vwc[1] = velc.y; vwc[2] = velc.z; vwc[3] = velc.w;
#pragma unroll
        for (int f = 0; f < NF; f++) {
          float xw[12];
          float4 ym[4], yp[4];
          load_window(st + M::HALO + f * kHaloFloats + hoff, xw, ym, yp);
          float sl[4];
          if (f == 0 && M::F0_VEL_INSIDE) {
            if constexpr (M::TQ)
              lap_velin(P.coef, xw, vw, ym, yp, vym, vyp, zs[f], sl);
            else
              lap_velin(P.coef, xw, vw, ym, yp, vym, vyp, q[f], sl);
#pragma unroll
            for (int c = 0; c < 4; c++)
              res[f][c] = M::INC0 ? sl[c] : __fadd_rn(__fadd_rn(sl[c], xw[4 + c]), xw[4 + c]);
          } else {
            if constexpr (M::TQ)
              lap_plain(P.coef, xw, ym, yp, zs[f], sl);
            else
              lap_plain(P.coef, xw, ym, yp, q[f], sl);
#pragma unroll
            for (int c = 0; c < 4; c++)
              res[f][c] = (f == 0 && M::INC0)
                              ? sl[c]
                              : __fadd_rn(__fmaf_rn(vwc[c], sl[c], xw[4 + c]), xw[4 + c]);
          }
          if (f == 0 && M::INC0) cur0 = make_float4(xw[4], xw[5], xw[6], xw[7]);
          prevv[f] = lds4(st + M::PREV + f * kCenterFloats + coff);
        }
        if (load_img) imgv = lds4(st + M::IMG + coff);
        if (M::HAS_AUX) auxv = lds4(st + M::AUX + coff);
      }
      // the stage is no longer read: hand it back to the producer
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&bar_empty[s]));

      float t[4] = {1.f, 1.f, 1.f, 1.f};
      float val[NF][4];
      const long long cell = rowoff + g.plane * z;
      if (active) {
        if (M::NEED_T) {
          if (P.ntab <= kTabSmem) {
            const int zd = min(z - 4, g.n3 - 4 - z);
#pragma unroll
            for (int c = 0; c < 4; c++) {
              const int ex = (int)((exy4 >> (8 * c)) & 255u);
              const int e = min(ex, zd);
              t[c] = (ex != 255 && e >= 0 && e < P.ntab) ? tab_s[e] : 1.0f;
            }
          } else {
#pragma unroll
            for (int c = 0; c < 4; c++) t[c] = sponge_full(P, x + c, y, z);
          }
        }
#pragma unroll
        for (int f = 0; f < NF; f++) {
          const int kp = (f == 0) ? M::KP0 : M::KW1;
#pragma unroll
          for (int c = 0; c < 4; c++) {
            if (f == 0 && MODE == kLinFwd) {          // dv_t = T (L(V v) + dv_{t-1})
              val[f][c] = __fmul_rn(__fadd_rn(res[f][c], comp(prevv[f], c)), t[c]);
            } else if (f == 0 && MODE == kLinAdj) {   // a_t = T a_{t+1} + V L(B)
              val[f][c] = __fmaf_rn(vwc[c], res[f][c], __fmul_rn(comp(prevv[f], c), t[c]));
            } else {
              float pv = comp(prevv[f], c);
              if (kp == 1) pv = damp_k<1>(pv, t[c]);
              if (kp == 2) pv = damp_k<2>(pv, t[c]);
              val[f][c] = __fsub_rn(res[f][c], pv);
              if (f == 0 && M::PRE0) val[f][c] = __fmul_rn(val[f][c], t[c]);
            }
          }
        }
        // source injection into the new field (ids in ascending order)
        if (M::SRC_INJ) {
          const int slot = src_sl;
          if (slot >= 0) {
            const int *mp = P.src.map + (long long)slot * g.n1 * g.n2 + (long long)y * g.n1 + x;
#pragma unroll
            for (int c = 0; c < 4; c++) {
              for (int id = __ldg(mp + c); id >= 0; id = __ldg(P.src.next + id))
                val[M::SRC_FIELD][c] = __fadd_rn(val[M::SRC_FIELD][c], __ldg(P.inj_s + id));
            }
          }
        }
        // receiver injection (adjoint): time-major traces, 8 taps
        if (M::REC_INJECT) {
          const int slot = rec_sl;
          if (slot >= 0) {
            const int *mp = P.rec.map + (long long)slot * g.n1 * g.n2 + (long long)y * g.n1 + x;
#pragma unroll
            for (int c = 0; c < 4; c++) {
              for (int id = __ldg(mp + c); id >= 0; id = __ldg(P.rec.next + id)) {
                const float *tr = P.trc + (long long)P.trc_id * P.nrec + id;
                float acc = __fmul_rn(__ldg(P.sinc_row), __ldg(tr));
#pragma unroll
                for (int k = 1; k < 8; k++)
                  acc = __fmaf_rn(__ldg(P.sinc_row + k), __ldg(tr + (long long)k * P.nrec), acc);
                val[0][c] = __fadd_rn(val[0][c], acc);
              }
            }
          }
        }
      }

      // snapshot block: scale from the block maximum of the new source field
      // (stored by kLinSrc, recomputed identically by kLinFwd)
      float sc = 1.f;
      long long blk = 0, eoff = 0;
      if (M::LIN) {
        const int ntx = (g.xe - g.xb + kTX - 1) / kTX, nty = (g.ye - g.yb) / kTY;
        blk = ((P.snap_index * (g.ze - g.zb) + (z - g.zb)) * nty + by) * ntx + bx;
        eoff = blk * kCenterFloats + row * kTX + 4 * xq;
      }
      if ((MODE == kLinSrc || MODE == kLinFwd) && P.do_snap && P.snap_prec != kSnapF32) {
        constexpr int sf = (MODE == kLinSrc) ? 0 : (NF - 1);
        float m = 0.f;
        if (active) {
#pragma unroll
          for (int c = 0; c < 4; c++) m = fmaxf(m, fabsf(val[sf][c]));
        }
        sc = snap_scale_of(consumer_max(m, red, warp, lane), P.snap_prec);
      }

      if (active) {
        const float s6 = (float)0.000001;
        float vpos[4];
        if (MODE == kLinAdj) {   // b_t = B_{t+1} + a_t
#pragma unroll
          for (int c = 0; c < 4; c++) vpos[c] = __fadd_rn(comp(cur0, c), val[0][c]);
        }
        if (MODE == kLinSrc && P.do_snap) {
          if (tid == 0) P.snap_scale[blk] = sc;
          if (P.snap_prec == kSnapF32) {
            *reinterpret_cast<float4 *>(reinterpret_cast<float *>(P.snap) + eoff) =
                make_float4(val[0][0], val[0][1], val[0][2], val[0][3]);
          } else {
            const float inv = __fdiv_rn(1.0f, sc);
            uint2 pk;
            pk.x = (uint32_t)snap_q(val[0][0], inv, P.snap_prec) |
                   ((uint32_t)snap_q(val[0][1], inv, P.snap_prec) << 16);
            pk.y = (uint32_t)snap_q(val[0][2], inv, P.snap_prec) |
                   ((uint32_t)snap_q(val[0][3], inv, P.snap_prec) << 16);
            *reinterpret_cast<uint2 *>(reinterpret_cast<unsigned short *>(P.snap) + eoff) = pk;
          }
        }
        if (MODE == kBornFwd || MODE == kLinFwd) {
          // Born scattering: rec += 1e-6 src img over x < xg, y < yg (kLinFwd:
          // with the snapshot value of the source field)
          if (P.do_scatter && y < g.yg) {
            float u[4];
#pragma unroll
            for (int c = 0; c < 4; c++) u[c] = val[NF - 1][c];
            if (MODE == kLinFwd && P.snap_prec != kSnapF32) {
              const float inv = __fdiv_rn(1.0f, sc);
#pragma unroll
              for (int c = 0; c < 4; c++)
                u[c] = snap_dq(snap_q(u[c], inv, P.snap_prec), sc, P.snap_prec);
            }
#pragma unroll
            for (int c = 0; c < 4; c++)
              if (x + c < g.xg)
                val[0][c] = __fmaf_rn(__fmul_rn(s6, u[c]), comp(imgv, c), val[0][c]);
          }
          if (MODE == kLinFwd) {   // position v_t = T v_{t-1} + dv_t (val[0] keeps dv_t)
#pragma unroll
            for (int c = 0; c < 4; c++)
              vpos[c] = __fadd_rn(__fmul_rn(comp(cur0, c), t[c]), val[0][c]);
          }
          const float *xv = (MODE == kLinFwd) ? vpos : val[0];
          // receiver extraction from the new scattered field
          const int slot = rec_sl;
          if (slot >= 0) {
            const int *mp = P.rec.map + (long long)slot * g.n1 * g.n2 + (long long)y * g.n1 + x;
#pragma unroll
            for (int c = 0; c < 4; c++) {
              for (int id = __ldg(mp + c); id >= 0; id = __ldg(P.rec.next + id)) {
                float *tr = P.trc + (long long)P.trc_id * P.nrec + id;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                  float *a = tr + (long long)k * P.nrec;
                  *a = __fmaf_rn(xv[c], __ldg(P.sinc_row + k), *a);
                }
              }
            }
          }
        }
        if (MODE == kRtmAdj || MODE == kRtmAdj1 || MODE == kLinAdj) {
          if (P.do_image && y < g.yg) {
            float4 src;
            if (MODE == kRtmAdj) {
              src = make_float4(val[1][0], val[1][1], val[1][2], val[1][3]);
            } else if (MODE == kRtmAdj1) {
              src = auxv;
            } else if (P.snap_prec == kSnapF32) {
              src = ldg4(reinterpret_cast<const float *>(P.snap) + eoff);
            } else {
              const float bsc = __ldg(P.snap_scale + blk);
              const uint2 pk =
                  __ldg(reinterpret_cast<const uint2 *>(reinterpret_cast<const unsigned short *>(P.snap) + eoff));
              src = make_float4(snap_dq((unsigned short)(pk.x & 0xffffu), bsc, P.snap_prec),
                                snap_dq((unsigned short)(pk.x >> 16), bsc, P.snap_prec),
                                snap_dq((unsigned short)(pk.y & 0xffffu), bsc, P.snap_prec),
                                snap_dq((unsigned short)(pk.y >> 16), bsc, P.snap_prec));
            }
            float o[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
              float iv = comp(imgv, c);
              const float w = (MODE == kLinAdj) ? vpos[c] : val[0][c];
              o[c] = (x + c < g.xg) ? __fmaf_rn(__fmul_rn(s6, w), comp(src, c), iv) : iv;
            }
            *reinterpret_cast<float4 *>(P.img + cell) = make_float4(o[0], o[1], o[2], o[3]);
          }
        }
        // increment-form field 0: position / increment pair
        if (M::INC0) {
          float pos[4];
#pragma unroll
          for (int c = 0; c < 4; c++)
            pos[c] = (MODE == kLinFwd) ? vpos[c] : __fmul_rn(vpos[c], t[c]);   // v_t | B_t = T b_t
          stcs4(P.out[0] + cell, make_float4(pos[0], pos[1], pos[2], pos[3]));
          stcs4(P.out2 + cell, make_float4(val[0][0], val[0][1], val[0][2], val[0][3]));
        }
        // write the new fields with the sponge applied
#pragma unroll
        for (int f = (M::INC0 ? 1 : 0); f < NF; f++) {
          const int kw = (f == 0) ? M::KW0 : M::KW1;
          float o[4];
#pragma unroll
          for (int c = 0; c < 4; c++) {
            float v = val[f][c];
            if (kw == 1) v = damp_k<1>(v, t[c]);
            if (kw == 2) v = damp_k<2>(v, t[c]);
            o[c] = v;
          }
          stcs4(P.out[f] + cell, make_float4(o[0], o[1], o[2], o[3]));
        }
        // advance the z-queues
        if (!M::TQ) {
#pragma unroll
          for (int f = 0; f < NF; f++)
#pragma unroll
            for (int j = 0; j < 8; j++) q[f][j] = q[f][j + 1];
        }
      }
    }
    // every tensor-memory store above completed before its registers were released
  }

  // Drain: never leave the CTA with bulk copies still writing its shared memory.
  __syncthreads();
  if (warp == kConsumerThreads / 32 && lane == 0) {
    for (int i = max(0, issued - STAGES); i < issued; i++) {
      if (!mbar_wait_bounded(smem_u32(&bar_full[i % STAGES]), (i / STAGES) & 1, P.err,
                             kErrDrainWait))
        break;
    }
  }
  __syncthreads();
  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_inval(smem_u32(&bar_full[s]));
      mbar_inval(smem_u32(&bar_empty[s]));
    }
  }
}

// Tensor memory of the z-queues (M::TQ): warp 0 allocates it once per CTA
// before any tile, and frees it after the last (a CTA may allocate only until
// it relinquishes its permit).  Shared memory per CTA bounds the resident CTAs
// (3, or 2 for the persistent kernel) so that 128 columns each fit the SM's 512.
template <int MODE>
__device__ __forceinline__ uint32_t tq_alloc(float *smem_slot) {
  using M = Mode<MODE>;
  if (!M::TQ) return 0;
  uint32_t *slot = reinterpret_cast<uint32_t *>(smem_slot);
  if (threadIdx.x < 32) {
    tc::tmem_alloc(smem_u32(slot), M::TQ_COLS);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  return *slot;
}
template <int MODE>
__device__ __forceinline__ void tq_free(uint32_t base) {
  using M = Mode<MODE>;
  if (!M::TQ) return;
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (threadIdx.x < 32) tc::tmem_dealloc(base, M::TQ_COLS);
}

// the 4-float block-max slot of the carve holds the tensor-memory address
// (a TQ mode that later uses the block max, the linearised forward, has read
// the address into a register before its first block max)
template <int MODE, int STAGES>
__device__ __forceinline__ float *tq_slot(float *smem) {
  return reinterpret_cast<float *>(reinterpret_cast<unsigned long long *>(
                                       smem + STAGES * Mode<MODE>::STAGE) + 2 * STAGES);
}

template <int MODE, int STAGES>
__global__ void __launch_bounds__(kThreads, Mode<MODE>::MINB)
    prop_step_kernel(const __grid_constant__ PropParams P) {
  extern __shared__ unsigned char smem_raw[];
  float *smem = smem_base<MODE, STAGES>(smem_raw);
  const uint32_t tq = tq_alloc<MODE>(tq_slot<MODE, STAGES>(smem));
  run_tile<MODE, STAGES>(P, P, blockIdx.x, blockIdx.y, blockIdx.z, smem, tq);
  tq_free<MODE>(tq);
}

// Many shots (or any set of grids) in one persistent launch: CTA b runs the
// tiles b, b + gridDim.x, ... of the item list.  Item = (shot, tile x, tile
// y, z-chunk), parameter set pstride*shot + the step's set; the parameter set's scalars are copied into shared
// memory and the step's values patched in (injection row, trace sample,
// sinc row, scattering / imaging switches), its tensor maps read from global
// memory.
// The batched kernel reads its scalars from shared memory (the single-launch
// kernel reads them as constant operands), so the two-field modes get the
// register budget of 2 CTAs per SM.
template <int MODE>
constexpr int batch_minb() {
  return (MODE == kBornFwd || MODE == kRtmAdj) ? 2 : Mode<MODE>::MINB;
}

template <int MODE, int STAGES>
__global__ void __launch_bounds__(kThreads, batch_minb<MODE>())
    prop_batch_kernel(const PropParams *__restrict__ params, const int4 *__restrict__ items,
                      int nitems, BatchStep step) {
  extern __shared__ unsigned char smem_raw[];
  float *smem = smem_base<MODE, STAGES>(smem_raw);
  PropParams *Ps = reinterpret_cast<PropParams *>(
      reinterpret_cast<unsigned char *>(smem) + ((smem_carve_bytes<MODE, STAGES>() + 63) & ~size_t(63)));
  const uint32_t tq = tq_alloc<MODE>(tq_slot<MODE, STAGES>(smem));
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int4 item = items[it];
    const PropParams *Pg = params + step.pstride * item.x + step.pset;
    const uint4 *src = reinterpret_cast<const uint4 *>(Pg);
    uint4 *dst = reinterpret_cast<uint4 *>(Ps);
    for (int i = threadIdx.x; i < (int)(sizeof(PropParams) / 16); i += kThreads) dst[i] = src[i];
    __syncthreads();
    if (threadIdx.x == 0) {
      Ps->inj_s = Pg->inj_s + (long long)step.inj_row * Pg->inj_stride;
      Ps->trc_id = step.trc_id;
      Ps->sinc_row = Pg->sinc_row + step.sinc_ii * 8;
      Ps->do_scatter = step.do_scatter;
      Ps->do_image = step.do_image;
    }
    __syncthreads();
    run_tile<MODE, STAGES>(*Ps, *Pg, item.y, item.z, item.w, smem, tq);
    __syncthreads();
  }
  tq_free<MODE>(tq);
}

// Up to kMaxMulti grids in one launch, parameters in parameter space.  The
// per-CTA grid lookup costs registers: the Born forward keeps the budget of 3
// CTAs per SM here (96 registers spill).
template <int MODE>
constexpr int multi_minb() {
  return MODE == kBornFwd ? 3 : Mode<MODE>::MINB;
}

template <int MODE, int STAGES>
__global__ void __launch_bounds__(kThreads, multi_minb<MODE>())
    prop_multi_kernel(const __grid_constant__ MultiParams mp) {
  extern __shared__ unsigned char smem_raw[];
  const int b = blockIdx.x;
  int s = 0;
  while (s + 1 < mp.nshot && b >= mp.tile_base[s + 1]) s++;
  const int local = b - mp.tile_base[s];
  const int ntx = mp.ntx[s], nty = mp.nty[s];
  const int bx = local % ntx, by = (local / ntx) % nty, bz = local / (ntx * nty);
  float *smem = smem_base<MODE, STAGES>(smem_raw);
  const uint32_t tq = tq_alloc<MODE>(tq_slot<MODE, STAGES>(smem));
  run_tile<MODE, STAGES>(mp.p[s], mp.p[s], bx, by, bz, smem, tq);
  tq_free<MODE>(tq);
}

template <int MODE, int STAGES>
constexpr size_t smem_bytes_of() {
  return smem_carve_bytes<MODE, STAGES>() + 128;
}
template <int MODE, int STAGES>
constexpr size_t batch_smem_bytes_of() {
  return ((smem_carve_bytes<MODE, STAGES>() + 63) & ~size_t(63)) + sizeof(PropParams) + 128;
}

template <int MODE, int STAGES>
static cudaError_t launch_mode(const PropParams &P, dim3 grid, cudaStream_t st) {
  const size_t smem = smem_bytes_of<MODE, STAGES>();
  auto kern = prop_step_kernel<MODE, STAGES>;
  static bool attr_done = false;   // per instantiation
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  kern<<<grid, kThreads, smem, st>>>(P);
  return cudaGetLastError();
}

// Host entry: launch one fused step.
cudaError_t launch_prop_step(int mode, const PropParams &P, cudaStream_t st) {
  const PropGeom &g = P.g;
  const int wx = g.xe - g.xb, wy = g.ye - g.yb, wz = g.ze - g.zb;
  if (wx <= 0 || wy <= 0 || wz <= 0) return cudaSuccess;
  dim3 grid((wx + kTX - 1) / kTX, (wy + kTY - 1) / kTY, (wz + g.zchunk - 1) / g.zchunk);
  switch (mode) {
    case kSrcProp: return launch_mode<kSrcProp, SEPX_SP_STAGES>(P, grid, st);
    case kBornFwd: return launch_mode<kBornFwd, SEPX_FWD_STAGES>(P, grid, st);
    case kRtmAdj: return launch_mode<kRtmAdj, SEPX_ADJ_STAGES>(P, grid, st);
    case kRtmAdj1: return launch_mode<kRtmAdj1, 3>(P, grid, st);
    case kLinSrc: return launch_mode<kLinSrc, 4>(P, grid, st);
    case kLinFwd: return launch_mode<kLinFwd, SEPX_LINFWD_STAGES>(P, grid, st);
    case kLinAdj: return launch_mode<kLinAdj, 3>(P, grid, st);
    default: return cudaErrorInvalidValue;
  }
}

// ---- batched launches ----
template <int MODE, int STAGES>
static cudaError_t launch_multi_mode(const MultiParams &mp, cudaStream_t st) {
  const size_t smem = smem_bytes_of<MODE, STAGES>();
  auto kern = prop_multi_kernel<MODE, STAGES>;
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  const int ntiles = mp.tile_base[mp.nshot];
  if (ntiles <= 0) return cudaSuccess;
  kern<<<ntiles, kThreads, smem, st>>>(mp);
  return cudaGetLastError();
}

template <int MODE, int STAGES>
static cudaError_t launch_batch_mode(const PropParams *params, const int4 *items, int nitems,
                                     const BatchStep &step, int grid, cudaStream_t st) {
  const size_t smem = batch_smem_bytes_of<MODE, STAGES>();
  auto kern = prop_batch_kernel<MODE, STAGES>;
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  kern<<<grid, kThreads, smem, st>>>(params, items, nitems, step);
  return cudaGetLastError();
}

// Resident CTAs per SM of the persistent kernel, from its registers and
// shared memory (every CTA of its grid must be resident at once), and for the
// tensor-memory z-queue modes from the 512 columns of an SM.
template <int MODE, int STAGES>
static int batch_occupancy_mode() {
  const size_t smem = batch_smem_bytes_of<MODE, STAGES>();
  auto kern = prop_batch_kernel<MODE, STAGES>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  cudaFuncAttributes fa;
  int dev = 0, smem_sm = 0, resv = 0, regs_sm = 0, thr_sm = 0;
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess)
    return 0;
  const size_t per_smem = ((smem + fa.sharedSizeBytes + 127) / 128) * 128 + (size_t)resv;
  // registers are allocated per warp in units of 256
  const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;
  const int per_regs = warp_regs * (kThreads / 32);
  int n = (int)((size_t)smem_sm / per_smem);
  n = std::min(n, regs_sm / std::max(per_regs, 1));
  n = std::min(n, thr_sm / kThreads);
  if (Mode<MODE>::TQ) n = std::min(n, (int)(512 / Mode<MODE>::TQ_COLS));
  return std::max(n, 0);
}

#define SEPX_BATCH_CASES(X)                                                                  \
  X(kSrcProp, 3) X(kSrcProp, 4) X(kBornFwd, 2) X(kBornFwd, 3) X(kBornFwd, 4) X(kRtmAdj, 3) \
  X(kRtmAdj, 4) X(kRtmAdj1, 3)

cudaError_t launch_prop_multi(int mode, int stages, const MultiParams &mp, cudaStream_t st) {
#define X(m, s) if (mode == m && stages == s) return launch_multi_mode<m, s>(mp, st);
  SEPX_BATCH_CASES(X)
#undef X
  return cudaErrorInvalidValue;
}

bool batch_supported(int mode, int stages) {
#define X(m, s) if (mode == m && stages == s) return true;
  SEPX_BATCH_CASES(X)
#undef X
  return false;
}

cudaError_t launch_prop_batch(int mode, int stages, const PropParams *params, const int4 *items,
                              int nitems, const BatchStep &step, int grid, cudaStream_t st) {
#define X(m, s) \
  if (mode == m && stages == s) return launch_batch_mode<m, s>(params, items, nitems, step, grid, st);
  SEPX_BATCH_CASES(X)
#undef X
  return cudaErrorInvalidValue;
}

int prop_batch_occupancy(int mode, int stages) {
#define X(m, s) if (mode == m && stages == s) return batch_occupancy_mode<m, s>();
  SEPX_BATCH_CASES(X)
#undef X
  return 0;
}

#include "sepx_prop2.inc"

size_t prop_smem_bytes(int mode) {
  switch (mode) {
    case kSrcProp: return smem_bytes_of<kSrcProp, SEPX_SP_STAGES>();
    case kBornFwd: return smem_bytes_of<kBornFwd, SEPX_FWD_STAGES>();
    case kRtmAdj: return smem_bytes_of<kRtmAdj, SEPX_ADJ_STAGES>();
    case kRtmAdj1: return smem_bytes_of<kRtmAdj1, 3>();
    case kLinSrc: return smem_bytes_of<kLinSrc, 4>();
    case kLinFwd: return smem_bytes_of<kLinFwd, SEPX_LINFWD_STAGES>();
    case kLinAdj: return smem_bytes_of<kLinAdj, 3>();
  }
  return 0;
}

}  // namespace sepx
