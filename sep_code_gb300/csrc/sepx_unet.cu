// sepx_unet.cu -- kernels of the learned preconditioner (a 3-D U-Net applied
// to the least-squares RTM search direction): 3x3x3 (or 1x1x1) convolutions
// as implicit GEMMs on the fifth-generation tensor cores -- BF16 operands in
// shared memory, FP32 accumulators in tensor memory -- for the forward pass,
// the data gradient (the same kernel with flipped, transposed weights) and the
// weight gradient; plus the memory-bound pieces around them (2x2x2 average
// pooling, nearest upsampling, ReLU masks, loss, Adam, weight packing).
//
// Activations are channel-last BF16 volumes: element (n, z, y, x, c) of a view
// lives at base[(((n*D + z)*H + y)*W + x)*cstride + coff + c]; channel counts,
// strides and offsets are multiples of 8, so 8 channels are one 16-byte load.
// Concatenation is a wider buffer whose channel slices are separate views.
//
// GEMM shapes: forward / data gradient  M = voxels (tiles of 128),
// N = output channels (16..128), K = taps x input channels (chunks of 64);
// weight gradient of the narrow layers (sepx_unet_wgrad.inc): M = (x shift,
// output channel), N = (y shift, input channel), K = the 128 voxels of a
// tile, nine taps per MMA; of the others (gather kernel below): M = taps x
// input channels (tiles of 128), N = output channels, K = voxels (chunks of
// 64, split over CTAs).  Both write per-CTA partial sums that a second kernel
// adds in a fixed order (the gather kernel adds with FP32 atomics only when
// the halo-staged kernels are switched off).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "sepx_common.h"
#include "sepx_device.cuh"
#include "sepx_tc.cuh"
#include "sepx_unet.h"

namespace sepx {

constexpr int kTM = 128;   // GEMM rows per CTA (tensor-memory lanes)
constexpr int kKC = 64;    // K per pipeline stage (8 K groups of 8)
constexpr int kUThreads = 128;
constexpr int kMaxN = 128;

struct View {
  const __nv_bfloat16 *p;
  int cstride, coff;
};

// ReLU backward fused into a data-gradient epilogue: the 8 outputs at acc
// become 0 where the activation (BF16, 8 channels at m) is not > 0 -- the
// same test as relu_mask_kernel, so the result is bit-identical
__device__ __forceinline__ void mask8(const __nv_bfloat16 *m, float *acc) {
  const uint4 q = *reinterpret_cast<const uint4 *>(m);
  const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
#pragma unroll
  for (int i = 0; i < 8; i++)
    if (!(__bfloat162float(h[i]) > 0.f)) acc[i] = 0.f;
}

// Voxel coordinates and the neighbour loads of the implicit GEMMs.  Volumes
// hold fewer than 2^31 voxels (checked on the host), so voxel indices are
// 32-bit; element offsets are formed from 64-bit row pointers.
struct Coord {
  int x, y, z;
};

__device__ __forceinline__ Coord coord_of(int v, int D, int H, int W) {
  Coord c;
  c.x = v % W;
  const int r = v / W;
  c.y = r % H;
  c.z = (r / H) % D;
  return c;
}

__device__ __forceinline__ void tap_delta(int t, int ntap, int &dz, int &dy, int &dx) {
  if (ntap == 1) {
    dz = dy = dx = 0;
  } else {
    const int q = (t * 57) >> 9;   // t / 9 for 0 <= t < 27
    dz = q - 1;
    const int r = t - 9 * q;
    const int q3 = (r * 11) >> 5;  // r / 3 for 0 <= r < 9
    dy = q3 - 1;
    dx = r - 3 * q3 - 1;
  }
}

// 16 bytes (8 channels from channel c0) of the neighbour (dz, dy, dx) of the
// voxel at (c) whose channel row starts at `row`, zeros outside the volume
__device__ __forceinline__ uint4 load_nb(const __nv_bfloat16 *row, const Coord &c, int dz, int dy,
                                         int dx, int D, int H, int W, int HWc, int Wc, int cs, int c0) {
  const int x2 = c.x + dx, y2 = c.y + dy, z2 = c.z + dz;
  if ((unsigned)x2 >= (unsigned)W || (unsigned)y2 >= (unsigned)H || (unsigned)z2 >= (unsigned)D)
    return make_uint4(0, 0, 0, 0);
  return *reinterpret_cast<const uint4 *>(row + (dz * HWc + dy * Wc + dx * cs + c0));
}

// 16-byte asynchronous copy global -> shared; src_bytes 0 fills zeros (src
// must still be a valid address)
__device__ __forceinline__ void cp_async16(void *dst, const void *src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

constexpr int kCS = 3;   // pipeline stages of the convolution kernels

// ---------------------------------------------------------------------------
// Forward (and data-gradient) convolution.
//   Y[v][n] = act( sum_{t, c} X[v + off(t)][c] * Wt[n][t*cin + c] + bias[n] )
// wp: packed weights [kchunks][8][np/8][8 n][8 k] BF16 (K-major operand B).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kUThreads) conv_fwd_kernel(
    View x, int nb, int D, int H, int W, int cin, int ntap, const __nv_bfloat16 *__restrict__ wp,
    int kchunks, const float *__restrict__ bias, int cout, int np, int relu, __nv_bfloat16 *y,
    int y_cstride, int y_coff, float *yf, const float *resid, int *err, int kper, float *kpart,
    View mask) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
  const int a_bytes = kTM * kKC * 2;      // 16 KB
  const int b_bytes = np * kKC * 2;       // <= 16 KB
  const int stage_bytes = a_bytes + b_bytes;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(sm + kCS * stage_bytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + kCS);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long V = (long long)nb * D * H * W;
  const long long v0 = (long long)blockIdx.x * kTM;
  const uint32_t ncols = np <= 32 ? 32 : (np <= 64 ? 64 : 128);
  // split K (kpart != NULL): this CTA sums K chunks kb .. kb + nk - 1 and
  // leaves its raw sums in kpart[blockIdx.y][v][np] for conv_finish_kernel
  const int kb = kpart ? (int)blockIdx.y * kper : 0;
  const int nk = kpart ? min(kper, kchunks - kb) : kchunks;
  if (nk <= 0) return;   // uniform for the CTA, before any allocation

  if (warp == 0) {
    tc::tmem_alloc(smem_u32(tslot), ncols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < kCS; i++) mbar_init(smem_u32(&bar[i]), 1);
    mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_bf16(kTM, np, false, false);
  const int ngn = np / 8;
  bool ok = true;
  int last = -1;   // last chunk whose MMAs were committed
  // this thread's output voxel (row `tid` of the tile) and its channel row
  const int vr = (int)min(v0 + tid, V - 1);
  const bool vin = v0 + tid < V;
  const Coord cv = coord_of(vr, D, H, W);
  const __nv_bfloat16 *xrow = x.p + (long long)vr * x.cstride + x.coff;
  const int Wc = W * x.cstride, HWc = H * Wc;
  // K position of the next K group to fetch: tap and channel
  int tap = (kb * kKC) / cin, c0 = (kb * kKC) % cin;

  // chunk j -> stage j % kCS: the A row of this thread (8 K groups of 8
  // channels of one tap, zeros outside the volume) and a share of the
  // chunk's packed weights, as asynchronous copies (one commit group)
  auto fetch = [&](int j) {
    unsigned char *A = sm + (j % kCS) * stage_bytes;
    unsigned char *Bm = A + a_bytes;
    const int r = tid;
#pragma unroll
    for (int kg = 0; kg < kKC / 8; kg++) {
      const __nv_bfloat16 *src = xrow;
      int nbytes = 0;
      if (vin && tap < ntap) {
        int dz, dy, dx;
        tap_delta(tap, ntap, dz, dy, dx);
        const int x2 = cv.x + dx, y2 = cv.y + dy, z2 = cv.z + dz;
        if ((unsigned)x2 < (unsigned)W && (unsigned)y2 < (unsigned)H && (unsigned)z2 < (unsigned)D) {
          src = xrow + (dz * HWc + dy * Wc + dx * x.cstride + c0);
          nbytes = 16;
        }
      }
      cp_async16(A + (kg * (kTM / 8) + (r >> 3)) * 128 + (r & 7) * 16, src, nbytes);
      c0 += 8;
      if (c0 >= cin) {
        c0 -= cin;
        tap++;
      }
    }
    const uint4 *wsrc = reinterpret_cast<const uint4 *>(wp + (size_t)(kb + j) * np * kKC);
    for (int i = tid; i < b_bytes / 16; i += kUThreads) cp_async16(Bm + 16 * i, wsrc + i, 16);
    cp_async_commit();
  };

  for (int j = 0; j < kCS - 1; j++) {
    if (j < nk) fetch(j);
    else cp_async_commit();
  }
  for (int j = 0; j < nk; j++) {
    cp_async_wait<kCS - 2>();   // this thread's copies of chunk j have landed
    tc::fence_proxy_async();
    if (!__syncthreads_and(ok)) break;
    if (tid == 0) {
      tc::fence_after_sync();
      unsigned char *A = sm + (j % kCS) * stage_bytes;
      const uint32_t a0 = smem_u32(A), b0 = smem_u32(A + a_bytes);
#pragma unroll
      for (int k16 = 0; k16 < kKC / 16; k16++) {
        const uint64_t ad = tc::smem_desc(a0 + k16 * 2 * (kTM / 8) * 128, (kTM / 8) * 128, 128);
        const uint64_t bd = tc::smem_desc(b0 + k16 * 2 * ngn * 128, ngn * 128, 128);
        tc::mma_bf16(tmem, ad, bd, idesc, (j > 0 || k16 > 0) ? 1u : 0u);
      }
      tc::mma_commit(smem_u32(&bar[j % kCS]));
    }
    last = j;
    // refill: chunk j + kCS - 1 reuses the stage of chunk j - 1
    const int jn = j + kCS - 1;
    if (jn < nk) {
      if (j >= 1 && !mbar_wait_bounded(smem_u32(&bar[(j - 1) % kCS]), ((j - 1) / kCS) & 1, err,
                                       kErrMmaWait))
        ok = false;
      if (ok) fetch(jn);
      else cp_async_commit();
    } else {
      cp_async_commit();
    }
  }
  cp_async_wait<0>();
  // all MMAs done (also on the error path, before the tensor memory is
  // freed): the last commit covers every earlier one
  if (last >= 0) {
    if (!mbar_wait_bounded(smem_u32(&bar[last % kCS]), (last / kCS) & 1, err, kErrMmaWait)) ok = false;
  }
  if (last != nk - 1) ok = false;
  ok = __syncthreads_and(ok);
  tc::fence_after_sync();
  if (ok) {
    // epilogue: warp w holds voxels 32w..32w+31 of the tile (TMEM lanes)
    const long long v = v0 + warp * 32 + lane;
    for (int n0 = 0; n0 < np; n0 += 16) {
      float acc[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + n0, acc);
      if (kpart) {
        if (v < V) {
          float4 *dst = reinterpret_cast<float4 *>(kpart + ((size_t)blockIdx.y * V + v) * np + n0);
#pragma unroll
          for (int i = 0; i < 4; i++) dst[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
        }
        continue;
      }
      if (v < V) {
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const int n = n0 + i;
          float o = acc[i] + ((n < cout && bias) ? bias[n] : 0.f);
          if (relu) o = fmaxf(o, 0.f);
          acc[i] = o;
        }
        if (mask.p) {
#pragma unroll
          for (int i = 0; i < 16; i += 8)
            if (n0 + i + 8 <= cout) mask8(mask.p + v * mask.cstride + mask.coff + n0 + i, acc + i);
        }
        if (y) {
#pragma unroll
          for (int i = 0; i < 16; i += 8) {
            if (n0 + i + 8 <= cout) {
              __align__(16) __nv_bfloat16 h[8];
#pragma unroll
              for (int e = 0; e < 8; e++) h[e] = __float2bfloat16_rn(acc[i + e]);
              *reinterpret_cast<uint4 *>(y + v * y_cstride + y_coff + n0 + i) =
                  *reinterpret_cast<const uint4 *>(h);
            }
          }
        }
        if (yf) {
#pragma unroll
          for (int i = 0; i < 16; i++)
            if (n0 + i < cout)
              yf[v * cout + n0 + i] = acc[i] + (resid ? resid[v * cout + n0 + i] : 0.f);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// Split-K epilogue: y = act(sum over the splits, in order, + bias); thread:
// one voxel and 8 output channels
__global__ void conv_finish_kernel(const float *__restrict__ kpart, int splits, long long V, int np,
                                   const float *__restrict__ bias, int cout, int relu, __nv_bfloat16 *y,
                                   int y_cstride, int y_coff, float *yf, const float *resid, View mask) {
  const int ng = (cout + 7) / 8;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < V * ng;
       e += (long long)gridDim.x * blockDim.x) {
    const long long v = e / ng;
    const int n0 = (int)(e % ng) * 8;
    float acc[8];
#pragma unroll
    for (int i = 0; i < 8; i++) acc[i] = 0.f;
    for (int k = 0; k < splits; k++) {
      const float4 *src = reinterpret_cast<const float4 *>(kpart + ((size_t)k * V + v) * np + n0);
      const float4 a = src[0], b = src[1];
      acc[0] += a.x; acc[1] += a.y; acc[2] += a.z; acc[3] += a.w;
      acc[4] += b.x; acc[5] += b.y; acc[6] += b.z; acc[7] += b.w;
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int n = n0 + i;
      float o = acc[i] + ((n < cout && bias) ? bias[n] : 0.f);
      acc[i] = relu ? fmaxf(o, 0.f) : o;
    }
    if (mask.p && n0 + 8 <= cout) mask8(mask.p + v * mask.cstride + mask.coff + n0, acc);
    if (y && n0 + 8 <= cout) {
      __align__(16) __nv_bfloat16 h[8];
#pragma unroll
      for (int i = 0; i < 8; i++) h[i] = __float2bfloat16_rn(acc[i]);
      *reinterpret_cast<uint4 *>(y + v * y_cstride + y_coff + n0) = *reinterpret_cast<const uint4 *>(h);
    }
    if (yf) {
#pragma unroll
      for (int i = 0; i < 8; i++)
        if (n0 + i < cout) yf[v * cout + n0 + i] = acc[i] + (resid ? resid[v * cout + n0 + i] : 0.f);
    }
  }
}

// ---------------------------------------------------------------------------
// Forward (and data-gradient) 3x3x3 convolution from a staged input halo.
// Output tile: 128 voxels = 16 rows (y) x 8 columns (x) of one z plane of one
// volume.  Its input halo -- 3 planes x 18 rows x 10 columns, every channel --
// is brought into shared memory by TMA once (zero fill outside the volume),
// channel group g (8 channels, 16 B) at g * kHaloGS bytes, voxel (z, y, x) of
// the halo at ((z * 18 + y) * 10 + x) * 16 within it.  For tap (dz, dy, dx)
// the A operand (M = 128 voxels, K = 16 channels) is a K-major no-swizzle view
// of that block: core matrix = 8 consecutive x of one row (128 B contiguous),
// M-group stride 160 B (next row), K-group stride kHaloGS (next 8 channels),
// start shifted by the tap.  So every input byte crosses L2 once per tile
// instead of once per tap.  All packed weights of the layer stay in shared
// memory; B for (tap t, channels 16s..16s+15) starts at K group t*cin/8 + 2s.
// One thread issues the 27 * cin/16 MMAs (M128, N = np, K16) into tensor
// memory; the CTA walks tiles (persistent), prefetching the next tile's halo
// into the other of two buffers while the current one is computed.
// ---------------------------------------------------------------------------
constexpr int kHaloX = 10, kHaloY = 18, kHaloZ = 3;
constexpr int kHaloGS = 8704;   // bytes per channel group (8640 rounded up to 128)
constexpr int kTileY = 16, kTileX = 8;

struct HaloArgs {
  int nb, D, H, W, cin, cout, np, relu;
  const float *bias;
  __nv_bfloat16 *y;
  int y_cstride, y_coff;
  float *yf;
  const float *resid;
  int *err;
  int ty, tx;          // tiles along y and x
  long long ntiles;
  uint32_t wbytes;     // packed weights of all taps
  int nbuf;            // halo buffers: 2 (prefetch during the MMAs) or 1
  View mask;           // ReLU-backward mask (mask.p NULL: none)
};

// channel groups held per halo buffer: cin/8 rounded up to even (an odd
// count gets one all-zero group, the channel box lying wholly outside x)
__host__ __device__ constexpr int halo_groups(int cin) { return ((cin / 8) + 1) & ~1; }

__host__ __device__ constexpr size_t halo_smem_bytes(int cin, uint32_t wbytes, int nbuf) {
  return (size_t)wbytes + (size_t)nbuf * (size_t)halo_groups(cin) * kHaloGS + 256 + 128;
}

// Warp roles: warp 4 (lane 0) loads the weights and the halos and issues the
// MMAs; warps 0-3 run the epilogue (warp w owns tensor-memory lanes
// 32w..32w+31 = tile rows).  Two accumulators in tensor memory: the MMAs of
// tile k+1 run while the epilogue of tile k reads the other one.
// Barriers: full[b] halo buffer b loaded (TMA), hfree[b] the MMAs reading
// halo buffer b are done (tcgen05.commit), acc[a] accumulator a complete
// (commit), afree[a] accumulator a read by the 4 epilogue warps, wbar weights.
constexpr int kHaloThreads = 160;
constexpr int kMaxPairs = 8;   // channel-group pairs of one halo (up to 128 channels)

__global__ void __launch_bounds__(kHaloThreads) conv_halo_kernel(const __grid_constant__ CUtensorMap tmx,
                                                                 const __nv_bfloat16 *__restrict__ wp,
                                                                 const HaloArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
  const int ngc = a.cin / 8;                       // channel groups of x
  const int ngh = halo_groups(a.cin);              // groups held (even)
  unsigned char *wsm = sm;                         // packed weights
  unsigned char *halo = sm + a.wbytes;             // a.nbuf halo buffers
  const uint32_t hbytes = (uint32_t)ngh * kHaloGS;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(halo + a.nbuf * hbytes);
  unsigned long long *full = bar, *hfree = bar + 2, *accb = bar + 4, *afree = bar + 6, *wbar = bar + 8;
  // one halo buffer: per pair of channel groups, loaded (pfull) and read by
  // its MMAs (pfree), so the next tile's halo streams in pair by pair
  unsigned long long *pfull = bar + 9, *pfree = bar + 9 + kMaxPairs;
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 9 + 2 * kMaxPairs);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t acols = a.np <= 32 ? 32 : (a.np <= 64 ? 64 : 128);   // per accumulator
  const uint32_t ncols = 2 * acols;
  if ((long long)blockIdx.x >= a.ntiles) return;   // uniform, before any allocation
  const int ntile = (int)((a.ntiles - 1 - blockIdx.x) / gridDim.x) + 1;   // tiles of this CTA

  if (warp == 0) {
    tc::tmem_alloc(smem_u32(tslot), ncols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < 2; i++) {
      mbar_init(smem_u32(&full[i]), 1);
      mbar_init(smem_u32(&hfree[i]), 1);
      mbar_init(smem_u32(&accb[i]), 1);
      mbar_init(smem_u32(&afree[i]), 4);
    }
    for (int i = 0; i < kMaxPairs; i++) {
      mbar_init(smem_u32(&pfull[i]), 1);
      mbar_init(smem_u32(&pfree[i]), 1);
    }
    mbar_init(smem_u32(wbar), 1);
    *abort_flag = 0;
    mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  // tile indices fit 32 bits (volumes hold fewer than 2^31 voxels): 32-bit
  // divisions, several times cheaper than 64-bit ones in the issuing lanes
  auto tile_pos = [&](int k, int &n, int &z, int &y0, int &x0) {
    const uint32_t tile = blockIdx.x + (uint32_t)k * gridDim.x;
    const uint32_t tx = (uint32_t)a.tx, ty = (uint32_t)a.ty, dd = (uint32_t)a.D;
    uint32_t r = tile / tx;
    const int bx = (int)(tile - r * tx);
    const uint32_t r2 = r / ty;
    const int by = (int)(r - r2 * ty);
    const uint32_t r3 = r2 / dd;
    z = (int)(r2 - r3 * dd);
    n = (int)r3;
    y0 = by * kTileY;
    x0 = bx * kTileX;
  };
  // halo copy k lands in buffer k % nbuf; its barrier phases alternate per use
  auto hbuf = [&](int k) { return a.nbuf == 2 ? (k & 1) : 0; };
  auto hpar = [&](int k) { return (uint32_t)((a.nbuf == 2 ? (k >> 1) : k) & 1); };

  if (warp == 4) {
    // ---------------- producer: TMA and MMA issue ----------------
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_bf16(kTM, a.np, false, false);
      const int ngn = a.np / 8;
      auto issue_halo = [&](int k) {
        int n, z, y0, x0;
        tile_pos(k, n, z, y0, x0);
        const uint32_t fb = smem_u32(&full[hbuf(k)]);
        mbar_arrive_expect_tx(fb, (uint32_t)ngh * (kHaloX * kHaloY * kHaloZ * 16));
        const uint32_t dst = smem_u32(halo + hbuf(k) * hbytes);
        for (int g = 0; g < ngh; g++)
          tma_load_5d(dst + g * kHaloGS, &tmx, 8 * g, x0 - 1, y0 - 1, z - 1, n, fb);
      };
      prefetch_tmap(&tmx);
      mbar_arrive_expect_tx(smem_u32(wbar), a.wbytes);
      bulk_load(smem_u32(wsm), wp, a.wbytes, smem_u32(wbar));
      if (a.nbuf == 1) {
        // ---- one buffer, pipelined by channel-group pair: pair j of tile k
        // is read by its 27 taps' MMAs, after which pair j of tile k+1 loads
        // while the MMAs of pair j+1 run (pair-major accumulation order)
        const int npair = ngh / 2;
        const uint32_t h0 = smem_u32(halo), w0 = smem_u32(wsm);
        auto issue_pair = [&](int k, int j) {
          int n, z, y0, x0;
          tile_pos(k, n, z, y0, x0);
          const uint32_t fb = smem_u32(&pfull[j]);
          mbar_arrive_expect_tx(fb, 2u * (kHaloX * kHaloY * kHaloZ * 16));
          for (int e = 0; e < 2; e++)
            tma_load_5d(h0 + (2 * j + e) * kHaloGS, &tmx, 8 * (2 * j + e), x0 - 1, y0 - 1, z - 1, n, fb);
        };
        int pi[kMaxPairs], pu[kMaxPairs];   // loads issued / consumed per pair
        for (int j = 0; j < npair; j++) {
          issue_pair(0, j);
          pi[j] = 1;
          pu[j] = 0;
        }
        bool ok = mbar_wait_bounded(smem_u32(wbar), 0, a.err, kErrFullWait);
        uint32_t last_bar = 0, last_par = 0;   // the latest commit
        for (int k = 0; ok && k < ntile; k++) {
          if (*abort_flag) { ok = false; break; }
          const int ab = k & 1;
          if (k >= 2 && !mbar_wait_bounded(smem_u32(&afree[ab]), ((k - 2) >> 1) & 1, a.err, kErrMmaWait)) { ok = false; break; }
          const uint32_t d = tmem + ab * acols;
          bool first = true;
          for (int j = 0; ok && j < npair; j++) {
            if (!mbar_wait_bounded(smem_u32(&pfull[j]), (uint32_t)(k & 1), a.err, kErrFullWait)) { ok = false; break; }
            pu[j]++;
            tc::fence_after_sync();
            for (int tp = 0; tp < 27; tp++) {
              const int q = (tp * 57) >> 9, r = tp - 9 * q, q3 = (r * 11) >> 5;
              const uint32_t tap_off = (uint32_t)(((q * kHaloY + q3) * kHaloX + (r - 3 * q3)) * 16);
              const uint64_t ad = tc::smem_desc(h0 + 2 * j * kHaloGS + tap_off, kHaloGS, kHaloX * 16);
              const uint64_t bd =
                  tc::smem_desc(w0 + (uint32_t)((tp * ngc + 2 * j) * ngn * 128), ngn * 128, 128);
              tc::mma_bf16(d, ad, bd, idesc, first ? 0u : 1u);
              first = false;
            }
            tc::mma_commit(smem_u32(&pfree[j]));
            last_bar = smem_u32(&pfree[j]);
            last_par = (uint32_t)(k & 1);
            // the previous pair's MMAs are queued ahead of these: refill it
            if (j >= 1 && k + 1 < ntile) {
              if (!mbar_wait_bounded(smem_u32(&pfree[j - 1]), (uint32_t)(k & 1), a.err, kErrMmaWait)) { ok = false; break; }
              issue_pair(k + 1, j - 1);
              pi[j - 1]++;
            }
          }
          if (!ok) break;
          tc::mma_commit(smem_u32(&accb[ab]));
          last_bar = smem_u32(&accb[ab]);
          last_par = (uint32_t)((k >> 1) & 1);
          if (k + 1 < ntile) {
            if (!mbar_wait_bounded(smem_u32(&pfree[npair - 1]), (uint32_t)(k & 1), a.err, kErrMmaWait)) { ok = false; break; }
            issue_pair(k + 1, npair - 1);
            pi[npair - 1]++;
          }
        }
        if (!ok) *abort_flag = 1;
        // never leave with a copy or an MMA in flight
        for (int j = 0; j < npair; j++)
          for (int i = pu[j]; i < pi[j]; i++)
            mbar_wait_bounded(smem_u32(&pfull[j]), (uint32_t)(i & 1), a.err, kErrDrainWait);
        if (last_bar) mbar_wait_bounded(last_bar, last_par, a.err, kErrDrainWait);
      } else {
      int issued = 0;
      for (; issued < a.nbuf && issued < ntile; issued++) issue_halo(issued);
      bool ok = mbar_wait_bounded(smem_u32(wbar), 0, a.err, kErrFullWait);
      int k = 0;
      for (; ok && k < ntile; k++) {
        if (*abort_flag) { ok = false; break; }
        // refill the buffer tile k-1 used, once its MMAs are done
        if (k >= 1 && issued < ntile && hbuf(issued) == hbuf(k - 1)) {
          if (!mbar_wait_bounded(smem_u32(&hfree[hbuf(k - 1)]), hpar(k - 1), a.err, kErrMmaWait)) { ok = false; break; }
          issue_halo(issued++);
        }
        const int ab = k & 1;
        if (!mbar_wait_bounded(smem_u32(&full[hbuf(k)]), hpar(k), a.err, kErrFullWait)) { ok = false; break; }
        if (k >= 2 && !mbar_wait_bounded(smem_u32(&afree[ab]), ((k - 2) >> 1) & 1, a.err, kErrMmaWait)) { ok = false; break; }
        tc::fence_after_sync();
        const uint32_t h0 = smem_u32(halo + hbuf(k) * hbytes), w0 = smem_u32(wsm);
        const uint32_t d = tmem + ab * acols;
        bool first = true;
        for (int t = 0; t < 27; t++) {
          const int q = (t * 57) >> 9, r = t - 9 * q, q3 = (r * 11) >> 5;   // t = 9 dz' + 3 dy' + dx'
          const uint32_t tap_off = (uint32_t)(((q * kHaloY + q3) * kHaloX + (r - 3 * q3)) * 16);
          // K16 step s: channel groups 2s, 2s + 1; for odd ngc the last step
          // pairs group ngc - 1 with the zero group, whose B partner (the
          // next tap's first group, or the zero padding after the last tap)
          // then multiplies zeros
          for (int s = 0; s < ngh / 2; s++) {
            const uint64_t ad = tc::smem_desc(h0 + 2 * s * kHaloGS + tap_off, kHaloGS, kHaloX * 16);
            const uint64_t bd =
                tc::smem_desc(w0 + (uint32_t)((t * ngc + 2 * s) * ngn * 128), ngn * 128, 128);
            tc::mma_bf16(d, ad, bd, idesc, first ? 0u : 1u);
            first = false;
          }
        }
        tc::mma_commit(smem_u32(&accb[ab]));
        tc::mma_commit(smem_u32(&hfree[hbuf(k)]));
        // single buffer: the next halo can only start once these MMAs are done
      }
      if (!ok) *abort_flag = 1;
      // never leave with a copy in flight: wait for every halo issued (each
      // was consumed above or is waited for here) and the weights
      for (int i = k; i < issued; i++) mbar_wait_bounded(smem_u32(&full[hbuf(i)]), hpar(i), a.err, kErrDrainWait);
      // and for the MMAs issued (the last commit covers all of them)
      if (k > 0) mbar_wait_bounded(smem_u32(&hfree[hbuf(k - 1)]), hpar(k - 1), a.err, kErrDrainWait);
      }
    }
  } else {
    // ---------------- epilogue warps 0-3 ----------------
    const int r = warp * 32 + lane;   // tile row = tensor-memory lane
    for (int k = 0; k < ntile; k++) {
      const int ab = k & 1;
      bool ok = mbar_wait_bounded(smem_u32(&accb[ab]), (k >> 1) & 1, a.err, kErrMmaWait);
      if (!__all_sync(0xffffffffu, ok) || *abort_flag) {   // tensor-memory loads are warp-wide
        *abort_flag = 1;
        break;
      }
      tc::fence_after_sync();
      int n, z, y0, x0;
      tile_pos(k, n, z, y0, x0);
      const int yy = y0 + (r >> 3), xx = x0 + (r & 7);
      const bool vin = yy < a.H && xx < a.W;
      const long long v = (((long long)n * a.D + z) * a.H + yy) * a.W + xx;
      for (int n0 = 0; n0 < a.np; n0 += 16) {
        float acc[16];
        tc::tmem_ld16(tmem + ab * acols + ((uint32_t)(warp * 32) << 16) + n0, acc);
        if (vin) {
#pragma unroll
          for (int i = 0; i < 16; i++) {
            const int c = n0 + i;
            float o = acc[i] + ((c < a.cout && a.bias) ? a.bias[c] : 0.f);
            if (a.relu) o = fmaxf(o, 0.f);
            acc[i] = o;
          }
          if (a.mask.p) {
#pragma unroll
            for (int i = 0; i < 16; i += 8)
              if (n0 + i + 8 <= a.cout)
                mask8(a.mask.p + v * a.mask.cstride + a.mask.coff + n0 + i, acc + i);
          }
          if (a.y) {
#pragma unroll
            for (int i = 0; i < 16; i += 8) {
              if (n0 + i + 8 <= a.cout) {
                __align__(16) __nv_bfloat16 h[8];
#pragma unroll
                for (int e = 0; e < 8; e++) h[e] = __float2bfloat16_rn(acc[i + e]);
                *reinterpret_cast<uint4 *>(a.y + v * a.y_cstride + a.y_coff + n0 + i) =
                    *reinterpret_cast<const uint4 *>(h);
              }
            }
          }
          if (a.yf) {
#pragma unroll
            for (int i = 0; i < 16; i++)
              if (n0 + i < a.cout)
                a.yf[v * a.cout + n0 + i] = acc[i] + (a.resid ? a.resid[v * a.cout + n0 + i] : 0.f);
          }
        }
      }
      // this warp has read accumulator ab: the producer may overwrite it
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&afree[ab]));
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// Weight gradient:  dW[m][n] += sum_v X[v + off(t)][c] * dY[v][n],  m = t*cin + c.
// A (M = taps x channels, K = voxels) and B (N = channels of dY, K = voxels)
// are MN-major: 8 consecutive channels of one voxel are one 16-byte row.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kUThreads) conv_wgrad_kernel(
    View x, int nb, int D, int H, int W, int cin, int ntap, View dy, int cout, int np,
    int vchunks_per_cta, float *dw, int *err, float *part) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *sm = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
  const int a_bytes = kTM * kKC * 2;
  const int b_bytes = np * kKC * 2;
  const int stage_bytes = a_bytes + b_bytes;
  unsigned long long *bar = reinterpret_cast<unsigned long long *>(sm + kCS * stage_bytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + kCS);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long V = (long long)nb * D * H * W;
  const int mtot = ntap * cin;
  const int m0 = blockIdx.x * kTM;
  const long long vchunks = (V + kKC - 1) / kKC;
  const long long jb = (long long)blockIdx.y * vchunks_per_cta;
  const int nch = (int)min((long long)vchunks_per_cta, vchunks - jb);
  const uint32_t ncols = np <= 32 ? 32 : (np <= 64 ? 64 : 128);
  if (nch <= 0) return;   // uniform for the CTA, before any allocation

  if (warp == 0) {
    tc::tmem_alloc(smem_u32(tslot), ncols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    for (int i = 0; i < kCS; i++) mbar_init(smem_u32(&bar[i]), 1);
    mbar_fence_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_bf16(kTM, np, true, true);
  const int ngn = np / 8;
  bool ok = true;
  int last = -1;
  // this thread's A pieces: M group (tid % 16) -- one tap, 8 channels -- for
  // the 8 consecutive voxels 8 * (tid / 16) .. +7 of every chunk
  const int mg = tid % (kTM / 8), kv0 = (tid / (kTM / 8)) * 8;
  const int m = m0 + mg * 8;
  const bool m_in = m < mtot;
  const int t_m = m_in ? m / cin : 0, c_m = m_in ? m - t_m * cin : 0;
  int dzm, dym, dxm;
  tap_delta(t_m, ntap, dzm, dym, dxm);
  const int Wc = W * x.cstride, HWc = H * Wc;

  // chunk jj (64 voxels) -> stage jj % kCS, asynchronous copies (one group)
  auto fetch = [&](int jj) {
    unsigned char *A = sm + (jj % kCS) * stage_bytes;
    unsigned char *Bm = A + a_bytes;
    const long long vb = (jb + jj) * kKC;
    int v = (int)(vb + kv0);
    Coord c = coord_of(min(v, (int)V - 1), D, H, W);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int kv = kv0 + i;
      const __nv_bfloat16 *row = x.p + (long long)min(v, (int)V - 1) * x.cstride + x.coff;
      const __nv_bfloat16 *src = row;
      int nbytes = 0;
      if (m_in && v < V) {
        const int x2 = c.x + dxm, y2 = c.y + dym, z2 = c.z + dzm;
        if ((unsigned)x2 < (unsigned)W && (unsigned)y2 < (unsigned)H && (unsigned)z2 < (unsigned)D) {
          src = row + (dzm * HWc + dym * Wc + dxm * x.cstride + c_m);
          nbytes = 16;
        }
      }
      cp_async16(A + ((kv >> 3) * (kTM / 8) + mg) * 128 + (kv & 7) * 16, src, nbytes);
      v++;
      if (++c.x == W) {
        c.x = 0;
        if (++c.y == H) {
          c.y = 0;
          if (++c.z == D) c.z = 0;
        }
      }
    }
    for (int p = tid; p < ngn * kKC; p += kUThreads) {
      const int ng = p % ngn, kv = p / ngn;
      const long long vv = vb + kv;
      const bool in = vv < V && ng * 8 < cout;
      const __nv_bfloat16 *src = dy.p + (in ? vv * dy.cstride + dy.coff + ng * 8 : dy.coff);
      cp_async16(Bm + ((kv >> 3) * ngn + ng) * 128 + (kv & 7) * 16, src, in ? 16 : 0);
    }
    cp_async_commit();
  };

  for (int jj = 0; jj < kCS - 1; jj++) {
    if (jj < nch) fetch(jj);
    else cp_async_commit();
  }
  for (int jj = 0; jj < nch; jj++) {
    cp_async_wait<kCS - 2>();
    tc::fence_proxy_async();
    if (!__syncthreads_and(ok)) break;
    if (tid == 0) {
      tc::fence_after_sync();
      unsigned char *A = sm + (jj % kCS) * stage_bytes;
      const uint32_t a0 = smem_u32(A), b0 = smem_u32(A + a_bytes);
#pragma unroll
      for (int k16 = 0; k16 < kKC / 16; k16++) {
        const uint64_t ad = tc::smem_desc(a0 + k16 * 2 * (kTM / 8) * 128, (kTM / 8) * 128, 128);
        const uint64_t bd = tc::smem_desc(b0 + k16 * 2 * ngn * 128, ngn * 128, 128);
        tc::mma_bf16(tmem, ad, bd, idesc, (jj > 0 || k16 > 0) ? 1u : 0u);
      }
      tc::mma_commit(smem_u32(&bar[jj % kCS]));
    }
    last = jj;
    const int jn = jj + kCS - 1;
    if (jn < nch) {
      if (jj >= 1 && !mbar_wait_bounded(smem_u32(&bar[(jj - 1) % kCS]), ((jj - 1) / kCS) & 1, err,
                                        kErrMmaWait))
        ok = false;
      if (ok) fetch(jn);
      else cp_async_commit();
    } else {
      cp_async_commit();
    }
  }
  cp_async_wait<0>();
  if (last >= 0) {
    if (!mbar_wait_bounded(smem_u32(&bar[last % kCS]), (last / kCS) & 1, err, kErrMmaWait)) ok = false;
  }
  if (last != nch - 1) ok = false;
  ok = __syncthreads_and(ok);
  tc::fence_after_sync();
  if (ok) {
    const int m = m0 + warp * 32 + lane;
    for (int n0 = 0; n0 < np; n0 += 16) {
      float acc[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + n0, acc);
      if (m < mtot) {
#pragma unroll
        for (int i = 0; i < 16; i++)
          if (n0 + i < cout) {
            // part: this split's sums, added in split order by wg_reduce_kernel
            if (part) part[((size_t)blockIdx.y * mtot + m) * cout + n0 + i] = acc[i];
            else atomicAdd(dw + (size_t)m * cout + n0 + i, acc[i]);
          }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

#include "sepx_unet_wgrad.inc"

// ---------------------------------------------------------------------------
// Weight packing.  w: FP32 master weights in the weight-gradient layout
// [ntap][cin_p][cout] (row m = t*cin_p + c).  Forward operand
// B[n = o][k = t*cin_p + c] = w[t][c][o]; data-gradient operand (transposed,
// taps flipped) B[n = c][k = t*cout_p + o] = w[ntap-1-t][c][o], cout_p = cout
// rounded up to 8.  Packed layout [kchunks][8][np/8][8 n][8 k], zero outside.
// ---------------------------------------------------------------------------
struct PackJob {
  const float *w;
  __nv_bfloat16 *out;
  int cout, cin_p, ntap, transpose, np, kchunks;
};

__device__ __forceinline__ void pack_one(const PackJob &J, long long e) {
  const int nout = J.transpose ? J.cin_p : J.cout;                   // GEMM N
  const int kin = J.transpose ? ((J.cout + 7) / 8) * 8 : J.cin_p;    // channels along K
  const int kk = (int)(e & 7);
  const int r = (int)((e >> 3) & 7);
  const long long rest = e >> 6;
  const int ng = (int)(rest % (J.np / 8));
  const long long rest2 = rest / (J.np / 8);
  const int kg = (int)(rest2 % 8);
  const int j = (int)(rest2 / 8);
  const int n = ng * 8 + r;
  const int k = j * kKC + kg * 8 + kk;
  const int t = k / kin, c = k - t * kin;
  float val = 0.f;
  if (n < nout && t < J.ntap) {
    if (!J.transpose)
      val = J.w[((size_t)t * J.cin_p + c) * J.cout + n];
    else if (c < J.cout)
      val = J.w[((size_t)(J.ntap - 1 - t) * J.cin_p + n) * J.cout + c];
  }
  J.out[e] = __float2bfloat16_rn(val);
}

__global__ void pack_weights_kernel(const PackJob J) {
  const long long total = (long long)J.kchunks * kKC * J.np;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x)
    pack_one(J, e);
}

// up to kMaxPackJobs packings in one launch: blockIdx.y picks the job
constexpr int kMaxPackJobs = 64;
struct PackJobs {
  PackJob j[kMaxPackJobs];
};
__global__ void pack_weights_many_kernel(const __grid_constant__ PackJobs P) {
  const PackJob &J = P.j[blockIdx.y];
  const long long total = (long long)J.kchunks * kKC * J.np;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x)
    pack_one(J, e);
}

// ---------------------------------------------------------------------------
// 1x1x1 layers with few channels (the output layer 16 -> 1 and its data
// gradient 8 -> 16): memory-bound, one thread per voxel, weights read once
// per block from the packed BF16 operand into shared memory, FP32 sums in
// ascending channel order.  The weight gradient of such a layer: per-thread
// products summed over the block, per-block partials summed in a fixed order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long packed_index(int n, int k, int np) {
  return ((((long long)(k / kKC) * 8 + (k % kKC) / 8) * (np / 8) + n / 8) * 8 + n % 8) * 8 + k % 8;
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(256, 3) conv1x1_kernel(View x, long long V, const __nv_bfloat16 *wp, int np,
                                                      const float *bias, int relu, __nv_bfloat16 *y,
                                                      int y_cstride, int y_coff, float *yf,
                                                      const float *resid, View mask) {
  __shared__ float w[COUT][CIN];
  __shared__ float bs[COUT];
  for (int i = threadIdx.x; i < COUT * CIN; i += blockDim.x) {
    const int n = i / CIN, k = i % CIN;
    w[n][k] = __bfloat162float(wp[packed_index(n, k, np)]);
  }
  for (int i = threadIdx.x; i < COUT; i += blockDim.x) bs[i] = bias ? bias[i] : 0.f;
  __syncthreads();
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
       v += (long long)gridDim.x * blockDim.x) {
    float xin[CIN];
#pragma unroll
    for (int g = 0; g < CIN / 8; g++) {
      const uint4 q = *reinterpret_cast<const uint4 *>(x.p + v * x.cstride + x.coff + 8 * g);
      const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
#pragma unroll
      for (int i = 0; i < 8; i++) xin[8 * g + i] = __bfloat162float(h[i]);
    }
    float acc[COUT];
    // weights re-read from shared memory per voxel (broadcast loads), not
    // held in registers: a memory-bound kernel needs its warps more
    const volatile float(*wv)[CIN] = w;
#pragma unroll
    for (int n = 0; n < COUT; n++) {
      float t = 0.f;
#pragma unroll
      for (int k = 0; k < CIN; k++) t = __fmaf_rn(wv[n][k], xin[k], t);
      t += bs[n];
      acc[n] = relu ? fmaxf(t, 0.f) : t;
    }
    if (mask.p) {
#pragma unroll
      for (int g = 0; g < COUT / 8; g++) mask8(mask.p + v * mask.cstride + mask.coff + 8 * g, acc + 8 * g);
    }
    if (y) {
#pragma unroll
      for (int g = 0; g < COUT / 8; g++) {
        __align__(16) __nv_bfloat16 h[8];
#pragma unroll
        for (int i = 0; i < 8; i++) h[i] = __float2bfloat16_rn(acc[8 * g + i]);
        *reinterpret_cast<uint4 *>(y + v * y_cstride + y_coff + 8 * g) = *reinterpret_cast<const uint4 *>(h);
      }
    }
    if (yf) {
#pragma unroll
      for (int n = 0; n < COUT; n++) yf[v * COUT + n] = acc[n] + (resid ? resid[v * COUT + n] : 0.f);
    }
  }
}

// part[block][(c, n)] = sum over the block's voxels of x[v][c] dy[v][n], and
// bpart[block][n] = sum of dy[v][n] (the bias gradient)
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) wgrad1x1_kernel(View x, View dy, long long V, float *part,
                                                       float *bpart) {
  constexpr int NP = CIN * COUT + COUT;
  __shared__ float red[8][NP];
  float acc[NP];
#pragma unroll
  for (int i = 0; i < NP; i++) acc[i] = 0.f;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
       v += (long long)gridDim.x * blockDim.x) {
    float xin[CIN], g[COUT];
#pragma unroll
    for (int q8 = 0; q8 < CIN / 8; q8++) {
      const uint4 q = *reinterpret_cast<const uint4 *>(x.p + v * x.cstride + x.coff + 8 * q8);
      const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
#pragma unroll
      for (int i = 0; i < 8; i++) xin[8 * q8 + i] = __bfloat162float(h[i]);
    }
#pragma unroll
    for (int n = 0; n < COUT; n++) g[n] = __bfloat162float(dy.p[v * dy.cstride + dy.coff + n]);
#pragma unroll
    for (int c = 0; c < CIN; c++)
#pragma unroll
      for (int n = 0; n < COUT; n++) acc[c * COUT + n] = __fmaf_rn(xin[c], g[n], acc[c * COUT + n]);
#pragma unroll
    for (int n = 0; n < COUT; n++) acc[CIN * COUT + n] += g[n];
  }
  // warp sums (fixed tree), then the 8 warps in order
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NP; i++) {
    float t = acc[i];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[wid][i] = t;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NP; i += blockDim.x) {
    float t = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += red[k][i];
    if (i < CIN * COUT) part[(size_t)blockIdx.x * (CIN * COUT) + i] = t;
    else bpart[(size_t)blockIdx.x * COUT + (i - CIN * COUT)] = t;
  }
}

// ---------------------------------------------------------------------------
// Memory-bound pieces.
// ---------------------------------------------------------------------------
// 2x2x2 average pooling: out (D/2, H/2, W/2)
// element e of a walk over (voxel, 8-channel group) of an nb x D x H x W
// volume -> group g, voxel v and its coordinates.  32-bit divisions where the
// walk is shorter than 2^31 (every U-Net volume): several times cheaper than
// the 64-bit ones, and these kernels are otherwise bound by them.
struct EV {
  long long v;
  int g, n, z, y, x;
};
template <typename I>
__device__ __forceinline__ EV decode_ev_t(I e, int cg, int D, int H, int W) {
  EV r;
  const I v = e / (I)cg;
  r.g = (int)(e - v * (I)cg);
  const I q1 = v / (I)W;
  r.x = (int)(v - q1 * (I)W);
  const I q2 = q1 / (I)H;
  r.y = (int)(q1 - q2 * (I)H);
  const I q3 = q2 / (I)D;
  r.z = (int)(q2 - q3 * (I)D);
  r.n = (int)q3;
  r.v = (long long)v;
  return r;
}
__device__ __forceinline__ EV decode_ev(long long e, bool narrow, int cg, int D, int H, int W) {
  return narrow ? decode_ev_t<uint32_t>((uint32_t)e, cg, D, H, W) : decode_ev_t<long long>(e, cg, D, H, W);
}

__global__ void avgpool_kernel(View x, int nb, int D, int H, int W, int c, __nv_bfloat16 *y,
                               int y_cstride, int y_coff) {
  const int D2 = D / 2, H2 = H / 2, W2 = W / 2, cg = c / 8;
  const long long total = (long long)nb * D2 * H2 * W2 * cg;
  const bool narrow = total < (1LL << 31);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const EV c4 = decode_ev(e, narrow, cg, D2, H2, W2);
    const int g = c4.g, xx = c4.x, yy = c4.y, zz = c4.z, n = c4.n;
    const long long v = c4.v;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int d = 0; d < 8; d++) {
      const long long vi = (((long long)n * D + 2 * zz + (d >> 2)) * H + 2 * yy + ((d >> 1) & 1)) * W +
                           2 * xx + (d & 1);
      const uint4 q = *reinterpret_cast<const uint4 *>(x.p + vi * x.cstride + x.coff + g * 8);
      const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
#pragma unroll
      for (int i = 0; i < 8; i++) acc[i] += __bfloat162float(h[i]);
    }
    __align__(16) __nv_bfloat16 o[8];
#pragma unroll
    for (int i = 0; i < 8; i++) o[i] = __float2bfloat16_rn(acc[i] * 0.125f);
    *reinterpret_cast<uint4 *>(y + v * y_cstride + y_coff + g * 8) = *reinterpret_cast<const uint4 *>(o);
  }
}

// gradient of avgpool: dx (D, H, W) = dy(parent) / 8
__global__ void avgpool_bwd_kernel(View dy, int nb, int D, int H, int W, int c, __nv_bfloat16 *dx,
                                   int dx_cstride, int dx_coff, int accumulate, View mask) {
  const int D2 = D / 2, H2 = H / 2, W2 = W / 2, cg = c / 8;
  const long long total = (long long)nb * D * H * W * cg;
  const bool narrow = total < (1LL << 31);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const EV c4 = decode_ev(e, narrow, cg, D, H, W);
    const int g = c4.g, xx = c4.x, yy = c4.y, zz = c4.z, n = c4.n;
    const long long v = c4.v;
    const long long vp = (((long long)n * D2 + zz / 2) * H2 + yy / 2) * W2 + xx / 2;
    const uint4 q = *reinterpret_cast<const uint4 *>(dy.p + vp * dy.cstride + dy.coff + g * 8);
    const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
    __nv_bfloat16 *dst = dx + v * dx_cstride + dx_coff + g * 8;
    __align__(16) __nv_bfloat16 o[8];
    const uint4 old = accumulate ? *reinterpret_cast<const uint4 *>(dst) : make_uint4(0, 0, 0, 0);
    const __nv_bfloat16 *ho = reinterpret_cast<const __nv_bfloat16 *>(&old);
#pragma unroll
    for (int i = 0; i < 8; i++)
      o[i] = __float2bfloat16_rn(__bfloat162float(h[i]) * 0.125f + (accumulate ? __bfloat162float(ho[i]) : 0.f));
    if (mask.p) {   // ReLU backward of the layer whose output this is (after the sum)
      const uint4 qm = *reinterpret_cast<const uint4 *>(mask.p + v * mask.cstride + mask.coff + g * 8);
      const __nv_bfloat16 *hm = reinterpret_cast<const __nv_bfloat16 *>(&qm);
#pragma unroll
      for (int i = 0; i < 8; i++)
        if (!(__bfloat162float(hm[i]) > 0.f)) o[i] = __float2bfloat16_rn(0.f);
    }
    *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(o);
  }
}

// nearest upsampling x2: out (2D, 2H, 2W)
__global__ void upsample_kernel(View x, int nb, int D, int H, int W, int c, __nv_bfloat16 *y,
                                int y_cstride, int y_coff) {
  const int cg = c / 8;
  const int D2 = 2 * D, H2 = 2 * H, W2 = 2 * W;
  const long long total = (long long)nb * D2 * H2 * W2 * cg;
  const bool narrow = total < (1LL << 31);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const EV c4 = decode_ev(e, narrow, cg, D2, H2, W2);
    const int g = c4.g, xx = c4.x, yy = c4.y, zz = c4.z, n = c4.n;
    const long long v = c4.v;
    const long long vs = (((long long)n * D + zz / 2) * H + yy / 2) * W + xx / 2;
    *reinterpret_cast<uint4 *>(y + v * y_cstride + y_coff + g * 8) =
        *reinterpret_cast<const uint4 *>(x.p + vs * x.cstride + x.coff + g * 8);
  }
}

// gradient of upsampling: dx (D, H, W) = sum of the 8 children
__global__ void upsample_bwd_kernel(View dy, int nb, int D, int H, int W, int c, __nv_bfloat16 *dx,
                                    int dx_cstride, int dx_coff, View mask) {
  const int cg = c / 8;
  const long long total = (long long)nb * D * H * W * cg;
  const bool narrow = total < (1LL << 31);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const EV c4 = decode_ev(e, narrow, cg, D, H, W);
    const int g = c4.g, xx = c4.x, yy = c4.y, zz = c4.z, n = c4.n;
    const long long v = c4.v;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int d = 0; d < 8; d++) {
      const long long vc = (((long long)n * 2 * D + 2 * zz + (d >> 2)) * 2 * H + 2 * yy + ((d >> 1) & 1)) *
                               2 * W + 2 * xx + (d & 1);
      const uint4 q = *reinterpret_cast<const uint4 *>(dy.p + vc * dy.cstride + dy.coff + g * 8);
      const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
#pragma unroll
      for (int i = 0; i < 8; i++) acc[i] += __bfloat162float(h[i]);
    }
    __align__(16) __nv_bfloat16 o[8];
#pragma unroll
    for (int i = 0; i < 8; i++) o[i] = __float2bfloat16_rn(acc[i]);
    if (mask.p) {
      const uint4 qm = *reinterpret_cast<const uint4 *>(mask.p + v * mask.cstride + mask.coff + g * 8);
      const __nv_bfloat16 *hm = reinterpret_cast<const __nv_bfloat16 *>(&qm);
#pragma unroll
      for (int i = 0; i < 8; i++)
        if (!(__bfloat162float(hm[i]) > 0.f)) o[i] = __float2bfloat16_rn(0.f);
    }
    *reinterpret_cast<uint4 *>(dx + v * dx_cstride + dx_coff + g * 8) = *reinterpret_cast<const uint4 *>(o);
  }
}

// dz = dy where y > 0 (ReLU backward), in place on dy's view
__global__ void relu_mask_kernel(View y, __nv_bfloat16 *dy, int dy_cstride, int dy_coff, long long V,
                                 int c) {
  const int cg = c / 8;
  const long long total = V * cg;
  const bool narrow = total < (1LL << 31);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long v = narrow ? (long long)((uint32_t)e / (uint32_t)cg) : e / cg;
    const int g = (int)(e - v * cg);
    const uint4 qy = *reinterpret_cast<const uint4 *>(y.p + v * y.cstride + y.coff + g * 8);
    __nv_bfloat16 *dst = dy + v * dy_cstride + dy_coff + g * 8;
    uint4 qd = *reinterpret_cast<const uint4 *>(dst);
    const __nv_bfloat16 *hy = reinterpret_cast<const __nv_bfloat16 *>(&qy);
    __nv_bfloat16 *hd = reinterpret_cast<__nv_bfloat16 *>(&qd);
#pragma unroll
    for (int i = 0; i < 8; i++)
      if (!(__bfloat162float(hy[i]) > 0.f)) hd[i] = __float2bfloat16_rn(0.f);
    *reinterpret_cast<uint4 *>(dst) = qd;
  }
}

// column sums of a BF16 gradient view (the bias gradient): db[c] += sum_v dy[v][c].
// Thread: one 8-channel group (16-byte loads) over a strided set of voxels,
// sums in registers; the block's partial per channel goes to part[block]
// and bias_sum_kernel adds the blocks in a fixed order.
constexpr int kBiasThreads = 256;
__global__ void __launch_bounds__(kBiasThreads) bias_grad_kernel(View dy, long long V, int c, float *part) {
  __shared__ float red[kBiasThreads][9];
  const int ng = (c + 7) / 8;
  const int lanes = kBiasThreads / ng;   // voxel lanes of the block (ng <= 16)
  const int g = threadIdx.x % ng, vl = threadIdx.x / ng;
  float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (vl < lanes) {
    for (long long v = blockIdx.x * (long long)lanes + vl; v < V; v += (long long)gridDim.x * lanes) {
      const uint4 q = *reinterpret_cast<const uint4 *>(dy.p + v * dy.cstride + dy.coff + 8 * g);
      const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&q);
#pragma unroll
      for (int i = 0; i < 8; i++) s[i] += __bfloat162float(h[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < 8; i++) red[threadIdx.x][i] = s[i];
  __syncthreads();
  for (int ch = threadIdx.x; ch < c; ch += kBiasThreads) {
    const int gg = ch / 8, i = ch % 8;
    float t = 0.f;
    for (int l = 0; l < lanes; l++) t += red[l * ng + gg][i];
    part[(size_t)blockIdx.x * c + ch] = t;
  }
}

// one warp per channel: lane l adds blocks l, l+32, ..; then a fixed shuffle tree
__global__ void bias_sum_kernel(const float *__restrict__ part, int blocks, int c, float *db) {
  const int ch = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (ch >= c) return;
  float t = 0.f;
  for (int b = lane; b < blocks; b += 32) t += part[(size_t)b * c + ch];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) db[ch] += t;
}

// FP32 volume (one channel) -> BF16 channel-last view channel 0, other
// channels of the 8-channel group zero; scale applied
__global__ void to_bf16_kernel(const float *in, long long V, float scale, __nv_bfloat16 *y,
                               int y_cstride, int y_coff) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
       v += (long long)gridDim.x * blockDim.x) {
    __align__(16) __nv_bfloat16 o[8];
    o[0] = __float2bfloat16_rn(in[v] * scale);
#pragma unroll
    for (int i = 1; i < 8; i++) o[i] = __float2bfloat16_rn(0.f);
    *reinterpret_cast<uint4 *>(y + v * y_cstride + y_coff) = *reinterpret_cast<const uint4 *>(o);
  }
}

// loss = mean (out - target)^2; grad (BF16, channel 0 of an 8-channel group) = 2 (out - target) / V
__global__ void mse_kernel(const float *out, const float *target, long long V, __nv_bfloat16 *g,
                           int g_cstride, double *loss) {
  double acc = 0.0;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V;
       v += (long long)gridDim.x * blockDim.x) {
    const float r = out[v] - target[v];
    acc += (double)r * r;
    __align__(16) __nv_bfloat16 o[8];
    o[0] = __float2bfloat16_rn(2.f * r / (float)V);
#pragma unroll
    for (int i = 1; i < 8; i++) o[i] = __float2bfloat16_rn(0.f);
    *reinterpret_cast<uint4 *>(g + v * g_cstride) = *reinterpret_cast<const uint4 *>(o);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
    atomicAdd(loss, t / (double)V);   // one atomic per block
  }
}

// hp (optional): {lr, b1, b2, eps, step} read when the kernel runs, so that a
// captured training step replays with the current learning rate and step;
// the bias corrections are formed here in both forms
__global__ void adam_kernel(float *p, const float *g, float *m, float *v, long long n,
                            const float *hp, float lr, float b1, float b2, float eps, int step,
                            int *err) {
  if (hp) {
    lr = hp[0]; b1 = hp[1]; b2 = hp[2]; eps = hp[3];
    const float s = hp[4];
    if (!(s >= 1.f)) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(err, 0, (int)kErrAdamStep);
      return;
    }
    step = (int)s;
  }
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

static int grid_for(long long n, int threads = 256) {
  long long g = (n + threads - 1) / threads;
  return (int)(g < 1 ? 1 : (g > 8 * 152 * 4 ? 8 * 152 * 4 : g));
}

// kCS stages of A (16 KB) and B (np x 128 B), barriers, the tensor-memory
// slot, alignment.  Resident CTAs per SM are bounded by this size, which also
// keeps their tensor memory (np <= 32: 32 columns, <= 64: 64, else 128) within
// the SM's 512 columns: 128 columns need np > 64, i.e. >= 78 KB, so at most 2
// such CTAs; 64 columns need >= 57 KB (at most 3); 32 columns >= 54 KB (4).
static size_t conv_smem(int np) {
  return (size_t)kCS * (kTM * kKC * 2 + np * kKC * 2) + 8 * kCS + 16 + 128;
}

}  // namespace sepx

using namespace sepx;

// ---------------------------------------------------------------------------
// C ABI (include/sepx_unet.h)
// ---------------------------------------------------------------------------
namespace {
int *g_unet_err = nullptr;
int unet_err_ptr(int **p) {
  if (!g_unet_err) {
    if (cudaMalloc((void **)&g_unet_err, sizeof(int)) != cudaSuccess) return -1;
    if (cudaMemset(g_unet_err, 0, sizeof(int)) != cudaSuccess) return -1;
  }
  *p = g_unet_err;
  return 0;
}
int check_conv_args(int cin, int cstride, int coff, int cout, int ntap) {
  if (cin <= 0 || cin % 8 || cstride % 8 || coff % 8 || coff + cin > cstride) return -1;
  if (cout <= 0 || cout > kMaxN) return -1;
  if (ntap != 1 && ntap != 27) return -1;
  return 0;
}
int np_of(int cout) { return ((cout + 15) / 16) * 16; }

// The halo-staged convolution takes 3x3x3 layers whose planes hold at least
// one 16 x 8 tile and whose weights and a halo buffer fit in the 227 KB of
// shared memory a CTA may have (one CTA per SM for the largest of them).
constexpr size_t kHaloMaxSmem = 227 * 1024;
bool g_halo_enabled = true;
int g_wgrad_form = 2;   // 2: z-walk, else per-tile TMA, else gather; 1: per-tile TMA, else gather; 0: gather
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
int g_num_sms = 0;
size_t g_smem_per_sm = 0, g_smem_reserved = 0;

// the tensor-map encoder and the device figures the persistent grids are sized from
int unet_dev_init() {
  if (g_encode) return 0;
  cudaDriverEntryPointQueryResult q;
  void *fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      !fn || q != cudaDriverEntryPointSuccess)
    return set_error("unet conv: cuTensorMapEncodeTiled is unavailable");
  int dev = 0, smem_sm = 0, resv = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess)
    return set_error("unet conv: cannot query the device");
  g_smem_per_sm = (size_t)smem_sm;
  g_smem_reserved = (size_t)resv;
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return 0;
}

// channel-last BF16 view as a 5-D tensor (channels, W, H, D, volumes) with a
// box of 8 channels x bx x by x bz x 1
int encode_view(CUtensorMap *tm, const void *p, int cstride, int coff, int chans, int nb, int D, int H,
                int W, int bx, int by, int bz, const char *what, int bc = 8) {
  const __nv_bfloat16 *base = (const __nv_bfloat16 *)p + coff;
  if (reinterpret_cast<uintptr_t>(base) % 16) return set_error("unet %s: view not 16-byte aligned", what);
  const cuuint64_t cs = (cuuint64_t)cstride * 2;
  cuuint64_t dims[5] = {(cuuint64_t)chans, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)nb};
  cuuint64_t strides[4] = {cs, cs * W, cs * W * H, cs * W * H * D};
  cuuint32_t box[5] = {(cuuint32_t)bc, (cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz, 1};
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUresult r = g_encode(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<__nv_bfloat16 *>(base), dims,
                        strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error("unet %s: cuTensorMapEncodeTiled failed (%d)", what, (int)r);
  return 0;
}

// Device scratch for partial sums, grown on demand (a call inside a CUDA-graph
// capture must not grow it: run the sequence once before capturing).  One
// buffer per (pool, stream) -- kScrConv for the split-K convolutions,
// kScrGrad for the weight and bias gradients -- so that calls on different
// streams never share one (the training step runs its weight gradients on
// streams beside the data gradients).
enum { kScrConv = 0, kScrGrad = 1 };
struct Scratch {
  cudaStream_t st;
  float *p;
  size_t n;
};
constexpr int kMaxScratch = 16;
Scratch g_scratch[2][kMaxScratch] = {};
std::mutex g_scratch_mu;   // host threads may enqueue on different streams
int unet_scratch(int pool, size_t floats, float **p, cudaStream_t st) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  Scratch *e = nullptr;
  for (int i = 0; i < kMaxScratch && !e; i++)
    if (g_scratch[pool][i].p && g_scratch[pool][i].st == st) e = &g_scratch[pool][i];
  for (int i = 0; i < kMaxScratch && !e; i++)
    if (!g_scratch[pool][i].p) e = &g_scratch[pool][i];
  if (!e) return set_error("unet: more than %d streams use the scratch buffers", kMaxScratch);
  if (floats > e->n || !e->p) {
    float *q = nullptr;
    if (cudaMalloc((void **)&q, std::max<size_t>(floats, 1) * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return set_error("unet: cannot allocate %zu floats of scratch", floats);
    }
    if (e->p) {
      cudaDeviceSynchronize();   // nothing may still read the old buffer
      cudaFree(e->p);
    }
    e->p = q;
    e->n = std::max<size_t>(floats, 1);
    e->st = st;
  }
  *p = e->p;
  return 0;
}

int conv_halo(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int cin,
              const void *wpacked, uint32_t wbytes, const float *bias, int cout, int np, int relu,
              void *y, int y_cstride, int y_coff, float *yf, const float *resid, View mask, int *err,
              cudaStream_t st) {
  if (unet_dev_init()) return -1;
  CUtensorMap tm;
  if (encode_view(&tm, x, x_cstride, x_coff, cin, nb, D, H, W, kHaloX, kHaloY, kHaloZ, "conv")) return -1;
  HaloArgs a;
  a.nb = nb; a.D = D; a.H = H; a.W = W; a.cin = cin; a.cout = cout; a.np = np; a.relu = relu;
  a.bias = bias; a.y = (__nv_bfloat16 *)y; a.y_cstride = y_cstride; a.y_coff = y_coff;
  a.yf = yf; a.resid = resid; a.err = err; a.mask = mask;
  a.ty = (H + kTileY - 1) / kTileY;
  a.tx = (W + kTileX - 1) / kTileX;
  a.ntiles = (long long)nb * D * a.ty * a.tx;
  if (a.ntiles >= (1LL << 31)) return set_error("unet conv: too many tiles");
  a.wbytes = wbytes;
  // resident CTAs per SM from the shared memory each needs (the CTAs of the
  // persistent grid must all be resident): two halo buffers unless one
  // buffer fits two CTAs per SM where two buffers fit only one
  auto fit = [&](int nbuf) {
    const size_t per = ((halo_smem_bytes(cin, wbytes, nbuf) + 127) / 128) * 128 + g_smem_reserved;
    return (int)(g_smem_per_sm / per);
  };
  // two or more channel-group pairs: one buffer pipelined pair by pair;
  // a single pair: two buffers where they still leave two CTAs per SM
  const bool two_fit = halo_smem_bytes(cin, wbytes, 2) <= kHaloMaxSmem;
  if (halo_groups(cin) >= 4) a.nbuf = 1;
  else a.nbuf = (two_fit && (fit(2) >= 2 || fit(1) < 2)) ? 2 : 1;
  int per_sm = fit(a.nbuf);
  if (per_sm < 1) return set_error("unet conv: the halo kernel does not fit an SM");
  if (per_sm > 8) per_sm = 8;
  const size_t smem = halo_smem_bytes(cin, wbytes, a.nbuf);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(conv_halo_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kHaloMaxSmem);
    // the persistent grid is sized from the occupancy query: ask for the
    // full shared-memory carve-out so that every CTA of the grid is resident
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(conv_halo_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return set_error("unet conv: %s", cudaGetErrorString(e));
    attr = true;
  }
  // tensor memory: two accumulators per CTA, at most 512 columns per SM
  const int ncols = 2 * (np <= 32 ? 32 : (np <= 64 ? 64 : 128));
  if (per_sm * ncols > 512) per_sm = 512 / ncols;
  long long grid = (long long)g_num_sms * per_sm;
  if (grid > a.ntiles) grid = a.ntiles;
  conv_halo_kernel<<<(unsigned)grid, kHaloThreads, smem, st>>>(tm, (const __nv_bfloat16 *)wpacked, a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : set_error("unet conv: %s", cudaGetErrorString(e));
}

// The z-walk form of the tap-stacked weight gradient (sepx_unet_wgrad.inc)
// for cin <= 48 and 8 ngo <= 40.  Returns 1 where it does not apply.
int conv_wgrad_zw(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int cin,
                  const void *dy, int dy_cstride, int dy_coff, int cout, float *dw, float *db, int *err,
                  cudaStream_t st) {
  const int ngi = cin / 8, ngo = (cout + 7) / 8;
  if (!g_halo_enabled || g_wgrad_form < 2 || 3 * ngo > 16 || ngi > 6) return 1;
  if (unet_dev_init()) return -1;
  ZwArgs a;
  a.nb = nb; a.D = D; a.H = H; a.W = W; a.cin = cin; a.cout = cout; a.ngi = ngi; a.ngo = ngo;
  a.np = ((8 * (3 * ngi + 1)) + 15) / 16 * 16;
  if (3 * a.np > 512) return 1;
  a.a_bytes = 3u * ngo * kWgBox;
  a.pl_bytes = (uint32_t)(a.np / 8) * kWgBox;
  a.rawb_bytes = 18u * 8u * (uint32_t)cin * 2u;
  a.rawa_bytes = 16u * 10u * 8u * (uint32_t)ngo * 2u;
  a.raw_bytes = (a.rawb_bytes + a.rawa_bytes + 127u) / 128u * 128u;
  const size_t fixed = 2 * (size_t)a.a_bytes + 4 * (size_t)a.pl_bytes + (2 * kZwMaxRaw + 12) * 8 + 16 + 128;
  if (fixed + 2 * (size_t)a.raw_bytes > kHaloMaxSmem) return 1;
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(3 * a.np)) ncols <<= 1;
  // raw slots: as many as keep the most CTAs per SM (by shared and tensor memory)
  auto per_sm_of = [&](int nr) {
    const size_t sm = fixed + (size_t)nr * a.raw_bytes;
    if (sm > kHaloMaxSmem) return 0;
    const int k = (int)(g_smem_per_sm / (((sm + 127) / 128) * 128 + g_smem_reserved));
    return std::min(k, 512 / (int)ncols);
  };
  a.nraw = 2;
  for (int nr = 3; nr <= kZwMaxRaw; nr++)
    if (per_sm_of(nr) >= per_sm_of(a.nraw)) a.nraw = nr;
  const size_t smem = fixed + (size_t)a.nraw * a.raw_bytes;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(conv_wgrad_zw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kHaloMaxSmem);
    if (e != cudaSuccess) return set_error("unet wgrad: %s", cudaGetErrorString(e));
    attr = true;
  }
  const int per_sm = per_sm_of(a.nraw);
  if (per_sm < 1) return 1;
  const long long slots = (long long)g_num_sms * per_sm;
  a.ty = (H + 15) / 16;
  a.tx = (W + 2 + 7) / 8;
  // planes per window: few windows leave SMs idle, short ones reload more
  // planes (zc + 2 per zc tiles); take the z run with the least work on the
  // busiest CTA, counting a plane as a third of a tile
  const long long cols = (long long)nb * a.ty * a.tx;
  double best = 1e300;
  for (int zc = D;; zc = (zc + 1) / 2) {
    const long long nzc = (D + zc - 1) / zc;
    const long long items = cols * nzc;
    const long long per = (items + slots - 1) / slots;
    const double cost = (double)per * (zc + 2.0 / 3.0);
    if (cost < best) {
      best = cost;
      a.zc = zc;
      a.nzc = (int)nzc;
    }
    if (zc <= 4) break;
  }
  a.nitems = cols * a.nzc;
  if (a.nitems >= (1LL << 31)) return 1;
  const long long grid = a.nitems < slots ? a.nitems : slots;
  a.err = err;
  a.mrows = 3 * 8 * ngo <= 64 ? 64 : 128;
  CUtensorMap tmx, tmy;
  if (encode_view(&tmx, x, x_cstride, x_coff, cin, nb, D, H, W, 8, 18, 1, "wgrad x", cin) ||
      encode_view(&tmy, dy, dy_cstride, dy_coff, 8 * ngo, nb, D, H, W, 10, 16, 1, "wgrad dy", 8 * ngo))
    return -1;
  const long long n = 27LL * cin * cout;
  float *scr;
  if (unet_scratch(kScrGrad, (size_t)grid * (size_t)(n + cout), &scr, st)) return -1;
  a.part = scr;
  a.bpart = scr + (size_t)grid * n;
  conv_wgrad_zw_kernel<<<(unsigned)grid, kZwThreads, smem, st>>>(tmx, tmy, a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error("unet wgrad: %s", cudaGetErrorString(e));
  wg_reduce_kernel<<<(unsigned)((n + cout + 31) / 32), 32 * kRedSlices, 0, st>>>(a.part, (int)grid, n, dw,
                                                                             a.bpart, cout, db);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : set_error("unet wgrad: %s", cudaGetErrorString(e));
}

// The tap-stacked TMA weight gradient (sepx_unet_wgrad.inc) for 3x3x3 layers
// with 3 x (cout rounded to 8) <= 128 rows and 3 x cin / 8 + 1 N groups <= 32.
// Returns 1 where it does not apply (the caller takes the gather kernel).
int conv_wgrad_tma(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int cin,
                   const void *dy, int dy_cstride, int dy_coff, int cout, float *dw, float *db, int *err,
                   cudaStream_t st) {
  const int ngi = cin / 8, ngo = (cout + 7) / 8;
  if (!g_halo_enabled || g_wgrad_form < 1 || 3 * ngo > 16 || 3 * ngi + 1 > 32) return 1;
  if (unet_dev_init()) return -1;
  const int np = ((8 * (3 * ngi + 1)) + 15) / 16 * 16;
  const uint32_t a_bytes = 3u * ngo * kWgBox;
  const size_t budget = kHaloMaxSmem - 256 - 128;
  int ndz = 0, stages = 0;
  uint32_t stage = 0;
  auto plan = [&](int nd) {
    if (nd * np > 512) return 0;
    const uint32_t sb = a_bytes + (uint32_t)nd * (np / 8) * kWgBox;
    const size_t slack = sb >= 16u * kWgBox ? 0 : 16u * kWgBox - sb;
    const size_t k = (budget - slack) / sb;
    return (int)(k > (size_t)kWgMaxStages ? kWgMaxStages : k);
  };
  // three dz per CTA where that still leaves three stages, else one
  for (int nd : {3, 1}) {
    const int k = plan(nd);
    if (k >= 3 || (nd == 1 && k >= 2)) {
      ndz = nd;
      stages = k;
      stage = a_bytes + (uint32_t)nd * (np / 8) * kWgBox;
      break;
    }
  }
  if (!ndz) return 1;
  const size_t slack = stage >= 16u * kWgBox ? 0 : 16u * kWgBox - stage;
  const size_t smem = (size_t)stages * stage + slack + 2 * kWgMaxStages * 8 + 16 + 128;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(conv_wgrad_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kHaloMaxSmem);
    if (e != cudaSuccess) return set_error("unet wgrad: %s", cudaGetErrorString(e));
    attr = true;
  }
  CUtensorMap tmx, tmy;
  if (encode_view(&tmx, x, x_cstride, x_coff, cin, nb, D, H, W, 8, 16, 1, "wgrad x") ||
      encode_view(&tmy, dy, dy_cstride, dy_coff, 8 * ngo, nb, D, H, W, 8, 16, 1, "wgrad dy"))
    return -1;
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(ndz * np)) ncols <<= 1;
  int per_sm = (int)(g_smem_per_sm / (((smem + 127) / 128) * 128 + g_smem_reserved));
  if (per_sm < 1) return 1;
  if (per_sm * (int)ncols > 512) per_sm = 512 / (int)ncols;
  const int nzg = 3 / ndz;
  WgArgs a;
  a.nb = nb; a.D = D; a.H = H; a.W = W; a.cin = cin; a.cout = cout; a.ngi = ngi; a.ngo = ngo;
  a.ndz = ndz; a.np = np;
  a.ty = (H + 15) / 16;
  a.tx = (W + 2 + 7) / 8;
  a.ntiles = (long long)nb * D * a.ty * a.tx;
  if (a.ntiles >= (1LL << 31)) return 1;
  a.groups = (g_num_sms * per_sm) / nzg;
  if (a.groups > a.ntiles) a.groups = (int)a.ntiles;
  if (a.groups < 1) a.groups = 1;
  a.stages = stages;
  a.a_bytes = a_bytes;
  a.b_bytes = (uint32_t)ndz * (np / 8) * kWgBox;
  a.stage_bytes = stage;
  a.err = err;
  a.mrows = 3 * 8 * ngo <= 64 ? 64 : 128;
  const long long n = 27LL * cin * cout;
  float *scr;
  if (unet_scratch(kScrGrad, (size_t)a.groups * (size_t)(n + cout), &scr, st)) return -1;
  a.part = scr;
  a.bpart = scr + (size_t)a.groups * n;
  conv_wgrad_tma_kernel<<<(unsigned)(a.groups * nzg), kWgThreads, smem, st>>>(tmx, tmy, a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error("unet wgrad: %s", cudaGetErrorString(e));
  const long long tot = n + cout;
  wg_reduce_kernel<<<(unsigned)((tot + 31) / 32), 32 * kRedSlices, 0, st>>>(a.part, a.groups, n, dw, a.bpart, cout, db);
  e = cudaGetLastError();
  return e == cudaSuccess ? 0 : set_error("unet wgrad: %s", cudaGetErrorString(e));
}

// db[c] += sum_v dy[v][c]: block partials in the scratch, summed in a fixed order
int bias_grad(const void *dy, int dy_cstride, int dy_coff, long long V, int c, float *db, cudaStream_t st) {
  const int ng = (c + 7) / 8;
  const int lanes = kBiasThreads / ng;
  long long blocks = (V + lanes - 1) / lanes;
  if (blocks > 2 * 152) blocks = 2 * 152;
  float *scr;
  if (unet_scratch(kScrGrad, (size_t)blocks * c, &scr, st)) return -1;
  View dv{(const __nv_bfloat16 *)dy, dy_cstride, dy_coff};
  bias_grad_kernel<<<(unsigned)blocks, kBiasThreads, 0, st>>>(dv, V, c, scr);
  bias_sum_kernel<<<(c + 3) / 4, 128, 0, st>>>(scr, (int)blocks, c, db);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet bias_grad: launch failed");
}
}  // namespace

namespace {
// a device operand the kernel dereferences: NULL is an error, never a launch
int need_dev(const void *p, const char *what) {
  return p ? 0 : sepx::set_error("unet: %s is NULL", what);
}
int need_dims(int nb, int D, int H, int W, const char *what) {
  return (nb >= 1 && D >= 1 && H >= 1 && W >= 1)
             ? 0
             : sepx::set_error("unet %s: empty volume %d x %d x %d x %d", what, nb, D, H, W);
}
}  // namespace

extern "C" {

int sepx_unet_set_wgrad_form(int form) {
  if (form < 0 || form > 2) return set_error("unet: weight-gradient form %d (0, 1 or 2)", form);
  const int prev = g_wgrad_form;
  g_wgrad_form = form;
  return prev;
}

int sepx_unet_set_halo(int enable) {
  const int prev = g_halo_enabled ? 1 : 0;
  g_halo_enabled = enable != 0;
  return prev;
}

int sepx_unet_packed_elems(int cout, int cin_p, int ntap, int transpose) {
  const int nout = transpose ? cin_p : cout, kin = transpose ? ((cout + 7) / 8) * 8 : cin_p;
  const int kch = (ntap * kin + kKC - 1) / kKC;
  return kch * kKC * np_of(nout);
}

int sepx_unet_pack_weights(const float *w, int cout, int cin_p, int ntap, int transpose, void *out,
                           void *stream) {
  if (need_dev(w, "pack weights w") || need_dev(out, "pack weights out")) return -1;
  const int nout = transpose ? cin_p : cout, kin = transpose ? ((cout + 7) / 8) * 8 : cin_p;
  if (cout < 1 || cin_p < 8 || nout > kMaxN || cin_p % 8 || (ntap != 1 && ntap != 27))
    return set_error("unet pack: channels (%d -> %d) unsupported", kin, nout);
  const int np = np_of(nout), kch = (ntap * kin + kKC - 1) / kKC;
  PackJob J{w, (__nv_bfloat16 *)out, cout, cin_p, ntap, transpose, np, kch};
  pack_weights_kernel<<<grid_for((long long)kch * kKC * np), 256, 0, (cudaStream_t)stream>>>(J);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : set_error("unet pack: %s", cudaGetErrorString(e));
}

int sepx_unet_pack_weights_many(int njobs, const float *const *w, void *const *out, const int *cout,
                                const int *cin_p, const int *ntap, const int *transpose, void *stream) {
  if (njobs < 0 || njobs > kMaxPackJobs) return set_error("unet pack: %d jobs (at most %d)", njobs, kMaxPackJobs);
  if (njobs == 0) return 0;
  if (!w || !out || !cout || !cin_p || !ntap || !transpose) return set_error("unet pack: NULL job array");
  PackJobs P;
  long long most = 0;
  for (int i = 0; i < njobs; i++) {
    if (need_dev(w[i], "pack weights w") || need_dev(out[i], "pack weights out")) return -1;
    const int tr = transpose[i] ? 1 : 0;
    const int nout = tr ? cin_p[i] : cout[i], kin = tr ? ((cout[i] + 7) / 8) * 8 : cin_p[i];
    if (cout[i] < 1 || cin_p[i] < 8 || nout > kMaxN || cin_p[i] % 8 || (ntap[i] != 1 && ntap[i] != 27))
      return set_error("unet pack: job %d: channels (%d -> %d) unsupported", i, kin, nout);
    const int np = np_of(nout), kch = (ntap[i] * kin + kKC - 1) / kKC;
    P.j[i] = PackJob{w[i], (__nv_bfloat16 *)out[i], cout[i], cin_p[i], ntap[i], tr, np, kch};
    most = std::max(most, (long long)kch * kKC * np);
  }
  const long long bx = std::min<long long>((most + 255) / 256, 64);
  pack_weights_many_kernel<<<dim3((unsigned)bx, (unsigned)njobs), 256, 0, (cudaStream_t)stream>>>(P);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : set_error("unet pack: %s", cudaGetErrorString(e));
}

int sepx_unet_conv_fwd(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int cin,
                       int ntap, const void *wpacked, const float *bias, int cout, int relu, void *y,
                       int y_cstride, int y_coff, float *yf, const float *resid, void *stream) {
  return sepx_unet_conv_fwd_masked(x, x_cstride, x_coff, nb, D, H, W, cin, ntap, wpacked, bias, cout, relu, y,
                                   y_cstride, y_coff, yf, resid, nullptr, 0, 0, stream);
}

int sepx_unet_conv_fwd_masked(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W,
                              int cin, int ntap, const void *wpacked, const float *bias, int cout, int relu,
                              void *y, int y_cstride, int y_coff, float *yf, const float *resid,
                              const void *mask, int mask_cstride, int mask_coff, void *stream) {
  if (need_dev(x, "conv x") || need_dev(wpacked, "conv weights") || need_dims(nb, D, H, W, "conv"))
    return -1;
  if (mask && (cout % 8 || mask_cstride % 8 || mask_coff % 8 || mask_coff + cout > mask_cstride))
    return set_error("unet conv: bad mask view");
  const View mv{(const __nv_bfloat16 *)mask, mask_cstride, mask_coff};
  if (!y && !yf) return set_error("unet conv: no output (y and yf are NULL)");
  if (check_conv_args(cin, x_cstride, x_coff, cout, ntap))
    return set_error("unet conv: bad channel arguments (cin %d cstride %d coff %d cout %d ntap %d)", cin,
                     x_cstride, x_coff, cout, ntap);
  if (y && (y_cstride % 8 || y_coff % 8 || cout % 8 || y_coff + cout > y_cstride))
    return set_error("unet conv: bad output view");
  int *err;
  if (unet_err_ptr(&err)) return set_error("unet conv: cannot allocate the status word");
  const int np = np_of(cout);
  const int kch = (ntap * cin + kKC - 1) / kKC;
  const long long V = (long long)nb * D * H * W;
  if (V >= (1LL << 31) || (long long)H * W * x_cstride >= (1LL << 30))
    return set_error("unet conv: volume too large (%lld voxels)", V);
  if (ntap == 27 && H >= kTileY && W >= kTileX && halo_groups(cin) / 2 <= kMaxPairs && g_halo_enabled) {
    // packed weights of the 27 taps, plus one K group for an odd group count
    // (the packing pads with zeros up to a multiple of 8 groups, and 27 * an
    // odd count is never one)
    const int ngc = cin / 8;
    const uint32_t wbytes = (uint32_t)((27 * ngc + (ngc & 1)) * (np / 8) * 128);
    if (halo_smem_bytes(cin, wbytes, 1) <= kHaloMaxSmem)
      return conv_halo(x, x_cstride, x_coff, nb, D, H, W, cin, wpacked, wbytes, bias, cout, np, relu, y,
                       y_cstride, y_coff, yf, resid, mv, err, (cudaStream_t)stream);
  }
  if (ntap == 1 && g_halo_enabled && ((cin == 16 && cout == 1 && !y) || (cin == 8 && cout == 16))) {
    View xv{(const __nv_bfloat16 *)x, x_cstride, x_coff};
    const unsigned grid = (unsigned)std::min<long long>((V + 255) / 256, 4 * 152);
    if (cin == 16)
      conv1x1_kernel<16, 1><<<grid, 256, 0, (cudaStream_t)stream>>>(
          xv, V, (const __nv_bfloat16 *)wpacked, np, bias, relu, nullptr, 0, 0, yf, resid, mv);
    else
      conv1x1_kernel<8, 16><<<grid, 256, 0, (cudaStream_t)stream>>>(
          xv, V, (const __nv_bfloat16 *)wpacked, np, bias, relu, (__nv_bfloat16 *)y, y_cstride, y_coff, yf,
          resid, mv);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : set_error("unet conv: %s", cudaGetErrorString(e));
  }
  const size_t smem = conv_smem(np);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(conv_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)conv_smem(kMaxN));
    if (e != cudaSuccess) return set_error("unet conv: %s", cudaGetErrorString(e));
    attr = true;
  }
  View xv{(const __nv_bfloat16 *)x, x_cstride, x_coff};
  const long long mt = (V + kTM - 1) / kTM;
  // few voxel tiles (the coarse levels): split K over CTAs so that about two
  // CTAs per SM run, at least two K chunks each; the splits' FP32 sums are
  // added in order by conv_finish_kernel
  int splits = 1, kper = kch;
  if (g_halo_enabled && mt < 2 * 152 && kch >= 4) {
    splits = (int)std::min<long long>((2 * 152 + mt - 1) / mt, kch / 2);
    kper = (kch + splits - 1) / splits;
    splits = (kch + kper - 1) / kper;
  }
  if (splits > 1) {
    float *kpart;
    if (unet_scratch(kScrConv, (size_t)splits * V * np, &kpart, (cudaStream_t)stream)) return -1;
    conv_fwd_kernel<<<dim3((unsigned)mt, (unsigned)splits), kUThreads, smem, (cudaStream_t)stream>>>(
        xv, nb, D, H, W, cin, ntap, (const __nv_bfloat16 *)wpacked, kch, bias, cout, np, relu,
        (__nv_bfloat16 *)y, y_cstride, y_coff, yf, resid, err, kper, kpart, mv);
    const long long work = V * ((cout + 7) / 8);
    conv_finish_kernel<<<(unsigned)std::min<long long>((work + 255) / 256, 8 * 152), 256, 0,
                         (cudaStream_t)stream>>>(kpart, splits, V, np, bias, cout, relu,
                                                 (__nv_bfloat16 *)y, y_cstride, y_coff, yf, resid, mv);
  } else {
    conv_fwd_kernel<<<(unsigned)mt, kUThreads, smem, (cudaStream_t)stream>>>(
        xv, nb, D, H, W, cin, ntap, (const __nv_bfloat16 *)wpacked, kch, bias, cout, np, relu,
        (__nv_bfloat16 *)y, y_cstride, y_coff, yf, resid, err, kch, nullptr, mv);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : set_error("unet conv: %s", cudaGetErrorString(e));
}

int sepx_unet_conv_wgrad(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W,
                         int cin, int ntap, const void *dy, int dy_cstride, int dy_coff, int cout,
                         float *dw, void *stream) {
  return sepx_unet_conv_wgrad_bias(x, x_cstride, x_coff, nb, D, H, W, cin, ntap, dy, dy_cstride, dy_coff,
                                   cout, dw, nullptr, stream);
}

int sepx_unet_conv_wgrad_bias(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W,
                              int cin, int ntap, const void *dy, int dy_cstride, int dy_coff, int cout,
                              float *dw, float *db, void *stream) {
  if (need_dev(x, "wgrad x") || need_dev(dy, "wgrad dy") || need_dev(dw, "wgrad dw") ||
      need_dims(nb, D, H, W, "wgrad"))
    return -1;
  if (check_conv_args(cin, x_cstride, x_coff, cout, ntap) || dy_cstride % 8 || dy_coff % 8 ||
      dy_coff + ((cout + 7) / 8) * 8 > dy_cstride)
    return set_error("unet wgrad: bad channel arguments");
  int *err;
  if (unet_err_ptr(&err)) return set_error("unet wgrad: cannot allocate the status word");
  const int np = np_of(cout);
  const long long V = (long long)nb * D * H * W;
  if (V >= (1LL << 31) || (long long)H * W * x_cstride >= (1LL << 30))
    return set_error("unet wgrad: volume too large (%lld voxels)", V);
  if (ntap == 27) {
    int rc = conv_wgrad_zw(x, x_cstride, x_coff, nb, D, H, W, cin, dy, dy_cstride, dy_coff, cout, dw, db,
                           err, (cudaStream_t)stream);
    if (rc <= 0) return rc;
    rc = conv_wgrad_tma(x, x_cstride, x_coff, nb, D, H, W, cin, dy, dy_cstride, dy_coff, cout, dw, db, err,
                        (cudaStream_t)stream);
    if (rc <= 0) return rc;
  }
  if (ntap == 1 && cin == 16 && cout == 1 && g_halo_enabled) {
    constexpr int NP = 16 * 1 + 1;
    const long long blocks = std::min<long long>((V + 255) / 256, 2 * 152);
    float *scr;
    if (unet_scratch(kScrGrad, (size_t)blocks * NP, &scr, (cudaStream_t)stream)) return -1;
    View xv{(const __nv_bfloat16 *)x, x_cstride, x_coff};
    View dv{(const __nv_bfloat16 *)dy, dy_cstride, dy_coff};
    float *bscr = scr + (size_t)blocks * 16;
    wgrad1x1_kernel<16, 1><<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(xv, dv, V, scr, bscr);
    // the same fixed-order sum as the tap-stacked kernels
    wg_reduce_kernel<<<1, 32 * kRedSlices, 0, (cudaStream_t)stream>>>(scr, (int)blocks, 16, dw, bscr, 1, db);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : set_error("unet wgrad: %s", cudaGetErrorString(e));
  }
  if (db && bias_grad(dy, dy_cstride, dy_coff, V, cout, db, (cudaStream_t)stream)) return -1;
  const long long vchunks = (V + kKC - 1) / kKC;
  const int mt = (ntap * cin + kTM - 1) / kTM;
  // enough CTAs to fill the GPU about twice, with at least 16 voxel chunks
  // each (fewer on the smallest volumes: at least 4, and 8 splits)
  long long per = (vchunks * mt + 2 * 152 * 4 - 1) / (2 * 152 * 4);
  per = std::max(per, std::max(4LL, std::min(16LL, vchunks / 8)));
  // with the halo-staged kernels on, each split writes its sums to a partial
  // buffer that wg_reduce_kernel adds in split order (repeatable bits, no
  // atomics); at least 8 voxel chunks per split keep the partials small
  float *part = nullptr;
  const long long mtot = (long long)ntap * cin;
  if (g_halo_enabled) {
    per = std::max(per, 8LL);
    while ((vchunks + per - 1) / per * mtot * cout > (16LL << 20)) per *= 2;
    if (unet_scratch(kScrGrad, (size_t)((vchunks + per - 1) / per * mtot * cout), &part, (cudaStream_t)stream))
      return -1;
  }
  const long long splits = (vchunks + per - 1) / per;
  const size_t smem = conv_smem(np);
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(conv_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)conv_smem(kMaxN));
    if (e != cudaSuccess) return set_error("unet wgrad: %s", cudaGetErrorString(e));
    attr = true;
  }
  View xv{(const __nv_bfloat16 *)x, x_cstride, x_coff};
  View dv{(const __nv_bfloat16 *)dy, dy_cstride, dy_coff};
  conv_wgrad_kernel<<<dim3(mt, (unsigned)splits), kUThreads, smem, (cudaStream_t)stream>>>(
      xv, nb, D, H, W, cin, ntap, dv, cout, np, (int)per, dw, err, part);
  if (part) {
    const long long n = mtot * cout;
    wg_reduce_kernel<<<(unsigned)((n + 31) / 32), 32 * kRedSlices, 0, (cudaStream_t)stream>>>(
        part, (int)splits, n, dw, nullptr, 0, nullptr);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : set_error("unet wgrad: %s", cudaGetErrorString(e));
}

int sepx_unet_avgpool(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int c,
                      void *y, int y_cstride, int y_coff, void *stream) {
  if (need_dev(x, "avgpool x") || need_dev(y, "avgpool y") || need_dims(nb, D, H, W, "avgpool"))
    return -1;
  if (c % 8 || D % 2 || H % 2 || W % 2) return set_error("unet avgpool: bad shape");
  View xv{(const __nv_bfloat16 *)x, x_cstride, x_coff};
  avgpool_kernel<<<grid_for((long long)nb * D * H * W / 8 * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
      xv, nb, D, H, W, c, (__nv_bfloat16 *)y, y_cstride, y_coff);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet avgpool: launch failed");
}

int sepx_unet_avgpool_bwd(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                          int c, void *dx, int dx_cstride, int dx_coff, int accumulate, void *stream) {
  return sepx_unet_avgpool_bwd_masked(dy, dy_cstride, dy_coff, nb, D, H, W, c, dx, dx_cstride, dx_coff,
                                      accumulate, nullptr, 0, 0, stream);
}

int sepx_unet_avgpool_bwd_masked(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                                 int c, void *dx, int dx_cstride, int dx_coff, int accumulate,
                                 const void *mask, int mask_cstride, int mask_coff, void *stream) {
  if (need_dev(dy, "avgpool_bwd dy") || need_dev(dx, "avgpool_bwd dx") ||
      need_dims(nb, D, H, W, "avgpool_bwd"))
    return -1;
  if (c % 8 || D % 2 || H % 2 || W % 2) return set_error("unet avgpool_bwd: bad shape");
  if (mask && (mask_cstride % 8 || mask_coff % 8 || mask_coff + c > mask_cstride))
    return set_error("unet avgpool_bwd: bad mask view");
  View dv{(const __nv_bfloat16 *)dy, dy_cstride, dy_coff};
  View mv{(const __nv_bfloat16 *)mask, mask_cstride, mask_coff};
  avgpool_bwd_kernel<<<grid_for((long long)nb * D * H * W * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
      dv, nb, D, H, W, c, (__nv_bfloat16 *)dx, dx_cstride, dx_coff, accumulate, mv);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet avgpool_bwd: launch failed");
}

int sepx_unet_upsample(const void *x, int x_cstride, int x_coff, int nb, int D, int H, int W, int c,
                       void *y, int y_cstride, int y_coff, void *stream) {
  if (need_dev(x, "upsample x") || need_dev(y, "upsample y") || need_dims(nb, D, H, W, "upsample"))
    return -1;
  if (c % 8) return set_error("unet upsample: bad shape");
  View xv{(const __nv_bfloat16 *)x, x_cstride, x_coff};
  upsample_kernel<<<grid_for((long long)nb * D * H * W * 8 * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
      xv, nb, D, H, W, c, (__nv_bfloat16 *)y, y_cstride, y_coff);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet upsample: launch failed");
}

int sepx_unet_upsample_bwd(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                           int c, void *dx, int dx_cstride, int dx_coff, void *stream) {
  return sepx_unet_upsample_bwd_masked(dy, dy_cstride, dy_coff, nb, D, H, W, c, dx, dx_cstride, dx_coff,
                                       nullptr, 0, 0, stream);
}

int sepx_unet_upsample_bwd_masked(const void *dy, int dy_cstride, int dy_coff, int nb, int D, int H, int W,
                                  int c, void *dx, int dx_cstride, int dx_coff, const void *mask,
                                  int mask_cstride, int mask_coff, void *stream) {
  if (need_dev(dy, "upsample_bwd dy") || need_dev(dx, "upsample_bwd dx") ||
      need_dims(nb, D, H, W, "upsample_bwd"))
    return -1;
  if (c % 8) return set_error("unet upsample_bwd: bad shape");
  if (mask && (mask_cstride % 8 || mask_coff % 8 || mask_coff + c > mask_cstride))
    return set_error("unet upsample_bwd: bad mask view");
  View dv{(const __nv_bfloat16 *)dy, dy_cstride, dy_coff};
  View mv{(const __nv_bfloat16 *)mask, mask_cstride, mask_coff};
  upsample_bwd_kernel<<<grid_for((long long)nb * D * H * W * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
      dv, nb, D, H, W, c, (__nv_bfloat16 *)dx, dx_cstride, dx_coff, mv);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet upsample_bwd: launch failed");
}

int sepx_unet_relu_mask(const void *y, int y_cstride, int y_coff, void *dy, int dy_cstride,
                        int dy_coff, long long V, int c, void *stream) {
  if (c % 8 || V < 0) return set_error("unet relu_mask: bad shape");
  if (V == 0 || c == 0) return 0;
  if (need_dev(y, "relu_mask y") || need_dev(dy, "relu_mask dy")) return -1;
  View yv{(const __nv_bfloat16 *)y, y_cstride, y_coff};
  relu_mask_kernel<<<grid_for(V * (c / 8)), 256, 0, (cudaStream_t)stream>>>(
      yv, (__nv_bfloat16 *)dy, dy_cstride, dy_coff, V, c);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet relu_mask: launch failed");
}

int sepx_unet_bias_grad(const void *dy, int dy_cstride, int dy_coff, long long V, int c, float *db,
                        void *stream) {
  if (c > kMaxN || c < 0 || V < 0) return set_error("unet bias_grad: bad shape");
  if (V == 0 || c == 0) return 0;
  if (need_dev(dy, "bias_grad dy") || need_dev(db, "bias_grad db")) return -1;
  if (dy_cstride % 8 || dy_coff % 8 || dy_coff + ((c + 7) / 8) * 8 > dy_cstride)
    return set_error("unet bias_grad: bad channel arguments");
  return bias_grad(dy, dy_cstride, dy_coff, V, c, db, (cudaStream_t)stream);
}

int sepx_unet_to_bf16(const float *in, long long V, float scale, void *y, int y_cstride, int y_coff,
                      void *stream) {
  if (V < 0) return set_error("unet to_bf16: negative length");
  if (V == 0) return 0;
  if (need_dev(in, "to_bf16 in") || need_dev(y, "to_bf16 y")) return -1;
  to_bf16_kernel<<<grid_for(V), 256, 0, (cudaStream_t)stream>>>(in, V, scale, (__nv_bfloat16 *)y,
                                                                y_cstride, y_coff);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet to_bf16: launch failed");
}

int sepx_unet_mse(const float *out, const float *target, long long V, void *g, int g_cstride,
                  double *loss, void *stream) {
  if (V < 0) return set_error("unet mse: negative length");
  if (V == 0) return 0;
  if (need_dev(out, "mse out") || need_dev(target, "mse target") || need_dev(g, "mse g") ||
      need_dev(loss, "mse loss"))
    return -1;
  mse_kernel<<<grid_for(V) < 2 * 152 ? grid_for(V) : 2 * 152, 256, 0, (cudaStream_t)stream>>>(
      out, target, V, (__nv_bfloat16 *)g, g_cstride, loss);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet mse: launch failed");
}

int sepx_unet_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1,
                   float b2, float eps, int step, void *stream) {
  if (n < 0 || step < 1) return set_error("unet adam: n %lld, step %d", n, step);
  if (n == 0) return 0;
  if (need_dev(p, "adam p") || need_dev(g, "adam g") || need_dev(m, "adam m") || need_dev(v, "adam v"))
    return -1;
  int *err;
  if (unet_err_ptr(&err)) return set_error("unet adam: cannot allocate the status word");
  adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, nullptr, lr, b1, b2, eps,
                                                              step, err);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet adam: launch failed");
}

int sepx_unet_adam_dev(float *p, const float *g, float *m, float *v, long long n, const float *hp,
                       void *stream) {
  if (n < 0) return set_error("unet adam: n %lld", n);
  if (n == 0) return 0;
  if (need_dev(p, "adam p") || need_dev(g, "adam g") || need_dev(m, "adam m") ||
      need_dev(v, "adam v") || need_dev(hp, "adam hyper-parameters"))
    return -1;
  int *err;
  if (unet_err_ptr(&err)) return set_error("unet adam: cannot allocate the status word");
  adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, hp, 0.f, 0.f, 0.f, 0.f, 1,
                                                              err);
  return cudaGetLastError() == cudaSuccess ? 0 : set_error("unet adam: launch failed");
}

int sepx_unet_capture_begin(void *stream) {
  if (!stream) return set_error("unet capture: the legacy stream cannot be captured");
  int *err;
  if (unet_err_ptr(&err)) return set_error("unet capture: cannot allocate the status word");
  cudaError_t e = cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal);
  return e == cudaSuccess ? 0 : set_error("unet capture: %s", cudaGetErrorString(e));
}

int sepx_unet_capture_end(void *stream, void **graph) {
  if (!stream || !graph) return set_error("unet capture: NULL stream or handle");
  *graph = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &g);
  if (e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return set_error("unet capture: %s", cudaGetErrorString(e != cudaSuccess ? e : cudaErrorUnknown));
  }
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_error("unet capture: instantiate: %s", cudaGetErrorString(e));
  *graph = (void *)x;
  return 0;
}

int sepx_unet_graph_launch(void *graph, void *stream) {
  if (!graph) return set_error("unet graph: NULL handle");
  cudaError_t e = cudaGraphLaunch((cudaGraphExec_t)graph, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : set_error("unet graph: %s", cudaGetErrorString(e));
}

int sepx_unet_graph_free(void *graph) {
  if (!graph) return 0;
  cudaError_t e = cudaGraphExecDestroy((cudaGraphExec_t)graph);
  return e == cudaSuccess ? 0 : set_error("unet graph: %s", cudaGetErrorString(e));
}

int sepx_unet_status(void) {
  if (!g_unet_err) return 0;
  int h = 0;
  if (cudaMemcpy(&h, g_unet_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return h;
}

}  // extern "C"
