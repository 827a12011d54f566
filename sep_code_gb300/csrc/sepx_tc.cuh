// sepx_tc.cuh -- fifth-generation tensor-core (tcgen05) building blocks for
// sm_103a: tensor-memory allocation, shared-memory matrix descriptors, the
// BF16 MMA with FP32 accumulation in tensor memory, and the loads that bring
// the accumulator back to registers.  Inline PTX only.
//
// Operand layout used throughout ("no swizzle" canonical layout): a core
// matrix is 8 rows x 16 bytes (8 BF16), stored contiguously (128 B).  For a
// K-major operand the rows are M (or N) and the 16 bytes run along K; for an
// MN-major operand the rows are K and the 16 bytes run along M (or N).  Core
// matrices are placed at  (kgroup * ngroups_mn + group_mn) * 128  bytes, so
// the stride between neighbouring MN groups is 128 B and the stride between
// neighbouring K groups is ngroups_mn * 128 B.
#pragma once
#include <cstdint>

namespace sepx {
namespace tc {

// ---- shared-memory matrix descriptor (64 bit) ----
// bits 0-13 start address >> 4; 16-29 leading-dimension byte offset >> 4;
// 32-45 stride-dimension byte offset >> 4; 46-47 descriptor version (1);
// 49-51 base offset (0); 52 LBO mode (0); 61-63 layout (0 = no swizzle).
// No swizzle, K-major:  LBO = stride between K groups, SBO = between M/N groups.
// No swizzle, MN-major: LBO = stride between K groups, SBO = between M/N groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// ---- instruction descriptor, kind::f16 with BF16 inputs and FP32 accumulator ----
// bits 4-5 D format (1 = F32); 7-9 A format (1 = BF16); 10-12 B format
// (1 = BF16); 15 A major (0 K, 1 MN); 16 B major; 17-22 N >> 3; 24-28 M >> 4.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- tensor memory ----
// One warp allocates `ncols` (a power of two >= 32) columns; the base address
// is written to shared memory at `dst`.
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 16, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// the mbarrier completes one phase once every MMA issued so far by this thread is done
__device__ __forceinline__ void mma_commit(uint32_t mbar_smem) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_smem)
      : "memory");
}

// 32 lanes x 16 columns of 32-bit accumulator: thread t of the warp receives
// lane (32 * (warp % 4) + t), columns col .. col+15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  // load and wait in one block: the registers are valid only after the wait
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Eight 32-lane x 4-column loads (columns col + 4j .. col + 4j + 3, j = 0..7,
// each naturally aligned) into q[0..7]; thread t reads lane (32 * (warp % 4)
// + t).  Loads and the wait in one block: the registers are valid after it.
__device__ __forceinline__ void tmem_ld32_q8(uint32_t taddr, float4 (&q)[9]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%4, %5, %6, %7}, [%33];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%8, %9, %10, %11}, [%34];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%12, %13, %14, %15}, [%35];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16, %17, %18, %19}, [%36];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%20, %21, %22, %23}, [%37];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%24, %25, %26, %27}, [%38];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%28, %29, %30, %31}, [%39];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr), "r"(taddr + 4), "r"(taddr + 8), "r"(taddr + 12), "r"(taddr + 16),
        "r"(taddr + 20), "r"(taddr + 24), "r"(taddr + 28)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; j++)
    q[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                       __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
}

// 32 lanes x 4 columns from the calling thread's float4
// The z-queues of two fields: 32 consecutive columns (8 planes of 4 floats)
// from each of a0 and a1 (one 32x32b.x32 load each), one wait for both.
__device__ __forceinline__ void tmem_ld32_q8_pair(uint32_t a0, uint32_t a1, float4 (&q0)[9],
                                                  float4 (&q1)[9]) {
  uint32_t r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%64];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, "
      "%42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, "
      "%60, %61, %62, %63}, [%65];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]),
        "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]),
        "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]),
        "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
        "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]),
        "=r"(r[62]), "=r"(r[63])
      : "r"(a0), "r"(a1)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; j++) {
    q0[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                        __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
    q1[j] = make_float4(__uint_as_float(r[32 + 4 * j]), __uint_as_float(r[32 + 4 * j + 1]),
                        __uint_as_float(r[32 + 4 * j + 2]), __uint_as_float(r[32 + 4 * j + 3]));
  }
}
// tcgen05.st reads its source registers asynchronously: they may be reused
// only after tcgen05.wait::st.  Storing and waiting inside one asm statement
// keeps the compiler from reusing them in between.  v goes to the 4 columns
// at a0 and to the 4 at a1.
__device__ __forceinline__ void tmem_st4x2_sync(uint32_t a0, uint32_t a1, float4 v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%2, %3, %4, %5};\n\t"
      "tcgen05.st.sync.aligned.32x32b.x4.b32 [%1], {%2, %3, %4, %5};\n\t"
      "tcgen05.wait::st.sync.aligned;" ::"r"(a0),
      "r"(a1), "r"(__float_as_uint(v.x)), "r"(__float_as_uint(v.y)), "r"(__float_as_uint(v.z)),
      "r"(__float_as_uint(v.w))
      : "memory");
}
__device__ __forceinline__ void tmem_st4(uint32_t taddr, float4 v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr),
               "r"(__float_as_uint(v.x)), "r"(__float_as_uint(v.y)), "r"(__float_as_uint(v.z)),
               "r"(__float_as_uint(v.w))
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

}  // namespace tc
}  // namespace sepx
