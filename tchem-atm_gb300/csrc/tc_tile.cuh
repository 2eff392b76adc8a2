// tcgen05 building blocks (5th-generation tensor cores, sm_100a / sm_103a): TMEM allocation,
// shared-memory matrix descriptors for the K-major no-swizzle canonical layout, the TF32
// instruction descriptor, MMA issue and commit, TMEM <-> register moves, and bounded mbarrier waits.
//
// Canonical K-major layout without swizzle (PTX ISA, tcgen05 shared memory descriptor): the
// operand is made of core matrices of 8 rows x 16 bytes (8 x 4 TF32 values), each stored as 128
// contiguous bytes, row r of the core matrix at r * 16 bytes. The descriptor's leading byte offset
// (LBO) is the distance between core matrices adjacent along K, its stride byte offset (SBO) the
// distance between 8-row groups along M (or N). One kind::tf32 MMA consumes K = 8, i.e. two core
// matrices along K.
#pragma once

#include <cstdint>

namespace tchem_gb {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (row, k) in a K-major no-swizzle operand with `kw` values of K per row
// (a multiple of 4): core matrix (row / 8, k / 4), LBO = 128, SBO = 32 * kw.
__host__ __device__ constexpr uint32_t kmajor_offset(int row, int k, int kw) {
  return static_cast<uint32_t>((row >> 3) * (32 * kw) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor: start address, LBO, SBO (bytes, multiples of 16), fixed
// version bits 46-48 = 0b001, base offset 0, no swizzle.
__host__ __device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16;
  d |= static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9 and 10-12
// = 2), optional negation of A (bit 13), both operands K-major (bits 15, 16 = 0), N >> 3 at
// bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N, bool negate_a) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((negate_a ? 1u : 0u) << 13) |
         (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
}

// Whole warp: allocates ncols TMEM columns (a power of two, 32..512); the address lands in *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

// Whole warp: frees the allocation.
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Orders this thread's generic-proxy shared-memory writes before later async-proxy reads (MMA operands).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One thread: D[tmem] (+)= op(A) * B, M x N x 8.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
      : "memory");
}

// One thread: the mbarrier receives one arrive when this thread's earlier MMAs have completed.
__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Polls the mbarrier's phase `parity` at most `limit` times; true when it completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, long long limit) {
  const uint32_t a = smem_addr(mbar);
  uint32_t done = 0;
  for (long long it = 0; it < limit && !done; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
  }
  return done != 0;
}

// Warp w of a 4-warp group: its 32 TMEM lanes (32 w .. 32 w + 31) x 16 columns from `col`;
// thread t gets lane 32 w + t.
__device__ __forceinline__ void tmem_ld16(uint32_t tbase, int warp, int col, float (&v)[16]) {
  const uint32_t a = tbase + (static_cast<uint32_t>(32 * (warp & 3)) << 16) + static_cast<uint32_t>(col);
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(a));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_st16(uint32_t tbase, int warp, int col, const float (&v)[16]) {
  const uint32_t a = tbase + (static_cast<uint32_t>(32 * (warp & 3)) << 16) + static_cast<uint32_t>(col);
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(a),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
      "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
      "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

}  // namespace tc
}  // namespace tchem_gb
