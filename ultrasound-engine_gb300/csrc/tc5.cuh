// tc5.cuh — the pieces of the fifth-generation tensor-core path shared by
// its kernels (gemm_tc5.cu, mv_tc.cu): shared-memory matrix descriptors for
// the 128-byte-swizzled K-major operand layout, the kind::f16 instruction
// descriptor, bounded mbarrier waits, and the byte offset of an element in
// the swizzled layout.
//
// Operand layout (both A and B K-major): blocks of 64 BF16 along K (128
// bytes per row); within a block, row r is 128 bytes at r * 128 and its
// 16-byte chunk j sits at chunk j ^ (r & 7); blocks of `rows` rows follow one
// another (rows * 128 bytes apart); 8-row atoms are 1024 bytes apart.
#pragma once

#include <cstdint>

namespace usxcu {

__device__ __forceinline__ unsigned su32(const void* p) { return static_cast<unsigned>(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 bytes apart (stride byte offset), version 1.
__device__ __forceinline__ uint64_t smem_desc(unsigned addr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFFu);          // start address
  d |= static_cast<uint64_t>(1u) << 16;                       // leading byte offset (unused with swizzle)
  d |= static_cast<uint64_t>((1024u >> 4) & 0x3FFFu) << 32;   // stride byte offset
  d |= static_cast<uint64_t>(1u) << 46;                       // version
  d |= static_cast<uint64_t>(2u) << 61;                       // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

// Byte offset of element (row r, k) of a K-major BF16 operand of `rows` rows
// in the swizzled layout.
__device__ __forceinline__ int sw128_offset(int rows, int r, int k) {
  return (k >> 6) * rows * 128 + r * 128 + ((((k & 63) >> 3) ^ (r & 7)) << 4) + ((k & 7) << 1);
}

// Waits for phase `parity` of the mbarrier; false after ~16M polls.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (long spin = 0; spin < (1L << 24); ++spin) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// One tcgen05.mma (cta_group::1, kind::f16) into the TMEM accumulator at
// `tmem`; `accumulate` = 0 overwrites it.
__device__ __forceinline__ void tc5_mma(unsigned tmem, uint64_t ad, uint64_t bd, uint32_t idesc, unsigned accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc5_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

// 32 consecutive TMEM columns of this warp's 32 lanes (one row per lane).
__device__ __forceinline__ void tc5_ld32(unsigned taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
        "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

}  // namespace usxcu
