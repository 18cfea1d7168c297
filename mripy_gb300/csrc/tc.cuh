// Fifth-generation tensor-core (tcgen05) primitives: tensor-memory (TMEM) allocation, loads
// and stores, shared-memory matrix descriptors, TF32 MMAs with the accumulator in TMEM, and
// commits to mbarriers.  Inline PTX for sm_103a.
//
// Conventions used by every caller:
// * TMEM addresses are (lane << 16) | column; a warp reaches the 32 lanes of its quarter
//   (warp % 4) only.  An M = 128 accumulator keeps row m in lane m, column n in column n.
// * A from TMEM (M = 128, kind::tf32): row m in lane m, element k in column k.
// * B in shared memory, K-major with the 128-byte swizzle: row n (of N) holds 32 TF32
//   elements (128 bytes); the 16-byte chunk c of row n sits at chunk c ^ (n % 8); eight rows
//   make a 1024-byte atom, atoms follow each other (stride 1024).  The buffer starts on a
//   1024-byte boundary.  The K step j (elements 8j .. 8j + 7) is addressed by advancing the
//   descriptor's start address by 32 j bytes; the hardware applies the swizzle.
#pragma once

#include <stdint.h>

#include "tma.cuh"

namespace gbn {

// ------------------------------------------------------------------ TMEM allocation
// one full warp; ncols a power of two in [32, 512]; the address lands in *dst
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// the warp that allocated, with the same column count
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ------------------------------------------------------------------ ordering
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// arrive (once) on the mbarrier when every earlier tcgen05 MMA of this thread has completed
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

// ------------------------------------------------------------------ descriptors
// Instruction descriptor, kind::tf32: D in F32, A and B TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t tc_idesc_tf32(int M, int N) {
    return (1u << 4)                       // D format: F32
           | (2u << 7)                     // A format: TF32
           | (2u << 10)                    // B format: TF32
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// Shared-memory descriptor of a K-major operand with the 128-byte swizzle (rows of 128
// bytes, 8-row atoms 1024 bytes apart); `addr` is the shared-state-space address of the
// K step's first byte.
__device__ __forceinline__ uint64_t tc_desc_sw128(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4)   // start address / 16
           | ((uint64_t)1 << 16)                // leading byte offset (unused with this swizzle)
           | ((uint64_t)(1024 >> 4) << 32)      // stride byte offset: next 8-row atom
           | ((uint64_t)1 << 46)                // descriptor version
           | ((uint64_t)2 << 61);               // swizzle: 128 bytes
}

// byte offset of element (row, k) of a K-major SW128 operand with 32 FP32/TF32 per row
__host__ __device__ __forceinline__ uint32_t sw128_offset(int row, int k) {
    return (uint32_t)row * 128u + ((uint32_t)(((k >> 2) ^ (row & 7))) << 4) + (uint32_t)(k & 3) * 4u;
}

// ------------------------------------------------------------------ MMA
// D[M x N] (+)= A[M x 8] * B[N x 8]^T, A in TMEM, B by descriptor; accumulate when `acc`
__device__ __forceinline__ void tc_mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                               uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(acc)
        : "memory");
}

// the same with A by descriptor
__device__ __forceinline__ void tc_mma_tf32_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                               uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(acc)
        : "memory");
}

// ------------------------------------------------------------------ TF32 split
// x = hi + lo with hi rounded to TF32 (nearest); lo = x - hi is exact in FP32 and is itself
// rounded to TF32 so the tensor core does not truncate it
__device__ __forceinline__ float tf32_round(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
__device__ __forceinline__ void tf32_split(float x, float &hi, float &lo) {
    hi = tf32_round(x);
    lo = tf32_round(x - hi);
}

// ------------------------------------------------------------------ TMEM loads and stores
// Shape 32x32b: thread t of the warp reaches lane (taddr lane + t); .xN covers N consecutive
// columns from the taddr column, one 32-bit register each.
__device__ __forceinline__ void tmem_st_x16(uint32_t taddr, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};" ::"r"(taddr),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}

__device__ __forceinline__ void tmem_st_x8(uint32_t taddr, const float (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                 : "memory");
}

__device__ __forceinline__ void tmem_ld_x8(uint32_t taddr, float (&v)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                 : "r"(taddr)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld_x16(uint32_t taddr, float (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
          "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
        : "r"(taddr)
        : "memory");
}

// every earlier tcgen05.st / tcgen05.ld of this thread has completed
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t tmem_lane_base(uint32_t base, int warp) {
    return base + ((uint32_t)((warp & 3) * 32) << 16);
}

}  // namespace gbn
