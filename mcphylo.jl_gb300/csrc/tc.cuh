// Fifth-generation tensor-core building blocks (tcgen05, sm_103a) used by the
// dense-state (K > 8) node updates: shared-memory operand tiles in the canonical
// no-swizzle K-major layout, TMEM allocation, single-thread MMA issue with
// completion on an mbarrier, and TMEM -> register loads.
//
// Operand tile (rows x KD 32-bit elements, KD a multiple of 8): "core matrices"
// of 8 rows x 16 bytes, stored as 128 contiguous bytes (row-major inside); core
// matrices adjacent along K are LBO = 128 bytes apart, groups of 8 rows are
// SBO = (KD / 4) * 128 bytes apart.  Element (row, k) therefore sits at byte
//     (row / 8) * SBO + (k / 4) * 128 + (row % 8) * 16 + (k % 4) * 4.
// One kind::tf32 MMA consumes K = 8 (two core matrices along K); step s of the
// K loop starts 2 * 128 * s bytes into both tiles.
//
// Accumulator: M = 128 rows (one per TMEM lane), N columns of FP32 starting at a
// column offset.  Warp w of a 4-warp group reads lanes 32 (w % 4) .. +31, so
// thread t of the CTA owns row t.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mcphy {
namespace tc {

constexpr int kCoreBytes = 128;

// 32-bit elements (TF32): 4 per 16-byte core-matrix row
__host__ __device__ constexpr int tile_sbo(int kd) { return (kd / 4) * kCoreBytes; }
__host__ __device__ constexpr int tile_bytes(int rows, int kd) { return rows * kd * 4; }
// byte offset of element (row, k) in a tile of KD columns
__host__ __device__ constexpr int tile_off(int row, int k, int kd) {
    return (row >> 3) * tile_sbo(kd) + (k >> 2) * kCoreBytes + (row & 7) * 16 + (k & 3) * 4;
}
// the same layout for ESZ-byte elements (2: BF16, 8 per core-matrix row)
template <int ESZ> __host__ __device__ constexpr int tile_sbo_e(int kd) {
    return (kd * ESZ / 16) * kCoreBytes;
}
template <int ESZ> __host__ __device__ constexpr int tile_off_e(int row, int k, int kd) {
    return (row >> 3) * tile_sbo_e<ESZ>(kd) + (k / (16 / ESZ)) * kCoreBytes + (row & 7) * 16 +
           (k % (16 / ESZ)) * ESZ;
}

// Shared-memory matrix descriptor (64 bit): start address >> 4 in bits [0,14),
// leading-dimension byte offset >> 4 in [16,30), stride-dimension byte offset >> 4
// in [32,46), descriptor version 1 in [46,48), base offset 0, swizzle mode 0 (none)
// in [61,64).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFFu) >> 4);
    d |= uint64_t((lbo & 0x3FFFFu) >> 4) << 16;
    d |= uint64_t((sbo & 0x3FFFFu) >> 4) << 32;
    d |= uint64_t(1) << 46;
    return d;
}

// Instruction descriptor of kind::tf32 with FP32 accumulation, both operands
// K-major: D format F32 (1) in [4,6), A and B format TF32 (2) in [7,10) and
// [10,13), N >> 3 in [17,23), M >> 4 in [24,29).
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}
// kind::f16 with BF16 operands (format 1) and FP32 accumulation, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// One whole warp: allocate `ncols` TMEM columns (power of two >= 32); the TMEM
// address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_addr(slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// One whole warp (the allocating one): release the columns.
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

// D[tmem] (+)= A[smem] * B[smem]^T, M x N x 8, issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate) : "memory");
}

// The same with BF16 operands: M x N x 16 (kind::f16).
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate) : "memory");
}

// Arrive once on the mbarrier when every MMA issued so far by this thread is done.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_addr(bar)) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4]) {
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(taddr) : "memory");
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// KD (16, 24 or 32) consecutive FP32 columns of this thread's TMEM lane, loaded and
// waited for in one asm statement: the outputs exist only after the wait.
template <int KD>
__device__ __forceinline__ void tmem_row_wait(uint32_t taddr, float (&v)[KD]) {
    uint32_t r[32];
    if constexpr (KD == 16) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
            "tcgen05.wait::ld.sync.aligned;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr) : "memory");
    } else if constexpr (KD == 24) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%24];\n\t"
            "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%25];\n\t"
            "tcgen05.wait::ld.sync.aligned;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
              "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23])
            : "r"(taddr), "r"(taddr + 16u) : "memory");
    } else {
        static_assert(KD == 32, "KD is 16, 24 or 32");
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
            "tcgen05.wait::ld.sync.aligned;"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
              "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
              "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
              "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
              "=r"(r[31])
            : "r"(taddr) : "memory");
    }
#pragma unroll
    for (int i = 0; i < KD; ++i) v[i] = __uint_as_float(r[i]);
}

// FP32 -> TF32 (round to nearest, ties away), kept in a 32-bit container.
__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

}  // namespace tc
}  // namespace mcphy
