// tc.cuh -- fifth-generation tensor core (tcgen05) helpers for the closure network:
// tensor-memory allocation, BF16 MMAs with operands in shared memory and the accumulator
// in tensor memory, completion through an mbarrier with a bounded wait, accumulator reads.
//
// Operand layout in shared memory: K-major without swizzle. A tile of R rows x K bf16
// columns is stored as 8-row x 8-column core matrices of 128 contiguous bytes (row r of a
// core matrix at byte 16 r); the core matrix of row group i and column group j starts at
// byte i * (K / 8) * 128 + j * 128, so core matrices adjacent in K are 128 bytes apart
// (leading byte offset) and row groups K / 8 * 128 bytes apart (stride byte offset). One
// MMA consumes K = 16, i.e. two column groups; the next one starts 256 bytes further.
//
// Accumulator layout in tensor memory (M = 128, cta_group::1): row i of D is lane i,
// column j of D is column (base + j), one float32 per lane and column. Warp w of the CTA
// may read lanes 32 (w % 4) .. 32 (w % 4) + 31 only.
#pragma once

#include <cstdint>

#include "clbm_internal.cuh"

namespace clbm {
namespace tc {

// Byte offset of element (row, k) in a K-major tile with `kdim` columns (bf16).
__device__ __forceinline__ uint32_t kmajor_offset(int row, int k, int kdim) {
    return (uint32_t)((row >> 3) * (kdim >> 3) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading byte offset (between core
// matrices adjacent in K), stride byte offset (between 8-row groups), descriptor version
// 1 (bits 46-47), no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 accumulator, both K-major,
// N at bits 17-22 (N / 8), M at bits 24-28 (M / 16).
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// The same with FP16 A and B (format fields 0).
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// One warp allocates `ncols` (a power of two >= 32) tensor-memory columns; the base
// address is written to *dst (shared memory).
__device__ __forceinline__ void alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_addr(dst)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

// D[taddr] (+)= A * B^T for one K = 16 slice; issued by one thread.
__device__ __forceinline__ void mma(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                    bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(taddr), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate) : "memory");
}

// Arrive on the mbarrier once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy stores to shared memory become visible to the tensor cores (async proxy).
__device__ __forceinline__ void fence_smem_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the given phase parity; false when the limit ran out.
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit && !done; ++it) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    }
    return done != 0;
}

// Read 32 consecutive float32 columns of this warp's 32 lanes (thread t gets lane
// 32 (warp % 4) + t), then wait for the read.
__device__ __forceinline__ void ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr) : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Tensor-memory address of column `col` for the lanes of warp `warp`.
__device__ __forceinline__ uint32_t lane_addr(uint32_t base, int warp, int col) {
    return base + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)col;
}

}  // namespace tc
}  // namespace clbm
