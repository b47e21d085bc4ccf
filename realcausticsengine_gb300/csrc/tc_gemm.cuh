// Fifth-generation tensor-core primitives (tcgen05, sm_100a/sm_103a) as inline PTX:
// TMEM allocation, BF16 x BF16 -> FP32 MMA from shared-memory operands, completion
// through an mbarrier, accumulator read-back with tcgen05.ld.
//
// Operand layout (no swizzle, K-major): a matrix of R rows x K bf16 is stored as
// core matrices of 8 rows x 8 elements (16 bytes per row, 128 bytes per core matrix);
// core matrix (i, j) (rows 8i.., columns 8j..) sits at byte offset (i * K/8 + j) * 128.
// In the shared-memory descriptor the leading-dimension byte offset is then the step
// between core matrices along K (128 B) and the stride-dimension byte offset the step
// between 8-row groups (K/8 * 128 B).
//
// One MMA computes D[M x N] (+)= A[M x K=16] * B[N x K=16]^T with M = 128: row r of D
// lives in TMEM lane r, column c in TMEM column base + c.  Warp w of the CTA reads
// lanes 32w .. 32w+31 with tcgen05.ld.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rc {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (row, k) in the K-major core-matrix layout (bf16 elements)
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int row, int k, int K) {
    return (uint32_t)(((row >> 3) * (K >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), version 1
// (bits 46-47), no swizzle (layout type 0 in bits 61-63).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    return d;
}

// Instruction descriptor for kind::f16: D = F32, A = B = BF16, both K-major,
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* smem_result, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                 :: "r"(smem_u32(smem_result)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         bool accumulate) {
    uint32_t acc = accumulate ? 1u : 0u;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.u32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n"
        :: "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(acc) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
                 :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" :: "r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Bounded wait for phase `parity`; returns false if it did not complete.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_tries) {
    const uint32_t addr = smem_u32(mbar);
    for (uint32_t i = 0; i < max_tries; ++i) {
        uint32_t done = 0;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done) : "r"(addr), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    // the load and its wait in one statement: the outputs are defined only after the wait
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// D[128 x N] (+)= A[128 x K] * B[N x K]^T, operands in the K-major core layout at
// a_smem / b_smem; issued by the calling thread, completion on `mbar`.
__device__ __forceinline__ void gemm_issue(uint32_t d_tmem, const void* a_smem, const void* b_smem, int K, int N,
                                           bool accumulate, uint64_t* mbar) {
    const uint32_t idesc = idesc_bf16_f32(128, N);
    const uint32_t a0 = smem_u32(a_smem), b0 = smem_u32(b_smem);
    const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
    for (int k = 0; k < K; k += 16) {
        // advancing K by 16 elements = two core matrices = 256 bytes
        const uint64_t ad = smem_desc(a0 + (uint32_t)(k >> 3) * 128u, 128u, sbo);
        const uint64_t bd = smem_desc(b0 + (uint32_t)(k >> 3) * 128u, 128u, sbo);
        mma_bf16(d_tmem, ad, bd, idesc, accumulate || k > 0);
    }
    mma_commit(mbar);
}

}  // namespace tc
}  // namespace rc
