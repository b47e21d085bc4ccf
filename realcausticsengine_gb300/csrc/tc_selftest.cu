// Self-check of the tcgen05 GEMM primitive: D[128 x N] = A[128 x K] * B[N x K]^T
// with BF16 operands staged into the K-major core-matrix layout and an FP32 TMEM
// accumulator, read back with tcgen05.ld.  The C ABI hook lets a test compare it with
// a host GEMM on the same BF16 inputs.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "realcaustics.h"
#include "tc_gemm.cuh"

namespace rc {
namespace {

constexpr uint32_t kWaitTries = 1u << 22;   // bounded mbarrier wait

__global__ void __launch_bounds__(128) k_tc_selftest(const __nv_bfloat16* __restrict__ A,
                                                     const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                     int K, int N, int* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* As = smem;                       // 128 x K
    unsigned char* Bs = smem + 128 * K * 2;         // N x K
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 128 * K; i += blockDim.x) {
        int r = i / K, k = i % K;
        *reinterpret_cast<__nv_bfloat16*>(As + tc::kmajor_offset(r, k, K)) = A[i];
    }
    for (int i = tid; i < N * K; i += blockDim.x) {
        int r = i / K, k = i % K;
        *reinterpret_cast<__nv_bfloat16*>(Bs + tc::kmajor_offset(r, k, K)) = B[i];
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 256);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t d_tmem = tmem_base;
    if (tid == 0) tc::gemm_issue(d_tmem, As, Bs, K, N, false, &mbar);
    bool ok = tc::mbar_wait(&mbar, 0, kWaitTries);
    if (!ok) {
        if (tid == 0) atomicOr(err, 1);
        tc::mbar_wait(&mbar, 0, kWaitTries);   // give in-flight MMAs a second bounded chance
    }
    tc::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + (tid & 31);
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tc::tmem_ld16(d_tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            for (int j = 0; j < 16 && c + j < N; ++j) D[row * N + c + j] = v[j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(d_tmem, 256);
}

// The timeout path of the bounded mbarrier wait that every tcgen05 kernel here uses:
// TMEM is allocated as in those kernels, no MMA is issued and nothing ever arrives on
// the barrier, so the wait must give up after `tries` polls, record the expiry and free
// the TMEM, leaving the context usable.
__global__ void __launch_bounds__(128) k_wait_selftest(uint32_t tries, int* err) {
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 32);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t d_tmem = tmem_base;
    const bool ok = tc::mbar_wait(&mbar, 0, tries);
    if (!ok && tid == 0) atomicOr(err, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(d_tmem, 32);
}

}  // namespace
}  // namespace rc

// Test hook: a bounded mbarrier wait that nothing completes, `tries` polls long (1 to
// 2^16).  Returns RC_E_TIMEOUT when the wait expired as it must (RC_OK would mean the
// barrier completed without an arrival).  No counterpart in the reference.
extern "C" int rc_tc_wait_selftest(unsigned tries) {
    if (tries < 1 || tries > (1u << 16)) return RC_E_INVALID;
    int* dErr = nullptr;
    if (cudaMalloc(&dErr, sizeof(int)) != cudaSuccess) return RC_E_CUDA;
    int rc = RC_OK;
    cudaMemset(dErr, 0, sizeof(int));
    rc::k_wait_selftest<<<1, 128>>>(tries, dErr);
    cudaError_t e = cudaDeviceSynchronize();
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, dErr, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = RC_E_CUDA;
    else if (h) rc = RC_E_TIMEOUT;
    cudaFree(dErr);
    return rc;
}

// Test hook: D (128 x N, FP32) = A (128 x K, BF16 bits, row-major) * B (N x K, BF16
// bits, row-major)^T on the tensor cores.  K in {16, 32, ..., 128}, N in {16, ..., 256}
// (multiples of 16).  No counterpart in the reference.
extern "C" int rc_tc_gemm_selftest(int K, int N, const unsigned short* A, const unsigned short* B, float* D) {
    if (K < 16 || K > 128 || (K % 16) || N < 16 || N > 256 || (N % 16) || !A || !B || !D) return RC_E_INVALID;
    __nv_bfloat16 *dA = nullptr, *dB = nullptr;
    float* dD = nullptr;
    int* dErr = nullptr;
    int rc = RC_OK;
    if (cudaMalloc(&dA, 2 * 128 * K) || cudaMalloc(&dB, 2 * N * K) || cudaMalloc(&dD, 4 * 128 * N) ||
        cudaMalloc(&dErr, sizeof(int))) {
        rc = RC_E_CUDA;
    } else {
        cudaMemcpy(dA, A, 2 * 128 * K, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B, 2 * N * K, cudaMemcpyHostToDevice);
        cudaMemset(dD, 0, 4 * 128 * N);
        cudaMemset(dErr, 0, sizeof(int));
        size_t smem = (size_t)(128 + N) * K * 2;
        cudaFuncSetAttribute(rc::k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        rc::k_tc_selftest<<<1, 128, smem>>>(dA, dB, dD, K, N, dErr);
        cudaError_t e = cudaDeviceSynchronize();
        int h = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&h, dErr, sizeof(int), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(D, dD, 4 * 128 * N, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = RC_E_CUDA;
        else if (h) rc = RC_E_TIMEOUT;
    }
    cudaFree(dA); cudaFree(dB); cudaFree(dD); cudaFree(dErr);
    return rc;
}
