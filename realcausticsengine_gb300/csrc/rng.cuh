// Counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011).  Each (seed, path, iteration, block, stream)
// tuple maps to 4 independent 32-bit words, so every photon/camera path draws its own
// primary samples without shared state - paths are reproducible in any launch order.
//
// Sample layout of one path (the reference's primary-sample vector, src/MLT_Sampler.h):
//   block 0: light pick, area u, area v, direction u     (Lights_list::sample_lights)
//   block 1: direction v, jitter x, jitter y, unused
//   block 2 + b: the 3 BSDF samples of bounce b, and the Russian-roulette draw of
//            bounce b (the reference takes that one from its global stream).
#pragma once
#include <cstdint>

namespace rc {

struct U4 { uint32_t a, b, c, d; };

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = mulhi32(M0, ctr.a), lo0 = M0 * ctr.a;
        uint32_t hi1 = mulhi32(M1, ctr.c), lo1 = M1 * ctr.c;
        ctr = {hi1 ^ ctr.b ^ k0, lo1, hi0 ^ ctr.d ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

// 24 random bits -> [0, 1)
__host__ __device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

enum : uint32_t { STREAM_LIGHT = 0u, STREAM_CAMERA = 1u, STREAM_MLT = 2u, STREAM_PROPOSAL = 3u };

struct PathRng {
    uint32_t k0, k1, path_lo, path_hi_stream, iter;
    __host__ __device__ __forceinline__ void init(uint64_t seed, uint64_t path, uint32_t iteration, uint32_t stream) {
        k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
        path_lo = (uint32_t)path;
        path_hi_stream = ((uint32_t)(path >> 32) & 0x00ffffffu) | (stream << 24);
        iter = iteration;
    }
    __host__ __device__ __forceinline__ U4 block(uint32_t b) const {
        return philox4x32_10(U4{path_lo, path_hi_stream, iter, b}, k0, k1);
    }
};

}  // namespace rc
