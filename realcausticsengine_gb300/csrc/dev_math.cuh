// Small float3 toolkit for the kernels.  All kernels are compiled with
// -fmad=false, so each expression rounds exactly as written: the same association
// order as the reference's vec3 operators (src/vec3.h) gives the same bits.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace rc {

struct F3 { float x, y, z; };

__device__ __forceinline__ F3 f3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ F3 f3(float a) { return {a, a, a}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator-(F3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ F3 operator*(F3 a, F3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float t) { return {a.x * t, a.y * t, a.z * t}; }
__device__ __forceinline__ F3 operator*(float t, F3 a) { return {a.x * t, a.y * t, a.z * t}; }
// vec3 / float multiplies by the reciprocal (src/vec3.h:154-157)
__device__ __forceinline__ F3 div_recip(F3 a, float t) { float r = 1.0f / t; return {a.x * r, a.y * r, a.z * r}; }
// vec3 /= float divides each component (src/vec3.h:79-85)
__device__ __forceinline__ F3 div_each(F3 a, float t) { return {a.x / t, a.y / t, a.z / t}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float abs_dot(F3 a, F3 b) { return fabsf(a.x * b.x + a.y * b.y + a.z * b.z); }
__device__ __forceinline__ F3 cross(F3 u, F3 v) {
    return {u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x};
}
__device__ __forceinline__ float length_sq(F3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ F3 normalize(F3 a) { return div_recip(a, sqrtf(length_sq(a))); }
__device__ __forceinline__ float max3(F3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
__device__ __forceinline__ bool is_zero(F3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
__device__ __forceinline__ F3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ F3 xyz(float4 v) { return {v.x, v.y, v.z}; }

// std::max(a, b) returns a unless a < b (argument order matters only for NaN)
__device__ __forceinline__ float ref_max(float a, float b) { return (a < b) ? b : a; }

// Frame (src/Frame.h:6-28), built from an unnormalised z
struct Frame {
    F3 x, y, z;
    __device__ __forceinline__ void set_from_z(F3 zz) {
        z = zz;
        F3 tx = (fabsf(zz.x) > 0.99f) ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
        y = normalize(cross(zz, tx));
        x = cross(y, zz);
    }
    __device__ __forceinline__ F3 to_world(F3 a) const { return x * a.x + y * a.y + z * a.z; }
    __device__ __forceinline__ F3 to_local(F3 a) const { return {dot(a, x), dot(a, y), dot(a, z)}; }
};

}  // namespace rc
