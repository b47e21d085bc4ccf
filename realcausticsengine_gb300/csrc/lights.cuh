// Light emission on the device (Lights_list::sample_lights, src/Light_list.cpp:10-30,
// Area_Light::sample_light, src/Lights.cpp:41-55, Sun_Light::sample_light,
// src/Lights.cpp:122-136).  The point light, a stub in the reference, emits uniformly
// over the sphere.
#pragma once
#include "bsdf.cuh"
#include "vm.cuh"

namespace rc {

// find_interval (src/utils.h:142-157)
__device__ __forceinline__ int light_find_interval(const float* cdf, int size, float u) {
    int first = 0, len = size;
    while (len > 0) {
        int half = len >> 1, middle = first + half;
        if (cdf[middle] < u) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    int v = first - 1;
    return v < 0 ? 0 : (v > size - 2 ? size - 2 : v);
}

// Picked light, emission position and the throughput before the direction factor.
struct LightSample {
    int idx;
    F3 o;
    F3 tp;      // colour * power * (pi for area lights, 4 pi for point lights) / pick pdf
};

__device__ __forceinline__ LightSample light_position(const LightsView& L, float u0, float u1, float u2) {
    LightSample s;
    s.idx = light_find_interval(L.cdf, L.count + 1, u0);
    const DevLight& l = L.lights[s.idx];
    const float pick = l.power / (L.count * L.integral);
    if (l.type == LIGHT_AREA) {
        s.o = ld3(l.bl) + ld3(l.hz) * u1 + ld3(l.vt) * u2;
        s.tp = div_each(f3(l.cr, l.cg, l.cb) * kPI, pick);
    } else if (l.type == LIGHT_SUN) {
        s.o = ld3(l.bl) + ld3(l.hz) * u1 + ld3(l.vt) * u2;
        s.tp = div_each(f3(l.cr, l.cg, l.cb), pick);
    } else {
        s.o = ld3(l.pos);
        s.tp = div_each(f3(l.cr, l.cg, l.cb) * (4.0f * kPI), pick);
    }
    return s;
}

// The light's own emission direction and its density (cosine-weighted about the
// emission normal for area lights, uniform sphere for point lights, a delta for the
// sun, reported as density 1).
__device__ __forceinline__ F3 light_direction(const DevLight& l, float u3, float u4) {
    if (l.type == LIGHT_AREA) {
        F3 local = cos_hemisphere(u3, u4);
        return ld3(l.fx) * local.x + ld3(l.fy) * local.y + ld3(l.fz) * local.z;
    }
    if (l.type == LIGHT_SUN) return ld3(l.fz);
    float z = 1.0f - 2.0f * u3;
    float r = sqrtf(ref_max(0.0f, 1.0f - z * z));
    float s, c;
    sincosf(kPI2 * u4, &s, &c);
    return f3(r * c, r * s, z);
}

__device__ __forceinline__ float light_direction_pdf(const DevLight& l, F3 w) {
    if (l.type == LIGHT_AREA) {
        const float c = dot(w, ld3(l.fz)) / sqrtf(length_sq(ld3(l.fz)));
        return c > 0.0f ? c * kInvPI : 0.0f;
    }
    if (l.type == LIGHT_SUN) return 1.0f;
    return 1.0f / (4.0f * kPI);
}

// Lights_list::sample_lights with the light's own direction sampling.
__device__ __forceinline__ void sample_light(const LightsView& L, float u0, float u1, float u2, float u3, float u4,
                                             F3& o, F3& d, F3& tp) {
    LightSample s = light_position(L, u0, u1, u2);
    o = s.o;
    d = light_direction(L.lights[s.idx], u3, u4);
    tp = s.tp;
}

}  // namespace rc
