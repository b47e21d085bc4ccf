// Flat records shared by the host code and the sm_103a kernels.
#pragma once
#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define RC_HD __host__ __device__ __forceinline__
#else
#define RC_HD inline
#endif

namespace rc {

// BSDF kinds, one per reference BxDF class (src/BXDF.h) plus the rough dielectric.
enum BsdfKind : int {
    BSDF_K_SPECULAR_REFLECTION = 0,     // Specular_Reflection        (metal, roughness < 0.01)
    BSDF_K_FRESNEL_SPECULAR = 1,        // Fresnel_Specular           (glass)
    BSDF_K_GGX_REFLECTION = 2,          // Microfacet_Reflection_GGX  (metal)
    BSDF_K_PLASTIC_GGX = 3,             // Fresnel_Microfacet_GGX     (plastic)
    BSDF_K_PLASTIC_SMOOTH = 4,          // Fresnel_Specular_Microfacet_GGX (plastic, roughness < 0.01)
    BSDF_K_LAMBERT = 5,                 // Lambertian_Reflection (no material uses it)
    BSDF_K_SPECULAR_TRANSMISSION = 6,   // Specular_Transmission (no material uses it)
    BSDF_K_GGX_DIELECTRIC = 7           // rough GGX dielectric (no counterpart in the reference)
};

// BxDFType bits (src/BXDF.h:16-24)
enum : int {
    EV_REFLECTION = 1, EV_TRANSMISSION = 2, EV_DIFFUSE = 4, EV_GLOSSY = 8, EV_SPECULAR = 16
};

struct DevMaterial {
    int kind;
    float r, g, b;        // R / T colour
    float ior;
    float a2;             // GGX alpha^2 as the reference stores it (a2 member)
    float s;              // plastic specular reflectance (specular * 0.08)
    float cont;           // max(0.05, max colour)  (mContiniationProb)
    float disp;           // per-channel IOR spread: R, G, B see ior - disp, ior, ior + disp
};

enum LightType : int { LIGHT_AREA = 0, LIGHT_SUN = 1, LIGHT_POINT = 2 };

struct DevLight {
    int type;
    float power;
    float cr, cg, cb;          // colour * power (Area_Light/Sun_Light constructors)
    float bl[3], hz[3], vt[3]; // bottom-left corner, horizontal, vertical edge
    float fx[3], fy[3], fz[3]; // emission frame (Frame::set_from_z of the rotated -z)
    float pos[3];              // point light position
};

struct DevCamera {
    int width, height;
    float origin[3], bottom_left[3], horizontal[3], vertical[3];
};

// Fixed integrator constants of the reference.
constexpr float kRayEps = 0.001f;          // src/Vertex_Merging.cpp:149,153
constexpr int kMaxDiffuse = 2;             // src/Vertex_Merging.cpp:184
constexpr int kRRDepth = 2;                // src/Vertex_Merging.cpp:60,112
constexpr float kPI = 3.14159265359f;      // src/main.cpp:42
constexpr float kInvPI = 0.31830988618f;   // src/main.cpp:48 (double literal rounded)
constexpr float kPI2 = 6.28318530718f;
constexpr float kPIOver2 = 1.57079632679f;
constexpr float kPIOver4 = 0.78539816339f;

}  // namespace rc
