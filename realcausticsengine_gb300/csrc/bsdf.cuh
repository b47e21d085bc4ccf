// BSDFs on the device: one switch over the reference's BxDF classes
// (src/BXDF.cpp:14-667, src/BXDF.h:461-505) plus a rough GGX dielectric.
// The reference allocates a BxDF with `new` at every hit; here the BSDF is a small
// register-resident struct built from the material record and the hit.
#pragma once
#include "dev_math.cuh"
#include "rc_device_types.h"

namespace rc {

// fresnel_dielectric_eta (src/BXDF.h:461-478)
__device__ __forceinline__ float fresnel_eta(float c, float eta) {
    float g = eta * eta - 1.0f + c * c;
    if (g > 0.0f) {
        g = sqrtf(g);
        float A = (g - c) / (g + c);
        float B = (c * (g + c) - 1.0f) / (c * (g - c) + 1.0f);
        return 0.5f * A * A * (1.0f + B * B);
    }
    return 1.0f;
}

// fresnel_dielectric_reflectance (src/BXDF.h:480-498)
__device__ __forceinline__ float fresnel_reflectance(float c, float refl) {
    if (refl >= 1.0f) return 1.0f;
    float n = (1.0f + sqrtf(refl)) / (1.0f - sqrtf(refl));
    float g = n * n - 1 + c * c;
    if (g > 0.0f) {
        g = sqrtf(g);
        float A = (g - c) / (g + c);
        float B = (c * (g + c) - 1.0f) / (c * (g - c) + 1.0f);
        return 0.5f * A * A * (1.0f + B * B);
    }
    return 1.0f;
}

// D and G2 (src/BXDF.cpp:286-300)
__device__ __forceinline__ float ggx_D(float NdotH, float a2) {
    float den = NdotH * NdotH * (a2 - 1.0f) + 1.0f;
    return a2 / (kPI * den * den);
}
__device__ __forceinline__ float ggx_G2(float NdotW, float NdotL, float a2) {
    float A = NdotW * sqrtf(a2 + (1.0f - a2) * NdotL * NdotL);
    float B = NdotL * sqrtf(a2 + (1.0f - a2) * NdotW * NdotW);
    return 2.0f * NdotL * NdotW / (A + B);
}

// sample_uniform_disk / sample_cos_hemisphere (src/Sampling.h:15-46)
__device__ __forceinline__ F3 cos_hemisphere(float e0, float e1) {
    float ox = 2.0f * e0 - 1.0f, oy = 2.0f * e1 - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (!(ox == 0.0f && oy == 0.0f)) {
        float theta, r;
        if (fabsf(ox) > fabsf(oy)) { r = ox; theta = kPIOver4 * (oy / ox); }
        else { r = oy; theta = kPIOver2 - kPIOver4 * (ox / oy); }
        float s, c;
        sincosf(theta, &s, &c);
        dx = r * c; dy = r * s;
    }
    float z = sqrtf(ref_max(0.0f, 1.0f - dx * dx - dy * dy));
    return {dx, dy, z};
}

// refract (src/vec3.h:185-200)
__device__ __forceinline__ bool refract(F3 wi, F3 n, float eta, F3& wo) {
    float ci = dot(n, wi);
    float s2i = ref_max(0.0f, 1.0f - ci * ci);
    float s2t = eta * eta * s2i;
    if (s2t >= 1.0f) return false;
    float ct = sqrtf(1.0f - s2t);
    wo = (-wi) * eta + n * (eta * ci - ct);
    return true;
}

// reflect (src/vec3.h:181-184)
__device__ __forceinline__ F3 reflect(F3 v, F3 n) { return v - n * (2 * dot(v, n)); }

// GGX half vector from two primary samples as the reference draws it
// (acos(sqrt(...)) then convert_from_spherical_coordinates, src/BXDF.cpp:311-314)
__device__ __forceinline__ F3 ggx_half(float e1, float e2, float a2) {
    float theta = acosf(sqrtf((1.0f - e1) / (e1 * (a2 - 1.0f) + 1.0f)));
    float phi = e2 * kPI2;
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    return {st * cp, st * sp, ct};
}

// Dispersion (per-channel IOR): a path that meets a dispersive material for the first
// time keeps one colour channel c (uniform, from sample block kChannelBlock + bounce),
// its throughput becomes 3 x that channel alone, and every dispersive interaction of the
// path then uses IOR ior + (c - 1) * disp.  channel < 0: not chosen yet.
constexpr uint32_t kChannelBlock = 48;

__device__ __forceinline__ int pick_channel(float u) {
    const int c = (int)(u * 3.0f);
    return c > 2 ? 2 : c;
}
__device__ __forceinline__ F3 keep_channel(F3 tp, int c) {
    return f3(c == 0 ? 3.0f * tp.x : 0.0f, c == 1 ? 3.0f * tp.y : 0.0f, c == 2 ? 3.0f * tp.z : 0.0f);
}
// IOR shift at a material for a path's channel (choosing it on first contact).
__device__ __forceinline__ float dispersion_shift(const DevMaterial& m, int& channel, F3& tp, float u) {
    if (!(m.disp > 0.0f)) return 0.0f;
    if (channel < 0) {
        channel = pick_channel(u);
        tp = keep_channel(tp, channel);
    }
    return (float)(channel - 1) * m.disp;
}

struct BsdfSample {
    F3 f;           // throughput factor; zero = sampling failed
    F3 wi;          // sampled world direction
    float fwd, rev; // forward / reverse pdf (solid angle)
    float cos_out;
    float cont;     // Russian-roulette continuation probability
    int event;      // EV_* bits
};

struct Bsdf {
    int kind;
    F3 R;
    float ior, a2, s, cont;
    Frame fr;
    F3 wo;          // local direction towards the previous vertex
    bool radiance;  // TransportMode::Radiance (camera) vs Importance (light)

    __device__ __forceinline__ void init(const DevMaterial& m, F3 ns, F3 ray_dir, bool radiance_mode,
                                         float ior_shift = 0.0f) {
        kind = m.kind;
        R = f3(m.r, m.g, m.b);
        ior = m.ior + ior_shift; a2 = m.a2; s = m.s; cont = m.cont;
        radiance = radiance_mode;
        fr.set_from_z(ns);
        wo = fr.to_local(-ray_dir);
    }
    __device__ __forceinline__ bool valid() const { return !(fabsf(wo.z) < 1e-6f); }
    __device__ __forceinline__ bool is_delta() const {
        return kind == BSDF_K_SPECULAR_REFLECTION || kind == BSDF_K_FRESNEL_SPECULAR ||
               kind == BSDF_K_SPECULAR_TRANSMISSION;
    }
    __device__ __forceinline__ float cos_theta_in() const { return fabsf(wo.z); }

    // dot(wi, Ng) * dot(to_world(wo), Ng) as the reference's hemisphere tests form it
    __device__ __forceinline__ float side(F3 wi, F3 ng) const { return dot(wi, ng) * dot(fr.to_world(wo), ng); }

    __device__ BsdfSample sample(float u0, float u1, float u2, F3 ng) const {
        BsdfSample o;
        o.f = f3(0.0f); o.wi = f3(0.0f); o.fwd = 0.0f; o.rev = 0.0f; o.cos_out = 0.0f; o.cont = 0.0f; o.event = 0;
        switch (kind) {
        case BSDF_K_SPECULAR_REFLECTION: {   // src/BXDF.cpp:25-53
            o.event = EV_REFLECTION | EV_GLOSSY | EV_SPECULAR;
            F3 wl = f3(-wo.x, -wo.y, wo.z);
            o.cos_out = fabsf(wl.z);
            if (o.cos_out < 1e-6f) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0.0f) return o;
            o.fwd = 1.0f; o.rev = 1.0f; o.cont = cont;
            o.f = R;
            return o;
        }
        case BSDF_K_SPECULAR_TRANSMISSION:   // src/BXDF.cpp:76-113
        case BSDF_K_FRESNEL_SPECULAR: {      // src/BXDF.cpp:136-205
            float eta = ior;
            if (wo.z > 0) eta = 1.0f / ior;
            float f = (kind == BSDF_K_FRESNEL_SPECULAR) ? fresnel_eta(fabsf(wo.z), 1 / eta) : 0.0f;
            if (kind == BSDF_K_FRESNEL_SPECULAR && u0 < f) {
                o.event = EV_GLOSSY | EV_SPECULAR | EV_REFLECTION;
                F3 wl = f3(-wo.x, -wo.y, wo.z);
                o.cos_out = fabsf(wl.z);
                if (o.cos_out < 1e-6f) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0.0f) return o;
                o.fwd = f; o.rev = f; o.cont = cont;
                o.f = R;
                return o;
            }
            o.event = EV_TRANSMISSION | EV_GLOSSY | EV_SPECULAR;
            F3 wl;
            if (!refract(wo, wo.z > 0 ? f3(0, 0, 1) : f3(0, 0, -1), eta, wl)) return o;
            o.cos_out = fabsf(wl.z);
            if (o.cos_out < 1e-6f) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) >= 0.0f) return o;
            if (kind == BSDF_K_FRESNEL_SPECULAR) { o.fwd = 1.0f - f; o.rev = 1.0f - f; }
            else { o.fwd = 1.0f; o.rev = 1.0f; }
            o.cont = cont;
            o.f = radiance ? R * eta * eta : R;
            return o;
        }
        case BSDF_K_LAMBERT: {               // src/BXDF.cpp:228-261
            o.event = EV_DIFFUSE;
            F3 wl = cos_hemisphere(u1, u2);
            o.cos_out = wl.z;
            if (o.cos_out < 1e-6f) return o;
            if (wo.z < 0) wl.z = -wl.z;
            o.wi = fr.to_world(wl);
            o.fwd = o.cos_out * kInvPI;
            o.rev = fabsf(wo.z) * kInvPI;
            o.cont = cont;
            o.f = R;
            return o;
        }
        case BSDF_K_GGX_REFLECTION: {        // src/BXDF.cpp:302-337
            o.event = EV_GLOSSY | EV_REFLECTION;
            F3 h = ggx_half(u1, u2, a2);
            if (wo.z < 0) h.z = -h.z;
            F3 wl = reflect(-wo, h);
            o.cos_out = fabsf(wl.z);
            if (o.cos_out < 1e-6f) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0.0f || wl.z * wo.z <= 0.0f) return o;
            float chn = fabsf(h.z);
            float d = ggx_D(chn, a2);
            o.fwd = o.rev = d * chn * 0.25f / abs_dot(h, wo);
            o.cont = cont;
            float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
            o.f = div_recip(R * g2 * abs_dot(wo, h), fabsf(wo.z) * chn);
            return o;
        }
        case BSDF_K_PLASTIC_GGX: {           // src/BXDF.cpp:384-489
            float f = fresnel_reflectance(fabsf(wo.z), s);
            if (u0 < f) {
                o.event = EV_GLOSSY | EV_REFLECTION;
                F3 h = ggx_half(u1, u2, a2);
                if (wo.z < 0) h.z = -h.z;
                F3 wl = reflect(-wo, h);
                o.cos_out = fabsf(wl.z);
                if (o.cos_out < 1e-6f) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0.0f || wl.z * wo.z <= 0.0f) return o;
                float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
                o.cont = ref_max(0.05f, f);
                float fdp = fabsf(wl.z) * kInvPI, rdp = fabsf(wo.z) * kInvPI;
                float chn = fabsf(h.z);
                float d = ggx_D(chn, a2);
                float sp = d * chn * 0.25f / abs_dot(wo, h);
                if (f > 1.0f) { o.fwd = o.rev = sp; }
                else { o.fwd = fdp * (1.0f - f) + sp * f; o.rev = rdp * (1.0f - f) + sp * f; }
                // the reference's fabs() is the double one here: exact double
                // denominator, one rounding of the quotient (src/BXDF.cpp:438)
                o.f = f3((float)((double)(g2 * abs_dot(wo, h)) / ((double)fabsf(wo.z) * (double)chn)));
                return o;
            }
            o.event = EV_DIFFUSE;
            F3 wl = cos_hemisphere(u1, u2);
            o.cos_out = wl.z;
            if (o.cos_out < 1e-6f) return o;
            if (wo.z < 0) wl.z = -wl.z;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0.0f || wl.z * wo.z <= 0.0f) return o;
            o.cont = ref_max(0.05f, max3(R * (1.0f - f)));
            float fdp = fabsf(wl.z) * kInvPI, rdp = fabsf(wo.z) * kInvPI;
            F3 h = normalize(wo + wl);
            float chn = fabsf(h.z);
            float d = ggx_D(chn, a2);
            float sp = d * chn * 0.25f / abs_dot(wo, h);
            if (f > 1.0f) { o.fwd = o.rev = sp; }
            else { o.fwd = fdp * (1.0f - f) + sp * f; o.rev = rdp * (1.0f - f) + sp * f; }
            o.f = R;
            return o;
        }
        case BSDF_K_PLASTIC_SMOOTH: {        // src/BXDF.cpp:568-632
            float f = fresnel_reflectance(fabsf(wo.z), s);
            if (u0 < f) {
                o.event = EV_SPECULAR | EV_REFLECTION | EV_GLOSSY;
                F3 wl = f3(-wo.x, -wo.y, wo.z);
                o.cos_out = fabsf(wl.z);
                if (o.cos_out < 1e-6f) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0.0f || wl.z * wo.z <= 0.0f) return o;
                o.fwd = f; o.rev = f;
                o.cont = ref_max(0.05f, f);
                o.f = f3(1.0f);
                return o;
            }
            o.event = EV_DIFFUSE;
            F3 wl = cos_hemisphere(u1, u2);
            o.cos_out = wl.z;
            if (o.cos_out < 1e-6f) return o;
            if (wo.z < 0) wl.z = -wl.z;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0.0f || wl.z * wo.z <= 0.0f) return o;
            o.fwd = fabsf(wl.z) * kInvPI;
            o.rev = fabsf(wo.z) * kInvPI;
            o.cont = ref_max(0.05f, max3(R * (1.0f - f)));
            o.f = R;
            return o;
        }
        case BSDF_K_GGX_DIELECTRIC: {
            // Rough dielectric (Walter, Marschner, Li, Torrance, EGSR 2007): microfacet
            // normal from the same GGX sampling as the reference's conductor, Fresnel
            // choice between reflection and refraction through it.
            float eta = (wo.z > 0) ? 1.0f / ior : ior;      // eta_wo / eta_wi
            F3 m = ggx_half(u1, u2, a2);
            if (wo.z < 0) m.z = -m.z;
            float c = dot(wo, m);
            if (c <= 0.0f) return o;
            float F = fresnel_eta(c, 1 / eta);
            float chn = fabsf(m.z);
            float Dm = ggx_D(chn, a2);
            F3 wl;
            if (u0 < F) {
                o.event = EV_GLOSSY | EV_REFLECTION;
                wl = reflect(-wo, m);
                o.cos_out = fabsf(wl.z);
                if (o.cos_out < 1e-6f) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0.0f || wl.z * wo.z <= 0.0f) return o;
                o.fwd = o.rev = F * Dm * chn * 0.25f / c;
                float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
                o.cont = cont;
                o.f = R * (g2 * c / (fabsf(wo.z) * chn));
                return o;
            }
            o.event = EV_GLOSSY | EV_TRANSMISSION;
            if (!refract(wo, m, eta, wl)) return o;
            o.cos_out = fabsf(wl.z);
            if (o.cos_out < 1e-6f) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) >= 0.0f || wl.z * wo.z >= 0.0f) return o;
            float ci = dot(wl, m);                 // < 0
            float den = eta * c + ci;
            o.fwd = (1.0f - F) * Dm * chn * fabsf(ci) / (den * den);
            float denr = ci / eta + c;             // reverse: from wi through m to wo
            o.rev = (1.0f - F) * Dm * chn * c / (denr * denr * eta * eta);
            float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
            o.cont = cont;
            F3 base = R * (g2 * c / (fabsf(wo.z) * chn));
            o.f = radiance ? base * eta * eta : base;
            return o;
        }
        default:
            return o;
        }
    }

    // BxDF::evaluate(wi, Ng): f * |cos| as the reference returns it
    __device__ F3 evaluate(F3 wi, F3 ng) const {
        switch (kind) {
        case BSDF_K_LAMBERT:
            if (side(wi, ng) <= 0.0f) return f3(0.0f);
            return R * kInvPI * abs_dot(wi, fr.z);
        case BSDF_K_GGX_REFLECTION: {        // src/BXDF.cpp:339-356
            if (side(wi, ng) <= 0.0f) return f3(0.0f);
            F3 wl = fr.to_local(wi);
            if (wl.z * wo.z <= 0.0f) return f3(0.0f);
            float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
            F3 h = normalize(wo + wl);
            float chn = fabsf(h.z);
            float d = ggx_D(chn, a2);
            return div_recip(R * d * g2 * 0.25f, fabsf(wo.z));
        }
        case BSDF_K_PLASTIC_GGX: {           // src/BXDF.cpp:491-519
            if (side(wi, ng) <= 0.0f) return f3(0.0f);
            float f = fresnel_reflectance(fabsf(wo.z), s);
            F3 wl = fr.to_local(wi);
            if (wl.z * wo.z <= 0.0f) return f3(0.0f);
            F3 h = normalize(wl + wo);
            F3 diffuse = R * kInvPI;
            float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
            float chn = fabsf(h.z);
            float d = ggx_D(chn, a2);
            float spec = f * d * g2 * 0.25f / fabsf(wo.z);
            return f3(diffuse.x + spec, diffuse.y + spec, diffuse.z + spec);
        }
        case BSDF_K_PLASTIC_SMOOTH:          // src/BXDF.cpp:634-648
            if (side(wi, ng) <= 0.0f) return f3(0.0f);
            if (fr.to_local(wi).z * wo.z <= 0.0f) return f3(0.0f);
            return R * kInvPI;
        case BSDF_K_GGX_DIELECTRIC: {
            F3 wl = fr.to_local(wi);
            float eta = (wo.z > 0) ? 1.0f / ior : ior;
            if (wl.z * wo.z > 0.0f) {
                if (side(wi, ng) <= 0.0f) return f3(0.0f);
                F3 m = normalize(wo + wl);
                float c = fabsf(dot(wo, m));
                float F = fresnel_eta(c, 1 / eta);
                float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
                float d = ggx_D(fabsf(m.z), a2);
                return R * (F * d * g2 * 0.25f / fabsf(wo.z));
            }
            if (side(wi, ng) >= 0.0f) return f3(0.0f);
            F3 m = normalize(wo * eta + wl);
            if (dot(m, wo) < 0.0f) m = -m;
            float c = dot(wo, m), ci = dot(wl, m);
            if (c <= 0.0f || ci >= 0.0f) return f3(0.0f);
            float F = fresnel_eta(c, 1 / eta);
            float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
            float d = ggx_D(fabsf(m.z), a2);
            float den = eta * c + ci;
            float v = (1.0f - F) * d * g2 * c * fabsf(ci) / (fabsf(wo.z) * den * den);
            F3 base = R * v;
            return radiance ? base * eta * eta : base;
        }
        default:
            return f3(0.0f);   // delta BSDFs evaluate to zero
        }
    }

    // evaluate() and pdf() for one incoming direction with their common subexpressions
    // computed once, for the gather's merges.  wo_ng = dot(fr.to_world(wo), Ng) (the
    // second factor of side()) and fwo = fresnel_reflectance(|wo.z|, s) (plastic kinds)
    // are the query's constants.  Every output is formed by the same operations, in the
    // same order, as evaluate() and pdf() form it.
    __device__ __forceinline__ void eval_pdf(F3 wi, F3 ng, float wo_ng, float fwo, F3& f, float& fwd,
                                             float& rev) const {
        f = f3(0.0f);
        fwd = 0.0f; rev = 0.0f;
        const float sd = dot(wi, ng) * wo_ng;
        switch (kind) {
        case BSDF_K_LAMBERT: {
            if (sd > 0.0f) f = R * kInvPI * abs_dot(wi, fr.z);
            fwd = fabsf(fr.to_local(wi).z) * kInvPI;
            rev = fabsf(wo.z) * kInvPI;
            return;
        }
        case BSDF_K_GGX_REFLECTION: {
            const F3 wl = fr.to_local(wi);
            const F3 h = normalize(wo + wl);
            const float chn = fabsf(h.z);
            const float d = ggx_D(chn, a2);
            fwd = rev = d * chn * 0.25f / abs_dot(h, wo);
            if (sd <= 0.0f || wl.z * wo.z <= 0.0f) return;
            const float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
            f = div_recip(R * d * g2 * 0.25f, fabsf(wo.z));
            return;
        }
        case BSDF_K_PLASTIC_GGX: {
            const F3 wl = fr.to_local(wi);
            const float fdp = fabsf(wl.z) * kInvPI, rdp = fabsf(wo.z) * kInvPI;
            const F3 h = normalize(wo + wl);
            const float chn = fabsf(h.z);
            const float d = ggx_D(chn, a2);
            const float sp = d * chn * 0.25f / abs_dot(h, wo);
            if (fwo > 1.0f) { fwd = rev = sp; }
            else { fwd = fdp * (1.0f - fwo) + sp * fwo; rev = rdp * (1.0f - fwo) + sp * fwo; }
            if (sd <= 0.0f || wl.z * wo.z <= 0.0f) return;
            const F3 diffuse = R * kInvPI;
            const float g2 = ggx_G2(fabsf(wo.z), fabsf(wl.z), a2);
            const float spec = fwo * d * g2 * 0.25f / fabsf(wo.z);
            f = f3(diffuse.x + spec, diffuse.y + spec, diffuse.z + spec);
            return;
        }
        case BSDF_K_PLASTIC_SMOOTH: {
            const F3 wl = fr.to_local(wi);
            if (!(fwo > 1.0f)) {
                fwd = fabsf(wl.z) * kInvPI * (1.0f - fwo);
                rev = fabsf(wo.z) * kInvPI * (1.0f - fwo);
            }
            if (sd <= 0.0f || wl.z * wo.z <= 0.0f) return;
            f = R * kInvPI;
            return;
        }
        case BSDF_K_GGX_DIELECTRIC:
            f = evaluate(wi, ng);
            pdf(wi, fwd, rev);
            return;
        default:
            return;   // delta BSDFs
        }
    }

    // BxDF::pdf(wi, forward, reverse)
    __device__ void pdf(F3 wi, float& fwd, float& rev) const {
        switch (kind) {
        case BSDF_K_LAMBERT: {
            fwd = fabsf(fr.to_local(wi).z) * kInvPI;
            rev = fabsf(wo.z) * kInvPI;
            return;
        }
        case BSDF_K_GGX_REFLECTION: {
            F3 wl = fr.to_local(wi);
            F3 h = normalize(wo + wl);
            float chn = fabsf(h.z);
            float d = ggx_D(chn, a2);
            fwd = rev = d * chn * 0.25f / abs_dot(h, wo);
            return;
        }
        case BSDF_K_PLASTIC_GGX: {
            F3 wl = fr.to_local(wi);
            float fdp = fabsf(wl.z) * kInvPI, rdp = fabsf(wo.z) * kInvPI;
            F3 h = normalize(wo + wl);
            float chn = fabsf(h.z);
            float d = ggx_D(chn, a2);
            float sp = d * chn * 0.25f / abs_dot(h, wo);
            float f = fresnel_reflectance(fabsf(wo.z), s);
            if (f > 1.0f) { fwd = rev = sp; }
            else { fwd = fdp * (1.0f - f) + sp * f; rev = rdp * (1.0f - f) + sp * f; }
            return;
        }
        case BSDF_K_PLASTIC_SMOOTH: {
            float f = fresnel_reflectance(fabsf(wo.z), s);
            if (f > 1.0f) { fwd = rev = 0.0f; return; }
            F3 wl = fr.to_local(wi);
            fwd = fabsf(wl.z) * kInvPI * (1.0f - f);
            rev = fabsf(wo.z) * kInvPI * (1.0f - f);
            return;
        }
        case BSDF_K_GGX_DIELECTRIC: {
            F3 wl = fr.to_local(wi);
            float eta = (wo.z > 0) ? 1.0f / ior : ior;
            fwd = rev = 0.0f;
            if (wl.z * wo.z > 0.0f) {
                F3 m = normalize(wo + wl);
                float c = fabsf(dot(wo, m));
                if (c <= 0.0f) return;
                float F = fresnel_eta(c, 1 / eta);
                float chn = fabsf(m.z);
                fwd = rev = F * ggx_D(chn, a2) * chn * 0.25f / c;
                return;
            }
            F3 m = normalize(wo * eta + wl);
            if (dot(m, wo) < 0.0f) m = -m;
            float c = dot(wo, m), ci = dot(wl, m);
            if (c <= 0.0f || ci >= 0.0f) return;
            float F = fresnel_eta(c, 1 / eta);
            float chn = fabsf(m.z);
            float Dm = ggx_D(chn, a2);
            float den = eta * c + ci;
            fwd = (1.0f - F) * Dm * chn * fabsf(ci) / (den * den);
            float denr = ci / eta + c;
            rev = (1.0f - F) * Dm * chn * c / (denr * denr * eta * eta);
            return;
        }
        default:
            fwd = 0.0f; rev = 0.0f;   // delta BSDFs
            return;
        }
    }
};

}  // namespace rc
