// Metropolis light sampling on the GPU: many independent chains in one launch.
//
// Primary-sample vectors follow MLT_Sampler (src/MLT_Sampler.h:25-61,
// src/MLT_Sampler.cpp:7-68): dims 0..4 drive the emission (light pick, area u, area v,
// direction u, direction v), dims 5+3b.. the BSDF samples of bounce b.  A small step
// moves each coordinate by +-e*exp(-1/m) (e uniform, sign with probability 1/2) and
// wraps it to [0,1) (MLT_Sampler::Mutate); the mutation size m adapts towards an
// acceptance rate of 0.234 (src/Vertex_Merging.cpp:269-270).  "Visible" means the path
// stored at least one photon.
//
// RC_SAMPLER_HYBRID - the reference's scheme (src/Vertex_Merging.cpp:231-282), one chain
//   per thread over a contiguous range of light-path indices: every index first traces
//   a large step (fresh uniform samples); if it stores no photon, the chain state falls
//   back to its last state, is mutated, and the mutation is traced and accepted if it
//   stores a photon.  All stored photons are kept; the estimator scales them by
//   V/N (visible large steps over light paths), applied here through VM_normalization.
// With the learned proposal (P.proposal_table), the emission direction is drawn from the
// tabulated proposal at the emission cell (dims 3, 4 and the extra last dim for the
// mixture choice) and the path throughput carries p_light / q; the chains then explore
// the primary-sample space of that emission.
//
// RC_SAMPLER_PSSMLT - a visibility-target primary-sample Metropolis chain: each step is
//   a large step with probability p_large, else a small step; a visible proposal is
//   accepted, an invisible one rejected.  Every step deposits the current state's
//   photons once: a state's photons are written with weight (number of steps the chain
//   stayed there) when the chain moves on, and the visible fraction b of large steps
//   scales all photons (a consistent estimator: states are distributed as the
//   visibility function, each weighted by the visible volume b).
#include "realcaustics.h"
#include "vm.cuh"
#include "bsdf.cuh"
#include "lights.cuh"
#include "proposal.cuh"
#include "rng.cuh"

namespace rc {

namespace {

constexpr int kMltMaxLen = 12;                        // longest path the sample vector covers
// (max_path_length + 2) * 3 + 2 dims as the reference, plus the proposal's mixture choice
constexpr int kMltDims = 5 + 3 * (kMltMaxLen + 1) + 1;
constexpr int kPhotonBuf = kMltMaxLen + 2;

struct PhotonRec { float4 pos, dir; float2 tp; };

// Trace one light path driven by the primary samples u[0..kMltDims); photons go to
// `out` (at most kPhotonBuf).  Russian roulette draws come from `rr` (the reference
// takes them from its global stream).  Returns the number of photons.
__device__ int trace_light_samples(const VMParams& P, const float* u, const PathRng& rr, int maxlen, PhotonRec* out) {
    F3 o, d, tp;
    if (P.proposal_table) {
        const LightSample ls = light_position(P.lights, u[0], u[1], u[2]);
        const DevLight& l = P.lights.lights[ls.idx];
        o = ls.o;
        tp = ls.tp;
        if (l.type == LIGHT_SUN) {
            d = light_direction(l, u[3], u[4]);
        } else {
            const float ratio = table_direction(ProposalTable{P.proposal_table, P.proposal_table_res}, l, ls.idx, u[1],
                                                u[2], u[3], u[4], u[kMltDims - 1], d);
            if (!(ratio > 0.0f)) return 0;
            tp = tp * ratio;
        }
    } else {
        sample_light(P.lights, u[0], u[1], u[2], u[3], u[4], o, d, tp);
    }
    int diffuse = 0, last = EV_DIFFUSE, n = 0, channel = -1;
    float dVM = 0.0f;
    for (int len = 0;; ++len) {
        F3 ro = o + d * kRayEps;
        HitRec h;
        if (!scene_hit(P.scene, ro, d, kRayEps, h, P.error + ERR_STACK)) break;
        Isect is;
        fill_isect(P.scene, h, ro, d, is);
        if ((unsigned)is.material >= (unsigned)P.num_materials) { atomicOr(P.error + ERR_MATERIAL, 1); break; }
        const DevMaterial& mat = P.materials[is.material];
        // dispersion channel from the Russian-roulette stream (outside the primary samples)
        const float shift = mat.disp > 0.0f
            ? dispersion_shift(mat, channel, tp, u01(rr.block(kChannelBlock + len).a)) : 0.0f;
        Bsdf b;
        b.init(mat, is.ns, is.dir, false, shift);
        if (!b.valid()) break;
        dVM /= fabsf(b.cos_theta_in());
        bool stored = false;
        if (!b.is_delta() && (last & EV_GLOSSY) && n < kPhotonBuf) {
            out[n].pos = make_float4(is.pos.x, is.pos.y, is.pos.z, dVM);
            out[n].dir = make_float4(-is.dir.x, -is.dir.y, -is.dir.z, tp.x);
            out[n].tp = make_float2(tp.y, tp.z);
            ++n;
            stored = true;
        }
        if (len > maxlen || diffuse > kMaxDiffuse) break;
        const float* s = u + 5 + 3 * len;
        BsdfSample smp = b.sample(s[0], s[1], s[2], is.ng);
        if (is_zero(smp.f)) break;
        F3 f = smp.f;
        if (len > kRRDepth) {
            if (u01(rr.block(2 + len).a) > smp.cont) break;
            f = div_each(f, smp.cont);
        }
        o = is.pos;
        d = smp.wi;
        if (smp.event & EV_DIFFUSE) diffuse++;
        tp = tp * f;
        last = smp.event;
        if (!stored) dVM *= (smp.cos_out / smp.fwd) * smp.rev;
        else dVM = (smp.cos_out / smp.fwd) * (1.0f + smp.rev * dVM);
    }
    return n;
}

__device__ __forceinline__ void store_photons(PhotonBuf& ph, const PhotonRec* r, int n, float weight, uint32_t path) {
    if (n <= 0) return;
    unsigned long long base = atomicAdd(ph.count, (unsigned long long)n);
    for (int k = 0; k < n; ++k) {
        unsigned long long slot = base + k;
        if (slot >= (unsigned long long)ph.capacity) break;
        float4 dir = r[k].dir;
        dir.w *= weight;
        ph.pos[slot] = r[k].pos;
        ph.dir[slot] = dir;
        ph.tp[slot] = make_float2(r[k].tp.x * weight, r[k].tp.y * weight);
        ph.path[slot] = path;
    }
}

// uniform samples of a large step (light-path index pidx)
__device__ __forceinline__ void uniform_samples(const VMParams& P, long long pidx, uint32_t salt, float* u) {
    PathRng g;
    g.init(P.seed, (uint64_t)pidx, P.iteration ^ (salt << 20), STREAM_LIGHT);
    for (int b = 0; b < (kMltDims + 3) / 4; ++b) {
        U4 r = g.block(b);
        float v[4] = {u01(r.a), u01(r.b), u01(r.c), u01(r.d)};
        for (int k = 0; k < 4 && 4 * b + k < kMltDims; ++k) u[4 * b + k] = v[k];
    }
}

// MLT_Sampler::Mutate with the random draws of step `key`
__device__ __forceinline__ void mutate(const VMParams& P, uint64_t key, float m, float* u) {
    PathRng g;
    g.init(P.seed, key, P.iteration, STREAM_MLT);
    const float scale = powf(0.36787944117f, 1.0f / m);
    for (int b = 0; b < (kMltDims + 1) / 2; ++b) {
        U4 r = g.block(b);
        float e0 = u01(r.a), s0 = u01(r.b), e1 = u01(r.c), s1 = u01(r.d);
        int i0 = 2 * b, i1 = 2 * b + 1;
        float d0 = s0 < 0.5f ? e0 * scale : -e0 * scale;
        u[i0] += d0;
        u[i0] -= floorf(u[i0]);
        if (i1 < kMltDims) {
            float d1 = s1 < 0.5f ? e1 * scale : -e1 * scale;
            u[i1] += d1;
            u[i1] -= floorf(u[i1]);
        }
    }
}

__global__ void __launch_bounds__(128) k_mlt_hybrid(const VMParams P, PhotonBuf ph, int chains,
                                                    unsigned long long* __restrict__ stats) {
    const int chain = blockIdx.x * blockDim.x + threadIdx.x;
    if (chain >= chains) return;
    const long long N = P.num_light_paths;
    const long long per = (N + chains - 1) / chains;
    const long long p0 = (long long)chain * per;
    const long long p1 = p0 + per < N ? p0 + per : N;
    if (p0 >= p1) return;
    const int maxlen = P.max_path_length < kMltMaxLen ? P.max_path_length : kMltMaxLen;
    float cur[kMltDims], prop[kMltDims];
    PhotonRec buf[kPhotonBuf];
    // MLT_Sampler constructor: uniform initial state
    uniform_samples(P, p0, 1u, cur);
    float m = 1.0f;
    int accepted = 1, mutated = 0;
    unsigned long long visible_large = 0;
    for (long long p = p0; p < p1; ++p) {
        // large step (Init_Uniform)
        uniform_samples(P, p, 0u, prop);
        PathRng rr;
        rr.init(P.seed, (uint64_t)p * 2u, P.iteration, STREAM_MLT + 1u);
        int n = trace_light_samples(P, prop, rr, maxlen, buf);
        if (n > 0) {
            ++visible_large;
            store_photons(ph, buf, n, 1.0f, (uint32_t)p);
            for (int k = 0; k < kMltDims; ++k) cur[k] = prop[k];
            continue;
        }
        // Reject the large step, Mutate from the last state, trace the mutation
        for (int k = 0; k < kMltDims; ++k) prop[k] = cur[k];
        mutate(P, (uint64_t)p, m, prop);
        ++mutated;
        rr.init(P.seed, (uint64_t)p * 2u + 1u, P.iteration, STREAM_MLT + 1u);
        n = trace_light_samples(P, prop, rr, maxlen, buf);
        if (n > 0) {
            ++accepted;
            store_photons(ph, buf, n, 1.0f, (uint32_t)p);
            for (int k = 0; k < kMltDims; ++k) cur[k] = prop[k];
        }
        const float R = (float)accepted / (float)mutated;
        m += (R - 0.234f) / (float)mutated;
    }
    atomicAdd(&stats[0], visible_large);
    atomicAdd(&stats[1], (unsigned long long)(p1 - p0));
}

__global__ void __launch_bounds__(128) k_mlt_pss(const VMParams P, PhotonBuf ph, int chains, float p_large,
                                                 unsigned long long* __restrict__ stats) {
    const int chain = blockIdx.x * blockDim.x + threadIdx.x;
    if (chain >= chains) return;
    const long long N = P.num_light_paths;
    const long long per = (N + chains - 1) / chains;
    const long long p0 = (long long)chain * per;
    const long long p1 = p0 + per < N ? p0 + per : N;
    if (p0 >= p1) return;
    const int maxlen = P.max_path_length < kMltMaxLen ? P.max_path_length : kMltMaxLen;
    float cur[kMltDims], prop[kMltDims];
    PhotonRec cur_ph[kPhotonBuf], tmp[kPhotonBuf];
    int cur_n = 0;
    unsigned long long large = 0, large_visible = 0;
    // burn-in: large steps until a visible state (bounded); they count as large steps
    long long step = 0;
    for (int t = 0; t < 256 && cur_n == 0; ++t) {
        uniform_samples(P, p0, 16u + (uint32_t)t, cur);
        PathRng rr;
        rr.init(P.seed, ((uint64_t)p0 << 9) | (uint64_t)t, P.iteration, STREAM_MLT + 2u);
        cur_n = trace_light_samples(P, cur, rr, maxlen, cur_ph);
        ++large;
        if (cur_n > 0) ++large_visible;
    }
    float m = 1.0f;
    int accepted = 1, mutated = 0;
    float dwell = 1.0f;
    for (long long p = p0 + 1; p < p1; ++p, ++step) {
        PathRng g;
        g.init(P.seed, (uint64_t)p, P.iteration, STREAM_MLT + 3u);
        const bool is_large = u01(g.block(0).a) < p_large;
        if (is_large) uniform_samples(P, p, 0u, prop);
        else {
            for (int k = 0; k < kMltDims; ++k) prop[k] = cur[k];
            mutate(P, (uint64_t)p, m, prop);
            ++mutated;
        }
        PathRng rr;
        rr.init(P.seed, (uint64_t)p * 2u, P.iteration, STREAM_MLT + 1u);
        const int n = trace_light_samples(P, prop, rr, maxlen, tmp);
        if (is_large) { ++large; if (n > 0) ++large_visible; }
        if (n > 0) {
            if (cur_n > 0) store_photons(ph, cur_ph, cur_n, dwell, (uint32_t)p);
            for (int k = 0; k < kMltDims; ++k) cur[k] = prop[k];
            for (int k = 0; k < n; ++k) cur_ph[k] = tmp[k];
            cur_n = n;
            dwell = 1.0f;
            if (!is_large) ++accepted;
        } else {
            dwell += 1.0f;
        }
        if (!is_large && mutated > 0) {
            const float R = (float)accepted / (float)mutated;
            m += (R - 0.234f) / (float)mutated;
        }
    }
    if (cur_n > 0) store_photons(ph, cur_ph, cur_n, dwell, (uint32_t)p0);
    atomicAdd(&stats[0], large_visible);
    atomicAdd(&stats[1], large);
}

}  // namespace

void launch_mlt_pass(const VMParams& p, PhotonBuf ph, int sampler, int chains, float p_large,
                     unsigned long long* stats, cudaStream_t s) {
    if (p.num_light_paths <= 0 || chains <= 0) return;
    cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned long long), s);
    const unsigned grid = (unsigned)((chains + 127) / 128);
    if (sampler == RC_SAMPLER_PSSMLT) k_mlt_pss<<<grid, 128, 0, s>>>(p, ph, chains, p_large, stats);
    else k_mlt_hybrid<<<grid, 128, 0, s>>>(p, ph, chains, stats);
}

}  // namespace rc
