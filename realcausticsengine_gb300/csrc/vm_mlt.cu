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

// One light path driven by the primary samples u[0..kMltDims), split into its emission
// (mlt_path_start: false when the emission carries nothing) and its segments
// (mlt_path_bounce: one closest hit and its shading; false when the path ends), so that
// a chain can advance its path one segment per loop iteration.  Photons go to `out` (at
// most kPhotonBuf).  Russian-roulette draws come from `rr` (the reference takes them
// from its global stream).
struct MltPath {
    F3 o, d, tp;
    float dVM;
    int diffuse, last, len, channel, n;
};

__device__ __forceinline__ bool mlt_path_start(const VMParams& P, const float* u, MltPath& t) {
    t.diffuse = 0; t.last = EV_DIFFUSE; t.len = 0; t.channel = -1; t.n = 0;
    t.dVM = 0.0f;
    if (P.proposal_table) {
        const LightSample ls = light_position(P.lights, u[0], u[1], u[2]);
        const DevLight& l = P.lights.lights[ls.idx];
        t.o = ls.o;
        t.tp = ls.tp;
        if (l.type == LIGHT_SUN) {
            t.d = light_direction(l, u[3], u[4]);
        } else {
            const float ratio = table_direction(ProposalTable{P.proposal_table, P.proposal_table_res}, l, ls.idx, u[1],
                                                u[2], u[3], u[4], u[kMltDims - 1], t.d);
            if (!(ratio > 0.0f)) return false;
            t.tp = t.tp * ratio;
        }
    } else {
        sample_light(P.lights, u[0], u[1], u[2], u[3], u[4], t.o, t.d, t.tp);
    }
    return true;
}

__device__ __forceinline__ bool mlt_path_bounce(const VMParams& P, const float* u, const PathRng& rr, int maxlen,
                                                MltPath& t, PhotonRec* out) {
    const F3 ro = t.o + t.d * kRayEps;
    HitRec h;
    if (!scene_hit(P.scene, ro, t.d, kRayEps, h, P.error + ERR_STACK)) return false;
    Isect is;
    fill_isect(P.scene, h, ro, t.d, is);
    if ((unsigned)is.material >= (unsigned)P.num_materials) { atomicOr(P.error + ERR_MATERIAL, 1); return false; }
    const DevMaterial& mat = P.materials[is.material];
    // dispersion channel from the Russian-roulette stream (outside the primary samples)
    const float shift = mat.disp > 0.0f
        ? dispersion_shift(mat, t.channel, t.tp, u01(rr.block(kChannelBlock + t.len).a)) : 0.0f;
    Bsdf b;
    b.init(mat, is.ns, is.dir, false, shift);
    if (!b.valid()) return false;
    t.dVM /= fabsf(b.cos_theta_in());
    bool stored = false;
    if (!b.is_delta() && (t.last & EV_GLOSSY) && t.n < kPhotonBuf) {
        out[t.n].pos = make_float4(is.pos.x, is.pos.y, is.pos.z, t.dVM);
        out[t.n].dir = make_float4(-is.dir.x, -is.dir.y, -is.dir.z, t.tp.x);
        out[t.n].tp = make_float2(t.tp.y, t.tp.z);
        ++t.n;
        stored = true;
    }
    if (t.len > maxlen || t.diffuse > kMaxDiffuse) return false;
    const float* sv = u + 5 + 3 * t.len;
    BsdfSample smp = b.sample(sv[0], sv[1], sv[2], is.ng);
    if (is_zero(smp.f)) return false;
    F3 f = smp.f;
    if (t.len > kRRDepth) {
        if (u01(rr.block(2 + t.len).a) > smp.cont) return false;
        f = div_each(f, smp.cont);
    }
    t.o = is.pos;
    t.d = smp.wi;
    if (smp.event & EV_DIFFUSE) t.diffuse++;
    t.tp = t.tp * f;
    t.last = smp.event;
    if (!stored) t.dVM *= (smp.cos_out / smp.fwd) * smp.rev;
    else t.dVM = (smp.cos_out / smp.fwd) * (1.0f + smp.rev * t.dVM);
    t.len++;
    return true;
}

// The whole path; returns the number of photons.
__device__ int trace_light_samples(const VMParams& P, const float* u, const PathRng& rr, int maxlen, PhotonRec* out) {
    MltPath t;
    if (!mlt_path_start(P, u, t)) return 0;
    while (mlt_path_bounce(P, u, rr, maxlen, t, out)) {}
    return t.n;
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

// PSSMLT, one chain per thread, advanced one path segment per loop iteration: lanes
// whose proposal's path has ended wait until kSettleLanes lanes of the warp (or all
// that still have steps) have, then settle their steps together (accept or reject,
// dwell, the adaptive mutation size) and start their chains' next proposals, so that
// the lanes of a warp neither wait for the warp's longest path at every step nor draw
// their proposals' random numbers (dozens of Philox blocks) a few lanes at a time.
// Each chain takes the same steps with the same random numbers in the same order as a
// step-at-a-time loop: burn-in large steps t = 0 .. (first visible, at most 256) from
// the chain's first path index, then one step per further path index.
// (gem cluster, 65,536 chains, 32M steps: 1, 4, 8, 16, 24 lanes -> 680, 681, 679, 700,
// 779 ms per iteration)
constexpr int kSettleLanes = 8;

__global__ void __launch_bounds__(128) k_mlt_pss(const VMParams P, PhotonBuf ph, int chains, float p_large,
                                                 unsigned long long* __restrict__ stats) {
    const int chain = blockIdx.x * blockDim.x + threadIdx.x;
    const long long N = P.num_light_paths;
    const long long per = (N + chains - 1) / chains;
    const long long p0 = (long long)chain * per;
    const long long p1 = p0 + per < N ? p0 + per : N;
    // lanes without a chain stay in the loop (its votes take the whole warp), idle
    bool alive = chain < chains && p0 < p1;
    const int maxlen = P.max_path_length < kMltMaxLen ? P.max_path_length : kMltMaxLen;
    // the current state and the proposal: sample vectors and photon lists, swapped on
    // acceptance
    float su[2][kMltDims];
    PhotonRec sph[2][kPhotonBuf];
    int ci = 0;                      // index of the current state
    int cur_n = 0;
    unsigned long long large = 0, large_visible = 0;
    float m = 1.0f;
    int accepted = 1, mutated = 0;
    float dwell = 1.0f;
    int t = 0;                       // burn-in step (t < 256), then main steps
    bool burn_in = true;
    long long p = p0 + 1;
    bool is_large = true;
    PathRng rr;
    MltPath path;
    path.n = 0;
    bool tracing = false;
    if (alive) {
        // first proposal: burn-in step 0
        uniform_samples(P, p0, 16u, su[ci ^ 1]);
        rr.init(P.seed, (uint64_t)p0 << 9, P.iteration, STREAM_MLT + 2u);
        tracing = mlt_path_start(P, su[ci ^ 1], path);
        if (!tracing) path.n = 0;
    }
    while (__any_sync(0xffffffffu, alive)) {
        if (alive && tracing) tracing = mlt_path_bounce(P, su[ci ^ 1], rr, maxlen, path, sph[ci ^ 1]);
        const unsigned waiting = __ballot_sync(0xffffffffu, alive && !tracing);
        const unsigned live = __ballot_sync(0xffffffffu, alive);
        if (!waiting || (__popc(waiting) < kSettleLanes && waiting != live)) continue;
        if (!(alive && !tracing)) continue;
        // the proposal's path has ended: settle its step
        const int n = path.n;
        if (burn_in) {
            ++large;
            if (n > 0) { ++large_visible; ci ^= 1; cur_n = n; burn_in = false; }
            else if (++t == 256) { ci ^= 1; cur_n = 0; burn_in = false; }   // go on from the last state tried
        } else {
            if (is_large) { ++large; if (n > 0) ++large_visible; }
            if (n > 0) {
                if (cur_n > 0) store_photons(ph, sph[ci], cur_n, dwell, (uint32_t)p);
                ci ^= 1;
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
            ++p;
        }
        // the next proposal
        if (burn_in) {
            uniform_samples(P, p0, 16u + (uint32_t)t, su[ci ^ 1]);
            rr.init(P.seed, ((uint64_t)p0 << 9) | (uint64_t)t, P.iteration, STREAM_MLT + 2u);
        } else {
            if (p >= p1) {
                alive = false;
                if (cur_n > 0) store_photons(ph, sph[ci], cur_n, dwell, (uint32_t)p0);
                atomicAdd(&stats[0], large_visible);
                atomicAdd(&stats[1], large);
                continue;
            }
            PathRng g;
            g.init(P.seed, (uint64_t)p, P.iteration, STREAM_MLT + 3u);
            is_large = u01(g.block(0).a) < p_large;
            if (is_large) uniform_samples(P, p, 0u, su[ci ^ 1]);
            else {
                for (int k = 0; k < kMltDims; ++k) su[ci ^ 1][k] = su[ci][k];
                mutate(P, (uint64_t)p, m, su[ci ^ 1]);
                ++mutated;
            }
            rr.init(P.seed, (uint64_t)p * 2u, P.iteration, STREAM_MLT + 1u);
        }
        tracing = mlt_path_start(P, su[ci ^ 1], path);
        if (!tracing) path.n = 0;
    }
}

// PSSMLT one step at a time per chain: the sampler as defined (propose, trace the whole
// path, accept or reject, adapt the mutation size), kept as a launch shape so that tests
// can check that k_mlt_pss (the same chains advanced one path segment per loop
// iteration) stores exactly its photons.
__global__ void __launch_bounds__(128) k_mlt_pss_steps(const VMParams P, PhotonBuf ph, int chains, float p_large,
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

int mlt_variants() { return 2; }

void launch_mlt_pass(const VMParams& p, PhotonBuf ph, int sampler, int chains, float p_large,
                     unsigned long long* stats, cudaStream_t s, int variant) {
    if (p.num_light_paths <= 0 || chains <= 0) return;
    cudaMemsetAsync(stats, 0, 2 * sizeof(unsigned long long), s);
    const unsigned grid = (unsigned)((chains + 127) / 128);
    if (sampler != RC_SAMPLER_PSSMLT) k_mlt_hybrid<<<grid, 128, 0, s>>>(p, ph, chains, stats);
    else if (variant == 1) k_mlt_pss_steps<<<grid, 128, 0, s>>>(p, ph, chains, p_large, stats);
    else k_mlt_pss<<<grid, 128, 0, s>>>(p, ph, chains, p_large, stats);
}

}  // namespace rc
