// Light pass, camera pass and the closest-hit parity kernel.
#include "vm.cuh"
#include "bsdf.cuh"
#include "lights.cuh"
#include "rng.cuh"

namespace rc {

namespace {

// Warp-aggregated append: one atomic per converged group of lanes.  kGrouped: the
// lanes may append to different counters (the batch passes, where a warp's lanes can
// hold paths of several scenes): one atomic per group of lanes sharing a counter.
template <bool kGrouped = false>
__device__ __forceinline__ unsigned long long warp_append(unsigned long long* counter) {
    unsigned m = __activemask();
    if (kGrouped) m = __match_any_sync(m, (unsigned long long)counter);
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    unsigned lower = m & ((1u << lane) - 1u);
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(lower);
}

// Persistent light pass with path regeneration: each loop iteration advances every
// live path by one bounce; lanes whose path ended fetch the next unstarted light path
// (one atomic per warp), so a warp's lanes stay busy until the pool is empty instead of
// waiting for the warp's longest path.  Photons, their order within a path and every
// random number are the same as one-thread-per-path execution (counter-based samples).
struct LightPath {
    F3 o, d, tp;
    float dVM;
    int diffuse, last, len;
    int channel;      // dispersion channel, -1 until a dispersive material is met
    long long idx;
    PathRng rng;
};

// Emission: the light's own direction sampling, or the learned proposal's direction
// with throughput factor p_light / q (0 when the direction leaves no emission).
__device__ __forceinline__ bool light_path_start(const VMParams& P, long long pidx, LightPath& s) {
    s.idx = pidx;
    s.rng.init(P.seed, (uint64_t)pidx, P.iteration, STREAM_LIGHT);
    U4 b0 = s.rng.block(0), b1 = s.rng.block(1);
    const LightSample ls = light_position(P.lights, u01(b0.a), u01(b0.b), u01(b0.c));
    s.o = ls.o;
    if (P.proposal) {
        const float4 pr = __ldg(&P.proposal[pidx]);
        if (!(pr.w > 0.0f)) return false;
        s.d = f3(pr.x, pr.y, pr.z);
        s.tp = ls.tp * pr.w;
    } else {
        s.d = light_direction(P.lights.lights[ls.idx], u01(b0.d), u01(b1.a));
        s.tp = ls.tp;
    }
    s.diffuse = 0;
    s.last = EV_DIFFUSE;
    s.dVM = 0.0f;
    s.len = 0;
    s.channel = -1;
    return true;
}

// One bounce of Vertex_Merging::trace_light_path (src/Vertex_Merging.cpp:140-194), in
// two halves: the closest hit of the path's next segment (false: the path ends), then
// the shading at that hit - photon store, BSDF sample, Russian roulette, dVM update -
// which returns false when the path ends.  The persistent pass runs both per bounce,
// the wavefront pass runs them in separate kernels.
template <class Stack>
__device__ __forceinline__ bool light_path_trace(const VMParams& P, const LightPath& s, HitRec& h, Stack& stack) {
    const F3 ro = s.o + s.d * kRayEps;
    return scene_hit(P.scene, ro, s.d, kRayEps, h, P.error + ERR_STACK, stack);
}

template <bool kGrouped = false>
__device__ __forceinline__ bool light_path_shade(const VMParams& P, const PhotonBuf& ph, LightPath& s,
                                                 const HitRec& h) {
    const F3 ro = s.o + s.d * kRayEps;
    Isect is;
    fill_isect(P.scene, h, ro, s.d, is);
    if ((unsigned)is.material >= (unsigned)P.num_materials) { atomicOr(P.error + ERR_MATERIAL, 1); return false; }
    const DevMaterial& mat = P.materials[is.material];
    const float shift = mat.disp > 0.0f
        ? dispersion_shift(mat, s.channel, s.tp, u01(s.rng.block(kChannelBlock + s.len).a)) : 0.0f;
    Bsdf b;
    b.init(mat, is.ns, is.dir, false, shift);
    if (!b.valid()) return false;
    s.dVM /= fabsf(b.cos_theta_in());
    bool stored = false;
    if (!b.is_delta() && (s.last & EV_GLOSSY)) {
        unsigned long long slot = warp_append<kGrouped>(ph.count);
        if (slot < (unsigned long long)ph.capacity) {
            ph.pos[slot] = make_float4(is.pos.x, is.pos.y, is.pos.z, s.dVM);
            ph.dir[slot] = make_float4(-is.dir.x, -is.dir.y, -is.dir.z, s.tp.x);
            ph.tp[slot] = make_float2(s.tp.y, s.tp.z);
            ph.path[slot] = (uint32_t)s.idx;
        }
        stored = true;
    }
    if (s.len > P.max_path_length || s.diffuse > kMaxDiffuse) return false;
    U4 bb = s.rng.block(2 + s.len);
    BsdfSample smp = b.sample(u01(bb.a), u01(bb.b), u01(bb.c), is.ng);
    if (is_zero(smp.f)) return false;
    F3 f = smp.f;
    if (s.len > kRRDepth) {
        if (u01(bb.d) > smp.cont) return false;
        f = div_each(f, smp.cont);
    }
    s.o = is.pos;
    s.d = smp.wi;
    if (smp.event & EV_DIFFUSE) s.diffuse++;
    s.tp = s.tp * f;
    s.last = smp.event;
    if (!stored) s.dVM *= (smp.cos_out / smp.fwd) * smp.rev;
    else s.dVM = (smp.cos_out / smp.fwd) * (1.0f + smp.rev * s.dVM);
    s.len++;
    return true;
}

template <bool kGrouped = false, class Stack>
__device__ __forceinline__ bool light_path_bounce(const VMParams& P, const PhotonBuf& ph, LightPath& s,
                                                  Stack& stack) {
    HitRec h;
    if (!light_path_trace(P, s, h, stack)) return false;
    return light_path_shade<kGrouped>(P, ph, s, h);
}

// Wavefront light pass: the same paths, bounces and photons as the persistent pass,
// with each bounce split over two kernels that every queued path passes through: a
// trace kernel (the closest hit only, so it keeps few registers and every lane holds a
// live ray) and a shade kernel that appends the paths that continue to the next queue.
// Path state between the kernels, per slot (slot = position in the light-path order):
//   o4 = origin | dVM, d4 = direction | tp.r, t2 = tp.gb,
//   m4 = path index, length, diffuse bounces, last event | (dispersion channel + 1) << 8,
//   hit = t, u, v, triangle slot (-1: the path ends).
struct WfState {
    float4* o4; float4* d4; float2* t2; int4* m4; float4* hit;
    uint32_t* queue[2];
    unsigned long long* count;   // [2] queue lengths
};

__device__ __forceinline__ void wf_store(const WfState& W, uint32_t slot, const LightPath& s) {
    W.o4[slot] = make_float4(s.o.x, s.o.y, s.o.z, s.dVM);
    W.d4[slot] = make_float4(s.d.x, s.d.y, s.d.z, s.tp.x);
    W.t2[slot] = make_float2(s.tp.y, s.tp.z);
    W.m4[slot] = make_int4((int)(uint32_t)s.idx, s.len, s.diffuse, (s.last & 0xff) | ((s.channel + 1) << 8));
}

__device__ __forceinline__ void wf_load(const VMParams& P, const WfState& W, uint32_t slot, LightPath& s) {
    const float4 o = W.o4[slot], d = W.d4[slot];
    const float2 t = W.t2[slot];
    const int4 m = W.m4[slot];
    s.o = f3(o.x, o.y, o.z); s.dVM = o.w;
    s.d = f3(d.x, d.y, d.z);
    s.tp = f3(d.w, t.x, t.y);
    s.idx = (long long)(uint32_t)m.x;
    s.len = m.y; s.diffuse = m.z;
    s.last = m.w & 0xff;
    s.channel = (m.w >> 8) - 1;
    s.rng.init(P.seed, (uint64_t)s.idx, P.iteration, STREAM_LIGHT);
}

__device__ __forceinline__ void wf_push(const WfState& W, int q, uint32_t slot) {
    W.queue[q][warp_append(&W.count[q])] = slot;
}

__global__ void k_wf_start(const VMParams P, WfState W) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= P.num_light_paths) return;
    const long long pidx = P.path_order ? (long long)__ldg(&P.path_order[i]) : i;
    LightPath s;
    if (!light_path_start(P, pidx, s)) return;
    wf_store(W, (uint32_t)i, s);
    wf_push(W, 0, (uint32_t)i);
}

template <int kMinBlocks>
__global__ void __launch_bounds__(128, kMinBlocks) k_wf_trace(const VMParams P, WfState W, int q) {
    const unsigned long long n = W.count[q];
    WarpStepStack stk;   // the lanes of a warp trace together here: step them together
    for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < n;
         j += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t slot = W.queue[q][j];
        const float4 o = W.o4[slot], d = W.d4[slot];
        LightPath s;
        s.o = f3(o.x, o.y, o.z);
        s.d = f3(d.x, d.y, d.z);
        HitRec h;
        if (!light_path_trace(P, s, h, stk)) h.slot = -1;
        W.hit[slot] = make_float4(h.t, h.u, h.v, __int_as_float(h.slot));
    }
}

// The paths still queued after the last wavefront round, each taken through all of its
// remaining bounces by one thread (few paths remain; one launch instead of a round per
// bounce, each of which waits for its longest traversal).
__global__ void __launch_bounds__(128, 8) k_wf_finish(const VMParams P, PhotonBuf ph, WfState W, int q) {
    const unsigned long long n = W.count[q];
    CallStack stk;
    for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < n;
         j += (unsigned long long)gridDim.x * blockDim.x) {
        LightPath s;
        wf_load(P, W, W.queue[q][j], s);
        while (light_path_bounce(P, ph, s, stk)) {}
    }
}

__global__ void __launch_bounds__(128) k_wf_shade(const VMParams P, PhotonBuf ph, WfState W, int q) {
    const unsigned long long n = W.count[q];
    for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < n;
         j += (unsigned long long)gridDim.x * blockDim.x) {
        const uint32_t slot = W.queue[q][j];
        const float4 hv = W.hit[slot];
        HitRec h{hv.x, hv.y, hv.z, __float_as_int(hv.w)};
        if (h.slot < 0) continue;
        LightPath s;
        wf_load(P, W, slot, s);
        if (!light_path_shade(P, ph, s, h)) continue;
        wf_store(W, slot, s);
        wf_push(W, q ^ 1, slot);
    }
}

// Light-path order: 4D Morton key of a path's emission samples (the same Philox draws
// light_path_start reads; with the learned proposal, the area samples and the proposed
// direction), counting-sorted.
constexpr int kOrderBits = 5;                      // cells per axis: 32
constexpr int kOrderCells = 1 << (4 * kOrderBits);

__global__ void k_light_keys(const VMParams P, uint32_t* __restrict__ keys, uint32_t* __restrict__ counts) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= P.num_light_paths) return;
    PathRng g;
    g.init(P.seed, (uint64_t)i, P.iteration, STREAM_LIGHT);
    const U4 b0 = g.block(0), b1 = g.block(1);
    float u[4] = {u01(b0.b), u01(b0.c), u01(b0.d), u01(b1.a)};
    if (P.proposal_table) {
        // emission about to be drawn from the tabulated proposal (mlp_proposal, in this
        // order): area cell, mixture component sample and the first direction sample, so
        // that a warp's lanes read the same table cells and lobes
        u[2] = u01(b1.b);
        u[3] = u01(b0.d);
    } else if (P.proposal) {
        // the learned proposal gives the direction: its octahedral coordinates instead
        const float4 pr = __ldg(&P.proposal[i]);
        const float l1 = fabsf(pr.x) + fabsf(pr.y) + fabsf(pr.z);
        float ox = l1 > 0.0f ? pr.x / l1 : 0.0f, oy = l1 > 0.0f ? pr.y / l1 : 0.0f;
        if (pr.z < 0.0f) {
            const float tx = (1.0f - fabsf(oy)) * (ox < 0.0f ? -1.0f : 1.0f);
            oy = (1.0f - fabsf(ox)) * (oy < 0.0f ? -1.0f : 1.0f);
            ox = tx;
        }
        u[2] = 0.5f * (ox + 1.0f);
        u[3] = 0.5f * (oy + 1.0f);
    }
    uint32_t key = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t c = min((uint32_t)(u[k] * (float)(1 << kOrderBits)), (uint32_t)((1 << kOrderBits) - 1));
#pragma unroll
        for (int bit = 0; bit < kOrderBits; ++bit) key |= ((c >> bit) & 1u) << (4 * bit + k);
    }
    keys[i] = key;
    atomicAdd(&counts[key], 1u);
}

__global__ void k_light_scatter(const uint32_t* __restrict__ keys, long long n, uint32_t* __restrict__ cursor,
                                uint32_t* __restrict__ order) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    order[atomicAdd(&cursor[keys[i]], 1u)] = (uint32_t)i;
}

constexpr int kRefillLanes = 24;

// kMinBlocks caps the registers per thread (resident blocks per SM the allocation must
// allow); traversal stacks are per-traversal local-memory arrays.
template <int kBlock, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_light_pass_persistent(const VMParams P, PhotonBuf ph,
                                                                               unsigned long long* __restrict__ next_path,
                                                                               unsigned long long* __restrict__ rays) {
    CallStack stk;
    const int lane = threadIdx.x & 31;
    LightPath s;
    bool alive = false;
    bool pool_left = true;
    unsigned traced = 0;      // closest-hit queries of this lane (one per bounce)
    while (true) {
        // refill lanes without a path, once at least kRefillLanes are free (or none has
        // a path): lanes refilled together take consecutive, coherent paths (the order
        // sorts paths by their emission samples), so a warp keeps groups of coherent
        // paths together for several bounces (measured on the water pool: refilling at
        // any free lane 14.2 ms, at 16 free 13.6, at 20-24 free 13.4, at 32 free 14.5;
        // with the children tested at the parent, per iteration at 20 / 24 / 28 / 32
        // free: 20.49 / 20.48 / 20.82 / 21.13 ms)
        const unsigned need = __ballot_sync(0xffffffffu, !alive);
        if (need && pool_left && (__popc(need) >= kRefillLanes || need == 0xffffffffu)) {
            unsigned long long base = 0;
            if (lane == __ffs(need) - 1) base = atomicAdd(next_path, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
            if (!alive) {
                const unsigned long long mine = base + __popc(need & ((1u << lane) - 1u));
                if (mine < (unsigned long long)P.num_light_paths)
                    alive = light_path_start(P, P.path_order ? (long long)__ldg(&P.path_order[mine]) : (long long)mine,
                                             s);
            }
            if (base + __popc(need) >= (unsigned long long)P.num_light_paths) pool_left = false;
        }
        if (!__any_sync(0xffffffffu, alive)) break;
        if (alive) { alive = light_path_bounce(P, ph, s, stk); ++traced; }
    }
    const unsigned w = __reduce_add_sync(0xffffffffu, traced);
    if (rays && lane == 0) atomicAdd(rays, (unsigned long long)w);
}

// Persistent camera pass with path regeneration (same scheme as the light pass).
struct CameraPath {
    F3 o, d, tp;
    float dVM;
    int len;
    int channel;      // dispersion channel, -1 until a dispersive material is met
    int target;
    PathRng rng;
};

// Generate_camera_sample + Image_Buffer::add_color's row mapping; false when the
// sample falls outside the image buffer (camera row 0, src/Image_Buffer.h:28-31).
__device__ __forceinline__ bool camera_path_start(const VMParams& P, long long pix, CameraPath& s) {
    const int W = P.camera.width, H = P.camera.height;
    s.rng.init(P.camera_seed, (uint64_t)pix, P.iteration, STREAM_CAMERA);
    U4 b1 = s.rng.block(1);
    const float x = (float)(int)(pix % W);
    const float y = (float)(int)(pix / W);
    const float sx = x + u01(b1.b), sy = y + u01(b1.c);
    if (sx < 0 || sx >= (float)W || sy < 0 || sy >= (float)H) return false;
    const int X = (int)sx, Y = H - (int)sy;
    const long long target = (long long)X + (long long)Y * W;
    if (target > (long long)W * H - 1) return false;
    F3 dir = ld3(P.camera.bottom_left) + ld3(P.camera.horizontal) * (sx / (float)W) +
             ld3(P.camera.vertical) * (sy / (float)H);
    dir = dir - ld3(P.camera.origin);
    s.o = ld3(P.camera.origin);
    s.d = normalize(dir);
    s.tp = f3(1.0f);
    s.dVM = 0.0f;
    s.len = 0;
    s.channel = -1;
    s.target = (int)target;
    return true;
}

template <bool kGrouped = false, class Stack>
__device__ __forceinline__ bool camera_path_bounce(const VMParams& P, const QueryBuf& qb, CameraPath& s,
                                                   Stack& stack) {
    F3 ro = s.o + s.d * kRayEps;
    HitRec h;
    if (!scene_hit(P.scene, ro, s.d, kRayEps, h, P.error + ERR_STACK, stack)) return false;
    Isect is;
    fill_isect(P.scene, h, ro, s.d, is);
    if ((unsigned)is.material >= (unsigned)P.num_materials) { atomicOr(P.error + ERR_MATERIAL, 1); return false; }
    const DevMaterial& mat = P.materials[is.material];
    const float shift = mat.disp > 0.0f
        ? dispersion_shift(mat, s.channel, s.tp, u01(s.rng.block(kChannelBlock + s.len).a)) : 0.0f;
    Bsdf b;
    b.init(mat, is.ns, is.dir, true, shift);
    if (!b.valid()) return false;
    s.dVM /= fabsf(b.cos_theta_in());
    if (!b.is_delta()) {
        unsigned long long slot = warp_append<kGrouped>(qb.count);
        if (slot < (unsigned long long)qb.capacity) {
            F3 w = s.tp * P.vm_norm;
            qb.q0[slot] = make_float4(is.pos.x, is.pos.y, is.pos.z, s.dVM);
            qb.q1[slot] = make_float4(is.ns.x, is.ns.y, is.ns.z, __int_as_float(is.material));
            qb.q2[slot] = make_float4(is.ng.x, is.ng.y, is.ng.z, __int_as_float(s.target));
            qb.q3[slot] = make_float4(w.x, w.y, w.z, 0.0f);
            qb.q4[slot] = make_float4(is.dir.x, is.dir.y, is.dir.z, __int_as_float(s.channel));
        }
    }
    if (s.len > P.max_path_length) return false;
    U4 bb = s.rng.block(2 + s.len);
    BsdfSample smp = b.sample(u01(bb.a), u01(bb.b), u01(bb.c), is.ng);
    if (is_zero(smp.f)) return false;
    F3 f = smp.f;
    if (s.len > kRRDepth) {
        if (u01(bb.d) > smp.cont) return false;
        f = div_each(f, smp.cont);
    }
    s.o = is.pos;
    s.d = smp.wi;
    s.tp = s.tp * f;
    if (smp.event & EV_SPECULAR) s.dVM *= (smp.cos_out / smp.fwd) * smp.rev;
    else s.dVM = (smp.cos_out / smp.fwd) * (1.0f + smp.rev * s.dVM);
    s.len++;
    return true;
}

template <int kBlock, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_camera_pass_persistent(const VMParams P, QueryBuf qb,
                                                                                unsigned long long* __restrict__ next_pixel) {
    CallStack stk;
    const int lane = threadIdx.x & 31;
    const long long npix = (long long)P.camera.width * P.camera.height;
    CameraPath s;
    bool alive = false;
    bool pool_left = true;
    while (true) {
        // refill as in the light pass: once kRefillLanes lanes are free (2.43 -> 2.35 ms on
        // the water pool), drawing again for samples that fall outside the buffer
        unsigned need = __ballot_sync(0xffffffffu, !alive);
        while (need && pool_left && (__popc(need) >= kRefillLanes || need == 0xffffffffu)) {
            unsigned long long base = 0;
            if (lane == __ffs(need) - 1) base = atomicAdd(next_pixel, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
            if (!alive) {
                const unsigned long long mine = base + __popc(need & ((1u << lane) - 1u));
                if (mine < (unsigned long long)npix) alive = camera_path_start(P, (long long)mine, s);
            }
            if (base + __popc(need) >= (unsigned long long)npix) pool_left = false;
            need = __ballot_sync(0xffffffffu, !alive);   // samples outside the buffer: draw again
        }
        if (!__any_sync(0xffffffffu, alive)) break;
        if (alive) alive = camera_path_bounce(P, qb, s, stk);
    }
}

// Batch passes: the persistent light and camera passes over the paths (pixels) of
// several resident scenes in one launch.  Work index g runs over the scenes' paths laid
// end to end (prefix[i] = first index of scene i, prefix[n] = total); a lane that takes
// index g finds its scene by binary search and runs that scene's path with the scene's
// own parameters and buffers (read from global memory: every lane of a warp that holds
// paths of one scene reads the same words).  Each path's samples, bounces and photons
// are those of the scene's own pass.
__device__ __forceinline__ int batch_scene_of(const long long* __restrict__ prefix, int n, long long g) {
    int lo = 0, hi = n - 1;   // the last scene whose range starts at or before g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&prefix[mid]) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int kBlock, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_light_pass_batch(const BatchScene* __restrict__ B,
                                                                         const long long* __restrict__ prefix, int n,
                                                                         unsigned long long* __restrict__ next_path) {
    CallStack stk;
    const int lane = threadIdx.x & 31;
    const unsigned long long total = (unsigned long long)__ldg(&prefix[n]);
    LightPath s;
    int sid = 0;
    bool alive = false;
    bool pool_left = true;
    while (true) {
        const unsigned need = __ballot_sync(0xffffffffu, !alive);
        if (need && pool_left && (__popc(need) >= kRefillLanes || need == 0xffffffffu)) {
            unsigned long long base = 0;
            if (lane == __ffs(need) - 1) base = atomicAdd(next_path, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
            if (!alive) {
                const unsigned long long mine = base + __popc(need & ((1u << lane) - 1u));
                if (mine < total) {
                    sid = batch_scene_of(prefix, n, (long long)mine);
                    const VMParams& P = B[sid].p;
                    const long long local = (long long)mine - __ldg(&prefix[sid]);
                    alive = light_path_start(P, P.path_order ? (long long)__ldg(&P.path_order[local]) : local, s);
                }
            }
            if (base + __popc(need) >= total) pool_left = false;
        }
        if (!__any_sync(0xffffffffu, alive)) break;
        if (alive) alive = light_path_bounce<true>(B[sid].p, B[sid].ph, s, stk);
    }
}

template <int kBlock, int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_camera_pass_batch(const BatchScene* __restrict__ B,
                                                                          const long long* __restrict__ prefix, int n,
                                                                          unsigned long long* __restrict__ next_pixel) {
    CallStack stk;
    const int lane = threadIdx.x & 31;
    const unsigned long long total = (unsigned long long)__ldg(&prefix[n]);
    CameraPath s;
    int sid = 0;
    bool alive = false;
    bool pool_left = true;
    while (true) {
        unsigned need = __ballot_sync(0xffffffffu, !alive);
        while (need && pool_left && (__popc(need) >= kRefillLanes || need == 0xffffffffu)) {
            unsigned long long base = 0;
            if (lane == __ffs(need) - 1) base = atomicAdd(next_pixel, (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
            if (!alive) {
                const unsigned long long mine = base + __popc(need & ((1u << lane) - 1u));
                if (mine < total) {
                    sid = batch_scene_of(prefix, n, (long long)mine);
                    alive = camera_path_start(B[sid].p, (long long)mine - __ldg(&prefix[sid]), s);
                }
            }
            if (base + __popc(need) >= total) pool_left = false;
            need = __ballot_sync(0xffffffffu, !alive);
        }
        if (!__any_sync(0xffffffffu, alive)) break;
        if (alive) alive = camera_path_bounce<true>(B[sid].p, B[sid].qb, s, stk);
    }
}

// Stack: CallStack (the persistent passes' traversal: children tested at the parent),
// WarpStepStack (the wavefront pass's warp-stepped one) or LocalStack (pop-and-test, the
// reference's own form).
template <class Stack>
__global__ void k_trace_rays(const SceneView S, int n, const float* __restrict__ o, const float* __restrict__ d,
                             float tmin, float* out_full, unsigned* out_words, int* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    F3 ro = f3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    F3 rd = f3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    HitRec h;
    Stack stk;
    bool hit = scene_hit(S, ro, rd, tmin, h, err, stk);
    Isect is;
    if (hit) fill_isect(S, h, ro, rd, is);
    if (out_words) {
        unsigned* w = out_words + 8 * i;
        w[0] = hit ? 1u : 0u;
        w[1] = __float_as_uint(h.t);
        w[2] = __float_as_uint(h.u);
        w[3] = __float_as_uint(h.v);
        w[4] = hit ? (unsigned)is.tri : 0xffffffffu;
        w[5] = hit ? (unsigned)is.material : 0xffffffffu;
        w[6] = hit ? (unsigned)is.mesh : 0xffffffffu;
        w[7] = 0u;
    }
    if (out_full) {
        float* f = out_full + 16 * i;
        f[0] = hit ? 1.0f : 0.0f;
        f[1] = h.t; f[2] = h.u; f[3] = h.v;
        if (hit) {
            f[4] = is.ng.x; f[5] = is.ng.y; f[6] = is.ng.z;
            f[7] = is.ns.x; f[8] = is.ns.y; f[9] = is.ns.z;
            f[10] = is.pos.x; f[11] = is.pos.y; f[12] = is.pos.z;
            f[13] = is.front ? 1.0f : 0.0f;
            f[14] = (float)is.material;
            f[15] = __int_as_float(is.tri);
        } else {
            for (int k = 4; k < 16; ++k) f[k] = 0.0f;
            f[14] = -1.0f;
            f[15] = __int_as_float(-1);
        }
    }
}

// Persistent grid for one shape: resident blocks per SM (occupancy with its dynamic
// shared memory) x SMs, capped by the work.
template <class K>
unsigned persistent_grid(K kernel, int block, size_t smem, long long work_items) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    const long long blocks = (long long)sms * (per_sm > 0 ? per_sm : 1);
    const long long need = (work_items + block - 1) / block;
    return (unsigned)(need < blocks ? need : blocks);
}

template <int B, int MB>
void launch_light_t(const VMParams& p, PhotonBuf ph, unsigned long long* next_path, unsigned long long* rays,
                    cudaStream_t s) {
    // per host thread: contexts on different threads launch concurrently
    static thread_local unsigned grid_cache = 0;
    static thread_local long long grid_for = -1;
    if (grid_for != p.num_light_paths) {
        grid_cache = persistent_grid(k_light_pass_persistent<B, MB>, B, 0, p.num_light_paths);
        grid_for = p.num_light_paths;
    }
    cudaMemsetAsync(next_path, 0, sizeof(unsigned long long), s);
    if (rays) cudaMemsetAsync(rays, 0, sizeof(unsigned long long), s);
    k_light_pass_persistent<B, MB><<<grid_cache, B, 0, s>>>(p, ph, next_path, rays);
}

template <int B, int MB>
void launch_camera_t(const VMParams& p, QueryBuf qb, unsigned long long* next_pixel, cudaStream_t s) {
    const long long n = (long long)p.camera.width * p.camera.height;
    // per host thread: contexts on different threads launch concurrently
    static thread_local unsigned grid_cache = 0;
    static thread_local long long grid_for = -1;
    if (grid_for != n) {
        grid_cache = persistent_grid(k_camera_pass_persistent<B, MB>, B, 0, n);
        grid_for = n;
    }
    cudaMemsetAsync(next_pixel, 0, sizeof(unsigned long long), s);
    k_camera_pass_persistent<B, MB><<<grid_cache, B, 0, s>>>(p, qb, next_pixel);
}

template <int B, int MB>
void launch_light_batch_t(const BatchScene* scenes, const long long* prefix, int n, long long total,
                          unsigned long long* next, cudaStream_t s) {
    static thread_local unsigned grid_cache = 0;
    static thread_local long long grid_for = -1;
    if (grid_for != total) {
        grid_cache = persistent_grid(k_light_pass_batch<B, MB>, B, 0, total);
        grid_for = total;
    }
    cudaMemsetAsync(next, 0, sizeof(unsigned long long), s);
    k_light_pass_batch<B, MB><<<grid_cache, B, 0, s>>>(scenes, prefix, n, next);
}

template <int B, int MB>
void launch_camera_batch_t(const BatchScene* scenes, const long long* prefix, int n, long long total,
                           unsigned long long* next, cudaStream_t s) {
    static thread_local unsigned grid_cache = 0;
    static thread_local long long grid_for = -1;
    if (grid_for != total) {
        grid_cache = persistent_grid(k_camera_pass_batch<B, MB>, B, 0, total);
        grid_for = total;
    }
    cudaMemsetAsync(next, 0, sizeof(unsigned long long), s);
    k_camera_pass_batch<B, MB><<<grid_cache, B, 0, s>>>(scenes, prefix, n, next);
}

}  // namespace

size_t light_order_scratch_bytes(long long n) {
    return 4 * (size_t)(n > 0 ? n : 1) + 4 * (size_t)kOrderCells + 4 * scan_scratch_words(kOrderCells) + 512;
}

void launch_light_order(const VMParams& p, void* scratch, uint32_t* order, cudaStream_t s) {
    const long long n = p.num_light_paths;
    if (n <= 0) return;
    uint32_t* keys = static_cast<uint32_t*>(scratch);
    uint32_t* counts = keys + ((n + 63) & ~63LL);
    cudaMemsetAsync(counts, 0, 4 * (size_t)kOrderCells, s);
    const unsigned g = (unsigned)((n + 255) / 256);
    k_light_keys<<<g, 256, 0, s>>>(p, keys, counts);
    launch_scan_counts(counts, kOrderCells, counts + kOrderCells, s);
    k_light_scatter<<<g, 256, 0, s>>>(keys, n, counts, order);
}

size_t light_wavefront_scratch_bytes(long long n) {
    const size_t m = (size_t)(n > 0 ? n : 1);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    return al(16 * m) * 4 + al(8 * m) + al(16 * m) + 2 * al(4 * m) + 256;
}

void launch_light_wavefront(const VMParams& p, PhotonBuf ph, void* scratch, cudaStream_t s, cudaEvent_t tail) {
    const long long n = p.num_light_paths;
    if (n <= 0) return;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char* c = static_cast<char*>(scratch);
    WfState W;
    W.o4 = (float4*)c; c += al(16 * (size_t)n);
    W.d4 = (float4*)c; c += al(16 * (size_t)n);
    W.m4 = (int4*)c; c += al(16 * (size_t)n);
    W.hit = (float4*)c; c += al(16 * (size_t)n);
    W.t2 = (float2*)c; c += al(8 * (size_t)n);
    W.queue[0] = (uint32_t*)c; c += al(4 * (size_t)n);
    W.queue[1] = (uint32_t*)c; c += al(4 * (size_t)n);
    W.count = (unsigned long long*)c;
    cudaMemsetAsync(W.count, 0, 2 * sizeof(unsigned long long), s);
    k_wf_start<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, W);
    static thread_local unsigned trace_grid = 0, shade_grid = 0, finish_grid = 0;
    if (!trace_grid) {
        trace_grid = persistent_grid(k_wf_trace<8>, 128, 0, 1LL << 40);
        shade_grid = persistent_grid(k_wf_shade, 128, 0, 1LL << 40);
        finish_grid = persistent_grid(k_wf_finish, 128, 0, 1LL << 40);
    }
    // a bounce per round for the first kWavefrontRounds bounces (most paths end by then),
    // then one launch finishes the rest
    constexpr int kWavefrontRounds = 4;
    int q = 0;
    for (int b = 0; b < kWavefrontRounds; ++b, q ^= 1) {
        k_wf_trace<8><<<trace_grid, 128, 0, s>>>(p, W, q);
        cudaMemsetAsync(W.count + (q ^ 1), 0, sizeof(unsigned long long), s);
        k_wf_shade<<<shade_grid, 128, 0, s>>>(p, ph, W, q);
    }
    if (tail) cudaEventRecord(tail, s);
    k_wf_finish<<<finish_grid, 128, 0, s>>>(p, ph, W, q);
}

int pass_variants() { return 6; }

const char* pass_variant_name(int v) {
    static const char* names[6] = {"256 threads, >= 3 blocks/SM (<= 85 registers)",
                                   "128 threads, >= 7 blocks/SM (<= 73 registers)",
                                   "128 threads, >= 8 blocks/SM (<= 64 registers)",
                                   "128 threads, >= 5 blocks/SM (<= 102 registers)",
                                   "128 threads, >= 10 blocks/SM (<= 51 registers)",
                                   "128 threads, >= 9 blocks/SM (<= 56 registers)"};
    if (v == 6) return "wavefront: closest-hit and shading kernels per bounce";
    return (v >= 0 && v < 6) ? names[v] : "?";
}

void launch_light_pass(const VMParams& p, PhotonBuf ph, unsigned long long* next_path, cudaStream_t s, int variant,
                       unsigned long long* rays) {
    long long n = p.num_light_paths;
    if (n <= 0) return;
    if (!next_path) return;
    switch (variant) {
    case 1: launch_light_t<128, 7>(p, ph, next_path, rays, s); break;
    case 2: launch_light_t<128, 8>(p, ph, next_path, rays, s); break;
    case 3: launch_light_t<128, 5>(p, ph, next_path, rays, s); break;
    case 4: launch_light_t<128, 10>(p, ph, next_path, rays, s); break;
    case 5: launch_light_t<128, 9>(p, ph, next_path, rays, s); break;
    default: launch_light_t<256, 3>(p, ph, next_path, rays, s); break;
    }
}

void launch_camera_pass(const VMParams& p, QueryBuf qb, unsigned long long* next_pixel, cudaStream_t s, int variant) {
    long long n = (long long)p.camera.width * p.camera.height;
    if (n <= 0) return;
    if (!next_pixel) return;
    switch (variant) {
    case 1: launch_camera_t<128, 7>(p, qb, next_pixel, s); break;
    case 2: launch_camera_t<128, 8>(p, qb, next_pixel, s); break;
    case 3: launch_camera_t<128, 5>(p, qb, next_pixel, s); break;
    case 4: launch_camera_t<128, 10>(p, qb, next_pixel, s); break;
    case 5: launch_camera_t<128, 9>(p, qb, next_pixel, s); break;
    default: launch_camera_t<256, 3>(p, qb, next_pixel, s); break;
    }
}

void launch_light_pass_batch(const BatchScene* scenes, const long long* path_prefix, int n, long long total_paths,
                             unsigned long long* next_path, cudaStream_t s, int variant) {
    if (n <= 0 || total_paths <= 0 || !next_path) return;
    switch (variant) {
    case 1: launch_light_batch_t<128, 7>(scenes, path_prefix, n, total_paths, next_path, s); break;
    case 2: launch_light_batch_t<128, 8>(scenes, path_prefix, n, total_paths, next_path, s); break;
    case 3: launch_light_batch_t<128, 5>(scenes, path_prefix, n, total_paths, next_path, s); break;
    case 4: launch_light_batch_t<128, 10>(scenes, path_prefix, n, total_paths, next_path, s); break;
    case 5: launch_light_batch_t<128, 9>(scenes, path_prefix, n, total_paths, next_path, s); break;
    default: launch_light_batch_t<256, 3>(scenes, path_prefix, n, total_paths, next_path, s); break;
    }
}

void launch_camera_pass_batch(const BatchScene* scenes, const long long* pixel_prefix, int n, long long total_pixels,
                              unsigned long long* next_pixel, cudaStream_t s, int variant) {
    if (n <= 0 || total_pixels <= 0 || !next_pixel) return;
    switch (variant) {
    case 1: launch_camera_batch_t<128, 7>(scenes, pixel_prefix, n, total_pixels, next_pixel, s); break;
    case 2: launch_camera_batch_t<128, 8>(scenes, pixel_prefix, n, total_pixels, next_pixel, s); break;
    case 3: launch_camera_batch_t<128, 5>(scenes, pixel_prefix, n, total_pixels, next_pixel, s); break;
    case 4: launch_camera_batch_t<128, 10>(scenes, pixel_prefix, n, total_pixels, next_pixel, s); break;
    case 5: launch_camera_batch_t<128, 9>(scenes, pixel_prefix, n, total_pixels, next_pixel, s); break;
    default: launch_camera_batch_t<256, 3>(scenes, pixel_prefix, n, total_pixels, next_pixel, s); break;
    }
}

// Debug views (src/Debug_scene.cpp:21-214, dispatched by src/main.cpp:172-180): one
// unjittered primary ray per pixel corner, closest hit with tmin 1e-4 from the camera
// origin, the colour added to the pixel Image_Buffer::add_color picks (row 0 dropped).
__global__ void __launch_bounds__(256) k_debug_view(const VMParams P, int mode, float ior, double* accum) {
    const long long pix = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int W = P.camera.width, H = P.camera.height;
    if (pix >= (long long)W * H) return;
    const float x = (float)(int)(pix % W);
    const float y = (float)(int)(pix / W);
    F3 dir = ld3(P.camera.bottom_left) + ld3(P.camera.horizontal) * (x / (float)W) +
             ld3(P.camera.vertical) * (y / (float)H);
    dir = dir - ld3(P.camera.origin);
    const F3 o = ld3(P.camera.origin);
    const F3 d = normalize(dir);
    HitRec h;
    if (!scene_hit(P.scene, o, d, 0.0001f, h, P.error + ERR_STACK)) return;
    Isect is;
    fill_isect(P.scene, h, o, d, is);
    F3 c;
    if (mode == 2) {
        c = is.ns;                                            // run_debug_normals
    } else if (mode == 3) {                                   // run_debug_facing
        const F3 base = is.front ? f3(0.0f, 0.0f, 1.0f) : f3(1.0f, 0.0f, 0.0f);
        c = base * fabsf(dot(d, is.ns));
    } else {                                                  // run_debug_materials
        Frame fr;
        fr.set_from_z(is.ns);
        const F3 dl = fr.to_local(-is.dir);
        float eta = ior;
        if (dl.z > 0.0f) eta = 1.0f / ior;
        c = f3(fresnel_eta(fabsf(dl.z), eta));
    }
    const int X = (int)x, Y = H - (int)y;
    const long long target = (long long)X + (long long)Y * W;
    if (target > (long long)W * H - 1) return;
    accum[3 * target] += (double)c.x;
    accum[3 * target + 1] += (double)c.y;
    accum[3 * target + 2] += (double)c.z;
}

void launch_debug_view(const VMParams& p, int mode, float ior, double* accum, cudaStream_t s) {
    const long long n = (long long)p.camera.width * p.camera.height;
    if (n <= 0) return;
    k_debug_view<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, mode, ior, accum);
}

// Running FP64 sum -> FP32 mean image (Vertex_Merging::run's final scale,
// src/Vertex_Merging.cpp:367-379, done at readback).
__global__ void k_image_mean(const double* __restrict__ acc, float* __restrict__ out, long long n, double scale) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)(acc[i] * scale);
}

void launch_image_mean(const double* acc, float* out, long long n, double scale, cudaStream_t s) {
    if (n <= 0) return;
    k_image_mean<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(acc, out, n, scale);
}

__global__ void k_pad_photons(float4* __restrict__ pos, const unsigned long long* __restrict__ count, long long cap,
                              float4 pad) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= cap || (unsigned long long)i < *count) return;
    pos[i] = pad;
}

__global__ void k_check_counts(const unsigned long long* photons, long long pcap, const unsigned long long* queries,
                               long long qcap, int* flag) {
    *flag = (*photons > (unsigned long long)pcap || *queries > (unsigned long long)qcap) ? 1 : 0;
}

void launch_pad_photons(float4* pos, const unsigned long long* count, long long capacity, float4 pad, cudaStream_t s) {
    if (capacity <= 0) return;
    k_pad_photons<<<(unsigned)((capacity + 255) / 256), 256, 0, s>>>(pos, count, capacity, pad);
}

void launch_check_counts(const unsigned long long* photons, long long photon_cap, const unsigned long long* queries,
                         long long query_cap, int* flag, cudaStream_t s) {
    k_check_counts<<<1, 1, 0, s>>>(photons, photon_cap, queries, query_cap, flag);
}

void launch_trace_rays(const SceneView& sv, int n, const float* o, const float* d, float tmin, float* out_full,
                       unsigned* out_words, int* err, cudaStream_t st, int shape) {
    if (n <= 0) return;
    if (shape == 1)
        k_trace_rays<WarpStepStack><<<(n + 127) / 128, 128, 0, st>>>(sv, n, o, d, tmin, out_full, out_words, err);
    else if (shape == 2)
        k_trace_rays<LocalStack><<<(n + 127) / 128, 128, 0, st>>>(sv, n, o, d, tmin, out_full, out_words, err);
    else
        k_trace_rays<CallStack><<<(n + 127) / 128, 128, 0, st>>>(sv, n, o, d, tmin, out_full, out_words, err);
}

}  // namespace rc
