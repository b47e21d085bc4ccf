// Radius gather at the camera vertices (Path_Vertices::get_contrib,
// src/Path_Vertices.h:46-68, over KD_Tree::find_closest_in_radius,
// src/KD_Tree.cpp:217-280).
//
// The photons the reference's query returns for a camera vertex q are exactly
// { p : ((dx*dx + dy*dy) + dz*dz) < r^2 } in FP32 without contraction: its descent
// prunes a side only when (q[axis] - split)^2 >= r^2, and every photon beyond that
// plane has a squared distance at least as large (rounding is monotonic), so pruning
// never drops a photon the predicate accepts.  The set does not depend on the tree's
// shape, so the gather may walk the photons in any order, as long as it skips only
// boxes that provably hold no accepted photon and tests every other photon with the
// reference's predicate.
//
// Layout (launch_kd_boxes).  The photons in tree order are cut into 2^Lc chunks, Lc
// being the shallowest level whose nodes hold at most 31 photons: chunk i is node
// (2^Lc + i)'s contiguous range plus the gap before the next chunk's range, which holds
// at most one inner node's median photon (that of the two nodes' lowest common
// ancestor), so a chunk holds at most 32 photons.  Each chunk has its photons' bounding
// box, with its first position and count in the spare .w words; every node above has
// the union of its children's boxes.
//
// Work split (k_gather).  Queries are sorted by Morton code (launch_query_order) and a
// warp owns G consecutive ones (a group), one per lane.  The warp descends the box hierarchy
// once for the whole group, E levels per step (lane j tests descendant j's box against
// the group's bounding box grown by the radius), down to the candidate chunks.  At a
// chunk each lane tests its own query's sphere against the chunk box (a ballot names the
// overlapping queries), each lane loads one of the chunk's photons, and for every
// overlapping query the warp tests all of the chunk's photons at once: a query x photon
// cross product, one photon per lane, the query broadcast from shared memory.  Accepted
// (query slot, photon) pairs collect in a per-warp pending list, and every 32 of them
// go to the sink with all lanes busy.  The render's sink evaluates the merges (the
// camera vertex's BSDF at the photon's direction, MIS weight, photon throughput) from
// per-query BSDF state staged in shared memory when the group starts, sums them per
// query in shared memory, and adds each query's sum into its FP64 pixel once.  The
// parity hook's sink records photon ids instead; both are the same kernel template.
#include "vm.cuh"
#include "bsdf.cuh"

namespace rc {

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr long long kChunkNode = 31;   // photons per chunk-level node (the chunk adds at most one median)
// DFS stack of subtree roots per warp.  Lc <= 24 for n < 2^28 photons, so a path from
// the root crosses at most ceil(24 / E) expansion steps, the last of which reaches the
// chunks (processed at once, never pushed): at most 4 x 31 + 1 = 125 (E = 5) or
// 5 x 15 + 1 = 76 (E = 4) pending roots.
constexpr int kRootStack = 128;
constexpr unsigned kFull = 0xffffffffu;

struct ChunkTree {
    const float4* __restrict__ lo;    // node boxes, heap order, levels [0, lc]; chunk level: .w = first position
    const float4* __restrict__ hi;    //                                          chunk level: .w = photon count
    const float4* __restrict__ pos;   // photon positions in tree order (TreePhotons::t0)
    int lc;                           // chunk level (-1: no photons)
};

// Squared distance from q to a box, formed like the acceptance test, so that it never
// exceeds the squared distance to any photon inside the box (rounding is monotonic).
__device__ __forceinline__ bool box_outside(F3 q, float4 lo, float4 hi, float r2) {
    const float dx = q.x < lo.x ? lo.x - q.x : (q.x > hi.x ? q.x - hi.x : 0.0f);
    const float dy = q.y < lo.y ? lo.y - q.y : (q.y > hi.y ? q.y - hi.y : 0.0f);
    const float dz = q.z < lo.z ? lo.z - q.z : (q.z > hi.z ? q.z - hi.z : 0.0f);
    return !(dx * dx + dy * dy + dz * dz < r2);
}

// The same bound between two boxes: never more than the squared distance from any
// point of the first (a query of the group) to any point of the second (a photon).
__device__ __forceinline__ bool gap_outside(float4 glo, float4 ghi, float4 lo, float4 hi, float r2) {
    const float dx = lo.x > ghi.x ? lo.x - ghi.x : (glo.x > hi.x ? glo.x - hi.x : 0.0f);
    const float dy = lo.y > ghi.y ? lo.y - ghi.y : (glo.y > hi.y ? glo.y - hi.y : 0.0f);
    const float dz = lo.z > ghi.z ? lo.z - ghi.z : (glo.z > hi.z ? glo.z - hi.z : 0.0f);
    return !(dx * dx + dy * dy + dz * dz < r2);
}

// Bounding box of the queries of the lanes with `in` set (all lanes call it).
__device__ __forceinline__ void warp_box(bool in, F3 q, float4& lo, float4& hi) {
    float lx = in ? q.x : INFINITY, ly = in ? q.y : INFINITY, lz = in ? q.z : INFINITY;
    float hx = in ? q.x : -INFINITY, hy = in ? q.y : -INFINITY, hz = in ? q.z : -INFINITY;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o)); ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
        lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o)); hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o)); hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
    }
    lo = make_float4(lx, ly, lz, 0.0f);
    hi = make_float4(hx, hy, hz, 0.0f);
}

// Lane holding the largest value (the lowest such lane on ties).
__device__ __forceinline__ int warp_argmax(float v) {
    int at = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oa = __shfl_xor_sync(0xffffffffu, at, o);
        if (ov > v || (ov == v && oa < at)) { v = ov; at = oa; }
    }
    return at;
}

// Surface of a box grown by `g` on every side (a proxy for how many chunk boxes it meets).
__device__ __forceinline__ float box_surface(float4 lo, float4 hi, float g) {
    const float ex = hi.x - lo.x + 2.0f * g, ey = hi.y - lo.y + 2.0f * g, ez = hi.z - lo.z + 2.0f * g;
    return ex * ey + ey * ez + ex * ez;
}

// The reference's acceptance test (src/KD_Tree.cpp:217-280): ((dx*dx + dy*dy) + dz*dz) < r2.
__device__ __forceinline__ bool in_radius(F3 q, float px, float py, float pz, float r2) {
    const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
    return dx * dx + dy * dy + dz * dz < r2;
}

// Camera-vertex state a merge evaluation needs, staged once per query.  29 words: an
// odd stride, so lanes reading different queries' fields hit different banks.
struct QState {
    int kind;
    float R[3], ior, a2, s;
    float fx[3], fy[3], fz[3];   // shading frame
    float wo[3];                 // local direction towards the previous camera vertex
    float ng[3];
    float wo_ng, fwo, dvm;       // dot(to_world(wo), Ng), plastic Fresnel at wo, camera dVM
    float tp[3];                 // camera throughput x VM normalisation
    float pad;
};
static_assert(sizeof(QState) == 29 * 4, "QState must keep an odd word stride");

template <bool Eval> struct GroupExtra {};
template <> struct GroupExtra<true> {
    QState qs[32];
    float acc[32][3];            // per-query merge sums (word stride 3: conflict-free)
};

template <bool Eval> struct WarpSmem {
    float4 qp[32];               // query positions (broadcast in the cross product)
    uint32_t qidx[32];           // query indices of the group's slots
    uint32_t pend_pos[64];       // accepted pairs: tree position ...
    uint8_t pend_slot[64];       // ... and query slot
    uint32_t stk[kRootStack];
    GroupExtra<Eval> g;
};

// The render's sink: merge evaluation (Path_Vertices::get_contrib, src/Path_Vertices.h:46-68)
// and FP64 pixel accumulation.
struct EvalSink {
    static constexpr bool kEval = true;
    VMParams P;
    QueryBuf qb;
    TreePhotons tp;
    const uint32_t* tree_id;
    double* accum;

    __device__ __forceinline__ void setup(WarpSmem<true>& sm, int lane, bool active, uint32_t qi) const {
        if (active) {
            const float dvm = qb.q0[qi].w;
            const float4 b = qb.q1[qi], c = qb.q2[qi], e = qb.q4[qi], g = qb.q3[qi];
            const DevMaterial& qm = P.materials[__float_as_int(b.w)];
            const int channel = __float_as_int(e.w);   // the camera path's dispersion channel
            Bsdf bs;
            bs.init(qm, xyz(b), xyz(e), true, (qm.disp > 0.0f && channel >= 0) ? (float)(channel - 1) * qm.disp : 0.0f);
            QState& st = sm.g.qs[lane];
            st.kind = bs.kind;
            st.R[0] = bs.R.x; st.R[1] = bs.R.y; st.R[2] = bs.R.z;
            st.ior = bs.ior; st.a2 = bs.a2; st.s = bs.s;
            st.fx[0] = bs.fr.x.x; st.fx[1] = bs.fr.x.y; st.fx[2] = bs.fr.x.z;
            st.fy[0] = bs.fr.y.x; st.fy[1] = bs.fr.y.y; st.fy[2] = bs.fr.y.z;
            st.fz[0] = bs.fr.z.x; st.fz[1] = bs.fr.z.y; st.fz[2] = bs.fr.z.z;
            st.wo[0] = bs.wo.x; st.wo[1] = bs.wo.y; st.wo[2] = bs.wo.z;
            st.ng[0] = c.x; st.ng[1] = c.y; st.ng[2] = c.z;
            st.wo_ng = dot(bs.fr.to_world(bs.wo), xyz(c));
            st.fwo = (bs.kind == BSDF_K_PLASTIC_GGX || bs.kind == BSDF_K_PLASTIC_SMOOTH)
                         ? fresnel_reflectance(fabsf(bs.wo.z), bs.s) : 0.0f;
            st.dvm = dvm;
            st.tp[0] = g.x * P.merge_scale; st.tp[1] = g.y * P.merge_scale; st.tp[2] = g.z * P.merge_scale;
        }
        sm.g.acc[lane][0] = 0.0f; sm.g.acc[lane][1] = 0.0f; sm.g.acc[lane][2] = 0.0f;
    }

    // Evaluate the first `count` pending pairs (lane j: pair j); sum each run of one
    // query's pairs across the lanes and add it to that query's shared sum.
    __device__ __forceinline__ void flush(WarpSmem<true>& sm, int lane, int count) const {
        F3 c = f3(0.0f);
        int s = -1;
        if (lane < count) {
            const uint32_t p = sm.pend_pos[lane];
            s = sm.pend_slot[lane];
            const QState& st = sm.g.qs[s];
            Bsdf bs;
            bs.kind = st.kind;
            bs.R = f3(st.R[0], st.R[1], st.R[2]);
            bs.ior = st.ior; bs.a2 = st.a2; bs.s = st.s; bs.cont = 0.0f;
            bs.fr.x = f3(st.fx[0], st.fx[1], st.fx[2]);
            bs.fr.y = f3(st.fy[0], st.fy[1], st.fy[2]);
            bs.fr.z = f3(st.fz[0], st.fz[1], st.fz[2]);
            bs.wo = f3(st.wo[0], st.wo[1], st.wo[2]);
            bs.radiance = true;
            const float4 p0 = __ldg(&tp.t0[p]);
            const float4 p1 = __ldg(&tp.t1[p]);
            const float2 p2 = __ldg(&tp.t2[p]);
            F3 ev;
            float fwd, rev;
            bs.eval_pdf(xyz(p1), f3(st.ng[0], st.ng[1], st.ng[2]), st.wo_ng, st.fwo, ev, fwd, rev);
            const float weight = 1.0f / (1.0f + st.dvm * rev + p0.w * fwd);
            c = ev * f3(p1.w, p2.x, p2.y) * weight;
            if (P.path_contrib) {
                // learned-proposal training signal: the squared luminance this merge adds
                // to its pixel, summed per light path
                const F3 img = f3(st.tp[0], st.tp[1], st.tp[2]) * c;
                const float lum = (fabsf(img.x) + fabsf(img.y) + fabsf(img.z)) * (1.0f / 3.0f);
                if (lum > 0.0f) atomicAdd(&P.path_contrib[__ldg(&P.photon_path[__ldg(&tree_id[p])])], lum * lum);
            }
        }
        // runs of equal slot, numbered by their heads (one query can form two runs in a
        // flush: its pairs from two chunks with another query's between them)
        const int sprev = __shfl_up_sync(kFull, s, 1);
        const unsigned heads = __ballot_sync(kFull, lane == 0 || sprev != s);
        const int run = __popc(heads & ((2u << lane) - 1u));
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float x = __shfl_up_sync(kFull, c.x, o);
            const float y = __shfl_up_sync(kFull, c.y, o);
            const float z = __shfl_up_sync(kFull, c.z, o);
            const int ro = __shfl_up_sync(kFull, run, o);
            if (lane >= o && ro == run) { c.x += x; c.y += y; c.z += z; }
        }
        const int snext = __shfl_down_sync(kFull, s, 1);
        if (s >= 0 && (lane == 31 || snext != s) && !is_zero(c)) {
            atomicAdd(&sm.g.acc[s][0], c.x);
            atomicAdd(&sm.g.acc[s][1], c.y);
            atomicAdd(&sm.g.acc[s][2], c.z);
        }
    }

    __device__ __forceinline__ void finish(WarpSmem<true>& sm, int lane, bool active, uint32_t qi) const {
        if (!active) return;
        const QState& st = sm.g.qs[lane];
        const F3 r = f3(st.tp[0], st.tp[1], st.tp[2]) * f3(sm.g.acc[lane][0], sm.g.acc[lane][1], sm.g.acc[lane][2]);
        if (is_zero(r)) return;
        const long long pixel = __float_as_int(qb.q2[qi].w);
        atomicAdd(&accum[3 * pixel + 0], (double)r.x);
        atomicAdd(&accum[3 * pixel + 1], (double)r.y);
        atomicAdd(&accum[3 * pixel + 2], (double)r.z);
    }
};

// The parity hook's sink: per query, the ids of the photons it accepts.  Without
// `offsets` it counts (counts[] zeroed by the caller), with them it writes the ids at
// offsets[q] + cursor[q]++ (cursor zeroed by the caller).
struct SetSink {
    static constexpr bool kEval = false;
    const uint32_t* tree_id;
    int* counts;
    const long long* offsets;
    int* cursor;
    int* idx;

    __device__ __forceinline__ void setup(WarpSmem<false>&, int, bool, uint32_t) const {}
    __device__ __forceinline__ void flush(WarpSmem<false>& sm, int lane, int count) const {
        if (lane >= count) return;
        const uint32_t qi = sm.qidx[sm.pend_slot[lane]];
        const uint32_t p = sm.pend_pos[lane];
        if (!offsets) atomicAdd(&counts[qi], 1);
        else idx[offsets[qi] + atomicAdd(&cursor[qi], 1)] = (int)__ldg(&tree_id[p]);
    }
    __device__ __forceinline__ void finish(WarpSmem<false>&, int, bool, uint32_t) const {}
};

// One group of G queries per warp.  MinBlocks (resident blocks per SM the register
// allocation must allow), G and E (levels per expansion step) are the launch shape the
// autotuner picks.  counters (optional, 4 u64 accumulated): accepted pairs, photon
// tests (chunk photons x overlapping queries), chunks tested, boxes tested.
template <int MinBlocks, int G, int E, class Sink>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, MinBlocks)
    k_gather(const ChunkTree t, const float* __restrict__ qpos, int qstride, const uint32_t* __restrict__ order,
             long long nq, const unsigned long long* __restrict__ nq_dev, const int* __restrict__ skip, float r2,
             const Sink sink, unsigned long long* __restrict__ counters, int* __restrict__ err) {
    static_assert(G == 16 || G == 32, "a group is a half or a whole warp of queries");
    static_assert(E >= 1 && E <= 5, "an expansion step tests at most 32 descendants");
    // device-side count (bounded by the capacity nq) and an iteration-wide skip flag,
    // for iterations enqueued without a host round trip
    if (skip && *skip) return;
    if (nq_dev) nq = (long long)min(*nq_dev, (unsigned long long)nq);
    __shared__ WarpSmem<Sink::kEval> smem[kWarpsPerBlock];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long first = ((long long)blockIdx.x * kWarpsPerBlock + warp) * G;
    if (first >= nq || t.lc < 0) return;
    WarpSmem<Sink::kEval>& sm = smem[warp];
    const int nslots = (int)min((long long)G, nq - first);
    const bool active = lane < nslots;
    const unsigned lt = (1u << lane) - 1u;
    uint32_t qi = 0;
    F3 q = f3(0.0f);
    if (active) {
        qi = __ldg(&order[first + lane]);
        const float* qp = qpos + (long long)qstride * qi;
        q = f3(qp[0], qp[1], qp[2]);
        sm.qidx[lane] = qi;
        sm.qp[lane] = make_float4(q.x, q.y, q.z, 0.0f);
    }
    sink.setup(sm, lane, active, qi);
    __syncwarp();
    // The group is traversed as one or more sub-groups (lane ranges [a, b) of the sorted
    // queries, `in` = this lane's query belongs to the current one, glo/ghi its box).
    bool in = false;
    float4 glo, ghi;

    int np = 0;
    unsigned n_acc = 0, n_tests = 0, n_chunks = 0, n_boxes = 0;

    // Append one chunk's accepted pairs: this lane's photon (tree position p) is accepted
    // by the queries whose bits are set in `am`.  Pairs go in query by query (runs of one
    // query), every 32 to the sink.
    auto emit = [&](uint32_t am, uint32_t p) {
        unsigned qa = __reduce_or_sync(kFull, am);
        while (qa) {
            const int s = __ffs(qa) - 1;
            qa &= qa - 1u;
            const bool acc = (am >> s) & 1u;
            const unsigned m = __ballot_sync(kFull, acc);
            if (acc) {
                const int at = np + __popc(m & lt);
                sm.pend_pos[at] = p;
                sm.pend_slot[at] = (uint8_t)s;
            }
            np += __popc(m);
            __syncwarp();
            if (np >= 32) {
                sink.flush(sm, lane, 32);
                n_acc += 32;
                __syncwarp();
                const int rest = np - 32;
                uint32_t vp = 0;
                uint8_t vs = 0;
                if (lane < rest) { vp = sm.pend_pos[32 + lane]; vs = sm.pend_slot[32 + lane]; }
                __syncwarp();
                if (lane < rest) { sm.pend_pos[lane] = vp; sm.pend_slot[lane] = vs; }
                np = rest;
                __syncwarp();
            }
        }
    };

    // The candidate chunks of one expansion step: lane j holds chunk j's box (blo, bhi;
    // .w = first position, count) and bm names the chunks that met the group box.  First
    // each candidate's mask of the group's queries whose sphere meets its box (kept by
    // lane j), then the photon tests chunk by chunk, the next chunk's photons loaded
    // while the current one's are tested; the queries of a chunk are tested two at a
    // time into a per-photon mask of accepting queries.
    auto chunks = [&](unsigned bm, float4 blo, float4 bhi) {
        uint32_t my_qm = 0;
        while (bm) {
            const int j = __ffs(bm) - 1;
            bm &= bm - 1u;
            const float4 lo = make_float4(__shfl_sync(kFull, blo.x, j), __shfl_sync(kFull, blo.y, j),
                                          __shfl_sync(kFull, blo.z, j), 0.0f);
            const float4 hi = make_float4(__shfl_sync(kFull, bhi.x, j), __shfl_sync(kFull, bhi.y, j),
                                          __shfl_sync(kFull, bhi.z, j), 0.0f);
            const unsigned qm = __ballot_sync(kFull, in && !box_outside(q, lo, hi, r2));
            if (lane == j) my_qm = qm;
        }
        unsigned cm = __ballot_sync(kFull, my_qm != 0u);
        if (!cm) return;
        int j = __ffs(cm) - 1;
        uint32_t start = __shfl_sync(kFull, __float_as_uint(blo.w), j);
        uint32_t cnt = __shfl_sync(kFull, __float_as_uint(bhi.w), j);
        float4 pp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if ((uint32_t)lane < cnt) pp = __ldg(&t.pos[start + lane]);
        for (;;) {
            const uint32_t qm = __shfl_sync(kFull, my_qm, j);
            cm &= cm - 1u;
            int jn = 0;
            uint32_t sn = 0, cn = 0;
            float4 pn = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (cm) {
                jn = __ffs(cm) - 1;
                sn = __shfl_sync(kFull, __float_as_uint(blo.w), jn);
                cn = __shfl_sync(kFull, __float_as_uint(bhi.w), jn);
                if ((uint32_t)lane < cn) pn = __ldg(&t.pos[sn + lane]);
            }
            ++n_chunks;
            n_tests += cnt * (unsigned)__popc(qm);
            uint32_t am = 0, qq = qm;
            while (qq) {
                const int s0 = __ffs(qq) - 1;
                qq &= qq - 1u;
                const int s1 = qq ? __ffs(qq) - 1 : s0;
                qq &= qq - 1u;
                const float4 a = sm.qp[s0], b = sm.qp[s1];
                if (in_radius(xyz(a), pp.x, pp.y, pp.z, r2)) am |= 1u << s0;
                if (in_radius(xyz(b), pp.x, pp.y, pp.z, r2)) am |= 1u << s1;
            }
            if ((uint32_t)lane >= cnt) am = 0u;
            emit(am, start + (uint32_t)lane);
            if (!cm) break;
            j = jn; start = sn; cnt = cn; pp = pn;
        }
    };

    const int lc = t.lc;
    const float4 rlo = __ldg(&t.lo[1]), rhi = __ldg(&t.hi[1]);
    // Sub-groups.  Consecutive queries of the Morton order can straddle a jump of the
    // curve, and a group holding two distant clusters would walk every chunk between
    // them.  A range is therefore split at its largest gap between consecutive queries
    // when the two parts' boxes, grown by 4 radii, have less than half the surface of the
    // whole range's; the parts are traversed one after another.
    const float grow = 4.0f * sqrtf(r2);
    int a = 0;
    while (a < nslots) {
        int b = nslots;
        warp_box(lane >= a && lane < b, q, glo, ghi);
        while (b - a >= 4) {
            const F3 qp = f3(__shfl_up_sync(kFull, q.x, 1), __shfl_up_sync(kFull, q.y, 1), __shfl_up_sync(kFull, q.z, 1));
            const float gap = (lane > a && lane < b) ? length_sq(q - qp) : -1.0f;
            const int c = warp_argmax(gap);
            float4 llo, lhi, rlo2, rhi2;
            warp_box(lane >= a && lane < c, q, llo, lhi);
            warp_box(lane >= c && lane < b, q, rlo2, rhi2);
            if (!(box_surface(llo, lhi, grow) + box_surface(rlo2, rhi2, grow) < 0.5f * box_surface(glo, ghi, grow)))
                break;
            b = c;
            glo = llo;
            ghi = lhi;
        }
        in = lane >= a && lane < b;
        ++n_boxes;
        if (!gap_outside(glo, ghi, rlo, rhi, r2)) {
        if (lc == 0) {
            chunks(1u, rlo, rhi);
        } else {
            if (lane == 0) sm.stk[0] = 1u;
            __syncwarp();
            int sp = 1;
            while (sp > 0) {
                --sp;
                const uint32_t e = sm.stk[sp];
                __syncwarp();
                const int L = 31 - __clz(e);
                const int k = (lc - L) < E ? (lc - L) : E;
                const uint32_t m = 1u << k;
                const uint32_t ce = (e << k) + (uint32_t)lane;
                bool keep = false;
                float4 blo = make_float4(0.0f, 0.0f, 0.0f, 0.0f), bhi = blo;
                if ((uint32_t)lane < m) {
                    blo = __ldg(&t.lo[ce]);
                    bhi = __ldg(&t.hi[ce]);
                    keep = !gap_outside(glo, ghi, blo, bhi, r2);
                }
                n_boxes += m;
                const unsigned bm = __ballot_sync(kFull, keep);
                if (L + k == lc) {
                    chunks(bm, blo, bhi);
                } else {
                    const int add = __popc(bm);
                    if (sp + add > kRootStack) {   // cannot happen (bound above); flagged, not silent
                        if (lane == 0 && err) atomicOr(err, 1);
                        break;
                    }
                    if (keep) sm.stk[sp + __popc(bm & lt)] = ce;
                    sp += add;
                    __syncwarp();
                }
            }
        }
        }
        a = b;
    }
    if (np > 0) {
        __syncwarp();
        sink.flush(sm, lane, np);
        n_acc += (unsigned)np;
    }
    __syncwarp();
    sink.finish(sm, lane, active, qi);
    if (counters && lane == 0) {
        atomicAdd(&counters[0], (unsigned long long)n_acc);
        atomicAdd(&counters[1], (unsigned long long)n_tests);
        atomicAdd(&counters[2], (unsigned long long)n_chunks);
        atomicAdd(&counters[3], (unsigned long long)n_boxes);
    }
}

// Exclusive scan of m counters in one CTA of 1024 threads (m up to a few million).
__global__ void __launch_bounds__(1024) k_scan_counts(uint32_t* counts, long long m) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long base = 0; base < m; base += 1024 * 8) {
        uint32_t v[8];
        uint32_t sum = 0;
        long long i0 = base + (long long)threadIdx.x * 8;
        for (int k = 0; k < 8; ++k) { v[k] = (i0 + k < m) ? counts[i0 + k] : 0u; sum += v[k]; }
        uint32_t incl = sum;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = warp_sums[lane], wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(kFull, wi, o);
                if (lane >= o) wi += y;
            }
            warp_sums[lane] = wi - w;
        }
        __syncthreads();
        uint32_t run = carry + warp_sums[wid] + incl - sum;
        for (int k = 0; k < 8; ++k) {
            if (i0 + k < m) counts[i0 + k] = run;
            run += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry = run;
        __syncthreads();
    }
}

// Multi-block form of the same scan for large m: each block scans one 8192-counter tile
// in place and writes its total, one block scans the totals, a third pass adds them.
constexpr long long kScanTile = 1024 * 8;
__global__ void __launch_bounds__(1024) k_scan_tile(uint32_t* counts, long long m, uint32_t* tile_sums) {
    __shared__ uint32_t warp_sums[32];
    const long long base = blockIdx.x * kScanTile;
    uint32_t v[8];
    uint32_t sum = 0;
    const long long i0 = base + (long long)threadIdx.x * 8;
    for (int k = 0; k < 8; ++k) { v[k] = (i0 + k < m) ? counts[i0 + k] : 0u; sum += v[k]; }
    uint32_t incl = sum;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = warp_sums[lane], wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(kFull, wi, o);
            if (lane >= o) wi += y;
        }
        warp_sums[lane] = wi - w;
        if (lane == 31) tile_sums[blockIdx.x] = wi;
    }
    __syncthreads();
    uint32_t run = warp_sums[wid] + incl - sum;
    for (int k = 0; k < 8; ++k) {
        if (i0 + k < m) counts[i0 + k] = run;
        run += v[k];
    }
}

__global__ void k_scan_tile_add(uint32_t* counts, long long m, const uint32_t* __restrict__ tile_offsets) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < m) counts[i] += tile_offsets[i / kScanTile];
}

// Query order: a stable LSD radix sort of the queries' 30-bit Morton codes (10 bits per
// axis over the queries' bounding box), three passes of 10-bit digits.  Consecutive
// queries of the sorted order are then close in space whatever the photon density (an
// order by KD cell is not: a cell of a sparsely lit region holds hundreds of queries).
constexpr int kRsBits = 10, kRsBins = 1 << kRsBits, kRsThreads = 256, kRsWarps = kRsThreads / 32;
constexpr int kRsPerWarp = 256;                        // keys a warp ranks per tile
constexpr long long kRsTile = kRsWarps * kRsPerWarp;   // keys per block

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t cell10(float v) {
    return v > 0.0f ? (v < 1023.0f ? (uint32_t)v : 1023u) : 0u;   // NaN -> 0
}

__global__ void k_query_keys(const float* __restrict__ qpos, int stride, long long nq,
                             const unsigned long long* __restrict__ nq_dev, QueryFrame f, uint32_t* __restrict__ keys,
                             uint32_t* __restrict__ vals) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (nq_dev) nq = (long long)min(*nq_dev, (unsigned long long)nq);
    if (i >= nq) return;
    const float* q = qpos + (long long)stride * i;
    const uint32_t cx = cell10((q[0] - f.lo[0]) * f.scale[0]);
    const uint32_t cy = cell10((q[1] - f.lo[1]) * f.scale[1]);
    const uint32_t cz = cell10((q[2] - f.lo[2]) * f.scale[2]);
    keys[i] = spread10(cx) | (spread10(cy) << 1) | (spread10(cz) << 2);
    vals[i] = (uint32_t)i;
}

// Per-block digit counts, digit-major (hist[d * blocks + b]), so that one exclusive scan
// of the whole array gives every (digit, block) its first output position.
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t* __restrict__ keys, long long nq,
                                                        const unsigned long long* __restrict__ nq_dev, int shift,
                                                        uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[kRsBins];
    for (int d = threadIdx.x; d < kRsBins; d += kRsThreads) cnt[d] = 0;
    __syncthreads();
    if (nq_dev) nq = (long long)min(*nq_dev, (unsigned long long)nq);
    const long long base = (long long)blockIdx.x * kRsTile;
    for (int k = threadIdx.x; k < kRsTile; k += kRsThreads) {
        const long long i = base + k;
        if (i < nq) atomicAdd(&cnt[(keys[i] >> shift) & (kRsBins - 1)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRsBins; d += kRsThreads) hist[(long long)d * gridDim.x + blockIdx.x] = cnt[d];
}

// Stable scatter of one block's tile: warp w ranks the keys [w * 256, (w + 1) * 256) of
// the tile in order (per-warp digit counts, a prefix over the warps per digit on top of
// the block's scanned offsets, then ranks by __match_any_sync round by round).
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t* __restrict__ keys_in,
                                                           const uint32_t* __restrict__ vals_in,
                                                           uint32_t* __restrict__ keys_out,
                                                           uint32_t* __restrict__ vals_out, long long nq,
                                                           const unsigned long long* __restrict__ nq_dev, int shift,
                                                           const uint32_t* __restrict__ offsets) {
    __shared__ uint32_t wc[kRsWarps][kRsBins];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int k = threadIdx.x; k < kRsWarps * kRsBins; k += kRsThreads) (&wc[0][0])[k] = 0;
    __syncthreads();
    if (nq_dev) nq = (long long)min(*nq_dev, (unsigned long long)nq);
    const long long wbase = (long long)blockIdx.x * kRsTile + (long long)warp * kRsPerWarp;
    for (int r = 0; r < kRsPerWarp / 32; ++r) {
        const long long i = wbase + r * 32 + lane;
        const bool valid = i < nq;
        const uint32_t d = valid ? (keys_in[i] >> shift) & (kRsBins - 1) : 0xffffffffu;
        const unsigned peers = __match_any_sync(kFull, d);
        if (valid && (peers & lt) == 0u) wc[warp][d] += (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRsBins; d += kRsThreads) {
        uint32_t run = offsets[(long long)d * gridDim.x + blockIdx.x];
        for (int w = 0; w < kRsWarps; ++w) {
            const uint32_t c = wc[w][d];
            wc[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    for (int r = 0; r < kRsPerWarp / 32; ++r) {
        const long long i = wbase + r * 32 + lane;
        const bool valid = i < nq;
        uint32_t key = 0, val = 0, d = 0xffffffffu;
        if (valid) {
            key = keys_in[i];
            val = vals_in[i];
            d = (key >> shift) & (kRsBins - 1);
        }
        const unsigned peers = __match_any_sync(kFull, d);
        uint32_t pos = 0;
        if (valid) pos = wc[warp][d] + (uint32_t)__popc(peers & lt);
        __syncwarp();
        if (valid) {
            keys_out[pos] = key;
            vals_out[pos] = val;
            if ((peers & lt) == 0u) wc[warp][d] += (uint32_t)__popc(peers);
        }
        __syncwarp();
    }
}

// Chunk boxes: one warp per chunk reduces its (at most 32) photons' coordinates.
__global__ void k_chunk_boxes(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z,
                              long long n, int lc, float4* __restrict__ lo, float4* __restrict__ hi) {
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long m = 1LL << lc;
    if (w >= m) return;
    const long long e = m + w;
    const long long s = kd_node_start(e, lc, n);
    const long long end = (w + 1 < m) ? kd_node_start(e + 1, lc, n) : n;
    const long long c = end - s;   // <= 32: the node's range plus at most one median
    float mnx = INFINITY, mny = INFINITY, mnz = INFINITY, mxx = -INFINITY, mxy = -INFINITY, mxz = -INFINITY;
    if (lane < c) {
        mnx = mxx = x[s + lane];
        mny = mxy = y[s + lane];
        mnz = mxz = z[s + lane];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(kFull, mnx, o)); mny = fminf(mny, __shfl_xor_sync(kFull, mny, o));
        mnz = fminf(mnz, __shfl_xor_sync(kFull, mnz, o)); mxx = fmaxf(mxx, __shfl_xor_sync(kFull, mxx, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(kFull, mxy, o)); mxz = fmaxf(mxz, __shfl_xor_sync(kFull, mxz, o));
    }
    if (lane == 0) {
        lo[e] = make_float4(mnx, mny, mnz, __uint_as_float((uint32_t)s));
        hi[e] = make_float4(mxx, mxy, mxz, __uint_as_float((uint32_t)c));
    }
}

// Boxes of the nodes on one level: the union of their children's.
__device__ __forceinline__ void unite_children(float4* lo, float4* hi, long long e) {
    const float4 a = lo[2 * e], b = lo[2 * e + 1], c = hi[2 * e], d = hi[2 * e + 1];
    lo[e] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
    hi[e] = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), 0.0f);
}
__global__ void k_level_boxes(int level, float4* lo, float4* hi) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < (1LL << level)) unite_children(lo, hi, (1LL << level) + i);
}
// levels [0, top] in one CTA, bottom-up
constexpr int kTopLevels = 11;
__global__ void __launch_bounds__(1024) k_top_boxes(int top, float4* lo, float4* hi) {
    for (int l = top; l >= 0; --l) {
        for (long long i = threadIdx.x; i < (1LL << l); i += blockDim.x) unite_children(lo, hi, (1LL << l) + i);
        __syncthreads();
    }
}

// Photon records gathered into tree order, so the gather reads them contiguously
// (positions only when ph.dir is null).
__global__ void k_tree_records(PhotonBuf ph, const uint32_t* __restrict__ id, long long n, TreePhotons tp) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t i = id[p];
    tp.t0[p] = ph.pos[i];
    if (ph.dir) {
        tp.t1[p] = ph.dir[i];
        tp.t2[p] = ph.tp[i];
    }
}

ChunkTree chunk_tree(const KdTree& tree, const float4* t0) {
    return ChunkTree{tree.box_lo, tree.box_hi, t0, (tree.n > 0 && tree.box_lo) ? tree.box_levels - 1 : -1};
}

// Launch shapes: (resident blocks per SM, queries per group, levels per expansion step).
struct Shape { int mb, g, e; };
constexpr Shape kShapes[] = {{2, 32, 5}, {3, 32, 5}, {4, 32, 5}, {3, 32, 4}, {4, 32, 4}, {3, 16, 5}, {4, 16, 4}, {4, 16, 5}};
constexpr int kNumShapes = (int)(sizeof(kShapes) / sizeof(kShapes[0]));
constexpr int kDefaultShape = 1;

template <int MB, int G, int E, class Sink>
void launch_shape(const ChunkTree& t, const float* qpos, int qstride, const uint32_t* order, long long nq,
                  const unsigned long long* nq_dev, const int* skip, float r2, const Sink& sink,
                  unsigned long long* counters, int* err, cudaStream_t s) {
    const long long warps = (nq + G - 1) / G;
    k_gather<MB, G, E, Sink><<<(unsigned)((warps + kWarpsPerBlock - 1) / kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(
        t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err);
}

template <class Sink>
void launch_variant(int v, const ChunkTree& t, const float* qpos, int qstride, const uint32_t* order, long long nq,
                    const unsigned long long* nq_dev, const int* skip, float r2, const Sink& sink,
                    unsigned long long* counters, int* err, cudaStream_t s) {
    switch (v) {
    case 0: launch_shape<2, 32, 5>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    case 2: launch_shape<4, 32, 5>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    case 3: launch_shape<3, 32, 4>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    case 4: launch_shape<4, 32, 4>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    case 5: launch_shape<3, 16, 5>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    case 6: launch_shape<4, 16, 4>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    case 7: launch_shape<4, 16, 5>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    default: launch_shape<3, 32, 5>(t, qpos, qstride, order, nq, nq_dev, skip, r2, sink, counters, err, s); break;
    }
}

}  // namespace

int kd_chunk_level(long long n) {
    if (n <= 0) return -1;
    int l = 0;
    while ((n >> l) > kChunkNode) ++l;
    return l;
}

int kd_box_levels(long long n) { return n > 0 ? kd_chunk_level(n) + 1 : 0; }

void launch_kd_boxes(const KdTree& tree, cudaStream_t s, int* launches) {
    if (tree.n <= 0 || !tree.box_lo) return;
    const int lc = tree.box_levels - 1;
    const long long chunks = 1LL << lc;
    k_chunk_boxes<<<(unsigned)((chunks * 32 + 255) / 256), 256, 0, s>>>(tree.x, tree.y, tree.z, tree.n, lc,
                                                                        tree.box_lo, tree.box_hi);
    int nl = 1;
    int l = lc - 1;
    for (; l > kTopLevels; --l) {
        k_level_boxes<<<(unsigned)(((1LL << l) + 255) / 256), 256, 0, s>>>(l, tree.box_lo, tree.box_hi);
        ++nl;
    }
    if (l >= 0) {
        k_top_boxes<<<1, 1024, 0, s>>>(l, tree.box_lo, tree.box_hi);
        ++nl;
    }
    if (launches) *launches += nl;
}

namespace {
long long rs_blocks(long long nq) { return (nq + kRsTile - 1) / kRsTile; }
}  // namespace

size_t query_order_scratch_bytes(long long nq) {
    const long long n = nq > 0 ? nq : 1;
    const long long m = rs_blocks(n) * kRsBins;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    return 3 * al(4 * (size_t)n) + al(4 * (size_t)m) + al(4 * scan_scratch_words(m));
}

QueryFrame query_frame(const float lo[3], const float hi[3]) {
    QueryFrame f;
    for (int k = 0; k < 3; ++k) {
        const float ext = hi[k] - lo[k];
        f.lo[k] = lo[k];
        f.scale[k] = ext > 0.0f ? 1023.99f / ext : 0.0f;
    }
    return f;
}

void launch_query_order(const float* qpos, int stride, long long nq, const QueryFrame& frame, void* scratch,
                        uint32_t* order, int* launches, cudaStream_t s, const unsigned long long* nq_dev) {
    if (nq <= 0) return;
    const long long B = rs_blocks(nq), m = B * kRsBins;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char* p = (char*)scratch;
    uint32_t* keys_a = (uint32_t*)p; p += al(4 * (size_t)nq);
    uint32_t* keys_b = (uint32_t*)p; p += al(4 * (size_t)nq);
    uint32_t* vals_a = (uint32_t*)p; p += al(4 * (size_t)nq);
    uint32_t* hist = (uint32_t*)p; p += al(4 * (size_t)m);
    uint32_t* tiles = (uint32_t*)p;
    k_query_keys<<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(qpos, stride, nq, nq_dev, frame, keys_a, vals_a);
    int nl = 1;
    // passes: a -> (keys_b, order), (keys_b, order) -> (keys_a, vals_a), (keys_a, vals_a) -> (keys_b, order)
    const uint32_t* kin[3] = {keys_a, keys_b, keys_a};
    const uint32_t* vin[3] = {vals_a, order, vals_a};
    uint32_t* kout[3] = {keys_b, keys_a, keys_b};
    uint32_t* vout[3] = {order, vals_a, order};
    for (int pass = 0; pass < 3; ++pass) {
        k_rs_hist<<<(unsigned)B, kRsThreads, 0, s>>>(kin[pass], nq, nq_dev, pass * kRsBits, hist);
        launch_scan_counts(hist, m, tiles, s);
        k_rs_scatter<<<(unsigned)B, kRsThreads, 0, s>>>(kin[pass], vin[pass], kout[pass], vout[pass], nq, nq_dev,
                                                         pass * kRsBits, hist);
        nl += 2 + (m > 4 * kScanTile ? 3 : 1);
    }
    if (launches) *launches += nl;
}

size_t scan_scratch_words(long long m) { return (size_t)(m / kScanTile + 2); }

void launch_scan_counts(uint32_t* counts, long long m, uint32_t* tile_scratch, cudaStream_t s) {
    if (m <= 0) return;
    if (m <= 4 * kScanTile || !tile_scratch) { k_scan_counts<<<1, 1024, 0, s>>>(counts, m); return; }
    const long long tiles = (m + kScanTile - 1) / kScanTile;
    k_scan_tile<<<(unsigned)tiles, 1024, 0, s>>>(counts, m, tile_scratch);
    k_scan_counts<<<1, 1024, 0, s>>>(tile_scratch, tiles);
    k_scan_tile_add<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(counts, m, tile_scratch);
}

void launch_tree_records(PhotonBuf ph, const KdTree& tree, TreePhotons tp, cudaStream_t s) {
    if (tree.n <= 0) return;
    k_tree_records<<<(unsigned)((tree.n + 255) / 256), 256, 0, s>>>(ph, tree.id, tree.n, tp);
}

int gather_variants() { return kNumShapes; }
int gather_default_variant() { return kDefaultShape; }

const char* gather_variant_name(int v) {
    static const char* names[kNumShapes] = {
        "blocks/SM>=2, 32 queries/group, 5-level steps", "blocks/SM>=3, 32 queries/group, 5-level steps",
        "blocks/SM>=4, 32 queries/group, 5-level steps", "blocks/SM>=3, 32 queries/group, 4-level steps",
        "blocks/SM>=4, 32 queries/group, 4-level steps", "blocks/SM>=3, 16 queries/group, 5-level steps",
        "blocks/SM>=4, 16 queries/group, 4-level steps", "blocks/SM>=4, 16 queries/group, 5-level steps"};
    return (v >= 0 && v < kNumShapes) ? names[v] : "?";
}

void launch_gather(const VMParams& p, const KdTree& tree, TreePhotons tp, QueryBuf qb, const uint32_t* order,
                   long long nq, double* accum, unsigned long long* counters, cudaStream_t s, int variant,
                   const unsigned long long* nq_dev, const int* skip) {
    if (nq <= 0 || tree.n <= 0) return;
    const EvalSink sink{p, qb, tp, tree.id, accum};
    launch_variant(variant, chunk_tree(tree, tp.t0), reinterpret_cast<const float*>(qb.q0), 4, order, nq, nq_dev,
                   skip, p.radius_sqr, sink, counters, p.error + ERR_GATHER, s);
}

void launch_gather_sets(const KdTree& tree, const float4* t0, const float* qpos, int qstride, const uint32_t* order,
                        long long nq, float r2, int* counts, const long long* offsets, int* cursor, int* idx,
                        int variant, unsigned long long* counters, int* err, cudaStream_t s) {
    if (nq <= 0 || tree.n <= 0) return;
    const SetSink sink{tree.id, counts, offsets, cursor, idx};
    launch_variant(variant, chunk_tree(tree, t0), qpos, qstride, order, nq, nullptr, nullptr, r2, sink, counters, err,
                   s);
}

}  // namespace rc
