// Radius gather at the camera vertices (Path_Vertices::get_contrib,
// src/Path_Vertices.h:46-68, over KD_Tree::find_closest_in_radius,
// src/KD_Tree.cpp:217-280), one merge query per warp.
//
// Queries are first ordered by the KD cell they fall in (launch_query_order), so the
// queries a warp processes one after another touch the same nodes and photons (L1/L2
// reuse).  For each query the warp runs the reference's descent uniformly (near side
// first; far side and an odd node's median photon only when (q[axis] - split)^2 < r^2)
// and, at a node of at most kBucket photons, tests the whole contiguous tree-order range
// at once, one photon per lane, with the reference's acceptance predicate
// ((dx*dx + dy*dy) + dz*dz) < r^2 in FP32 without contraction.  Accepted photons are
// compacted in shared memory and their MIS-weighted BSDF contributions are evaluated
// lane-parallel, then summed across the warp.
//
// The set of photons a query accepts is exactly the reference's: the descent is the
// reference's own, a bucket is tested exhaustively, and pruning never drops a photon
// inside the radius (rounding is monotonic, so |q - p|^2 >= (q[axis] - split)^2 holds in
// floats too).  Accumulation order differs from the reference's recursion, so
// contributions agree to FP32 rounding.
#include "vm.cuh"
#include "bsdf.cuh"

namespace rc {

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kStack = 64;
constexpr int kQueriesPerWarp = 16;
constexpr int kBucket = 32;   // photons tested per bucket (kBucket / 32 per lane)

struct KdNav {
    const uint2* __restrict__ nodes;
    const float* __restrict__ x;
    const float* __restrict__ y;
    const float* __restrict__ z;
    const uint32_t* __restrict__ id;
    const float4* __restrict__ box_lo;   // per node down to the bucket level (nullptr: none)
    const float4* __restrict__ box_hi;
    int box_levels;                      // boxes exist for levels [0, box_levels)
    long long n;
};

// Squared distance from q to a box, formed like the acceptance test so that it never
// exceeds the squared distance to any photon inside the box (rounding is monotonic).
__device__ __forceinline__ bool box_outside(F3 q, float4 lo, float4 hi, float r2) {
    float dx = q.x < lo.x ? lo.x - q.x : (q.x > hi.x ? q.x - hi.x : 0.0f);
    float dy = q.y < lo.y ? lo.y - q.y : (q.y > hi.y ? q.y - hi.y : 0.0f);
    float dz = q.z < lo.z ? lo.z - q.z : (q.z > hi.z ? q.z - hi.z : 0.0f);
    return !(dx * dx + dy * dy + dz * dz < r2);
}

__device__ __forceinline__ bool in_radius(F3 q, float px, float py, float pz, float r2) {
    float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
    return dx * dx + dy * dy + dz * dz < r2;
}

// Warp-uniform traversal; fn(tree position) runs on each lane for each photon its
// query accepts.  `stack` is this warp's shared-memory stack (kStack (e, start) pairs).
struct VisitCounts { unsigned nodes, buckets, tests; };

// Hand the first 32 pending entries to `flush` once there are 32 or more, and move the
// rest (at most 31) to the front, so that every flush but a warp's last is a full one.
template <class Flush>
__device__ __forceinline__ void drain32(uint32_t* pend, int& np, Flush& flush) {
    if (np < 32) return;
    flush(32, pend);
    __syncwarp();
    const int lane = threadIdx.x & 31, rest = np - 32;
    const uint32_t v = lane < rest ? pend[32 + lane] : 0u;
    __syncwarp();
    if (lane < rest) pend[lane] = v;
    np = rest;
    __syncwarp();
}

// One query per warp.  The traversal is the reference's descent for that single query
// (uniform across the warp): near side first, far side and an odd node's median photon
// only when (q[axis] - split)^2 < r^2.  The stack lives in registers spread over the
// lanes (entry k in lane k % 32 of register pair k / 32); push and pop are uniform.
// A node of at most kBucket photons is a bucket, tested kBucket/32 photons per lane.
// Accepted tree positions are appended to the warp's pending list in shared memory;
// `flush(count, list)` runs on all lanes whenever the list holds 32 or more entries
// and once at the end, so the per-photon work is spread over the lanes.
template <class Flush>
__device__ __forceinline__ void kd_query_warp(const KdNav& t, F3 q, float r2, uint2 start_node, uint32_t* pend,
                                              int& np, uint32_t tag, VisitCounts& vc, Flush&& flush) {
    const int lane = threadIdx.x & 31;
    if (t.n <= 0) return;
    uint32_t se0 = 0, ss0 = 0, se1 = 0, ss1 = 0;   // stack entries lane and lane+32
    if (lane == 0) { se0 = start_node.x; ss0 = start_node.y; }
    {
        const int l0 = 31 - __clz(start_node.x);
        if (l0 < t.box_levels && box_outside(q, __ldg(&t.box_lo[start_node.x]), __ldg(&t.box_hi[start_node.x]), r2))
            return;
    }
    int sp = 1;
    const uint32_t n32 = (uint32_t)t.n;   // photon counts stay below 2^28 (28-bit index field)
    while (sp) {
        --sp;
        uint32_t e, start;
        if (sp < 32) { e = __shfl_sync(0xffffffffu, se0, sp); start = __shfl_sync(0xffffffffu, ss0, sp); }
        else { e = __shfl_sync(0xffffffffu, se1, sp - 32); start = __shfl_sync(0xffffffffu, ss1, sp - 32); }
        const int level = 31 - __clz(e);
        const uint32_t c = n32 >> level;
        if (c <= (uint32_t)kBucket) {
            if (level < t.box_levels && box_outside(q, __ldg(&t.box_lo[e]), __ldg(&t.box_hi[e]), r2)) continue;
            vc.buckets++;
            vc.tests += c;
#pragma unroll
            for (int k = 0; k < kBucket / 32; ++k) {
                const uint32_t i = (uint32_t)(k * 32 + lane);
                bool acc = false;
                if (i < c) {
                    const uint32_t p = start + i;
                    acc = in_radius(q, __ldg(&t.x[p]), __ldg(&t.y[p]), __ldg(&t.z[p]), r2);
                }
                const unsigned m = __ballot_sync(0xffffffffu, acc);
                if (acc) pend[np + __popc(m & ((1u << lane) - 1u))] = (start + i) | tag;
                np += __popc(m);
                __syncwarp();
                drain32(pend, np, flush);
            }
            continue;
        }
        vc.nodes++;
        const uint2 nd = __ldg(&t.nodes[e]);
        const uint32_t ax = nd.x & 0x60000000u;
        const float split = __uint_as_float(nd.y);
        const float qa = ax == 0 ? q.x : (ax == 0x20000000u ? q.y : q.z);
        const float d = qa - split;
        const uint32_t half = c >> 1, odd = c & 1u;
        const bool left_near = d < 0;
        const bool within = d * d < r2;
        if (odd && within) {
            const uint32_t p = start + half;
            const bool a = in_radius(q, __ldg(&t.x[p]), __ldg(&t.y[p]), __ldg(&t.z[p]), r2);
            if (a && lane == 0) pend[np] = p | tag;
            np += a ? 1 : 0;
            __syncwarp();
            drain32(pend, np, flush);
        }
        const uint32_t le = 2u * e, ls = start;
        const uint32_t re = 2u * e + 1u, rs = start + half + odd;
        // far side first (when within), then the near side, which is popped next
        if (within && sp < kStack) {
            const uint32_t fe = left_near ? re : le, fs = left_near ? rs : ls;
            if ((sp & 31) == lane) { if (sp < 32) { se0 = fe; ss0 = fs; } else { se1 = fe; ss1 = fs; } }
            ++sp;
        }
        if (sp < kStack) {
            const uint32_t ne = left_near ? le : re, ns = left_near ? ls : rs;
            if ((sp & 31) == lane) { if (sp < 32) { se0 = ne; ss0 = ns; } else { se1 = ne; ss1 = ns; } }
            ++sp;
        }
    }
    __syncwarp();
}

// Lane-parallel variant of the same query, used when node boxes exist down to the bucket
// level Lb (every node at level Lb holds n >> Lb <= kBucket photons).  A subtree root at
// level L < Lb is expanded k = min(E, Lb - L) levels at once (E = 4 or 5, a launch-shape
// parameter): lane j box-tests the j-th descendant at level L + k and survivors are
// pushed as new roots, while lanes test the median photons of the 2^k - 1 inner nodes in
// between (odd counts only).  Roots at
// level >= Lb are scanned like buckets.  The accepted set is the reference's: every
// photon of the start node's range lies in a bucket or is an inner node's median; a
// culled box holds no photon within the radius (box distance <= photon distance under
// monotonic rounding), a median outside its node's split slab fails the predicate
// (its distance >= |q[axis] - split|), and every photon that is tested is tested with
// the reference's predicate.  DFS over roots keeps at most 2^E - 1 pending roots per
// expansion level: with n < 2^28 (Lb <= 27) at most 6 x 31 + 1 = 187 (E = 5) or
// 7 x 15 + 1 = 106 (E = 4) < kRootStack.  (On the 1920x1080 water pool 4 levels per
// step beat 5; 3 lost to both: 6.9 / 7.1 / 8.2 ms per gather.)
constexpr int kRootStack = 256;

template <int E, class Flush>
__device__ __forceinline__ void kd_query_expand(const KdNav& t, F3 q, float r2, uint2 start_node, uint32_t* pend,
                                                uint2* stk, int& np, uint32_t tag, VisitCounts& vc, Flush&& flush) {
    const int lane = threadIdx.x & 31;
    if (t.n <= 0) return;
    const uint32_t n32 = (uint32_t)t.n;
    const int Lb = t.box_levels - 1;
    {
        const int l0 = 31 - __clz(start_node.x);
        if (l0 <= Lb && box_outside(q, __ldg(&t.box_lo[start_node.x]), __ldg(&t.box_hi[start_node.x]), r2)) return;
    }
    auto append = [&](bool acc, uint32_t p) {
        const unsigned m = __ballot_sync(0xffffffffu, acc);
        if (acc) pend[np + __popc(m & ((1u << lane) - 1u))] = p | tag;
        np += __popc(m);
        __syncwarp();
        drain32(pend, np, flush);
    };
    if (lane == 0) stk[0] = start_node;
    __syncwarp();
    int sp = 1;
    while (sp) {
        --sp;
        const uint2 rt = stk[sp];
        __syncwarp();
        const uint32_t e = rt.x, start = rt.y;
        const int L = 31 - __clz(e);
        if (L >= Lb) {
            const uint32_t c = n32 >> L;
            vc.buckets++;
            vc.tests += c;
#pragma unroll
            for (int k = 0; k < kBucket / 32; ++k) {
                const uint32_t i = (uint32_t)(k * 32 + lane);
                bool acc = false;
                if (i < c) acc = in_radius(q, __ldg(&t.x[start + i]), __ldg(&t.y[start + i]), __ldg(&t.z[start + i]), r2);
                append(acc, start + i);
            }
            continue;
        }
        const int k = (Lb - L) < E ? (Lb - L) : E;
        const uint32_t m = 1u << k;
        vc.nodes += m - 1;
        {
            // median photons of the inner nodes at levels L .. L+k-1 (1-based BFS index)
            bool acc = false;
            uint32_t p = 0;
            if ((uint32_t)lane < m - 1) {
                const uint32_t i1 = (uint32_t)lane + 1u;
                const int li = 31 - __clz(i1);
                const uint32_t pi = i1 - (1u << li);
                const uint32_t c = n32 >> (L + li);
                if (c & 1u) {
                    uint32_t st = start;
                    for (int b = 0; b < li; ++b) {
                        const uint32_t cl = n32 >> (L + b);
                        if ((pi >> (li - 1 - b)) & 1u) st += (cl >> 1) + (cl & 1u);
                    }
                    p = st + (c >> 1);
                    acc = in_radius(q, __ldg(&t.x[p]), __ldg(&t.y[p]), __ldg(&t.z[p]), r2);
                }
            }
            append(acc, p);
        }
        {
            // the 2^k descendants at level L + k: box test, survivors become roots
            bool keep = false;
            uint32_t st = start;
            const uint32_t ce = (e << k) + (uint32_t)lane;
            if ((uint32_t)lane < m) {
                for (int b = 0; b < k; ++b) {
                    const uint32_t cl = n32 >> (L + b);
                    if (((uint32_t)lane >> (k - 1 - b)) & 1u) st += (cl >> 1) + (cl & 1u);
                }
                keep = !box_outside(q, __ldg(&t.box_lo[ce]), __ldg(&t.box_hi[ce]), r2);
            }
            const unsigned bm = __ballot_sync(0xffffffffu, keep);
            if (keep) stk[sp + __popc(bm & ((1u << lane) - 1u))] = make_uint2(ce, st);
            sp += __popc(bm);
            __syncwarp();
        }
    }
    __syncwarp();
}

// Accepted tree positions go to the warp's pending list `pend` (count `np`, uniform,
// carried across the queries of a warp) with `tag` in their top bits; the list is
// handed to `flush` whenever it holds 32 or more entries.  The caller flushes the rest.
template <int E = 5, class Flush>
__device__ __forceinline__ void kd_query(const KdNav& t, F3 q, float r2, uint2 start_node, uint32_t* pend, uint2* stk,
                                         int& np, uint32_t tag, VisitCounts& vc, Flush&& flush) {
    if (t.box_levels > 0) kd_query_expand<E>(t, q, r2, start_node, pend, stk, np, tag, vc, flush);
    else kd_query_warp(t, q, r2, start_node, pend, np, tag, vc, flush);
}

// Traversal half of the gather.  MinBlocks (resident blocks per SM the register
// allocation must allow) and QPW (consecutive sorted queries per warp) are the autotuned
// shape parameters.  The warp's queries share the pending list (entry = query slot << 28
// | tree position); every 32 accepted photons become 32 pairs (query index, position) in
// the merge buffer, in query order.
template <int MinBlocks, int QPW, int E>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, MinBlocks) k_gather(const VMParams P, const KdNav t,
                                                                         QueryBuf qb,
                                                                         const uint32_t* __restrict__ order,
                                                                         const uint2* __restrict__ start_nodes,
                                                                         long long nq, MergeBuf mb,
                                                                         unsigned long long* __restrict__ counters,
                                                                         const unsigned long long* __restrict__ nq_dev,
                                                                         const int* __restrict__ skip) {
    static_assert(QPW <= 16, "a pending entry keeps its query slot in its top 4 bits");
    // device-side count (bounded by the capacity nq) and an iteration-wide skip flag,
    // for iterations enqueued without a host round trip
    if (skip && *skip) return;
    if (nq_dev) nq = (long long)min(*nq_dev, (unsigned long long)nq);
    __shared__ uint32_t pend[kWarpsPerBlock][64];
    __shared__ uint2 stk[kWarpsPerBlock][kRootStack];
    __shared__ uint32_t qidx[kWarpsPerBlock][QPW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long w = blockIdx.x * (long long)kWarpsPerBlock + warp;
    const long long first = w * QPW;
    if (first >= nq) return;
    const int nslots = (int)((first + QPW < nq ? first + QPW : nq) - first);
    VisitCounts vc{0u, 0u, 0u};
    unsigned accepted = 0;
    auto flush = [&](int n, const uint32_t* list) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(mb.count, (unsigned long long)n);
        base = __shfl_sync(0xffffffffu, base, 0);
        for (int j = lane; j < n; j += 32) {
            const unsigned long long at = base + (unsigned long long)j;
            const uint32_t entry = list[j];
            if (at < (unsigned long long)mb.cap) mb.pairs[at] = make_uint2(qidx[warp][entry >> 28], entry & 0x0fffffffu);
        }
        accepted += (unsigned)n;
    };
    int np = 0;
    for (int k = 0; k < nslots; ++k) {
        const uint32_t qi = __ldg(&order[first + k]);
        if (lane == 0) qidx[warp][k] = qi;
        const uint2 sn = __ldg(&start_nodes[qi]);
        const float4 a = qb.q0[qi];
        __syncwarp();
        kd_query<E>(t, xyz(a), P.radius_sqr, sn, pend[warp], stk[warp], np, (uint32_t)k << 28, vc, flush);
    }
    if (np > 0) flush(np, pend[warp]);
    if (counters && lane == 0) {
        atomicAdd(&counters[0], (unsigned long long)accepted);
        atomicAdd(&counters[1], (unsigned long long)vc.tests);
        atomicAdd(&counters[2], (unsigned long long)vc.buckets);
        atomicAdd(&counters[3], (unsigned long long)vc.nodes);
    }
}

// Merge half of the gather (Path_Vertices::get_contrib, src/Path_Vertices.h:46-68): per
// pair, the camera vertex's BSDF at the photon's direction, the MIS weight
// 1 / (1 + dVM_cam pdf_rev + dVM_light pdf_fwd), times the photon throughput.  A
// warp's pairs come in runs of one query (each traversal flush writes its pairs in query
// order), so a segmented scan over the lanes sums each run and its last lane adds the
// run, times the camera throughput, to the pixel's FP64 sum.
constexpr int kMergeThreads = 256;
__global__ void __launch_bounds__(kMergeThreads) k_merge(const VMParams P, TreePhotons tp, QueryBuf qb,
                                                         const uint32_t* __restrict__ tree_id, MergeBuf mb,
                                                         double* __restrict__ accum, const int* __restrict__ skip) {
    if (skip && *skip) return;
    const unsigned long long n = *mb.count;
    if (n > (unsigned long long)mb.cap) {
        if (mb.overflow && blockIdx.x == 0 && threadIdx.x == 0) *mb.overflow = 1;
        return;
    }
    const int lane = threadIdx.x & 31;
    const unsigned long long stride = (unsigned long long)gridDim.x * kMergeThreads;
    // whole warps step together (the scan below needs every lane)
    for (unsigned long long i0 = (unsigned long long)blockIdx.x * kMergeThreads + (threadIdx.x & ~31u); i0 < n;
         i0 += stride) {
        const unsigned long long i = i0 + (unsigned long long)lane;
        const bool valid = i < n;
        const uint2 pr = valid ? mb.pairs[i] : make_uint2(0xffffffffu, 0u);
        const uint32_t qi = pr.x;
        F3 cpair = f3(0.0f);
        if (valid) {
            const uint32_t p = pr.y;
            const float4 a = qb.q0[qi], b = qb.q1[qi], c = qb.q2[qi], e = qb.q4[qi];
            const F3 ng = xyz(c);
            Bsdf bs;
            const DevMaterial& qm = P.materials[__float_as_int(b.w)];
            const int channel = __float_as_int(e.w);   // the camera path's dispersion channel
            bs.init(qm, xyz(b), xyz(e), true, (qm.disp > 0.0f && channel >= 0) ? (float)(channel - 1) * qm.disp : 0.0f);
            const float wo_ng = dot(bs.fr.to_world(bs.wo), ng);
            const float fwo = (bs.kind == BSDF_K_PLASTIC_GGX || bs.kind == BSDF_K_PLASTIC_SMOOTH)
                                  ? fresnel_reflectance(fabsf(bs.wo.z), bs.s) : 0.0f;
            const float4 p0 = __ldg(&tp.t0[p]);
            const float4 p1 = __ldg(&tp.t1[p]);
            const float2 p2 = __ldg(&tp.t2[p]);
            float fwd, rev;
            F3 ev;
            bs.eval_pdf(xyz(p1), ng, wo_ng, fwo, ev, fwd, rev);
            const float weight = 1.0f / (1.0f + a.w * rev + p0.w * fwd);
            cpair = ev * f3(p1.w, p2.x, p2.y) * weight;
            if (P.path_contrib) {
                // learned-proposal training signal: the squared luminance this merge adds
                // to its pixel, summed per light path
                const F3 img = xyz(qb.q3[qi]) * cpair;
                const float lum = (fabsf(img.x) + fabsf(img.y) + fabsf(img.z)) * (1.0f / 3.0f);
                if (lum > 0.0f) atomicAdd(&P.path_contrib[__ldg(&P.photon_path[__ldg(&tree_id[p])])], lum * lum);
            }
        }
        // runs of equal query index, numbered by their heads: a query's pairs may form two
        // runs in one window (its warp's flushes need not be adjacent in the buffer), and
        // the scan must not join them across another query's run
        const uint32_t qprev = __shfl_up_sync(0xffffffffu, qi, 1);
        const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || qprev != qi);
        const int run = __popc(heads & ((2u << lane) - 1u));
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float x = __shfl_up_sync(0xffffffffu, cpair.x, o);
            const float y = __shfl_up_sync(0xffffffffu, cpair.y, o);
            const float z = __shfl_up_sync(0xffffffffu, cpair.z, o);
            const int ro = __shfl_up_sync(0xffffffffu, run, o);
            if (lane >= o && ro == run) { cpair.x += x; cpair.y += y; cpair.z += z; }
        }
        const uint32_t qnext = __shfl_down_sync(0xffffffffu, qi, 1);
        if (valid && (lane == 31 || qnext != qi)) {   // last lane of its query's run
            const F3 r = xyz(qb.q3[qi]) * cpair;
            if (r.x != 0.0f || r.y != 0.0f || r.z != 0.0f) {
                const long long pixel = __float_as_int(qb.q2[qi].w);
                atomicAdd(&accum[3 * pixel + 0], (double)r.x);
                atomicAdd(&accum[3 * pixel + 1], (double)r.y);
                atomicAdd(&accum[3 * pixel + 2], (double)r.z);
            }
        }
    }
}

__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_kd_query(const KdNav t, int q, const float* __restrict__ qpos,
                                                                   const uint32_t* __restrict__ order,
                                                                   const uint2* __restrict__ start_nodes, float r2,
                                                                   int* counts, const long long* offsets, int* idx) {
    __shared__ uint32_t pend[kWarpsPerBlock][64];
    __shared__ uint2 stk[kWarpsPerBlock][kRootStack];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long w = blockIdx.x * (long long)kWarpsPerBlock + warp;
    const long long first = w * kQueriesPerWarp;
    if (first >= q) return;
    const long long last = first + kQueriesPerWarp < q ? first + kQueriesPerWarp : q;
    VisitCounts vc{0u, 0u, 0u};
    for (long long slot = first; slot < last; ++slot) {
        const long long j = order[slot];
        const F3 p = f3(qpos[3 * j], qpos[3 * j + 1], qpos[3 * j + 2]);
        const long long off = offsets ? offsets[j] : 0;
        int n = 0, np = 0;
        auto flush = [&](int cnt, const uint32_t* list) {
            if (idx)
                for (int k = lane; k < cnt; k += 32) idx[off + n + k] = (int)__ldg(&t.id[list[k]]);
            n += cnt;
        };
        kd_query(t, p, r2, start_nodes[j], pend[warp], stk[warp], np, 0u, vc, flush);
        if (np > 0) flush(np, pend[warp]);
        __syncwarp();
        if (lane == 0) counts[j] = n;
    }
}

// Query ordering: each query descends the tree's near sides to `level` (cells of
// n >> level photons); a counting sort by cell puts neighbouring queries in the same
// warp, which keeps the union of a warp's tree paths close to one query's path.
// The same descent also finds where the reference's traversal for this query first
// branches: the shallowest node on the near path with (q[axis] - split)^2 < r^2.  Above
// it the traversal only follows near sides and tests no median photon, so starting
// there visits exactly the same photons.  start_nodes[i] = (node, first position).
__global__ void k_query_cells(const KdNav t, const float* __restrict__ qpos, int stride, long long nq,
                              const unsigned long long* __restrict__ nq_dev, int level,
                              float r2, uint32_t* __restrict__ keys, uint32_t* __restrict__ counts,
                              uint2* __restrict__ start_nodes) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (nq_dev) nq = (long long)min(*nq_dev, (unsigned long long)nq);
    if (i >= nq) return;
    F3 q = f3(qpos[stride * i], qpos[stride * i + 1], qpos[stride * i + 2]);
    uint32_t e = 1;
    long long st = 0, c = t.n;
    uint2 start = make_uint2(0u, 0u);
    bool found = false;
    int l = 0;
    for (; l < level || !found; ++l) {
        if (c <= kBucket) {                       // reached a bucket without branching
            if (!found) { start = make_uint2(e, (uint32_t)st); found = true; }
            break;
        }
        uint2 nd = __ldg(&t.nodes[e]);
        uint32_t ax = nd.x & 0x60000000u;
        float split = __uint_as_float(nd.y);
        float qa = ax == 0 ? q.x : (ax == 0x20000000u ? q.y : q.z);
        float d = qa - split;
        if (!found && d * d < r2) { start = make_uint2(e, (uint32_t)st); found = true; }
        long long half = c >> 1, odd = c & 1;
        if (d < 0) { e = 2 * e; }
        else { e = 2 * e + 1; st += half + odd; }
        c = half;
        if (l + 1 >= level && found) { ++l; break; }
    }
    // cell key at `level` (continue the near descent if the start was found early)
    uint32_t ek = e;
    int lk = l;
    long long ck = c;
    while (lk < level) {
        if (ck <= 1) break;
        uint2 nd = __ldg(&t.nodes[ek]);
        uint32_t ax = nd.x & 0x60000000u;
        float split = __uint_as_float(nd.y);
        float qa = ax == 0 ? q.x : (ax == 0x20000000u ? q.y : q.z);
        ek = 2 * ek + ((qa - split) < 0 ? 0u : 1u);
        ck >>= 1;
        ++lk;
    }
    while (lk < level) { ek = 2 * ek; ++lk; }
    if (lk > level) ek >>= (lk - level);
    uint32_t key = ek - (1u << level);
    keys[i] = key;
    start_nodes[i] = start;
    atomicAdd(&counts[key], 1u);
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
            uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = warp_sums[lane], wi = w;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
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
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = warp_sums[lane], wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
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

__global__ void k_scatter_queries(const uint32_t* __restrict__ keys, long long nq,
                                  const unsigned long long* __restrict__ nq_dev, uint32_t* __restrict__ cursor,
                                  uint32_t* __restrict__ order) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (nq_dev) nq = (long long)min(*nq_dev, (unsigned long long)nq);
    if (i >= nq) return;
    uint32_t pos = atomicAdd(&cursor[keys[i]], 1u);
    order[pos] = (uint32_t)i;
}

// Node bounding boxes, bottom-up: a warp per node on the lowest boxed level reduces
// its contiguous photon range; each upper node unites its children and its median.
__global__ void k_leaf_boxes(const KdNav t, int level, float4* lo, float4* hi) {
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long first = 1LL << level;
    if (w >= first) return;
    const long long e = first + w;
    const long long c = t.n >> level;
    const long long s = kd_node_start(e, level, t.n);
    float mnx = INFINITY, mny = INFINITY, mnz = INFINITY, mxx = -INFINITY, mxy = -INFINITY, mxz = -INFINITY;
    for (long long i = lane; i < c; i += 32) {
        float x = t.x[s + i], y = t.y[s + i], z = t.z[s + i];
        mnx = fminf(mnx, x); mny = fminf(mny, y); mnz = fminf(mnz, z);
        mxx = fmaxf(mxx, x); mxy = fmaxf(mxy, y); mxz = fmaxf(mxz, z);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o)); mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, o)); mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o)); mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, o));
    }
    if (lane == 0) { lo[e] = make_float4(mnx, mny, mnz, 0.0f); hi[e] = make_float4(mxx, mxy, mxz, 0.0f); }
}

__global__ void k_parent_boxes(const KdNav t, int level, float4* lo, float4* hi) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long first = 1LL << level;
    if (i >= first) return;
    const long long e = first + i;
    float4 a = lo[2 * e], b = lo[2 * e + 1], c = hi[2 * e], d = hi[2 * e + 1];
    float4 l = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
    float4 h = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), 0.0f);
    const long long cnt = t.n >> level;
    if (cnt & 1) {
        const long long p = kd_node_start(e, level, t.n) + (cnt >> 1);
        l.x = fminf(l.x, t.x[p]); l.y = fminf(l.y, t.y[p]); l.z = fminf(l.z, t.z[p]);
        h.x = fmaxf(h.x, t.x[p]); h.y = fmaxf(h.y, t.y[p]); h.z = fmaxf(h.z, t.z[p]);
    }
    lo[e] = l;
    hi[e] = h;
}

// Photon records gathered into tree order, so the gather reads them contiguously.
__global__ void k_tree_records(PhotonBuf ph, const uint32_t* __restrict__ id, long long n, TreePhotons tp) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    uint32_t i = id[p];
    tp.t0[p] = ph.pos[i];
    tp.t1[p] = ph.dir[i];
    tp.t2[p] = ph.tp[i];
}

KdNav nav_of(const KdTree& tr) {
    return KdNav{tr.nodes, tr.x, tr.y, tr.z, tr.id, tr.box_lo, tr.box_hi, tr.box_lo ? tr.box_levels : 0, tr.n};
}

}  // namespace

int kd_box_levels(long long n) {
    // boxes for every level whose nodes hold more than half a bucket: the bucket level
    // (nodes of at most kBucket photons) and everything above it
    if (n <= 0) return 0;
    int l = 0;
    while ((n >> l) > kBucket) ++l;
    return l + 1;
}

void launch_kd_boxes(const KdTree& tree, cudaStream_t s, int* launches) {
    if (tree.n <= 0 || !tree.box_lo) return;
    KdNav t = nav_of(tree);
    const int lb = tree.box_levels - 1;
    const long long nodes = 1LL << lb;
    k_leaf_boxes<<<(unsigned)((nodes * 32 + 255) / 256), 256, 0, s>>>(t, lb, tree.box_lo, tree.box_hi);
    int nl = 1;
    for (int l = lb - 1; l >= 0; --l) {
        const long long cnt = 1LL << l;
        k_parent_boxes<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(t, l, tree.box_lo, tree.box_hi);
        ++nl;
    }
    if (launches) *launches += nl;
}

int query_order_level(long long nq, const KdTree& tree) {
    if (tree.n < 64 || nq <= 0) return 0;
    int lq = 0;
    while ((nq >> (lq + 1)) >= 16) ++lq;
    int lmax = tree.levels - 5;      // cells keep at least 32 photons
    if (lq > lmax) lq = lmax;
    if (lq > 24) lq = 24;
    return lq < 0 ? 0 : lq;
}

size_t query_order_scratch_bytes(long long nq, const KdTree& tree) {
    int lq = query_order_level(nq, tree);
    return 4 * (size_t)(nq > 0 ? nq : 1) + 4 * ((size_t)1 << lq) + 4 * scan_scratch_words(1LL << lq) + 512;
}

void launch_query_order(const KdTree& tree, const float* qpos, int stride, long long nq, float r2, void* scratch,
                        uint32_t* order, uint2* start_nodes, int* launches, cudaStream_t s,
                        const unsigned long long* nq_dev) {
    if (nq <= 0) return;
    int lq = query_order_level(nq, tree);
    uint32_t* keys = (uint32_t*)scratch;
    uint32_t* counts = keys + ((nq + 63) & ~63LL);
    long long m = 1LL << lq;
    cudaMemsetAsync(counts, 0, 4 * (size_t)m, s);
    unsigned g = (unsigned)((nq + 255) / 256);
    k_query_cells<<<g, 256, 0, s>>>(nav_of(tree), qpos, stride, nq, nq_dev, lq, r2, keys, counts, start_nodes);
    launch_scan_counts(counts, m, counts + ((m + 63) & ~63LL), s);
    k_scatter_queries<<<g, 256, 0, s>>>(keys, nq, nq_dev, counts, order);
    if (launches) *launches += m > 4 * kScanTile ? 5 : 3;
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

template <int MB, int QPW, int E>
void launch_gather_t(const VMParams& p, const KdNav& nav, QueryBuf qb, const uint32_t* order,
                     const uint2* start_nodes, long long nq, MergeBuf mb, unsigned long long* counters,
                     cudaStream_t s, const unsigned long long* nq_dev, const int* skip) {
    const long long warps = (nq + QPW - 1) / QPW;
    k_gather<MB, QPW, E><<<(unsigned)((warps + kWarpsPerBlock - 1) / kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(
        p, nav, qb, order, start_nodes, nq, mb, counters, nq_dev, skip);
}

unsigned merge_grid() {
    static thread_local unsigned g = 0;
    if (!g) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_merge, kMergeThreads, 0);
        g = (unsigned)(sms * (per_sm > 0 ? per_sm : 1));
    }
    return g;
}

int gather_variants() { return 8; }

const char* gather_variant_name(int v) {
    static const char* names[8] = {
        "blocks/SM>=2, 8 queries/warp, 5-level steps", "blocks/SM>=2, 16 queries/warp, 5-level steps",
        "blocks/SM>=3, 8 queries/warp, 5-level steps", "blocks/SM>=3, 16 queries/warp, 5-level steps",
        "blocks/SM>=4, 8 queries/warp, 5-level steps", "blocks/SM>=4, 16 queries/warp, 5-level steps",
        "blocks/SM>=3, 8 queries/warp, 4-level steps", "blocks/SM>=4, 8 queries/warp, 4-level steps"};
    return (v >= 0 && v < 8) ? names[v] : "?";
}

void launch_gather(const VMParams& p, const KdTree& tree, TreePhotons tp, QueryBuf qb, const uint32_t* order,
                   const uint2* start_nodes, long long nq, double* accum, unsigned long long* counters, MergeBuf mb,
                   cudaStream_t s, int variant, const unsigned long long* nq_dev, const int* skip) {
    if (nq <= 0) return;
    const KdNav nav = nav_of(tree);
    cudaMemsetAsync(mb.count, 0, sizeof(unsigned long long), s);
    switch (variant) {
    case 0: launch_gather_t<2, 8, 5>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    case 1: launch_gather_t<2, 16, 5>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    case 2: launch_gather_t<3, 8, 5>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    case 4: launch_gather_t<4, 8, 5>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    case 5: launch_gather_t<4, 16, 5>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    case 6: launch_gather_t<3, 8, 4>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    case 7: launch_gather_t<4, 8, 4>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    default: launch_gather_t<3, 16, 5>(p, nav, qb, order, start_nodes, nq, mb, counters, s, nq_dev, skip); break;
    }
    k_merge<<<merge_grid(), kMergeThreads, 0, s>>>(p, tp, qb, tree.id, mb, accum, skip);
}

void launch_kd_query(const KdTree& tree, int q, const float* qpos, const uint32_t* order, const uint2* start_nodes,
                     float r2, int* counts, const long long* offsets, int* idx, cudaStream_t s) {
    if (q <= 0) return;
    long long warps = (q + kQueriesPerWarp - 1) / kQueriesPerWarp;
    k_kd_query<<<(unsigned)((warps + kWarpsPerBlock - 1) / kWarpsPerBlock), 32 * kWarpsPerBlock, 0, s>>>(
        nav_of(tree), q, qpos, order, start_nodes, r2, counts, offsets, idx);
}

}  // namespace rc
