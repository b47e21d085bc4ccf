// Per-mesh SAH BVH build on the device (bvh_build.h).
//
// Why the result equals the host build bit for bit:
// * Box unions.  The host folds boxes with (b < a) ? b : a and (a < b) ? b : a in
//   array order.  Over finite values without -0.0 that is the minimum / maximum in any
//   order, so the reductions here run on order-preserving unsigned keys (redux.sync,
//   integer atomics).  k_prim_boxes flags every other input for the host build.
// * Split choice.  Bucket index, bucket costs (int count x float area, the 0.16874
//   constant added in double) and the first-minimum selection use the host's
//   expressions in the host's order (device code is compiled with -fmad=false).
// * Partition order.  std::partition (libstdc++, bidirectional form) swaps the k-th
//   element failing the predicate, counted from the left, with the k-th element
//   passing it, counted from the right, until the two scans meet.  Both ranks come
//   from scans of the predicate, so every moved element knows its slot.
// * Pre-order numbering.  Every node covers a contiguous range [start, end) of the
//   triangle order.  Node v follows every node whose range starts before start(v) and
//   its own ancestors with the same start (a chain of left children), so
//   pre(v) = #{nodes with start < start(v)} + depth(v) - depth(chain top at start(v)).
//   The right child of v starts at mid(v) and tops its chain:
//   pre(right) = #{nodes with start < mid(v)}; the left child is pre(v) + 1.
// * Traversal cost.  Bottom-up from the leaves: of the two children, the one that
//   finishes second computes the parent (per-node arrival counter; nothing waits).
//
// Work split.  Segments of more than kSmall (256) triangles go through level passes
// over 2048-triangle chunks (bounds, bins, decision, partition, swap); smaller segments
// are finished by one warp each, depth first, with the pending right halves on a stack
// kept in the segment's own slice of a global array.  (A warp walks its subtree node by
// node at L2 latency, so the per-warp size is kept small enough for thousands of warps
// to share the subtrees.)
#include "bvh_build.h"

#include <algorithm>
#include <cstring>

#include "realcaustics.h"

namespace rc {

namespace {

constexpr int kBins = 12;
constexpr int kSmall = 256;
constexpr int kChunk = 2048;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxGrid = 152 * 8;
constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kKeyPosInf = 0xFF800000u;   // key(+inf): identity of a minimum
constexpr uint32_t kKeyNegInf = 0x007FFFFFu;   // key(-inf): identity of a maximum
constexpr int kFlagInput = 1;     // non-finite or -0.0 box coordinate: host build
constexpr int kFlagPool = 2;      // node record pool exhausted
constexpr int kFlagIndex = 4;     // an index failed its range check (not expected)

// Monotone map float -> unsigned: a < b (as floats, no NaN, no -0.0) iff key(a) < key(b).
__device__ __forceinline__ uint32_t fkey(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float kfloat(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__host__ __device__ constexpr bool key_is_min(int j) { return (j % 6) < 3; }

// 12 keys: box min xyz, box max xyz, centroid min xyz, centroid max xyz.
struct Keys12 {
    uint32_t v[12];
};

__device__ __forceinline__ void keys_init(Keys12& k) {
#pragma unroll
    for (int j = 0; j < 12; ++j) k.v[j] = key_is_min(j) ? kKeyPosInf : kKeyNegInf;
}

// Prim center: (box.mn + box.mx) * (1 / 2.0f)  (the host's build_mesh_bvh)
__device__ __forceinline__ float3 centroid(const float4& lo, const float4& hi) {
    return make_float3((lo.x + hi.x) * 0.5f, (lo.y + hi.y) * 0.5f, (lo.z + hi.z) * 0.5f);
}
__device__ __forceinline__ float comp(const float3& c, int d) { return d == 0 ? c.x : (d == 1 ? c.y : c.z); }

__device__ __forceinline__ void keys_add(Keys12& k, const float4& lo, const float4& hi) {
    const float3 c = centroid(lo, hi);
    k.v[0] = min(k.v[0], fkey(lo.x)); k.v[1] = min(k.v[1], fkey(lo.y)); k.v[2] = min(k.v[2], fkey(lo.z));
    k.v[3] = max(k.v[3], fkey(hi.x)); k.v[4] = max(k.v[4], fkey(hi.y)); k.v[5] = max(k.v[5], fkey(hi.z));
    k.v[6] = min(k.v[6], fkey(c.x)); k.v[7] = min(k.v[7], fkey(c.y)); k.v[8] = min(k.v[8], fkey(c.z));
    k.v[9] = max(k.v[9], fkey(c.x)); k.v[10] = max(k.v[10], fkey(c.y)); k.v[11] = max(k.v[11], fkey(c.z));
}

__device__ __forceinline__ void keys_warp_reduce(Keys12& k) {
#pragma unroll
    for (int j = 0; j < 12; ++j) k.v[j] = key_is_min(j) ? __reduce_min_sync(kFull, k.v[j]) : __reduce_max_sync(kFull, k.v[j]);
}

// aabb::SurfaceArea (src/aabb.cpp:54-58)
__device__ __forceinline__ float surface_area(float mnx, float mny, float mnz, float mxx, float mxy, float mxz) {
    const float dx = mxx - mnx, dy = mxy - mny, dz = mxz - mnz;
    return 2.0f * (dx * dy + dx * dz + dy * dz);
}
__device__ __forceinline__ float surface_area(const float4& lo, const float4& hi) {
    return surface_area(lo.x, lo.y, lo.z, hi.x, hi.y, hi.z);
}
__device__ __forceinline__ float keys_box_area(const Keys12& k) {
    return surface_area(kfloat(k.v[0]), kfloat(k.v[1]), kfloat(k.v[2]), kfloat(k.v[3]), kfloat(k.v[4]), kfloat(k.v[5]));
}

// aabb::MaximumExtent (src/aabb.cpp:60-69) of the centroid bounds
__device__ __forceinline__ int keys_split_axis(const Keys12& k, float& lo, float& hi) {
    const float mnx = kfloat(k.v[6]), mny = kfloat(k.v[7]), mnz = kfloat(k.v[8]);
    const float mxx = kfloat(k.v[9]), mxy = kfloat(k.v[10]), mxz = kfloat(k.v[11]);
    const float dx = mxx - mnx, dy = mxy - mny, dz = mxz - mnz;
    int d = 2;
    if (dx > dy && dx > dz) d = 0;
    else if (dy > dz) d = 1;
    lo = d == 0 ? mnx : (d == 1 ? mny : mnz);
    hi = d == 0 ? mxx : (d == 1 ? mxy : mxz);
    return d;
}

// Bucket of a centroid coordinate (src/BVH/BVH_mesh.cpp:98-101)
__device__ __forceinline__ int bucket_of(float c, float lo, float hi) {
    const float o = (c - lo) / (hi - lo);
    const int b = (int)(12.0f * o);
    return b == 12 ? 11 : b;
}

// Bucket costs and the split choice (src/BVH/BVH_mesh.cpp:103-131) with lane j < 12
// holding bucket j (count, box keys); lanes >= 12 hold empty buckets.  Returns the
// chosen bucket (the split puts buckets <= it on the left) or -1 for a leaf, in every
// lane.
__device__ int warp_choose_split(int cnt, const uint32_t (&bk)[6], float sa, int n, int lane) {
    int pc = cnt, sc = cnt;
    uint32_t p[6], q[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) { p[j] = bk[j]; q[j] = bk[j]; }
    // inclusive prefix (buckets 0..lane) and suffix (buckets lane..11) unions
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
        const int pu = __shfl_up_sync(kFull, pc, off);
        const int sd = __shfl_down_sync(kFull, sc, off);
        if (lane >= off) pc += pu;
        if (lane + off < 32) sc += sd;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const uint32_t u = __shfl_up_sync(kFull, p[j], off);
            const uint32_t d = __shfl_down_sync(kFull, q[j], off);
            if (lane >= off) p[j] = j < 3 ? min(p[j], u) : max(p[j], u);
            if (lane + off < 32) q[j] = j < 3 ? min(q[j], d) : max(q[j], d);
        }
    }
    const int c1 = __shfl_down_sync(kFull, sc, 1);
    uint32_t r[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) r[j] = __shfl_down_sync(kFull, q[j], 1);
    float cost = 0.0f;
    if (lane < kBins - 1) {
        const float a0 = surface_area(kfloat(p[0]), kfloat(p[1]), kfloat(p[2]), kfloat(p[3]), kfloat(p[4]), kfloat(p[5]));
        const float a1 = surface_area(kfloat(r[0]), kfloat(r[1]), kfloat(r[2]), kfloat(r[3]), kfloat(r[4]), kfloat(r[5]));
        // cost[i] = 0.16874 + (c0 * SA(b0) + c1 * SA(b1)) / SA(node), stored as float
        const float num = (float)pc * a0 + (float)c1 * a1;
        cost = (float)(0.16874 + (double)(num / sa));
    }
    float min_cost = __shfl_sync(kFull, cost, 0);
    int mb = 0;
    for (int i = 1; i < kBins - 1; ++i) {
        const float ci = __shfl_sync(kFull, cost, i);
        if (ci < min_cost) { min_cost = ci; mb = i; }
    }
    return (min_cost < (float)n) ? mb : -1;   // leaf cost = number of triangles
}

struct __align__(16) NodeRec {
    float4 lo;         // box min xyz
    float4 hi;         // box max xyz
    int start, depth;  // range start; depth below the mesh root (< 0: unused slot)
    int count, mid;    // count > 0: leaf of `count` triangles; count < 0: split at mid
};

struct SegState {
    int start, end, depth, chunk0;
    int nchunks, split, mid, T;
    int K, pad0, pad1, pad2;
    uint32_t keys[12];
    int count[kBins];
    uint32_t bin[kBins][6];
};

struct View {
    uint32_t* perm;
    const float4* blo;
    const float4* bhi;
    uint32_t* tf; int* pf;   // failing elements left of the split: triangle, position (by rank)
    uint32_t* tt; int* pt;   // passing elements right of the split: triangle, position (by rank)
    int4* stack;
    NodeRec* small_pool;
    NodeRec* large_pool;
    int* large_count;
    int large_cap;
    int* cnt;                // nodes starting at each position
    int* topd;               // smallest depth of a node starting at each position
    int* flags;
    int n;
    int next_cap, small_cap;   // capacities of the next-level and per-warp segment lists
};

__device__ __forceinline__ void record_node(NodeRec* rec, const Keys12& k, int start, int depth, int count, int mid,
                                            int* cnt, int* topd) {
    NodeRec r;
    r.lo = make_float4(kfloat(k.v[0]), kfloat(k.v[1]), kfloat(k.v[2]), 0.0f);
    r.hi = make_float4(kfloat(k.v[3]), kfloat(k.v[4]), kfloat(k.v[5]), 0.0f);
    r.start = start; r.depth = depth; r.count = count; r.mid = mid;
    *rec = r;
    atomicAdd(&cnt[start], 1);
    atomicMin(&topd[start], depth);
}

__device__ __forceinline__ int find_mesh(const uint32_t* tri_off, int M, uint32_t t) {
    int lo = 0, hi = M - 1;
    while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (tri_off[m] <= t) lo = m; else hi = m - 1;
    }
    return lo;
}

__device__ __forceinline__ float ref_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float ref_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ bool plain(float f) { return isfinite(f) && __float_as_uint(f) != 0x80000000u; }

// Triangle::bounding_box (src/Triangle.cpp:90-106) per triangle, in triangle order.
__global__ void k_prim_boxes(const float* __restrict__ wpos, const uint32_t* __restrict__ tri,
                             const uint32_t* __restrict__ tri_off, const uint32_t* __restrict__ vert_off, int M, int N,
                             float4* blo, float4* bhi, uint32_t* perm, int* flags) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
        const uint32_t vo = vert_off[find_mesh(tri_off, M, (uint32_t)t)];
        const size_t ia = 3 * (size_t)(tri[3 * (size_t)t] + vo);
        const size_t ib = 3 * (size_t)(tri[3 * (size_t)t + 1] + vo);
        const size_t ic = 3 * (size_t)(tri[3 * (size_t)t + 2] + vo);
        const float ax = wpos[ia], ay = wpos[ia + 1], az = wpos[ia + 2];
        const float bx = wpos[ib], by = wpos[ib + 1], bz = wpos[ib + 2];
        const float cx = wpos[ic], cy = wpos[ic + 1], cz = wpos[ic + 2];
        const float4 lo = make_float4(ref_min(ref_min(ax, bx), cx), ref_min(ref_min(ay, by), cy),
                                      ref_min(ref_min(az, bz), cz), 0.0f);
        const float4 hi = make_float4(ref_max(ref_max(ax, bx), cx), ref_max(ref_max(ay, by), cy),
                                      ref_max(ref_max(az, bz), cz), 0.0f);
        const float3 c = centroid(lo, hi);
        const bool ok = plain(lo.x) && plain(lo.y) && plain(lo.z) && plain(hi.x) && plain(hi.y) && plain(hi.z) &&
                        plain(c.x) && plain(c.y) && plain(c.z);
        if (!ok) atomicOr(flags, kFlagInput);
        blo[t] = lo;
        bhi[t] = hi;
        perm[t] = (uint32_t)t;
    }
}

// Inclusive warp scan of ints.
__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int u = __shfl_up_sync(kFull, v, off);
        if (lane >= off) v += u;
    }
    return v;
}

// Block-wide exclusive scan (NT threads); `total` receives the block sum.  Ends with a
// barrier, so the scratch can be reused right away.
template <int NT>
__device__ __forceinline__ int block_excl_scan(int v, int& total, int* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int incl = warp_incl_scan(v, lane);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int w = lane < NT / 32 ? s_warp[lane] : 0;
        const int wi = warp_incl_scan(w, lane);
        if (lane < NT / 32) s_warp[lane] = wi - w;
        if (lane == 31) s_warp[NT / 32] = wi;
    }
    __syncthreads();
    const int r = s_warp[warp] + incl - v;
    total = s_warp[NT / 32];
    __syncthreads();
    return r;
}

// ---- level passes over segments of more than kSmall triangles ----------------------

// Segment states and the chunk list of one level.
// The level's segment count is read on the device (levels are enqueued several at a
// time; a level without segments does nothing); the next level's list is emptied here.
__global__ void __launch_bounds__(1024) k_lvl_setup(const int4* segs, const int* nseg_ptr, int* next_count,
                                                    SegState* st, int2* chunks, int* nchunks, int* levels) {
    __shared__ int s_warp[33];
    __shared__ int s_base;
    const int nseg = *nseg_ptr;
    if (threadIdx.x == 0) {
        s_base = 0;
        *next_count = 0;
        if (nseg > 0) atomicAdd(levels, 1);
    }
    __syncthreads();
    for (int t0 = 0; t0 < nseg; t0 += blockDim.x) {
        const int i = t0 + threadIdx.x;
        int4 sg = make_int4(0, 0, 0, 0);
        int nc = 0;
        if (i < nseg) {
            sg = segs[i];
            nc = (sg.y - sg.x + kChunk - 1) / kChunk;
        }
        int total;
        const int excl = block_excl_scan<1024>(nc, total, s_warp);
        if (i < nseg) {
            SegState& s = st[i];
            s.start = sg.x; s.end = sg.y; s.depth = sg.z;
            s.chunk0 = s_base + excl; s.nchunks = nc;
            s.split = -1; s.mid = -1; s.T = 0; s.K = 0;
            for (int j = 0; j < 12; ++j) s.keys[j] = key_is_min(j) ? kKeyPosInf : kKeyNegInf;
            for (int b = 0; b < kBins; ++b) {
                s.count[b] = 0;
                for (int j = 0; j < 6; ++j) s.bin[b][j] = j < 3 ? kKeyPosInf : kKeyNegInf;
            }
            for (int c = 0; c < nc; ++c) chunks[s.chunk0 + c] = make_int2(i, sg.x + c * kChunk);
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *nchunks = s_base;
}

// Box and centroid bounds of every segment.
__global__ void __launch_bounds__(kThreads) k_lvl_bounds(SegState* st, const int2* chunks, const int* nchunks, View V) {
    __shared__ uint32_t red[kWarps][12];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nc = *nchunks;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int2 ch = chunks[c];
        SegState& s = st[ch.x];
        const int end = min(ch.y + kChunk, s.end);
        Keys12 k;
        keys_init(k);
        for (int i = ch.y + threadIdx.x; i < end; i += kThreads) {
            const uint32_t t = V.perm[i];
            keys_add(k, V.blo[t], V.bhi[t]);
        }
        keys_warp_reduce(k);
        if (lane == 0)
            for (int j = 0; j < 12; ++j) red[warp][j] = k.v[j];
        __syncthreads();
        if (threadIdx.x < 12) {
            const int j = threadIdx.x;
            uint32_t v = red[0][j];
            for (int w = 1; w < kWarps; ++w) v = key_is_min(j) ? min(v, red[w][j]) : max(v, red[w][j]);
            if (key_is_min(j)) atomicMin(&s.keys[j], v);
            else atomicMax(&s.keys[j], v);
        }
        __syncthreads();
    }
}

// Bucket counts and boxes of every segment (and per chunk, the counts).
__global__ void __launch_bounds__(kThreads) k_lvl_bins(SegState* st, const int2* chunks, const int* nchunks, View V,
                                                       int* chunk_cnt) {
    __shared__ int s_cnt[kBins];
    __shared__ uint32_t s_bin[kBins][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nc = *nchunks;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int2 ch = chunks[c];
        SegState& s = st[ch.x];
        Keys12 sk;
#pragma unroll
        for (int j = 6; j < 12; ++j) sk.v[j] = s.keys[j];
        float clo, chi;
        const int dim = keys_split_axis(sk, clo, chi);
        if (clo == chi) continue;   // leaf (same for every thread of the block)
        const int end = min(ch.y + kChunk, s.end);
        if (threadIdx.x < kBins) {
            s_cnt[threadIdx.x] = 0;
            for (int j = 0; j < 6; ++j) s_bin[threadIdx.x][j] = j < 3 ? kKeyPosInf : kKeyNegInf;
        }
        __syncthreads();
        for (int base = ch.y + warp * 32; base < end; base += kThreads) {
            const int i = base + lane;
            const bool valid = i < end;
            float4 lo = make_float4(0, 0, 0, 0), hi = lo;
            int bkt = 0;
            if (valid) {
                const uint32_t t = V.perm[i];
                lo = V.blo[t];
                hi = V.bhi[t];
                bkt = bucket_of(comp(centroid(lo, hi), dim), clo, chi);
            }
            unsigned pending = __ballot_sync(kFull, valid);
            while (pending) {
                const int leader = __ffs(pending) - 1;
                const int bl = __shfl_sync(kFull, bkt, leader);
                const bool in = valid && bkt == bl;
                const unsigned m = __ballot_sync(kFull, in);
                const uint32_t r0 = __reduce_min_sync(kFull, in ? fkey(lo.x) : kKeyPosInf);
                const uint32_t r1 = __reduce_min_sync(kFull, in ? fkey(lo.y) : kKeyPosInf);
                const uint32_t r2 = __reduce_min_sync(kFull, in ? fkey(lo.z) : kKeyPosInf);
                const uint32_t r3 = __reduce_max_sync(kFull, in ? fkey(hi.x) : kKeyNegInf);
                const uint32_t r4 = __reduce_max_sync(kFull, in ? fkey(hi.y) : kKeyNegInf);
                const uint32_t r5 = __reduce_max_sync(kFull, in ? fkey(hi.z) : kKeyNegInf);
                if (lane == leader) {
                    atomicAdd(&s_cnt[bl], __popc(m));
                    atomicMin(&s_bin[bl][0], r0); atomicMin(&s_bin[bl][1], r1); atomicMin(&s_bin[bl][2], r2);
                    atomicMax(&s_bin[bl][3], r3); atomicMax(&s_bin[bl][4], r4); atomicMax(&s_bin[bl][5], r5);
                }
                pending &= ~m;
            }
        }
        __syncthreads();
        if (threadIdx.x < kBins) {
            const int b = threadIdx.x;
            chunk_cnt[(size_t)c * kBins + b] = s_cnt[b];
            if (s_cnt[b]) {
                atomicAdd(&s.count[b], s_cnt[b]);
                for (int j = 0; j < 3; ++j) atomicMin(&s.bin[b][j], s_bin[b][j]);
                for (int j = 3; j < 6; ++j) atomicMax(&s.bin[b][j], s_bin[b][j]);
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void push_child(int a, int b, int depth, int4* next, int* nnext, int4* small, int* nsmall,
                                           const View& V) {
    if (b - a > kSmall) {
        const int i = atomicAdd(nnext, 1);
        if (i < V.next_cap) next[i] = make_int4(a, b, depth, 0);
        else atomicOr(V.flags, kFlagIndex);
    } else {
        const int i = atomicAdd(nsmall, 1);
        if (i < V.small_cap) small[i] = make_int4(a, b, depth, 0);
        else atomicOr(V.flags, kFlagIndex);
    }
}

// One warp: split choice of a segment, its node record, its children, and the
// per-chunk rank offsets of its partition.
__device__ void decide_segment(SegState& s, const int* chunk_cnt, int* chunk_off, const View& V, int4* next,
                               int* nnext, int4* small, int* nsmall) {
    const int lane = threadIdx.x & 31;
    const int n = s.end - s.start;
    Keys12 k;
#pragma unroll
    for (int j = 0; j < 12; ++j) k.v[j] = s.keys[j];
    float clo, chi;
    keys_split_axis(k, clo, chi);
    int mb = -1, T = 0;
    if (clo != chi) {
        const int bc = lane < kBins ? s.count[lane] : 0;
        uint32_t bk[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) bk[j] = lane < kBins ? s.bin[lane][j] : (j < 3 ? kKeyPosInf : kKeyNegInf);
        mb = warp_choose_split(bc, bk, keys_box_area(k), n, lane);
        if (mb >= 0) T = __reduce_add_sync(kFull, lane <= mb ? bc : 0);
        if (mb >= 0 && (T <= 0 || T >= n)) {   // a chosen split has both sides non-empty
            if (lane == 0) atomicOr(V.flags, kFlagIndex);
            mb = -1;
        }
    }
    const int mid = mb >= 0 ? s.start + T : -1;
    if (mb >= 0) {
        int run = 0;
        for (int c0 = 0; c0 < s.nchunks; c0 += 32) {
            const int c = c0 + lane;
            int tr = 0;
            if (c < s.nchunks)
                for (int b = 0; b <= mb; ++b) tr += chunk_cnt[(size_t)(s.chunk0 + c) * kBins + b];
            const int incl = warp_incl_scan(tr, lane);
            if (c < s.nchunks) chunk_off[s.chunk0 + c] = run + incl - tr;
            run += __shfl_sync(kFull, incl, 31);
        }
    }
    if (lane == 0) {
        s.split = mb;
        s.mid = mid;
        s.T = T;
        const int idx = atomicAdd(V.large_count, 1);
        if (idx < V.large_cap) record_node(V.large_pool + idx, k, s.start, s.depth, mb < 0 ? n : -1, mid, V.cnt, V.topd);
        else atomicOr(V.flags, kFlagPool);
        if (mb >= 0) {
            push_child(s.start, mid, s.depth + 1, next, nnext, small, nsmall, V);
            push_child(mid, s.end, s.depth + 1, next, nnext, small, nsmall, V);
        }
    }
}

// One warp per segment.
__global__ void __launch_bounds__(kThreads) k_lvl_decide(SegState* st, const int* nseg_ptr, const int* chunk_cnt,
                                                         int* chunk_off, View V, int4* next, int* nnext, int4* small,
                                                         int* nsmall) {
    const int nseg = *nseg_ptr;
    for (int w = blockIdx.x * kWarps + (threadIdx.x >> 5); w < nseg; w += gridDim.x * kWarps)
        decide_segment(st[w], chunk_cnt, chunk_off, V, next, nnext, small, nsmall);
}

// Ranks of the elements that move, written to the swap tables.
__global__ void __launch_bounds__(kThreads) k_lvl_partition(SegState* st, const int2* chunks, const int* nchunks,
                                                            const int* chunk_off, View V) {
    __shared__ int s_warp[kWarps + 1];
    __shared__ int s_run, s_kfl;
    const int nc = *nchunks;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int2 ch = chunks[c];
        SegState& s = st[ch.x];
        const int mb = s.split;
        if (mb < 0) continue;
        Keys12 sk;
#pragma unroll
        for (int j = 6; j < 12; ++j) sk.v[j] = s.keys[j];
        float clo, chi;
        const int dim = keys_split_axis(sk, clo, chi);
        const int start = s.start, mid = s.mid, T = s.T;
        const int end = min(ch.y + kChunk, s.end);
        if (threadIdx.x == 0) { s_run = 0; s_kfl = 0; }
        __syncthreads();
        const int off = chunk_off[c];
        for (int base = ch.y; base < end; base += kThreads) {
            const int i = base + threadIdx.x;
            const bool valid = i < end;
            uint32_t t = 0;
            bool pred = false;
            if (valid) {
                t = V.perm[i];
                pred = bucket_of(comp(centroid(V.blo[t], V.bhi[t]), dim), clo, chi) <= mb;
            }
            int total;
            const int excl = block_excl_scan<kThreads>(pred ? 1 : 0, total, s_warp);
            const int true_rank = off + s_run + excl;
            const bool left_fail = valid && i < mid && !pred;
            if (left_fail) {
                const int kk = (i - start) - true_rank;
                if (kk >= 0 && start + kk < s.end) { V.tf[start + kk] = t; V.pf[start + kk] = i; }
                else atomicOr(V.flags, kFlagIndex);
            }
            if (valid && i >= mid && pred) {
                const int kk = T - 1 - true_rank;
                if (kk >= 0 && start + kk < s.end) { V.tt[start + kk] = t; V.pt[start + kk] = i; }
                else atomicOr(V.flags, kFlagIndex);
            }
            const unsigned lf = __ballot_sync(kFull, left_fail);
            if ((threadIdx.x & 31) == 0 && lf) atomicAdd(&s_kfl, __popc(lf));
            __syncthreads();
            if (threadIdx.x == 0) s_run += total;
            __syncthreads();
        }
        if (threadIdx.x == 0 && s_kfl) atomicAdd(&s.K, s_kfl);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads) k_lvl_swap(SegState* st, const int2* chunks, const int* nchunks, View V) {
    const int nc = *nchunks;
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int2 ch = chunks[c];
        const SegState& s = st[ch.x];
        if (s.split < 0) continue;
        const int start = s.start, K = s.K;
        const int end = min(ch.y + kChunk, s.end);
        for (int i = ch.y + threadIdx.x; i < end; i += kThreads) {
            const int kk = i - start;
            if (kk >= K) break;
            const int pf = V.pf[start + kk], pt = V.pt[start + kk];
            if (pf < start || pf >= s.end || pt < start || pt >= s.end) { atomicOr(V.flags, kFlagIndex); continue; }
            V.perm[pf] = V.tt[start + kk];
            V.perm[pt] = V.tf[start + kk];
        }
    }
}

// ---- one warp per segment of at most kSmall triangles -------------------------------

__global__ void __launch_bounds__(kThreads) k_small_build(const int4* segs, const int* nsegs, View V) {
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * kWarps;
    const int count = *nsegs;
    for (int w = blockIdx.x * kWarps + (threadIdx.x >> 5); w < count; w += nw) {
        const int4 sg = segs[w];
        const int s0 = sg.x, e0 = sg.y;
        NodeRec* pool = V.small_pool + 2 * (size_t)s0;
        int4* stack = V.stack + s0;
        int sp = 0, slot = 0;
        int a = sg.x, b = sg.y, depth = sg.z;
        bool bad = false;
        while (true) {
            const int n = b - a;
            Keys12 k;
            keys_init(k);
            for (int i = a + lane; i < b; i += 32) {
                const uint32_t t = V.perm[i];
                keys_add(k, V.blo[t], V.bhi[t]);
            }
            keys_warp_reduce(k);
            int split_mid = -1;
            if (n > 1) {
                float clo, chi;
                const int dim = keys_split_axis(k, clo, chi);
                if (clo != chi) {
                    if (n == 2) {
                        // two triangles: ordered by centroid (src/BVH/BVH_mesh.cpp:80-88)
                        if (lane == 0) {
                            const uint32_t t0 = V.perm[a], t1 = V.perm[a + 1];
                            const float c0 = comp(centroid(V.blo[t0], V.bhi[t0]), dim);
                            const float c1 = comp(centroid(V.blo[t1], V.bhi[t1]), dim);
                            if (!(c0 < c1)) { V.perm[a] = t1; V.perm[a + 1] = t0; }
                        }
                        __syncwarp();
                        split_mid = a + 1;
                    } else {
                        int bc = 0;
                        uint32_t bk[6] = {kKeyPosInf, kKeyPosInf, kKeyPosInf, kKeyNegInf, kKeyNegInf, kKeyNegInf};
                        for (int base = a; base < b; base += 32) {
                            const int i = base + lane;
                            const bool valid = i < b;
                            float4 lo = make_float4(0, 0, 0, 0), hi = lo;
                            int bkt = 0;
                            if (valid) {
                                const uint32_t t = V.perm[i];
                                lo = V.blo[t];
                                hi = V.bhi[t];
                                bkt = bucket_of(comp(centroid(lo, hi), dim), clo, chi);
                            }
                            unsigned pending = __ballot_sync(kFull, valid);
                            while (pending) {
                                const int leader = __ffs(pending) - 1;
                                const int bl = __shfl_sync(kFull, bkt, leader);
                                const bool in = valid && bkt == bl;
                                const unsigned m = __ballot_sync(kFull, in);
                                const uint32_t r0 = __reduce_min_sync(kFull, in ? fkey(lo.x) : kKeyPosInf);
                                const uint32_t r1 = __reduce_min_sync(kFull, in ? fkey(lo.y) : kKeyPosInf);
                                const uint32_t r2 = __reduce_min_sync(kFull, in ? fkey(lo.z) : kKeyPosInf);
                                const uint32_t r3 = __reduce_max_sync(kFull, in ? fkey(hi.x) : kKeyNegInf);
                                const uint32_t r4 = __reduce_max_sync(kFull, in ? fkey(hi.y) : kKeyNegInf);
                                const uint32_t r5 = __reduce_max_sync(kFull, in ? fkey(hi.z) : kKeyNegInf);
                                if (lane == bl) {
                                    bc += __popc(m);
                                    bk[0] = min(bk[0], r0); bk[1] = min(bk[1], r1); bk[2] = min(bk[2], r2);
                                    bk[3] = max(bk[3], r3); bk[4] = max(bk[4], r4); bk[5] = max(bk[5], r5);
                                }
                                pending &= ~m;
                            }
                        }
                        int mb = warp_choose_split(bc, bk, keys_box_area(k), n, lane);
                        const int T = __reduce_add_sync(kFull, (mb >= 0 && lane <= mb) ? bc : 0);
                        if (mb >= 0 && (T <= 0 || T >= n)) { bad = true; mb = -1; }
                        if (mb >= 0) {
                            const int m = a + T;
                            int run = 0, kfl = 0;
                            for (int base = a; base < b; base += 32) {
                                const int i = base + lane;
                                const bool valid = i < b;
                                uint32_t t = 0;
                                bool pred = false;
                                if (valid) {
                                    t = V.perm[i];
                                    pred = bucket_of(comp(centroid(V.blo[t], V.bhi[t]), dim), clo, chi) <= mb;
                                }
                                const unsigned bt = __ballot_sync(kFull, pred);
                                const int true_rank = run + __popc(bt & ((1u << lane) - 1u));
                                const bool left_fail = valid && i < m && !pred;
                                if (left_fail) {
                                    const int kk = (i - a) - true_rank;
                                    if (kk >= 0 && kk < n) { V.tf[a + kk] = t; V.pf[a + kk] = i; }
                                    else bad = true;
                                }
                                if (valid && i >= m && pred) {
                                    const int kk = T - 1 - true_rank;
                                    if (kk >= 0 && kk < n) { V.tt[a + kk] = t; V.pt[a + kk] = i; }
                                    else bad = true;
                                }
                                kfl += __popc(__ballot_sync(kFull, left_fail));
                                run += __popc(bt);
                            }
                            __syncwarp();
                            for (int kk = lane; kk < kfl && kk < n; kk += 32) {
                                const int pf = V.pf[a + kk], pt = V.pt[a + kk];
                                if (pf < a || pf >= b || pt < a || pt >= b) { bad = true; continue; }
                                V.perm[pf] = V.tt[a + kk];
                                V.perm[pt] = V.tf[a + kk];
                            }
                            __syncwarp();
                            split_mid = m;
                        }
                    }
                }
            }
            if (slot >= 2 * (e0 - s0) || (split_mid >= 0 && sp >= e0 - s0)) { bad = true; break; }
            if (lane == 0) record_node(pool + slot, k, a, depth, split_mid < 0 ? n : -1, split_mid, V.cnt, V.topd);
            ++slot;
            if (split_mid >= 0) {
                if (lane == 0) stack[sp] = make_int4(split_mid, b, depth + 1, 0);
                ++sp;
                b = split_mid;
                depth += 1;
            } else {
                if (sp == 0) break;
                --sp;
                __syncwarp();
                const int4 e = stack[sp];
                a = e.x; b = e.y; depth = e.z;
            }
        }
        if (__any_sync(kFull, bad) && lane == 0) atomicOr(V.flags, kFlagIndex);
    }
}

// ---- node numbering, output ----------------------------------------------------------

constexpr int kScanTile = 4096;   // 1024 threads x 4

__global__ void __launch_bounds__(1024) k_scan_tiles(const int* in, int n, int* out, int* tile_sum) {
    __shared__ int s_warp[33];
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    int v[4], sum = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) { v[j] = base + j < n ? in[base + j] : 0; sum += v[j]; }
    int total;
    int run = block_excl_scan<1024>(sum, total, s_warp);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int* tile_sum, int ntiles, int* out, int n) {
    __shared__ int s_warp[33];
    __shared__ int s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int t0 = 0; t0 < ntiles; t0 += 1024) {
        const int i = t0 + threadIdx.x;
        const int v = i < ntiles ? tile_sum[i] : 0;
        int total;
        const int e = block_excl_scan<1024>(v, total, s_warp);
        if (i < ntiles) tile_sum[i] = s_carry + e;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = s_carry;
}

__global__ void __launch_bounds__(1024) k_scan_add(int* out, int n, const int* tile_off) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * 4;
    const int o = tile_off[blockIdx.x];
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (base + j < n) out[base + j] += o;
}

__global__ void k_emit(const NodeRec* small_pool, long long nsmall, const NodeRec* large_pool, const int* large_count,
                       int large_cap, const int* prefix, const int* topd, long long nn, float4* nodes, int* parent,
                       int* flags) {
    const long long total = nsmall + min(*large_count, large_cap);
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < total;
         r += (long long)gridDim.x * blockDim.x) {
        const NodeRec rec = r < nsmall ? small_pool[r] : large_pool[r - nsmall];
        if (rec.depth < 0) continue;
        const long long pre = (long long)prefix[rec.start] + rec.depth - topd[rec.start];
        uint32_t w0, w1;
        if (rec.count > 0) {
            w0 = 0x80000000u | (uint32_t)rec.count;
            w1 = (uint32_t)rec.start;
        } else {
            const long long right = prefix[rec.mid];
            if (pre + 1 >= nn || right >= nn) { atomicOr(flags, kFlagIndex); continue; }
            w0 = (uint32_t)(pre + 1);
            w1 = (uint32_t)right;
            parent[pre + 1] = (int)pre;
            parent[right] = (int)pre;
        }
        if (pre < 0 || pre >= nn) { atomicOr(flags, kFlagIndex); continue; }
        nodes[2 * pre] = make_float4(rec.lo.x, rec.lo.y, rec.lo.z, __uint_as_float(w0));
        nodes[2 * pre + 1] = make_float4(rec.hi.x, rec.hi.y, rec.hi.z, __uint_as_float(w1));
    }
}

// CostOfTraversing (src/BVH/BVH_mesh.cpp:286-305) bottom-up.
__global__ void k_cost(const float4* __restrict__ nodes, const int* __restrict__ parent, long long nn, int* arrive,
                       float* cost, int* flags) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nn; v += (long long)gridDim.x * blockDim.x) {
        const uint32_t w0 = __float_as_uint(nodes[2 * v].w);
        if (!(w0 & 0x80000000u)) continue;
        float c = (float)(w0 & 0x7fffffffu);
        __stcg(&cost[v], c);
        long long cur = v;
        for (long long steps = 0;; ++steps) {
            const int p = parent[cur];
            if (p < 0) break;
            if (steps >= nn) { atomicOr(flags, kFlagIndex); break; }   // a cycle: not a tree
            if (p >= nn) { atomicOr(flags, kFlagIndex); break; }
            __threadfence();
            if (atomicAdd(&arrive[p], 1) == 0) break;   // the sibling subtree finishes the parent
            __threadfence();
            const float4 pl = nodes[2 * p], ph = nodes[2 * p + 1];
            const uint32_t l = __float_as_uint(pl.w), r = __float_as_uint(ph.w);
            if (l >= nn || r >= nn) { atomicOr(flags, kFlagIndex); break; }
            const float a = surface_area(pl, ph);
            const float la = surface_area(nodes[2 * l], nodes[2 * l + 1]);
            const float ra = surface_area(nodes[2 * r], nodes[2 * r + 1]);
            c = (float)(0.16874 + (double)((__ldcg(&cost[l]) * la + __ldcg(&cost[r]) * ra) / a));
            __stcg(&cost[p], c);
            cur = p;
        }
    }
}

// Triangle records in leaf order (the upload layout of the host path).
__global__ void k_pack_tris(const uint32_t* __restrict__ perm, const float* __restrict__ wpos,
                            const float* __restrict__ wnrm, const uint32_t* __restrict__ tri,
                            const uint32_t* __restrict__ mat, const uint32_t* __restrict__ tri_off,
                            const uint32_t* __restrict__ vert_off, int M, int N, float4* tris, float4* n0,
                            float4* n1, float4* n2) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
        const uint32_t t = perm[j];
        const int m = find_mesh(tri_off, M, t);
        const uint32_t vo = vert_off[m];
        const size_t ia = 3 * (size_t)(tri[3 * (size_t)t] + vo);
        const size_t ib = 3 * (size_t)(tri[3 * (size_t)t + 1] + vo);
        const size_t ic = 3 * (size_t)(tri[3 * (size_t)t + 2] + vo);
        const float ax = wpos[ia], ay = wpos[ia + 1], az = wpos[ia + 2];
        tris[3 * (size_t)j] = make_float4(ax, ay, az, __uint_as_float(t));
        tris[3 * (size_t)j + 1] = make_float4(wpos[ib] - ax, wpos[ib + 1] - ay, wpos[ib + 2] - az, __uint_as_float(mat[t]));
        tris[3 * (size_t)j + 2] =
            make_float4(wpos[ic] - ax, wpos[ic + 1] - ay, wpos[ic + 2] - az, __uint_as_float((uint32_t)m));
        n0[j] = make_float4(wnrm[ia], wnrm[ia + 1], wnrm[ia + 2], 0.0f);
        n1[j] = make_float4(wnrm[ib], wnrm[ib + 1], wnrm[ib + 2], 0.0f);
        n2[j] = make_float4(wnrm[ic], wnrm[ic + 1], wnrm[ic + 2], 0.0f);
    }
}

__global__ void k_mesh_results(const uint32_t* tri_off, int M, const int* prefix, const float4* nodes,
                               const float* cost, float* out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const int root = prefix[tri_off[m]];
    const float4 l = nodes[2 * (size_t)root], h = nodes[2 * (size_t)root + 1];
    float* o = out + 8 * (size_t)m;
    o[0] = l.x; o[1] = l.y; o[2] = l.z; o[3] = h.x; o[4] = h.y; o[5] = h.z;
    o[6] = cost[root];
    o[7] = __int_as_float(root);
}

template <class T>
struct Buf {
    T* p = nullptr;
    size_t n = 0;
    // grow-only with 1/8 headroom: the builder lives for the process, and a batch of
    // scenes of similar sizes then allocates once
    cudaError_t reserve(size_t count) {
        count = std::max<size_t>(count, 1);
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr; n = 0;
        const size_t want = count + count / 8;
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

int grid_for(long long items, int threads) {
    return (int)std::max<long long>(1, std::min<long long>((items + threads - 1) / threads, kMaxGrid * 4));
}

}  // namespace

struct GpuBvhBuilder::Bufs {
    Buf<float> wpos, wnrm, results, cost;
    Buf<uint32_t> tri, mat, tri_off, vert_off, perm, tf, tt;
    Buf<float4> blo, bhi;
    Buf<int> pf, pt, chunk_cnt, chunk_off, cnt, topd, prefix, tile, parent, arrive, ctr;
    Buf<int4> stack, lvl0, lvl1, small;
    Buf<SegState> seg;
    Buf<int2> chunks;
    Buf<NodeRec> small_pool, large_pool;
    int large_cap = 0;
    void release() {
        wpos.release(); wnrm.release(); results.release(); cost.release();
        tri.release(); mat.release(); tri_off.release(); vert_off.release(); perm.release(); tf.release(); tt.release();
        blo.release(); bhi.release();
        pf.release(); pt.release(); chunk_cnt.release(); chunk_off.release(); cnt.release(); topd.release();
        prefix.release(); tile.release(); parent.release(); arrive.release(); ctr.release();
        stack.release(); lvl0.release(); lvl1.release(); small.release(); seg.release(); chunks.release();
        small_pool.release(); large_pool.release();
    }
};

#define BVH_CUDA(call)                                                                \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            err = std::string("device BVH build: ") + #call + ": " + cudaGetErrorString(e_); \
            return RC_E_CUDA;                                                         \
        }                                                                             \
    } while (0)

void GpuBvhBuilder::release() {
    if (b_) { b_->release(); delete b_; b_ = nullptr; }
    num_nodes_ = num_tris_ = 0;
}

int GpuBvhBuilder::build(const std::vector<GpuMeshSrc>& meshes, cudaStream_t s, bool& supported, std::string& err) {
    supported = false;
    levels = 0;
    const int M = (int)meshes.size();
    long long N = 0, NV = 0;
    for (const GpuMeshSrc& m : meshes) {
        if (m.num_tris == 0) return RC_OK;   // a mesh without triangles: host build
        N += m.num_tris;
        NV += m.num_verts;
    }
    if (M == 0 || N >= (1ll << 30) || NV >= (1ll << 31) / 3) return RC_OK;
    if (!b_) b_ = new Bufs();
    Bufs& B = *b_;
    num_tris_ = N;
    num_meshes_ = M;
    std::vector<uint32_t> tri_off(M + 1), vert_off(M);
    std::vector<int4> large0, small0;
    {
        uint32_t t = 0, v = 0;
        for (int m = 0; m < M; ++m) {
            tri_off[m] = t;
            vert_off[m] = v;
            const int4 seg = make_int4((int)t, (int)(t + meshes[m].num_tris), 0, 0);
            (meshes[m].num_tris > (uint32_t)kSmall ? large0 : small0).push_back(seg);
            t += meshes[m].num_tris;
            v += meshes[m].num_verts;
        }
        tri_off[M] = t;
    }
    const size_t n = (size_t)N;
    const size_t max_seg = n / kSmall + M + 2;
    const size_t max_chunks = n / kChunk + max_seg + 2;
    B.large_cap = (int)std::min<size_t>(n / 2 + 1024, (size_t)1 << 30);
    BVH_CUDA(B.wpos.reserve(3 * (size_t)NV)); BVH_CUDA(B.wnrm.reserve(3 * (size_t)NV));
    BVH_CUDA(B.tri.reserve(3 * n)); BVH_CUDA(B.mat.reserve(n));
    BVH_CUDA(B.tri_off.reserve(M + 1)); BVH_CUDA(B.vert_off.reserve(M));
    BVH_CUDA(B.blo.reserve(n)); BVH_CUDA(B.bhi.reserve(n)); BVH_CUDA(B.perm.reserve(n));
    BVH_CUDA(B.tf.reserve(n)); BVH_CUDA(B.tt.reserve(n)); BVH_CUDA(B.pf.reserve(n)); BVH_CUDA(B.pt.reserve(n));
    BVH_CUDA(B.stack.reserve(n)); BVH_CUDA(B.small.reserve(n + M));
    BVH_CUDA(B.lvl0.reserve(max_seg)); BVH_CUDA(B.lvl1.reserve(max_seg)); BVH_CUDA(B.seg.reserve(max_seg));
    BVH_CUDA(B.chunks.reserve(max_chunks)); BVH_CUDA(B.chunk_cnt.reserve(max_chunks * kBins));
    BVH_CUDA(B.chunk_off.reserve(max_chunks));
    BVH_CUDA(B.small_pool.reserve(2 * n)); BVH_CUDA(B.large_pool.reserve(B.large_cap));
    BVH_CUDA(B.cnt.reserve(n)); BVH_CUDA(B.topd.reserve(n)); BVH_CUDA(B.prefix.reserve(n + 1));
    BVH_CUDA(B.tile.reserve(n / kScanTile + 2)); BVH_CUDA(B.ctr.reserve(8));
    for (int m = 0; m < M; ++m) {
        const GpuMeshSrc& src = meshes[m];
        BVH_CUDA(cudaMemcpyAsync(B.wpos.p + 3 * (size_t)vert_off[m], src.wpos, 12 * (size_t)src.num_verts,
                                 cudaMemcpyHostToDevice, s));
        BVH_CUDA(cudaMemcpyAsync(B.wnrm.p + 3 * (size_t)vert_off[m], src.wnrm, 12 * (size_t)src.num_verts,
                                 cudaMemcpyHostToDevice, s));
        BVH_CUDA(cudaMemcpyAsync(B.tri.p + 3 * (size_t)tri_off[m], src.tri, 12 * (size_t)src.num_tris,
                                 cudaMemcpyHostToDevice, s));
        BVH_CUDA(cudaMemcpyAsync(B.mat.p + tri_off[m], src.mat, 4 * (size_t)src.num_tris, cudaMemcpyHostToDevice, s));
    }
    BVH_CUDA(cudaMemcpyAsync(B.tri_off.p, tri_off.data(), 4 * (M + 1), cudaMemcpyHostToDevice, s));
    BVH_CUDA(cudaMemcpyAsync(B.vert_off.p, vert_off.data(), 4 * M, cudaMemcpyHostToDevice, s));
    // ctr: [0] chunks of the level, [1]/[5] segment counts of the two level lists,
    // [2] per-warp segments, [3] large node records, [4] flags, [6] non-empty levels
    int h_ctr[8] = {0, (int)large0.size(), (int)small0.size(), 0, 0, 0, 0, 0};
    BVH_CUDA(cudaMemcpyAsync(B.ctr.p, h_ctr, sizeof(h_ctr), cudaMemcpyHostToDevice, s));
    if (!large0.empty())
        BVH_CUDA(cudaMemcpyAsync(B.lvl0.p, large0.data(), sizeof(int4) * large0.size(), cudaMemcpyHostToDevice, s));
    if (!small0.empty())
        BVH_CUDA(cudaMemcpyAsync(B.small.p, small0.data(), sizeof(int4) * small0.size(), cudaMemcpyHostToDevice, s));
    BVH_CUDA(cudaMemsetAsync(B.cnt.p, 0, 4 * n, s));
    BVH_CUDA(cudaMemsetAsync(B.topd.p, 0x7f, 4 * n, s));
    BVH_CUDA(cudaMemsetAsync(B.small_pool.p, 0xff, sizeof(NodeRec) * 2 * n, s));
    int* flags = B.ctr.p + 4;
    // (flagged input is still built - every index is range-checked - and then discarded)
    k_prim_boxes<<<grid_for(N, 256), 256, 0, s>>>(B.wpos.p, B.tri.p, B.tri_off.p, B.vert_off.p, M, (int)N, B.blo.p,
                                                  B.bhi.p, B.perm.p, flags);
    BVH_CUDA(cudaGetLastError());

    View V{};
    V.perm = B.perm.p; V.blo = B.blo.p; V.bhi = B.bhi.p;
    V.tf = B.tf.p; V.pf = B.pf.p; V.tt = B.tt.p; V.pt = B.pt.p;
    V.stack = B.stack.p; V.small_pool = B.small_pool.p; V.large_pool = B.large_pool.p;
    V.large_count = B.ctr.p + 3; V.large_cap = B.large_cap;
    V.cnt = B.cnt.p; V.topd = B.topd.p; V.flags = flags; V.n = (int)N;
    V.next_cap = (int)max_seg; V.small_cap = (int)(n + M);

    // level passes, kLevelsPerSync at a time between reads of the remaining count
    constexpr int kLevelsPerSync = 4;
    const int g = (int)std::min<long long>(N / kChunk + max_seg + 1, kMaxGrid);
    const int gd = (int)std::min<long long>((max_seg + kWarps - 1) / kWarps, kMaxGrid);
    int4* list[2] = {B.lvl0.p, B.lvl1.p};
    int* count[2] = {B.ctr.p + 1, B.ctr.p + 5};
    int cur = 0, remaining = (int)large0.size(), launched = 0;
    while (remaining > 0) {
        for (int k = 0; k < kLevelsPerSync; ++k, cur ^= 1) {
            k_lvl_setup<<<1, 1024, 0, s>>>(list[cur], count[cur], count[cur ^ 1], B.seg.p, B.chunks.p, B.ctr.p + 0,
                                           B.ctr.p + 6);
            k_lvl_bounds<<<g, kThreads, 0, s>>>(B.seg.p, B.chunks.p, B.ctr.p + 0, V);
            k_lvl_bins<<<g, kThreads, 0, s>>>(B.seg.p, B.chunks.p, B.ctr.p + 0, V, B.chunk_cnt.p);
            k_lvl_decide<<<gd, kThreads, 0, s>>>(B.seg.p, count[cur], B.chunk_cnt.p, B.chunk_off.p, V, list[cur ^ 1],
                                                 count[cur ^ 1], B.small.p, B.ctr.p + 2);
            k_lvl_partition<<<g, kThreads, 0, s>>>(B.seg.p, B.chunks.p, B.ctr.p + 0, B.chunk_off.p, V);
            k_lvl_swap<<<g, kThreads, 0, s>>>(B.seg.p, B.chunks.p, B.ctr.p + 0, V);
        }
        BVH_CUDA(cudaGetLastError());
        BVH_CUDA(cudaMemcpyAsync(&remaining, count[cur], sizeof(int), cudaMemcpyDeviceToHost, s));
        BVH_CUDA(cudaStreamSynchronize(s));
        if (remaining > (int)max_seg) { err = "device BVH build: segment list overflow"; return RC_E_INVALID; }
        if ((launched += kLevelsPerSync) > (1 << 20)) { err = "device BVH build: no progress"; return RC_E_INVALID; }
    }
    {
        // one warp per remaining segment (the count is read on the device)
        const int gs = (int)std::min<long long>((n + M + kWarps - 1) / kWarps, kMaxGrid);
        k_small_build<<<gs, kThreads, 0, s>>>(B.small.p, B.ctr.p + 2, V);
        BVH_CUDA(cudaGetLastError());
    }
    const int ntiles = (int)((n + kScanTile - 1) / kScanTile);
    k_scan_tiles<<<ntiles, 1024, 0, s>>>(B.cnt.p, (int)N, B.prefix.p, B.tile.p);
    k_scan_sums<<<1, 1024, 0, s>>>(B.tile.p, ntiles, B.prefix.p, (int)N);
    k_scan_add<<<ntiles, 1024, 0, s>>>(B.prefix.p, (int)N, B.tile.p);
    BVH_CUDA(cudaGetLastError());
    int total_nodes = 0;
    BVH_CUDA(cudaMemcpyAsync(&total_nodes, B.prefix.p + N, sizeof(int), cudaMemcpyDeviceToHost, s));
    BVH_CUDA(cudaMemcpyAsync(h_ctr, B.ctr.p, sizeof(h_ctr), cudaMemcpyDeviceToHost, s));
    BVH_CUDA(cudaStreamSynchronize(s));
    levels = h_ctr[6];
    if (h_ctr[4]) {
        // input outside the device build's domain, or (not expected) an exhausted pool or
        // a failed range check: the host build runs instead
        if (h_ctr[4] & kFlagIndex) err = "device BVH build: inconsistent ranks";
        else if (h_ctr[4] & kFlagPool) err = "device BVH build: node pool full";
        return RC_OK;
    }
    num_nodes_ = total_nodes;
    supported = true;
    return RC_OK;
}

int GpuBvhBuilder::emit(float4* nodes, float4* tris, float4* n0, float4* n1, float4* n2, cudaStream_t s,
                        std::string& err) {
    if (!b_ || num_nodes_ <= 0) { err = "device BVH build: nothing built"; return RC_E_INVALID; }
    Bufs& B = *b_;
    const long long nn = num_nodes_;
    const int N = (int)num_tris_, M = num_meshes_;
    int* flags = B.ctr.p + 4;
    BVH_CUDA(B.parent.reserve(nn)); BVH_CUDA(B.arrive.reserve(nn)); BVH_CUDA(B.cost.reserve(nn));
    BVH_CUDA(B.results.reserve(8 * (size_t)M));
    BVH_CUDA(cudaMemsetAsync(B.parent.p, 0xff, 4 * nn, s));
    BVH_CUDA(cudaMemsetAsync(B.arrive.p, 0, 4 * nn, s));
    k_emit<<<grid_for(2ll * N + B.large_cap, 256), 256, 0, s>>>(B.small_pool.p, 2ll * N, B.large_pool.p, B.ctr.p + 3,
                                                                 B.large_cap, B.prefix.p, B.topd.p, nn, nodes, B.parent.p,
                                                                 flags);
    k_cost<<<grid_for(nn, 256), 256, 0, s>>>(nodes, B.parent.p, nn, B.arrive.p, B.cost.p, flags);
    k_pack_tris<<<grid_for(N, 256), 256, 0, s>>>(B.perm.p, B.wpos.p, B.wnrm.p, B.tri.p, B.mat.p, B.tri_off.p,
                                                 B.vert_off.p, M, N, tris, n0, n1, n2);
    k_mesh_results<<<(M + 127) / 128, 128, 0, s>>>(B.tri_off.p, M, B.prefix.p, nodes, B.cost.p, B.results.p);
    BVH_CUDA(cudaGetLastError());
    std::vector<float> res(8 * (size_t)M);
    int h_flags = 0;
    BVH_CUDA(cudaMemcpyAsync(res.data(), B.results.p, sizeof(float) * res.size(), cudaMemcpyDeviceToHost, s));
    BVH_CUDA(cudaMemcpyAsync(&h_flags, flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    BVH_CUDA(cudaStreamSynchronize(s));
    if (h_flags & kFlagIndex) { err = "device BVH build: node numbering out of range"; return RC_E_INVALID; }
    mesh_root.resize(M);
    mesh_box.resize(6 * (size_t)M);
    mesh_cost.resize(M);
    for (int m = 0; m < M; ++m) {
        for (int j = 0; j < 6; ++j) mesh_box[6 * (size_t)m + j] = res[8 * (size_t)m + j];
        mesh_cost[m] = res[8 * (size_t)m + 6];
        int root;
        std::memcpy(&root, &res[8 * (size_t)m + 7], 4);
        mesh_root[m] = root;
    }
    return RC_OK;
}

}  // namespace rc
