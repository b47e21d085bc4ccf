// GPU photon KD-tree build by parallel median splits (see kdtree.cuh for the tree).
//
// Levels whose nodes hold more than kSmemSeg photons are split with global passes,
// one pass per step over all photons (SoA x/y/z/id, double buffered):
//   bbox      per-node extent -> axis (largest extent)
//   hist x4   8-bit radix select of the rank-count/2 key along the node's axis (the
//             leading digits the node's box fixes are skipped)
//   partition photons below / equal / above the median key to their halves
// A CTA covers T x kItems consecutive positions (T = 256 threads on levels whose nodes
// hold more than 2048 photons, else 128); because nodes on these levels hold more
// than that many photons, a chunk meets at most two nodes (and one ancestor median
// between them), so histograms and counters stay in shared memory and only their
// totals go to global memory.
// From the first level with at most kSmemSeg photons per node, one CTA per node
// loads its photons into shared memory and finishes the whole subtree there: one
// sort along x, y and z (key, then local index), then stable splits of the three
// lists per level, writing nodes and final order.
#include "kdtree.cuh"
#include "dev_once.h"
#include <cmath>
#include <cstdio>
#include <mutex>

namespace rc {

namespace {

constexpr int kSmemSeg = 1024;      // largest node finished in shared memory (~66 KB: 3 CTAs per SM)
constexpr int kItems = 8;           // positions per thread in the global passes
constexpr int kThreads = 128;       // CTA size of the global passes (kThreads x kItems <= kSmemSeg)
constexpr int kWideThreads = 256;   // CTA size on levels whose nodes hold more than its positions
constexpr int kSmemThreads = 256;
constexpr float kSplitBias = 1.175494e-38f;   // src/KD_Tree.cpp:150

__device__ __forceinline__ uint32_t f2key(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key2f(uint32_t k) {
    uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}
// order-preserving int encoding for atomicMin/Max on floats
__device__ __forceinline__ int f2ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : (i ^ 0x7fffffff);
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : (i ^ 0x7fffffff)); }

__device__ __forceinline__ uint32_t odd_mask(int axis) { return axis == 0 ? 0x90000000u : (axis == 1 ? 0xb0000000u : 0xf0000000u); }
__device__ __forceinline__ uint32_t even_mask(int axis) { return axis == 0 ? 0x80000000u : (axis == 1 ? 0xa0000000u : 0xe0000000u); }

// aproximate_biggest_axis's final choice (src/KD_Tree.cpp:90-94)
__device__ __forceinline__ int biggest_axis(float ex, float ey, float ez) {
    float b = fmaxf(fmaxf(ex, ey), ez);
    return b == ex ? 0 : (b == ey ? 1 : 2);
}

// Node on `level` whose range holds position i; returns 0 if i is the median photon
// of an ancestor.  *start receives the node's first position.
__device__ __forceinline__ long long locate(long long i, int level, long long n, long long* start) {
    long long e = 1, s = 0, c = n;
    for (int j = 0; j < level; ++j) {
        long long half = c >> 1, odd = c & 1;
        if (i < s + half) { e = 2 * e; }
        else if (odd && i == s + half) { *start = 0; return 0; }
        else { e = 2 * e + 1; s += half + odd; }
        c = half;
    }
    *start = s;
    return e;
}

struct NodeSel {
    uint32_t prefix;   // selected high bits of the median key
    int krem;          // remaining rank inside the selected bin
    int eq;            // photons whose key equals the median key
    int axis;
    int cnt[3];        // partition cursors (below / equal / above)
    int first;         // first digit pass that runs (earlier digits fixed by the node's box)
};

struct Buffers {
    float* x[2]; float* y[2]; float* z[2]; uint32_t* id[2];
};

// One half of the double buffer, picked with selects: indexing the kernel parameter
// with a runtime value would copy all of it to local memory in every thread.
struct Side {
    float* x; float* y; float* z; uint32_t* id;
};
__device__ __forceinline__ Side side(const Buffers& B, int k) {
    return k ? Side{B.x[1], B.y[1], B.z[1], B.id[1]} : Side{B.x[0], B.y[0], B.z[0], B.id[0]};
}

// Chunk -> at most two nodes A, B on `level`.
struct ChunkNodes {
    long long eA, sA, eB, sB, c;
};

__device__ __forceinline__ void chunk_nodes(long long a, long long chunk, int level, long long n, ChunkNodes& cn) {
    long long c = n >> level;
    long long s;
    long long e = locate(a, level, n, &s);
    if (e == 0) e = locate(a + 1, level, n, &s);
    cn.eA = e; cn.sA = s; cn.c = c;
    long long endA = s + c;
    cn.eB = 0; cn.sB = -1;
    if (endA < a + chunk && endA < n) {
        long long s2;
        long long e2 = locate(endA, level, n, &s2);
        if (e2 == 0 && endA + 1 < n) e2 = locate(endA + 1, level, n, &s2);
        if (e2) { cn.eB = e2; cn.sB = s2; }
    }
}

// 0 = node A, 1 = node B, -1 = not inside a node on this level
__device__ __forceinline__ int which(long long i, const ChunkNodes& cn) {
    if (i >= cn.sA && i < cn.sA + cn.c) return 0;
    if (cn.eB && i >= cn.sB && i < cn.sB + cn.c) return 1;
    return -1;
}

__global__ void k_level_init(int level, long long first, long long count, int* nbox, NodeSel* sel, long long n) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= count) return;
    int* b = nbox + 6 * t;
    b[0] = b[1] = b[2] = 0x7fffffff;
    b[3] = b[4] = b[5] = (int)0x80000000;
    NodeSel& s = sel[t];
    s.prefix = 0; s.krem = (int)((n >> level) >> 1); s.eq = 0; s.axis = 0;
    s.cnt[0] = s.cnt[1] = s.cnt[2] = 0;
    s.first = 0;
}

template <int T>
__global__ void __launch_bounds__(T) k_bbox(Buffers B, int cur, int level, long long n, long long first, int* nbox) {
    __shared__ ChunkNodes cn;
    __shared__ int sb[2][6];
    long long a = blockIdx.x * (long long)(T * kItems);
    if (threadIdx.x == 0) chunk_nodes(a, T * kItems, level, n, cn);
    if (threadIdx.x < 12) sb[threadIdx.x / 6][threadIdx.x % 6] = (threadIdx.x % 6) < 3 ? 0x7fffffff : (int)0x80000000;
    __syncthreads();
    int mn[2][3], mx[2][3];
    for (int q = 0; q < 2; ++q) for (int k = 0; k < 3; ++k) { mn[q][k] = 0x7fffffff; mx[q][k] = (int)0x80000000; }
    float px[kItems], py[kItems], pz[kItems];
    int wh[kItems];
    const Side S = side(B, cur);
#pragma unroll
    for (int it = 0; it < kItems; ++it) {   // loads of all rounds in flight together
        long long i = a + it * T + threadIdx.x;
        wh[it] = i < n ? which(i, cn) : -1;
        const long long j = wh[it] >= 0 ? i : a;
        px[it] = S.x[j]; py[it] = S.y[j]; pz[it] = S.z[j];
    }
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int w = wh[it];
        if (w < 0) continue;
        int vx = f2ord(px[it]), vy = f2ord(py[it]), vz = f2ord(pz[it]);
        if (w == 0) {
            mn[0][0] = min(mn[0][0], vx); mn[0][1] = min(mn[0][1], vy); mn[0][2] = min(mn[0][2], vz);
            mx[0][0] = max(mx[0][0], vx); mx[0][1] = max(mx[0][1], vy); mx[0][2] = max(mx[0][2], vz);
        } else {
            mn[1][0] = min(mn[1][0], vx); mn[1][1] = min(mn[1][1], vy); mn[1][2] = min(mn[1][2], vz);
            mx[1][0] = max(mx[1][0], vx); mx[1][1] = max(mx[1][1], vy); mx[1][2] = max(mx[1][2], vz);
        }
    }
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 3; ++k) {
            int v = mn[q][k], u = mx[q][k];
            for (int o = 16; o > 0; o >>= 1) {
                v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
                u = max(u, __shfl_xor_sync(0xffffffffu, u, o));
            }
            if ((threadIdx.x & 31) == 0) { atomicMin(&sb[q][k], v); atomicMax(&sb[q][3 + k], u); }
        }
    __syncthreads();
    if (threadIdx.x < 12) {
        int q = threadIdx.x / 6, k = threadIdx.x % 6;
        long long e = q == 0 ? cn.eA : cn.eB;
        if (e) {
            int* dst = nbox + 6 * (e - first) + k;
            if (k < 3) atomicMin(dst, sb[q][k]); else atomicMax(dst, sb[q][k]);
        }
    }
}

__device__ __forceinline__ int node_axis(const int* nbox, long long t) {
    const int* b = nbox + 6 * t;
    float ex = ord2f(b[3]) - ord2f(b[0]);
    float ey = ord2f(b[4]) - ord2f(b[1]);
    float ez = ord2f(b[5]) - ord2f(b[2]);
    return biggest_axis(ex, ey, ez);
}

// The node's split axis.  Every key of the node lies between the keys of its box's
// ends along that axis (both orders are IEEE total order), so the whole leading digits
// those two keys share are the median's digits too: they go into the prefix, and the
// radix-select passes over them are skipped (the last pass always runs: it writes the
// split and the count of keys equal to the median).
__global__ void k_axis(long long count, const int* nbox, NodeSel* sel) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int a = node_axis(nbox, t);
    const uint32_t lo = f2key(ord2f(nbox[6 * t + a])), hi = f2key(ord2f(nbox[6 * t + 3 + a]));
    const int d = min(__clz(lo ^ hi) >> 3, 3);
    NodeSel& s = sel[t];
    s.axis = a;
    s.first = d;
    s.prefix = lo & ~(0xffffffffu >> (8 * d));
}

__device__ __forceinline__ float coord(const Side& S, long long i, int axis) {
    return axis == 0 ? S.x[i] : (axis == 1 ? S.y[i] : S.z[i]);
}

template <int T>
__global__ void __launch_bounds__(T) k_hist(Buffers B, int cur, int level, long long n, long long first,
                                                   const NodeSel* sel, uint32_t* hist, int pass) {
    __shared__ ChunkNodes cn;
    __shared__ uint32_t sh[2][256];
    __shared__ uint32_t pre[2];
    __shared__ int ax[2];
    __shared__ bool live[2];   // the node's digit for this pass is not fixed by its box
    long long a = blockIdx.x * (long long)(T * kItems);
    if (threadIdx.x == 0) {
        chunk_nodes(a, T * kItems, level, n, cn);
        const NodeSel* sa = sel + (cn.eA - first);
        ax[0] = sa->axis; pre[0] = sa->prefix; live[0] = pass >= sa->first;
        live[1] = false;
        if (cn.eB) {
            const NodeSel* sb = sel + (cn.eB - first);
            ax[1] = sb->axis; pre[1] = sb->prefix; live[1] = pass >= sb->first;
        }
    }
    for (int k = threadIdx.x; k < 512; k += T) (&sh[0][0])[k] = 0;
    __syncthreads();
    if (!live[0] && !live[1]) return;
    const int shift = 24 - 8 * pass;
    // all rounds' coordinates first (independent loads in flight together), then bins
    float val[kItems];
    int wh[kItems];
    const Side S = side(B, cur);
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        long long i = a + it * T + threadIdx.x;
        const int w = i < n ? which(i, cn) : -1;
        wh[it] = w >= 0 && live[w] ? w : -1;
        val[it] = wh[it] >= 0 ? coord(S, i, ax[wh[it]]) : 0.0f;
    }
#pragma unroll
    for (int it = 0; it < kItems; ++it) {   // every lane runs every round (full-warp match)
        unsigned slot = 0xffffffffu;
        const int w = wh[it];
        if (w >= 0) {
            uint32_t key = f2key(val[it]);
            if (pass == 0 || (key >> (shift + 8)) == (pre[w] >> (shift + 8)))
                slot = (unsigned)w * 256u + ((key >> shift) & 255u);
        }
        // lanes with the same bin add once (the top digits of nearby coordinates
        // coincide, so per-lane atomics would serialise on a few bins)
        const unsigned peers = __match_any_sync(0xffffffffu, slot);
        if (slot != 0xffffffffu && (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1))
            atomicAdd(&(&sh[0][0])[slot], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 512; k += T) {
        int q = k >> 8;
        uint32_t v = (&sh[0][0])[k];
        long long e = q == 0 ? cn.eA : cn.eB;
        if (v && e) atomicAdd(&hist[(e - first) * 256 + (k & 255)], v);
    }
}

// One warp per node: find the bin holding rank krem, narrow the prefix, clear the
// histogram for the next pass.  After the last pass, write the node's split.
__global__ void k_select(long long count, long long first, int level, long long n, NodeSel* sel, uint32_t* hist,
                         int pass, uint2* nodes, int* err) {
    long long t = blockIdx.x * (long long)(blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (t >= count) return;
    if (pass < sel[t].first) return;   // digit fixed by the node's box (k_axis); no counts
    uint32_t* h = hist + t * 256;
    uint32_t v[8];
    uint32_t sum = 0;
    for (int k = 0; k < 8; ++k) { v[k] = h[lane * 8 + k]; sum += v[k]; h[lane * 8 + k] = 0; }
    uint32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    uint32_t excl = incl - sum;
    int krem = sel[t].krem;
    // lane whose range [excl, incl) contains krem
    bool mine = (uint32_t)krem >= excl && (uint32_t)krem < incl;
    unsigned bal = __ballot_sync(0xffffffffu, mine);
    int owner = __ffs(bal) - 1;
    if (owner < 0) {
        if (lane == 0) atomicOr(err, 1);   // histogram does not hold rank krem
        return;
    }
    if (lane == owner) {
        uint32_t cum = excl;
        int bin = 0;
        for (int k = 0; k < 8; ++k) {
            if ((uint32_t)krem < cum + v[k]) { bin = lane * 8 + k; break; }
            cum += v[k];
        }
        NodeSel& s = sel[t];
        s.krem = krem - (int)cum;
        s.prefix |= (uint32_t)bin << (24 - 8 * pass);
        if (pass == 3) {
            s.eq = (int)v[bin - lane * 8];
            long long c = n >> level;
            float m = key2f(s.prefix);
            long long e = first + t;
            nodes[e].y = __float_as_uint((c & 1) ? m : m + kSplitBias);
            if (!(c & 1)) nodes[e].x = even_mask(s.axis);
        }
    }
}

template <int T>
__global__ void __launch_bounds__(T) k_partition(Buffers B, int cur, int level, long long n, long long first,
                                                        NodeSel* sel, uint2* nodes, int* err) {
    __shared__ ChunkNodes cn;
    __shared__ int ax[2], krem[2], eq[2];
    __shared__ uint32_t med[2];
    __shared__ int base[6];
    __shared__ int woff[kItems][T / 32][6];
    long long a = blockIdx.x * (long long)(T * kItems);
    if (threadIdx.x == 0) {
        chunk_nodes(a, T * kItems, level, n, cn);
        NodeSel s = sel[cn.eA - first];
        ax[0] = s.axis; krem[0] = s.krem; eq[0] = s.eq; med[0] = s.prefix;
        if (cn.eB) {
            s = sel[cn.eB - first];
            ax[1] = s.axis; krem[1] = s.krem; eq[1] = s.eq; med[1] = s.prefix;
        }
    }
    __syncthreads();
    const int dst = cur ^ 1;
    // coalesced rounds of T consecutive positions; the rank of a photon in its
    // class (node A/B x below/equal/above) follows position order inside the CTA:
    // ballots within a warp, then per-(round, warp) offsets
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    // the photons of all rounds are loaded once, up front (independent loads in flight
    // together); position past n: -2, ancestor median (stays in place): -1
    float px[kItems], py[kItems], pz[kItems];
    uint32_t pid[kItems];
    int cls[kItems], rank[kItems];
    const Side S = side(B, cur), D = side(B, dst);
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const long long i = a + it * T + threadIdx.x;
        const long long j = i < n ? i : a;
        px[it] = S.x[j]; py[it] = S.y[j]; pz[it] = S.z[j]; pid[it] = S.id[j];
        cls[it] = i < n ? which(i, cn) : -2;
    }
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const int w = cls[it];   // node A (0) / B (1), or -1 / -2 as above
        int q = w;
        if (w >= 0) {
            const int axw = ax[w];
            const uint32_t key = f2key(axw == 0 ? px[it] : (axw == 1 ? py[it] : pz[it]));
            q = w * 3 + (key < med[w] ? 0 : (key == med[w] ? 1 : 2));
        }
        cls[it] = q;
        rank[it] = 0;
#pragma unroll
        for (int cq = 0; cq < 6; ++cq) {
            const unsigned m = __ballot_sync(0xffffffffu, q == cq);
            if (q == cq) rank[it] = __popc(m & lt_mask);
            if (lane == 0) woff[it][wid][cq] = __popc(m);
        }
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int q = threadIdx.x;
        int run = 0;
        for (int it = 0; it < kItems; ++it)
            for (int w = 0; w < T / 32; ++w) {
                const int v = woff[it][w][q];
                woff[it][w][q] = run;
                run += v;
            }
        long long e = q < 3 ? cn.eA : cn.eB;
        base[q] = (e && run) ? atomicAdd(&sel[e - first].cnt[q % 3], run) : 0;
    }
    __syncthreads();
    const long long c = cn.c;
    const long long k = c >> 1, odd = c & 1;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        long long i = a + it * T + threadIdx.x;
        int q = cls[it];
        if (q == -2) continue;
        const float xv = px[it], yv = py[it], zv = pz[it];
        const uint32_t idv = pid[it];
        long long d;
        if (q < 0) {
            d = i;   // ancestor median: stays in place
        } else {
            int w = q / 3, cl = q % 3;
            long long s = w == 0 ? cn.sA : cn.sB;
            long long r = base[q] + woff[it][wid][q] + rank[it];
            long long kl = krem[w];
            long long lt = k - kl;
            if (cl == 0) d = s + r;
            else if (cl == 1) {
                if (r < kl) d = s + lt + r;
                else if (odd && r == kl) {
                    d = s + k;
                    long long e = w == 0 ? cn.eA : cn.eB;
                    nodes[e].x = idv | odd_mask(ax[w]);
                } else d = s + k + odd + (r - kl - odd);
            } else d = s + k + odd + (eq[w] - kl - odd) + r;
            if (d < s || d >= s + c) { atomicOr(err, 2); continue; }   // inconsistent counts
        }
        D.x[d] = xv; D.y[d] = yv; D.z[d] = zv; D.id[d] = idv;
    }
}

__global__ void k_load(const float4* __restrict__ pos4, long long n, Buffers B) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos4[i];
    B.x[0][i] = p.x; B.y[0][i] = p.y; B.z[0][i] = p.z; B.id[0][i] = (uint32_t)i;
}

// Copy the median photons of levels < level0 from buffer `src` to buffer 0.
__global__ void k_copy_medians(Buffers B, int src, int level0, long long n) {
    long long e = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (1LL << level0)) return;
    int lv = 63 - __clzll(e);
    long long c = n >> lv;
    if (!(c & 1)) return;
    long long p = kd_node_start(e, lv, n) + (c >> 1);
    const Side S = side(B, src);
    B.x[0][p] = S.x[p]; B.y[0][p] = S.y[p]; B.z[0][p] = S.z[p]; B.id[0][p] = S.id[p];
}

// Shared-memory subtree builder: one CTA per node on level0 (at most kSmemSeg photons).
// The photons are sorted once along x, y and z (three index lists; bitonic on the key
// (coordinate, local index)).  Every level then reads each sub-node's extents (first
// and last entry of each list) and its median (middle entry of the chosen axis's list)
// off the lists, and splits all three lists stably into left / median / right.  A
// sub-node of c photons has exactly c/2 photons on each side, so the rank of a photon
// inside its sub-node's class is a block-wide prefix count minus s * (c/2).
struct SmemLayout {
    static constexpr size_t xs = 0;                                  // photons by local index
    static constexpr size_t ys = xs + 4 * kSmemSeg;
    static constexpr size_t zs = ys + 4 * kSmemSeg;
    static constexpr size_t ids = zs + 4 * kSmemSeg;
    static constexpr size_t v = ids + 4 * kSmemSeg;                  // 3 x kSmemSeg uint64 sort keys,
    static constexpr size_t lists = v;                               // then 3 x kSmemSeg uint32 lists
    static constexpr size_t temp = v + 4 * 3 * kSmemSeg;             // and 3 x kSmemSeg uint32 split output
    static constexpr size_t cls = v + 8 * 3 * kSmemSeg;              // class per photon (0 left, 1 median, 2 right)
    static constexpr size_t segs = cls + 4 * kSmemSeg;               // sub-node starts (up to kSmemSeg)
    static constexpr size_t axes = segs + 4 * kSmemSeg;              // split axis per sub-node (up to kSmemSeg / 2)
    static constexpr size_t warp = axes + 4 * (kSmemSeg / 2);        // block scan scratch
    static constexpr size_t total = warp + 4 * 6 * (kSmemThreads / 32);
};

__device__ __forceinline__ float axis_coord(const float* X, const float* Y, const float* Z, int a, uint32_t q) {
    return a == 0 ? X[q] : (a == 1 ? Y[q] : Z[q]);
}

// Compare-exchange of a thread's keys E0 < E1 (positions 4t + E0, 4t + E1) in all three
// lists, ascending where bit k of the position is clear.
template <int E0, int E1>
__device__ __forceinline__ void sort_pair(unsigned long long (&key)[3][4], int tid, int k) {
    const bool up = ((4 * tid + E0) & k) == 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const unsigned long long lo = key[a][E0], hi = key[a][E1];
        const bool swap = (lo > hi) == up;
        key[a][E0] = swap ? hi : lo;
        key[a][E1] = swap ? lo : hi;
    }
}

__global__ void __launch_bounds__(kSmemThreads) k_smem_build(Buffers B, int src, int level0, long long n, uint2* nodes) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* X = (float*)(smem + SmemLayout::xs);
    float* Y = (float*)(smem + SmemLayout::ys);
    float* Z = (float*)(smem + SmemLayout::zs);
    uint32_t* I = (uint32_t*)(smem + SmemLayout::ids);
    unsigned long long* V = (unsigned long long*)(smem + SmemLayout::v);
    uint32_t* L = (uint32_t*)(smem + SmemLayout::lists);   // current lists: L[a * kSmemSeg + p]
    uint32_t* T = (uint32_t*)(smem + SmemLayout::temp);    // split output (swapped with L per level)
    int* cls = (int*)(smem + SmemLayout::cls);
    int* segs = (int*)(smem + SmemLayout::segs);
    int* axes = (int*)(smem + SmemLayout::axes);
    int (*wsum)[6] = (int (*)[6])(smem + SmemLayout::warp);

    const long long e0 = (1LL << level0) + blockIdx.x;
    const long long s0 = kd_node_start(e0, level0, n);
    const int c0 = (int)(n >> level0);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, wid = tid >> 5;
    const Side S = side(B, src);
    for (int i = tid; i < c0; i += nt) {
        X[i] = S.x[s0 + i]; Y[i] = S.y[s0 + i]; Z[i] = S.z[s0 + i]; I[i] = S.id[s0 + i];
    }
    __syncthreads();
    // three sorted lists: a bitonic network over kSmemSeg keys (coordinate key, local
    // index) per list, padding keys ~0 sorting last.  Thread t holds keys 4t..4t+3 of
    // every list in registers: strides 1 and 2 are exchanged in registers, 4..64 with
    // warp shuffles (partner lane t ^ stride/4), 128 and up through shared memory.
    static_assert(kSmemSeg == 4 * kSmemThreads, "four keys per thread and list");
    unsigned long long key[3][4];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int p = 4 * tid + e;
            key[a][e] = p < c0 ? ((unsigned long long)f2key(axis_coord(X, Y, Z, a, p)) << 32) | (unsigned)p : ~0ull;
        }
    for (int k = 2; k <= kSmemSeg; k <<= 1) {
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            if (jj >= 4) {
                const bool smem_stage = jj >= 128;
                if (smem_stage) {
#pragma unroll
                    for (int a = 0; a < 3; ++a)
#pragma unroll
                        for (int e = 0; e < 4; ++e) V[a * kSmemSeg + 4 * tid + e] = key[a][e];
                    __syncthreads();
                }
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int i = 4 * tid + e;
                    // the lower index of a pair keeps the minimum in an ascending run
                    const bool keep_min = ((i & jj) == 0) == ((i & k) == 0);
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const unsigned long long other =
                            smem_stage ? V[a * kSmemSeg + (i ^ jj)]
                                       : (unsigned long long)__shfl_xor_sync(0xffffffffu, (long long)key[a][e], jj >> 2);
                        const unsigned long long mine = key[a][e];
                        key[a][e] = keep_min ? (mine < other ? mine : other) : (mine < other ? other : mine);
                    }
                }
                if (smem_stage) __syncthreads();
            } else if (jj == 2) {
                sort_pair<0, 2>(key, tid, k);
                sort_pair<1, 3>(key, tid, k);
            } else {
                sort_pair<0, 1>(key, tid, k);
                sort_pair<2, 3>(key, tid, k);
            }
        }
    }
    // keys -> index lists (the lists overlay the keys; the last shared-memory stage
    // ended with a barrier)
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int p = 4 * tid + e;
            if (p < c0) L[a * kSmemSeg + p] = (uint32_t)(key[a][e] & 0xffffffffu);
        }
    __syncthreads();
    for (int j = 0;; ++j) {
        const int c = c0 >> j;
        const int nsub = 1 << j;
        for (int s = tid; s < nsub; s += nt) {
            int st = 0, cc = c0;
            for (int b = j - 1; b >= 0; --b) {
                int half = cc >> 1;
                if ((s >> b) & 1) st += half + (cc & 1);
                cc = half;
            }
            segs[s] = st;
        }
        __syncthreads();
        if (c <= 1) {
            for (int s = tid; s < nsub; s += nt) nodes[(e0 << j) + s] = make_uint2(I[L[segs[s]]], 0u);
            break;
        }
        const int k = c >> 1, odd = c & 1;
        // node records: extents and median read off the lists
        for (int s = tid; s < nsub; s += nt) {
            const int st = segs[s];
            const float ex = X[L[st + c - 1]] - X[L[st]];
            const float ey = Y[L[kSmemSeg + st + c - 1]] - Y[L[kSmemSeg + st]];
            const float ez = Z[L[2 * kSmemSeg + st + c - 1]] - Z[L[2 * kSmemSeg + st]];
            const int a = biggest_axis(ex, ey, ez);
            const uint32_t q = L[a * kSmemSeg + st + k];
            const float m = axis_coord(X, Y, Z, a, q);
            const long long e = (e0 << j) + s;
            if (odd) nodes[e] = make_uint2(I[q] | odd_mask(a), __float_as_uint(m));
            else nodes[e] = make_uint2(even_mask(a), __float_as_uint(m + kSplitBias));
            axes[s] = a;
        }
        __syncthreads();
        // class of every photon (0 left, 1 median, 2 right) from its place in its
        // sub-node's axis list
        const int nv = nsub * c;
        for (int v = tid; v < nv; v += nt) {
            const int s = v / c, off = v - s * c;
            cls[L[axes[s] * kSmemSeg + segs[s] + off]] = off < k ? 0 : ((odd && off == k) ? 1 : 2);
        }
        __syncthreads();
        // stable split of the three lists: thread t takes positions v = 4t..4t+3 of the
        // level's index space v -> (sub-node s = v / c, offset v % c)
        int cnt[6] = {0, 0, 0, 0, 0, 0};
        int cl[3][4];
        uint32_t qq[3][4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int v = 4 * tid + r;
            const int s = v / c, off = v - s * c;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                cl[a][r] = -1;
                if (v < nv) {
                    const uint32_t q = L[a * kSmemSeg + segs[s] + off];
                    qq[a][r] = q;
                    cl[a][r] = cls[q];
                    cnt[2 * a] += cl[a][r] == 0;
                    cnt[2 * a + 1] += cl[a][r] == 2;
                }
            }
        }
        // block-wide exclusive prefix of the 6 counters
        int excl[6];
#pragma unroll
        for (int u = 0; u < 6; ++u) {
            int x = cnt[u];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            excl[u] = x - cnt[u];
            if (lane == 31) wsum[wid][u] = x;
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 6; ++u) {
            int before = 0;
            for (int w = 0; w < wid; ++w) before += wsum[w][u];
            excl[u] += before;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int v = 4 * tid + r;
            if (v >= nv) break;
            const int s = v / c;
            const int st = segs[s];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const int c2 = cl[a][r];
                int dst;
                if (c2 == 0) dst = st + (excl[2 * a]++ - s * k);
                else if (c2 == 1) dst = st + k;
                else dst = st + k + odd + (excl[2 * a + 1]++ - s * k);
                T[a * kSmemSeg + dst] = qq[a][r];
                // a median keeps its place for good, outside every later sub-node: it
                // goes into both buffers (this level's reads of L ended at the barrier)
                if (c2 == 1) L[a * kSmemSeg + dst] = qq[a][r];
            }
        }
        __syncthreads();
        uint32_t* const done = L;   // the split lists become the current ones
        L = T;
        T = done;
    }
    __syncthreads();
    for (int i = tid; i < c0; i += nt) {
        const uint32_t q = L[i];
        B.x[0][s0 + i] = X[q]; B.y[0][s0 + i] = Y[q]; B.z[0][s0 + i] = Z[q]; B.id[0][s0 + i] = I[q];
    }
}

int first_smem_level(long long n) {
    int l = 0;
    while ((n >> l) > kSmemSeg) ++l;
    return l;
}

}  // namespace

long long kd_node_array_len(long long n) {
    if (n <= 0) return 0;
    // kdtree.resize(std::pow(2, (int)(std::log2f(size) + 1)))  (src/KD_Tree.cpp:186)
    long long ref = (long long)std::pow(2.0, (int)(std::log2f((float)n) + 1));
    int L = 63 - __builtin_clzll((unsigned long long)n);
    long long need = 1LL << (L + 1);
    return ref > need ? ref : need;
}

size_t kd_scratch_bytes(long long n) {
    if (n <= 0) return 256;
    int l0 = first_smem_level(n);
    long long maxnodes = l0 > 0 ? (1LL << (l0 - 1)) : 1;
    size_t b = 0;
    b += 16 * (size_t)n;                      // second buffer x/y/z/id
    b += 24 * (size_t)maxnodes;               // boxes
    b += sizeof(NodeSel) * (size_t)maxnodes;  // selection state
    b += 1024 * (size_t)maxnodes;             // histograms
    return b + 1024;
}

int kd_build(const float4* pos4, long long n, KdTree& tree, void* scratch, size_t scratch_bytes,
             cudaStream_t stream, int* launches, int* err) {
    int nl = 0;
    tree.n = n;
    if (n <= 0) { tree.levels = 0; tree.num_nodes = 0; if (launches) *launches = 0; return 0; }
    tree.levels = 63 - __builtin_clzll((unsigned long long)n);
    tree.num_nodes = kd_node_array_len(n);
    if (scratch_bytes < kd_scratch_bytes(n)) return -1;
    int l0 = first_smem_level(n);
    long long maxnodes = l0 > 0 ? (1LL << (l0 - 1)) : 1;
    char* p = (char*)scratch;
    Buffers B;
    B.x[0] = tree.x; B.y[0] = tree.y; B.z[0] = tree.z; B.id[0] = tree.id;
    B.x[1] = (float*)p; p += 4 * (size_t)n;
    B.y[1] = (float*)p; p += 4 * (size_t)n;
    B.z[1] = (float*)p; p += 4 * (size_t)n;
    B.id[1] = (uint32_t*)p; p += 4 * (size_t)n;
    p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
    int* nbox = (int*)p; p += 24 * (size_t)maxnodes;
    p = (char*)(((uintptr_t)p + 15) & ~(uintptr_t)15);
    NodeSel* sel = (NodeSel*)p; p += sizeof(NodeSel) * (size_t)maxnodes;
    p = (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255);
    uint32_t* hist = (uint32_t*)p;

    cudaMemsetAsync(tree.nodes, 0, sizeof(uint2) * (size_t)tree.num_nodes, stream);
    k_load<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(pos4, n, B);
    nl++;
    if (l0 > 0) cudaMemsetAsync(hist, 0, 1024 * (size_t)maxnodes, stream);
    int cur = 0;
    for (int l = 0; l < l0; ++l) {
        long long first = 1LL << l, count = 1LL << l;
        unsigned g = (unsigned)((count + 255) / 256);
        // half as many CTAs, each twice as wide, while a wide chunk still meets at most
        // two nodes: the passes' per-CTA fixed cost (chunk location, shared-memory
        // reduction) is paid half as often
        const bool wide = (n >> l) > (long long)kWideThreads * kItems;
        const long long span = (long long)(wide ? kWideThreads : kThreads) * kItems;
        const unsigned chunks = (unsigned)((n + span - 1) / span);
        k_level_init<<<g, 256, 0, stream>>>(l, first, count, nbox, sel, n);
        if (wide) k_bbox<kWideThreads><<<chunks, kWideThreads, 0, stream>>>(B, cur, l, n, first, nbox);
        else k_bbox<kThreads><<<chunks, kThreads, 0, stream>>>(B, cur, l, n, first, nbox);
        k_axis<<<g, 256, 0, stream>>>(count, nbox, sel);
        nl += 3;
        for (int pass = 0; pass < 4; ++pass) {
            if (wide) k_hist<kWideThreads><<<chunks, kWideThreads, 0, stream>>>(B, cur, l, n, first, sel, hist, pass);
            else k_hist<kThreads><<<chunks, kThreads, 0, stream>>>(B, cur, l, n, first, sel, hist, pass);
            k_select<<<(unsigned)((count + 7) / 8), 256, 0, stream>>>(count, first, l, n, sel, hist, pass, tree.nodes,
                                                                       err);
            nl += 2;
        }
        if (wide) k_partition<kWideThreads><<<chunks, kWideThreads, 0, stream>>>(B, cur, l, n, first, sel, tree.nodes, err);
        else k_partition<kThreads><<<chunks, kThreads, 0, stream>>>(B, cur, l, n, first, sel, tree.nodes, err);
        nl++;
        cur ^= 1;
    }
    if (cur == 1 && l0 > 0) {
        long long cnt = (1LL << l0) - 1;
        k_copy_medians<<<(unsigned)((cnt + 255) / 256), 256, 0, stream>>>(B, 1, l0, n);
        nl++;
    }
    size_t smem = SmemLayout::total;
    // once per device: later builds may be recorded into a CUDA graph, and contexts on
    // several threads build concurrently
    static std::once_flag attr_set[kOnceDevices];
    once_per_device(attr_set, [&] { cudaFuncSetAttribute(k_smem_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); });
    k_smem_build<<<(unsigned)(1LL << l0), kSmemThreads, smem, stream>>>(B, cur, l0, n, tree.nodes);
    nl++;
    if (launches) *launches = nl;
    return 0;
}

}  // namespace rc
