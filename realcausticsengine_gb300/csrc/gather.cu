// Radius gather at the camera vertices (Path_Vertices::get_contrib,
// src/Path_Vertices.h:46-68, over KD_Tree::find_closest_in_radius,
// src/KD_Tree.cpp:217-280).
//
// Descent: the reference's near-side-first recursion with the far side (and an odd
// node's median photon) visited only when (q[axis] - split)^2 < r^2.  Once a node
// holds at most kBucket photons its whole contiguous range is tested.  Every photon
// that reaches the test is accepted by the reference's own predicate
// ((dx*dx + dy*dy) + dz*dz) < r^2 in FP32 without contraction, so the set of photons
// found is exactly the reference's: pruning never drops a photon inside the radius
// (rounding is monotonic, so |q - p|^2 >= (q[axis] - split)^2 holds in floats too).
#include "vm.cuh"
#include "bsdf.cuh"

namespace rc {

namespace {

constexpr int kBucket = 8;

struct KdNav {
    const uint2* __restrict__ nodes;
    const float* __restrict__ x;
    const float* __restrict__ y;
    const float* __restrict__ z;
    const uint32_t* __restrict__ id;
    long long n;
};

__device__ __forceinline__ bool in_radius(F3 q, float px, float py, float pz, float r2) {
    float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
    return dx * dx + dy * dy + dz * dz < r2;
}

// Visit every photon within the radius: fn(tree position).
template <class Fn>
__device__ __forceinline__ void kd_visit(const KdNav& t, F3 q, float r2, Fn&& fn) {
    if (t.n <= 0) return;
    struct Item { long long e, start; int level; };
    Item stack[64];
    int sp = 0;
    stack[sp++] = {1, 0, 0};
    while (sp) {
        Item it = stack[--sp];
        long long c = t.n >> it.level;
        if (c <= kBucket) {
            for (long long p = it.start; p < it.start + c; ++p)
                if (in_radius(q, __ldg(&t.x[p]), __ldg(&t.y[p]), __ldg(&t.z[p]), r2)) fn(p);
            continue;
        }
        uint2 nd = __ldg(&t.nodes[it.e]);
        uint32_t ax = nd.x & 0x60000000u;
        float split = __uint_as_float(nd.y);
        float qa = ax == 0 ? q.x : (ax == 0x20000000u ? q.y : q.z);
        float dist = qa - split;
        long long half = c >> 1, odd = c & 1;
        Item left = {2 * it.e, it.start, it.level + 1};
        Item right = {2 * it.e + 1, it.start + half + odd, it.level + 1};
        bool go_left_first = dist < 0;
        if (dist * dist < r2) {
            if (odd) {
                long long p = it.start + half;
                if (in_radius(q, __ldg(&t.x[p]), __ldg(&t.y[p]), __ldg(&t.z[p]), r2)) fn(p);
            }
            if (sp < 63) stack[sp++] = go_left_first ? right : left;
        }
        if (sp < 64) stack[sp++] = go_left_first ? left : right;
    }
}

__global__ void __launch_bounds__(256) k_gather(const VMParams P, const KdNav t, PhotonBuf ph, QueryBuf qb,
                                                long long nq, double* __restrict__ accum) {
    long long qi = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    float4 a = qb.q0[qi], b = qb.q1[qi], c = qb.q2[qi], w = qb.q3[qi], e = qb.q4[qi];
    F3 q = xyz(a);
    float cam_dVM = a.w;
    int mat = __float_as_int(b.w);
    int pixel = __float_as_int(c.w);
    F3 ng = xyz(c);
    Bsdf bs;
    bs.init(P.materials[mat], xyz(b), xyz(e), true);
    F3 color = f3(0.0f);
    kd_visit(t, q, P.radius_sqr, [&](long long p) {
        uint32_t i = __ldg(&t.id[p]);
        float4 pp = __ldg(&ph.pos[i]);
        float4 pd = __ldg(&ph.dir[i]);
        float2 pt = __ldg(&ph.tp[i]);
        F3 wi = xyz(pd);
        float fwd, rev;
        bs.pdf(wi, fwd, rev);
        float weight = 1.0f / (1.0f + cam_dVM * rev + pp.w * fwd);
        F3 ev = bs.evaluate(wi, ng);
        color = color + ev * f3(pd.w, pt.x, pt.y) * weight;
    });
    F3 r = xyz(w) * color;
    if (r.x != 0.0f || r.y != 0.0f || r.z != 0.0f) {
        atomicAdd(&accum[3 * (long long)pixel + 0], (double)r.x);
        atomicAdd(&accum[3 * (long long)pixel + 1], (double)r.y);
        atomicAdd(&accum[3 * (long long)pixel + 2], (double)r.z);
    }
}

__global__ void k_kd_query(const KdNav t, int q, const float* __restrict__ qpos, float r2, int* counts,
                           const long long* offsets, int* idx) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= q) return;
    F3 p = f3(qpos[3 * j], qpos[3 * j + 1], qpos[3 * j + 2]);
    int n = 0;
    long long off = offsets ? offsets[j] : 0;
    kd_visit(t, p, r2, [&](long long pos) {
        if (idx) idx[off + n] = (int)__ldg(&t.id[pos]);
        ++n;
    });
    counts[j] = n;
}

KdNav nav_of(const KdTree& tr) { return KdNav{tr.nodes, tr.x, tr.y, tr.z, tr.id, tr.n}; }

}  // namespace

void launch_gather(const VMParams& p, const KdTree& tree, PhotonBuf ph, QueryBuf qb, long long nq, double* accum,
                   cudaStream_t s) {
    if (nq <= 0) return;
    k_gather<<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(p, nav_of(tree), ph, qb, nq, accum);
}

void launch_kd_query(const KdTree& tree, int q, const float* qpos, float r2, int* counts, const long long* offsets,
                     int* idx, cudaStream_t s) {
    if (q <= 0) return;
    k_kd_query<<<(q + 127) / 128, 128, 0, s>>>(nav_of(tree), q, qpos, r2, counts, offsets, idx);
}

}  // namespace rc
