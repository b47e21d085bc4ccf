// Closest-hit traversal of the reference's two-level SAH BVH on sm_103a.
//
// Bit-exact restatement of Scene::hit (src/Scene.cpp:154-189) ->
// CacheBVHNode_world::hit (src/BVH/BVH_world.cpp:267-283) -> Mesh::hit
// (src/mesh.cpp:70-105) -> CacheBVHNode_mesh::hit (src/BVH/BVH_mesh.cpp:265-283) ->
// aabb::hit (src/aabb.cpp:6-41) and Triangle::hit (src/Triangle.cpp:20-88):
//  * stack DFS, right child pushed before left, so the left subtree is visited first;
//  * every box is tested against the current closest distance of its own level (the
//    warp-stepped mesh traversal tests both children's boxes at their parent and keeps
//    the right one's entry distance on the stack: mesh_traverse_steps says why that is
//    the same test);
//  * a world leaf starts a fresh record (distance = inf) and, if any of its meshes is
//    hit, OVERWRITES the running result - so the answer is the last hit world leaf's
//    closest triangle, exactly as the reference returns it;
//  * ties keep the first triangle found (strict t < closest).
// Vertices are pre-transformed on upload with the reference's operation order, which
// gives the same floats the reference recomputes per test.
#pragma once
#include "dev_math.cuh"

namespace rc {

// Device view of the scene.  Nodes: two float4 per node (min.xyz|w0, max.xyz|w1), the
// mesh nodes interleaved in one array (node i at nodes[2i], nodes[2i+1]: one 32-byte
// sector per visit).  Mesh-level inner nodes hold global child indices; mesh-level
// leaves hold (0x80000000|count, first triangle slot).  World leaves hold
// (0x80000000|count, first slot in world_mesh).  Triangles are stored in leaf order,
// the three records a test reads interleaved (slot j at tris[3j .. 3j+2]).
struct SceneView {
    const float4* __restrict__ nodes;       // mesh BVH nodes, 2 per node
    const float4* __restrict__ wnode_lo;
    const float4* __restrict__ wnode_hi;
    const int* __restrict__ world_mesh;     // mesh id per world-leaf slot
    const int* __restrict__ mesh_root;      // global root node per mesh
    const float4* __restrict__ tris;        // 3 per triangle: v0.xyz | global triangle id,
                                            // (v1 - v0).xyz | material, (v2 - v0).xyz | mesh id
    const float4* __restrict__ tri_n0;      // vertex normals (normalised, world space)
    const float4* __restrict__ tri_n1;
    const float4* __restrict__ tri_n2;
    int num_world_nodes;
    int num_meshes;
};

constexpr int kStackSize = 64;   // BVH_STACK_SIZE in the reference

// Traversal stacks.  LocalStack / LocalPairStack: per-thread arrays (local memory),
// declared by each mesh traversal when the caller passes the CallStack or
// WarpStepStack tag, so that their lifetime is the traversal.  (Stacks held for a
// whole persistent kernel, or kept in shared memory as [kStackSize][block] columns,
// measured 1.5-3.6x slower on the water workload.)  Any type with int& operator[] can
// serve as the stack of mesh_traverse_impl.
struct LocalStack {
    int s[kStackSize];
    __device__ __forceinline__ int& operator[](int i) { return s[i]; }
};
// CallStack: the tag of the persistent passes' traversal (mesh_traverse_children).
struct CallStack {};
// WarpStepStack: the tag of the warp-stepped traversal (mesh_traverse_steps), for
// kernels whose lanes all trace at once; its per-traversal stack holds node index and
// box entry distance (float bits) per entry.
struct WarpStepStack {};
struct LocalPairStack {
    int2 s[kStackSize];
    __device__ __forceinline__ int2& operator[](int i) { return s[i]; }
};

struct HitRec {
    float t, u, v;
    int slot;       // triangle slot (leaf order) of the reported hit, -1 if none
};

// aabb::hit with the per-ray reciprocals (1/d computed once: the same division the
// reference repeats per box).  NaN and -0 behaviour follows the ternaries as written.
__device__ __forceinline__ bool box_hit(float4 lo, float4 hi, F3 o, F3 inv, float tmin, float tmax) {
    float t0 = (lo.x - o.x) * inv.x, t1 = (hi.x - o.x) * inv.x;
    if (inv.x < 0) { float s = t0; t0 = t1; t1 = s; }
    tmin = t0 > tmin ? t0 : tmin;
    tmax = t1 < tmax ? t1 : tmax;
    if (tmax < tmin) return false;
    t0 = (lo.y - o.y) * inv.y; t1 = (hi.y - o.y) * inv.y;
    if (inv.y < 0) { float s = t0; t0 = t1; t1 = s; }
    tmin = t0 > tmin ? t0 : tmin;
    tmax = t1 < tmax ? t1 : tmax;
    if (tmax < tmin) return false;
    t0 = (lo.z - o.z) * inv.z; t1 = (hi.z - o.z) * inv.z;
    if (inv.z < 0) { float s = t0; t0 = t1; t1 = s; }
    tmin = t0 > tmin ? t0 : tmin;
    tmax = t1 < tmax ? t1 : tmax;
    if (tmax < tmin) return false;
    return true;
}

// box_hit in two parts: the same slab arithmetic, with the box's entry distance n
// (tmin and the three near-slab distances, NaNs skipped, as box_hit folds them) kept.
// box_hit's early exits never change its answer (the interval only narrows), so it
// equals !(far < near) over all three slabs: box_entry returns exactly box_hit(tmax),
// and for any tmax' <= tmax, box_hit(tmax') == box_entry(tmax) && !(tmax' < n).
__device__ __forceinline__ bool box_entry(float4 lo, float4 hi, F3 o, F3 inv, float tmin, float tmax, float& n) {
    float a = tmin, b = tmax;
    float t0 = (lo.x - o.x) * inv.x, t1 = (hi.x - o.x) * inv.x;
    if (inv.x < 0) { float s = t0; t0 = t1; t1 = s; }
    a = t0 > a ? t0 : a;
    b = t1 < b ? t1 : b;
    t0 = (lo.y - o.y) * inv.y; t1 = (hi.y - o.y) * inv.y;
    if (inv.y < 0) { float s = t0; t0 = t1; t1 = s; }
    a = t0 > a ? t0 : a;
    b = t1 < b ? t1 : b;
    t0 = (lo.z - o.z) * inv.z; t1 = (hi.z - o.z) * inv.z;
    if (inv.z < 0) { float s = t0; t0 = t1; t1 = s; }
    a = t0 > a ? t0 : a;
    b = t1 < b ? t1 : b;
    n = a;
    return !(b < a);
}

// Möller-Trumbore as src/Triangle.cpp:44-66 computes it.
__device__ __forceinline__ bool tri_hit(const SceneView& s, int slot, F3 o, F3 d, float tmin, float tmax,
                                        float& t_out, float& u_out, float& v_out) {
    float4 a = __ldg(&s.tris[3 * slot]);
    float4 b = __ldg(&s.tris[3 * slot + 1]);
    float4 c = __ldg(&s.tris[3 * slot + 2]);
    F3 v0 = xyz(a), e1 = xyz(b), e2 = xyz(c);
    F3 pvec = cross(d, e2);
    float det = dot(e1, pvec);
    if (fabsf(det) < 0.0000001f) return false;
    float inv_det = 1.0f / det;
    F3 tvec = o - v0;
    float u = dot(tvec, pvec) * inv_det;
    if (u < 0.0f || u > 1.0f) return false;
    F3 qvec = cross(tvec, e1);
    float v = dot(d, qvec) * inv_det;
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = dot(e2, qvec) * inv_det;
    if (t > tmin && t < tmax) {
        t_out = t; u_out = u; v_out = v;
        return true;
    }
    return false;
}

// Mesh::hit on one mesh with the running record of the current world leaf.
// Returns false (and sets *overflow) if the stack would exceed kStackSize.
template <class Stack>
__device__ __forceinline__ bool mesh_traverse(const SceneView& s, int mesh, F3 o, F3 d, F3 inv, float tmin,
                                              HitRec& rec, bool& any, int* overflow, Stack& stack);

template <class Stack>
__device__ __forceinline__ bool mesh_traverse_impl(const SceneView& s, int mesh, F3 o, F3 d, F3 inv, float tmin,
                                                   HitRec& rec, bool& any, int* overflow, Stack& stack) {
    int sp = 0;
    stack[sp++] = __ldg(&s.mesh_root[mesh]);
    while (sp) {
        int id = stack[--sp];
        float4 lo = __ldg(&s.nodes[2 * id]);
        float4 hi = __ldg(&s.nodes[2 * id + 1]);
        if (!box_hit(lo, hi, o, inv, tmin, rec.t)) continue;
        uint32_t w0 = __float_as_uint(lo.w), w1 = __float_as_uint(hi.w);
        if (w0 & 0x80000000u) {
            int cnt = (int)(w0 & 0x7fffffffu);
            for (int k = 0; k < cnt; ++k) {
                int slot = (int)w1 + k;
                float t, u, v;
                if (tri_hit(s, slot, o, d, tmin, rec.t, t, u, v)) {
                    rec.t = t; rec.u = u; rec.v = v; rec.slot = slot;
                    any = true;
                }
            }
        } else {
            if (sp + 2 > kStackSize) { *overflow = 1; return false; }
            stack[sp++] = (int)w1;   // right first ...
            stack[sp++] = (int)w0;   // ... so the left child is popped first
        }
    }
    return true;
}

// Mesh::hit (src/mesh.cpp:70-105) visits nodes in left-first DFS order and tests each
// box when it is popped, against the running distance then.  mesh_traverse_children
// (the persistent passes, one lane per ray) and mesh_traverse_steps (the wavefront
// pass, a warp's lanes stepping together) test both children's boxes at their parent
// instead, with the same outcome (below).  Measured on the water pool (light pass per
// iteration): pop-and-test (mesh_traverse_impl) 13.3 ms, children tested at the parent
// 11.9 ms, the same with a warp's lanes stepping together (mesh_traverse_steps) 13.3
// ms, four-wide records of grandchildren tested at the grandparent 14.7 ms.
template <class Stack>
__device__ __forceinline__ bool mesh_traverse_children(const SceneView& s, int mesh, F3 o, F3 d, F3 inv,
                                                       float tmin, HitRec& rec, bool& any, int* overflow,
                                                       Stack& stack) {
    const int root = __ldg(&s.mesh_root[mesh]);
    float4 lo = __ldg(&s.nodes[2 * root]);
    float4 hi = __ldg(&s.nodes[2 * root + 1]);
    float n;
    bool active = box_entry(lo, hi, o, inv, tmin, rec.t, n);
    int sp = 0;
    while (active) {
        const uint32_t w0 = __float_as_uint(lo.w), w1 = __float_as_uint(hi.w);
        bool descend = false;
        if (!(w0 & 0x80000000u)) {
            // both children's boxes (two independent loads in flight) at the distance now;
            // the left one is the reference's next test exactly, the right one waits with
            // its entry distance
            const float4 llo = __ldg(&s.nodes[2 * w0]), lhi = __ldg(&s.nodes[2 * w0 + 1]);
            const float4 rlo = __ldg(&s.nodes[2 * w1]), rhi = __ldg(&s.nodes[2 * w1 + 1]);
            float nl, nr;
            const bool hl = box_entry(llo, lhi, o, inv, tmin, rec.t, nl);
            const bool hr = box_entry(rlo, rhi, o, inv, tmin, rec.t, nr);
            if (hl && hr) {
                if (sp >= kStackSize) { *overflow = 1; return false; }
                stack[sp++] = make_int2((int)w1, __float_as_int(nr));
            }
            descend = hl || hr;
            lo = hl ? llo : rlo;
            hi = hl ? lhi : rhi;
        } else {
            const int cnt = (int)(w0 & 0x7fffffffu);
            for (int k = 0; k < cnt; ++k) {
                const int slot = (int)w1 + k;
                float t, u, v;
                if (tri_hit(s, slot, o, d, tmin, rec.t, t, u, v)) {
                    rec.t = t; rec.u = u; rec.v = v; rec.slot = slot;
                    any = true;
                }
            }
        }
        if (!descend) {
            // pop pending right children until one whose box the current distance reaches
            int next = -1;
            while (sp > 0 && next < 0) {
                const int2 e = stack[--sp];
                if (!(rec.t < __int_as_float(e.y))) next = e.x;
            }
            active = next >= 0;
            if (active) {
                lo = __ldg(&s.nodes[2 * next]);
                hi = __ldg(&s.nodes[2 * next + 1]);
            }
        }
    }
    return true;
}

// Why testing the children at their parent gives the reference's result: the left
// child is the node the reference pops next, with the same distance, so its test is
// the reference's; the right child is popped only after the left subtree, when the
// distance may have shrunk.  The distance never grows, so a right box that fails now
// fails then too (box_hit is monotone in tmax) and is not pushed; one that passes is
// pushed with its entry distance n, and at its pop the reference's test is
// !(distance < n) (box_entry).  Same nodes, same triangles, same order.
template <class Stack>
__device__ __forceinline__ bool mesh_traverse_steps(const SceneView& s, int mesh, F3 o, F3 d, F3 inv, float tmin,
                                                   HitRec& rec, bool& any, int* overflow, Stack& stack) {
    // the lanes that arrive together step together: one node per lane per round, the
    // round ending in a vote, so that a warp's lanes meet again after every node
    const unsigned lanes = __activemask();
    const int root = __ldg(&s.mesh_root[mesh]);
    float4 lo = __ldg(&s.nodes[2 * root]);
    float4 hi = __ldg(&s.nodes[2 * root + 1]);
    float n;
    bool active = box_entry(lo, hi, o, inv, tmin, rec.t, n);
    int sp = 0;
    bool ok = true;
    while (__any_sync(lanes, active)) {
        if (!active) continue;
        const uint32_t w0 = __float_as_uint(lo.w), w1 = __float_as_uint(hi.w);
        bool descend = false;
        if (!(w0 & 0x80000000u)) {
            const float4 llo = __ldg(&s.nodes[2 * w0]), lhi = __ldg(&s.nodes[2 * w0 + 1]);
            const float4 rlo = __ldg(&s.nodes[2 * w1]), rhi = __ldg(&s.nodes[2 * w1 + 1]);
            float nl, nr;
            const bool hl = box_entry(llo, lhi, o, inv, tmin, rec.t, nl);
            const bool hr = box_entry(rlo, rhi, o, inv, tmin, rec.t, nr);
            if (hl && hr) {
                if (sp < kStackSize) stack[sp++] = make_int2((int)w1, __float_as_int(nr));
                else { *overflow = 1; ok = false; active = false; continue; }
            }
            descend = hl || hr;
            lo = hl ? llo : rlo;
            hi = hl ? lhi : rhi;
        } else {
            const int cnt = (int)(w0 & 0x7fffffffu);
            for (int k = 0; k < cnt; ++k) {
                const int slot = (int)w1 + k;
                float t, u, v;
                if (tri_hit(s, slot, o, d, tmin, rec.t, t, u, v)) {
                    rec.t = t; rec.u = u; rec.v = v; rec.slot = slot;
                    any = true;
                }
            }
        }
        if (!descend) {
            // pop pending right children until one whose box the current distance reaches
            int next = -1;
            while (sp > 0 && next < 0) {
                const int2 e = stack[--sp];
                if (!(rec.t < __int_as_float(e.y))) next = e.x;
            }
            active = next >= 0;
            if (active) {
                lo = __ldg(&s.nodes[2 * next]);
                hi = __ldg(&s.nodes[2 * next + 1]);
            }
        }
    }
    return ok;
}

template <class Stack>
__device__ __forceinline__ bool mesh_traverse(const SceneView& s, int mesh, F3 o, F3 d, F3 inv, float tmin,
                                              HitRec& rec, bool& any, int* overflow, Stack& stack) {
    return mesh_traverse_impl(s, mesh, o, d, inv, tmin, rec, any, overflow, stack);
}
template <>
__device__ __forceinline__ bool mesh_traverse<CallStack>(const SceneView& s, int mesh, F3 o, F3 d, F3 inv,
                                                         float tmin, HitRec& rec, bool& any, int* overflow,
                                                         CallStack&) {
    LocalPairStack st;
    return mesh_traverse_children(s, mesh, o, d, inv, tmin, rec, any, overflow, st);
}
template <>
__device__ __forceinline__ bool mesh_traverse<WarpStepStack>(const SceneView& s, int mesh, F3 o, F3 d, F3 inv,
                                                             float tmin, HitRec& rec, bool& any, int* overflow,
                                                             WarpStepStack&) {
    LocalPairStack st;
    return mesh_traverse_steps(s, mesh, o, d, inv, tmin, rec, any, overflow, st);
}

// Scene::hit.  `out` is the reported record (t = inf when nothing was hit).  `stack`
// serves the mesh levels; the world level (several world leaves only) uses its own.
template <class Stack>
__device__ __forceinline__ bool scene_hit(const SceneView& s, F3 o, F3 d, float tmin, HitRec& out, int* overflow,
                                          Stack& stack) {
    F3 inv = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    out.t = INFINITY; out.u = 0.0f; out.v = 0.0f; out.slot = -1;
    bool hit = false;
    if (s.num_world_nodes == 1) {
        // single world leaf: the common case (one leaf holding every mesh)
        float4 lo = __ldg(&s.wnode_lo[0]);
        float4 hi = __ldg(&s.wnode_hi[0]);
        if (!box_hit(lo, hi, o, inv, tmin, out.t)) return false;
        uint32_t w0 = __float_as_uint(lo.w), w1 = __float_as_uint(hi.w);
        int cnt = (int)(w0 & 0x7fffffffu);
        HitRec leaf = {INFINITY, 0.0f, 0.0f, -1};
        bool any = false;
        for (int k = 0; k < cnt; ++k) {
            int mesh = __ldg(&s.world_mesh[w1 + k]);
            bool mesh_any = false;
            if (!mesh_traverse(s, mesh, o, d, inv, tmin, leaf, mesh_any, overflow, stack)) return false;
            any |= mesh_any;
        }
        if (any) out = leaf;
        return any;
    }
    int wstack[kStackSize];
    int sp = 0;
    wstack[sp++] = 0;
    while (sp) {
        int id = wstack[--sp];
        float4 lo = __ldg(&s.wnode_lo[id]);
        float4 hi = __ldg(&s.wnode_hi[id]);
        if (!box_hit(lo, hi, o, inv, tmin, out.t)) continue;
        uint32_t w0 = __float_as_uint(lo.w), w1 = __float_as_uint(hi.w);
        if (w0 & 0x80000000u) {
            int cnt = (int)(w0 & 0x7fffffffu);
            HitRec leaf = {INFINITY, 0.0f, 0.0f, -1};   // fresh Isect temp_rec
            bool any = false;
            for (int k = 0; k < cnt; ++k) {
                int mesh = __ldg(&s.world_mesh[w1 + k]);
                bool mesh_any = false;
                if (!mesh_traverse(s, mesh, o, d, inv, tmin, leaf, mesh_any, overflow, stack)) return false;
                any |= mesh_any;
            }
            if (any) { out = leaf; hit = true; }   // unconditional overwrite (world-leaf quirk)
        } else {
            if (sp + 2 > kStackSize) { *overflow = 1; return false; }
            wstack[sp++] = (int)w1;
            wstack[sp++] = (int)w0;
        }
    }
    return hit;
}

// Scene::hit with per-traversal local-memory stacks.
__device__ __forceinline__ bool scene_hit(const SceneView& s, F3 o, F3 d, float tmin, HitRec& out, int* overflow) {
    CallStack st;
    return scene_hit(s, o, d, tmin, out, overflow, st);
}

// Attributes Triangle::hit fills in (src/Triangle.cpp:68-80), for the reported triangle.
struct Isect {
    F3 ng, ns, pos, dir;
    float t, u, v;
    bool front;
    int material;
    int tri;     // global triangle id
    int mesh;
};

__device__ __forceinline__ void fill_isect(const SceneView& s, const HitRec& h, F3 o, F3 d, Isect& is) {
    float4 a = __ldg(&s.tris[3 * h.slot]);
    float4 b = __ldg(&s.tris[3 * h.slot + 1]);
    float4 c = __ldg(&s.tris[3 * h.slot + 2]);
    F3 e1 = xyz(b), e2 = xyz(c);
    is.t = h.t; is.u = h.u; is.v = h.v;
    is.ng = normalize(cross(e1, e2));
    F3 n0 = xyz(__ldg(&s.tri_n0[h.slot]));
    F3 n1 = xyz(__ldg(&s.tri_n1[h.slot]));
    F3 n2 = xyz(__ldg(&s.tri_n2[h.slot]));
    float w = 1 - h.u - h.v;
    is.ns = n0 * w + n1 * h.u + n2 * h.v;
    is.front = dot(is.ns, d) < 0;
    is.pos = o + d * h.t;
    is.dir = d;
    is.tri = (int)__float_as_uint(a.w);
    is.material = (int)__float_as_uint(b.w);
    is.mesh = (int)__float_as_uint(c.w);
}

}  // namespace rc
