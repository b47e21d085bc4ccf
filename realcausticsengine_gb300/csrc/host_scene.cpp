// Host-side scene construction: Blender mesh ingest, reference-identical two-level
// SAH BVH, light and material conversion.
//
// Every floating-point expression below keeps the reference's operation order and
// types (float vs double) so that the BVH boxes, split decisions and the world-space
// triangles are bit-identical to what the reference computes; the GPU traversal then
// returns bit-identical hits.  This file is compiled with -ffp-contract=off.
#include "host_scene.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <utility>

namespace rc {

namespace {

inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul(const V3& a, float t) { return {a.x * t, a.y * t, a.z * t}; }
inline float dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& u, const V3& v) {
    return {u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x};
}
// vec3 / float is a reciprocal multiply in the reference (src/vec3.h:154-157)
inline V3 normalize(const V3& u) {
    float len = std::sqrt(u.x * u.x + u.y * u.y + u.z * u.z);
    return mul(u, 1 / len);
}
inline float comp(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
// std::min / std::max argument order as the reference calls them
inline float fmin_ref(float a, float b) { return (b < a) ? b : a; }
inline float fmax_ref(float a, float b) { return (a < b) ? b : a; }

inline Box box_union(const Box& a, const Box& b) {
    Box r;
    r.mn = {fmin_ref(a.mn.x, b.mn.x), fmin_ref(a.mn.y, b.mn.y), fmin_ref(a.mn.z, b.mn.z)};
    r.mx = {fmax_ref(a.mx.x, b.mx.x), fmax_ref(a.mx.y, b.mx.y), fmax_ref(a.mx.z, b.mx.z)};
    return r;
}
inline Box box_union(const Box& a, const V3& p) {
    Box r;
    r.mn = {fmin_ref(a.mn.x, p.x), fmin_ref(a.mn.y, p.y), fmin_ref(a.mn.z, p.z)};
    r.mx = {fmax_ref(a.mx.x, p.x), fmax_ref(a.mx.y, p.y), fmax_ref(a.mx.z, p.z)};
    return r;
}
// aabb::SurfaceArea (src/aabb.cpp:54-58)
inline float surface_area(const Box& b) {
    V3 d = sub(b.mx, b.mn);
    return 2 * (d.x * d.y + d.x * d.z + d.y * d.z);
}
// aabb::MaximumExtent (src/aabb.cpp:60-69)
inline int max_extent(const Box& b) {
    V3 d = sub(b.mx, b.mn);
    if (d.x > d.y && d.x > d.z) return 0;
    if (d.y > d.z) return 1;
    return 2;
}
// aabb::Offset(p)[dim] followed by the bucket computation (src/BVH/BVH_mesh.cpp:98-101)
inline int bucket_of(const Box& cb, const V3& c, int dim) {
    float o = (comp(c, dim) - comp(cb.mn, dim)) / (comp(cb.mx, dim) - comp(cb.mn, dim));
    int b = (int)(12 * o);
    return b == 12 ? 11 : b;
}

struct Prim {
    uint32_t index;
    Box box;
    V3 center;
    int cost;   // world level only (aabb_temp_world::cost is an int)
};

// Hoare-style partition with the element order std::partition produces for
// random-access ranges in libstdc++: scan from the front for the first element
// failing the predicate, from the back for the last one passing it, swap, repeat.
template <class Pred>
size_t hoare_partition(std::vector<Prim>& v, size_t first, size_t last, Pred pred) {
    while (true) {
        while (true) {
            if (first == last) return first;
            if (pred(v[first])) ++first; else break;
        }
        --last;
        while (true) {
            if (first == last) return first;
            if (!pred(v[last])) --last; else break;
        }
        std::swap(v[first], v[last]);
        ++first;
    }
}

struct TmpNode {
    Box box;
    bool leaf = false;
    int left = -1, right = -1;     // indices into the temporary node pool
    uint32_t first = 0, count = 0; // leaf contents: prims [first, first + count) in order
};

// The recursive binned SAH build shared by both levels.  `world` selects the world
// variant (per-mesh traversal-cost weights, leaf cost summed over the first 11
// buckets, src/BVH/BVH_world.cpp:25-159) instead of the mesh variant
// (src/BVH/BVH_mesh.cpp:28-155).
// Subtrees of at least kParallelPrims primitives, down to kParallelDepth levels of
// splitting, are built concurrently (up to 2^kParallelDepth threads).
constexpr size_t kParallelPrims = 16384;
constexpr int kParallelDepth = 4;
thread_local int g_par_depth = 0;

// Order-independent reduction (box unions, counts) over [start, end) on several
// threads for large ranges: `acc(R&, i)` folds item i, `merge(R&, const R&)` joins.
constexpr size_t kParallelLoop = 131072;
template <class R, class Acc, class Merge>
R par_reduce(size_t start, size_t end, const R& init, Acc&& acc, Merge&& merge) {
    const size_t n = end - start;
    static const unsigned hw = std::thread::hardware_concurrency();   // queried once
    const unsigned nt = hw < 1 ? 1 : (hw > 16 ? 16 : hw);
    if (n < kParallelLoop || nt == 1) {
        R r = init;
        for (size_t i = start; i < end; ++i) acc(r, i);
        return r;
    }
    std::vector<R> part(nt, init);
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < nt; ++t)
        ts.emplace_back([&, t]() {
            const size_t a = start + n * t / nt, b = start + n * (t + 1) / nt;
            R local = init;   // thread-local accumulator (no shared cache lines while folding)
            for (size_t i = a; i < b; ++i) acc(local, i);
            part[t] = local;
        });
    for (auto& t : ts) t.join();
    R r = init;
    for (const R& q : part) merge(r, q);
    return r;
}

// fn(begin, end) over [0, n) in contiguous pieces on several threads for large n
// (per-element work only: the results do not depend on the split).
template <class Fn>
void par_for(size_t n, Fn&& fn) {
    static const unsigned hw = std::thread::hardware_concurrency();
    const unsigned nt = hw < 1 ? 1 : (hw > 16 ? 16 : hw);
    if (n < kParallelLoop || nt == 1) { fn(0, n); return; }
    std::vector<std::thread> ts;
    for (unsigned t = 1; t < nt; ++t) ts.emplace_back([&, t]() { fn(n * t / nt, n * (t + 1) / nt); });
    fn(0, n / nt);
    for (auto& t : ts) t.join();
}

int sah_recurse(std::vector<Prim>& p, size_t start, size_t end, bool world, std::vector<TmpNode>& pool) {
    const Box bbox = par_reduce(start, end, Box{}, [&](Box& b, size_t i) { b = box_union(b, p[i].box); },
                                [](Box& a, const Box& b) { a = box_union(a, b); });
    size_t n = end - start;
    int me = (int)pool.size();
    pool.emplace_back();
    pool[me].box = bbox;
    if (n == 1) {
        pool[me].leaf = true;
        pool[me].first = (uint32_t)start;
        pool[me].count = 1;
        return me;
    }
    const Box cb = par_reduce(start, end, Box{}, [&](Box& b, size_t i) { b = box_union(b, p[i].center); },
                              [](Box& a, const Box& b) { a = box_union(a, b); });
    int dim = max_extent(cb);
    size_t mid = (start + end) / 2;
    auto make_leaf = [&]() {
        // the range is final: later splits only permute other (disjoint) ranges
        pool[me].leaf = true;
        pool[me].first = (uint32_t)start;
        pool[me].count = (uint32_t)n;
        return me;
    };
    if (comp(cb.mx, dim) == comp(cb.mn, dim)) return make_leaf();
    if (n == 2) {
        if (!(comp(p[start].center, dim) < comp(p[end - 1].center, dim))) std::swap(p[start], p[end - 1]);
    } else {
        constexpr int nb = 12;
        int count[nb] = {0};
        Box bb[nb];
        float travers[nb] = {0};
        if (world || n < kParallelLoop) {
            for (size_t i = start; i < end; ++i) {
                int b = bucket_of(cb, p[i].center, dim);
                count[b]++;
                bb[b] = box_union(bb[b], p[i].box);
                if (world) travers[b] += p[i].cost;   // float sums: kept sequential
            }
        } else {
            struct Bins { int count[nb]; Box bb[nb]; };
            Bins z{};
            for (int k = 0; k < nb; ++k) z.bb[k] = Box{};
            const Bins r = par_reduce(start, end, z, [&](Bins& bs, size_t i) {
                const int b = bucket_of(cb, p[i].center, dim);
                bs.count[b]++;
                bs.bb[b] = box_union(bs.bb[b], p[i].box);
            }, [](Bins& a, const Bins& b) {
                for (int k = 0; k < nb; ++k) { a.count[k] += b.count[k]; a.bb[k] = box_union(a.bb[k], b.bb[k]); }
            });
            for (int k = 0; k < nb; ++k) { count[k] = r.count[k]; bb[k] = r.bb[k]; }
        }
        float cost[nb - 1];
        float sa = surface_area(bbox);
        for (int i = 0; i < nb - 1; ++i) {
            Box b0, b1;
            int c0 = 0, c1 = 0;
            int t0 = 0, t1 = 0;
            for (int j = 0; j <= i; ++j) {
                b0 = box_union(b0, bb[j]);
                c0 += count[j];
                if (world) t0 += travers[j];   // int += float, as the reference
            }
            for (int j = i + 1; j < nb; ++j) {
                b1 = box_union(b1, bb[j]);
                c1 += count[j];
                if (world) t1 += travers[j];
            }
            if (world)
                cost[i] = 0.16874 + (surface_area(b0) * t0 + surface_area(b1) * t1) / sa;
            else
                cost[i] = 0.16874 + (c0 * surface_area(b0) + c1 * surface_area(b1)) / sa;
        }
        float min_cost = cost[0];
        float min_bucket = 0;   // float in the reference
        float leaf_cost = 0;
        for (int i = 0; i < nb - 1; ++i) {
            if (world) leaf_cost += travers[i];
            if (cost[i] < min_cost) { min_cost = cost[i]; min_bucket = i; }
        }
        if (!world) leaf_cost = (float)n;
        if (min_cost < leaf_cost) {
            size_t m = hoare_partition(p, start, end, [&](const Prim& q) {
                return bucket_of(cb, q.center, dim) <= min_bucket;
            });
            mid = m;
        } else {
            return make_leaf();
        }
    }
    int l, r;
    if (n >= kParallelPrims && g_par_depth < kParallelDepth) {
        // the two halves touch disjoint ranges of `p`: build the left one on another
        // thread into its own pool, then splice it in (child links re-based); node
        // numbering in the pool does not reach the output, which flatten() orders by
        // the tree's own pre-order
        std::vector<TmpNode> lpool;
        lpool.reserve((mid - start) * 2);
        int lroot = -1;
        const int depth = g_par_depth + 1;
        std::thread t([&]() {
            g_par_depth = depth;
            lroot = sah_recurse(p, start, mid, world, lpool);
        });
        g_par_depth = depth;
        r = sah_recurse(p, mid, end, world, pool);
        g_par_depth = depth - 1;
        t.join();
        const int base = (int)pool.size();
        for (TmpNode& tn : lpool) {
            if (!tn.leaf) { tn.left += base; tn.right += base; }
            pool.push_back(std::move(tn));
        }
        l = lroot + base;
    } else {
        l = sah_recurse(p, start, mid, world, pool);
        r = sah_recurse(p, mid, end, world, pool);
    }
    pool[me].left = l;
    pool[me].right = r;
    return me;
}

// Depth-first flattening (populate_cache_friendly_bvh, src/BVH/BVH_mesh.cpp:199-261):
// pre-order node numbering, left child = parent + 1, 1-based item list.
void flatten(const std::vector<TmpNode>& pool, const std::vector<Prim>& prims, int t, uint32_t& idx_nodes,
             uint32_t& idx_items, std::vector<BvhNode>& nodes, std::vector<int>& items) {
    const TmpNode& n = pool[t];
    uint32_t cur = idx_nodes;
    nodes[cur].box = n.box;
    if (!n.leaf) {
        uint32_t l = ++idx_nodes;
        flatten(pool, prims, n.left, idx_nodes, idx_items, nodes, items);
        uint32_t r = ++idx_nodes;
        flatten(pool, prims, n.right, idx_nodes, idx_items, nodes, items);
        nodes[cur].w0 = l;
        nodes[cur].w1 = r;
    } else {
        nodes[cur].w0 = 0x80000000u | n.count;
        nodes[cur].w1 = idx_items;
        for (uint32_t k = 0; k < n.count; ++k) items[++idx_items] = (int)prims[n.first + k].index;
    }
}

void build_flat(std::vector<Prim>& prims, bool world, std::vector<BvhNode>& nodes, std::vector<int>& items, Box& root_box) {
    std::vector<TmpNode> pool;
    pool.reserve(prims.size() * 2);
    int root = sah_recurse(prims, 0, prims.size(), world, pool);
    root_box = pool[root].box;
    size_t nitems = 0;
    for (const TmpNode& t : pool) nitems += t.count;
    nodes.assign(pool.size(), BvhNode{});
    items.assign(nitems + 1, 0);
    uint32_t in = 0, ii = 0;
    flatten(pool, prims, root, in, ii, nodes, items);
}

// Inverse (src/matrix.cpp:4-63): cofactor expansion in double, rounded to float.
void inverse4(const float* mf, float* out) {
    double m[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) m[i][j] = mf[4 * i + j];
    double A2323 = m[2][2] * m[3][3] - m[2][3] * m[3][2];
    double A1323 = m[2][1] * m[3][3] - m[2][3] * m[3][1];
    double A1223 = m[2][1] * m[3][2] - m[2][2] * m[3][1];
    double A0323 = m[2][0] * m[3][3] - m[2][3] * m[3][0];
    double A0223 = m[2][0] * m[3][2] - m[2][2] * m[3][0];
    double A0123 = m[2][0] * m[3][1] - m[2][1] * m[3][0];
    double A2313 = m[1][2] * m[3][3] - m[1][3] * m[3][2];
    double A1313 = m[1][1] * m[3][3] - m[1][3] * m[3][1];
    double A1213 = m[1][1] * m[3][2] - m[1][2] * m[3][1];
    double A2312 = m[1][2] * m[2][3] - m[1][3] * m[2][2];
    double A1312 = m[1][1] * m[2][3] - m[1][3] * m[2][1];
    double A1212 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
    double A0313 = m[1][0] * m[3][3] - m[1][3] * m[3][0];
    double A0213 = m[1][0] * m[3][2] - m[1][2] * m[3][0];
    double A0312 = m[1][0] * m[2][3] - m[1][3] * m[2][0];
    double A0212 = m[1][0] * m[2][2] - m[1][2] * m[2][0];
    double A0113 = m[1][0] * m[3][1] - m[1][1] * m[3][0];
    double A0112 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    double det = m[0][0] * (m[1][1] * A2323 - m[1][2] * A1323 + m[1][3] * A1223)
               - m[0][1] * (m[1][0] * A2323 - m[1][2] * A0323 + m[1][3] * A0223)
               + m[0][2] * (m[1][0] * A1323 - m[1][1] * A0323 + m[1][3] * A0123)
               - m[0][3] * (m[1][0] * A1223 - m[1][1] * A0223 + m[1][2] * A0123);
    det = 1.0 / det;
    out[0] = (float)(det * (m[1][1] * A2323 - m[1][2] * A1323 + m[1][3] * A1223));
    out[1] = (float)(det * -(m[0][1] * A2323 - m[0][2] * A1323 + m[0][3] * A1223));
    out[2] = (float)(det * (m[0][1] * A2313 - m[0][2] * A1313 + m[0][3] * A1213));
    out[3] = (float)(det * -(m[0][1] * A2312 - m[0][2] * A1312 + m[0][3] * A1212));
    out[4] = (float)(det * -(m[1][0] * A2323 - m[1][2] * A0323 + m[1][3] * A0223));
    out[5] = (float)(det * (m[0][0] * A2323 - m[0][2] * A0323 + m[0][3] * A0223));
    out[6] = (float)(det * -(m[0][0] * A2313 - m[0][2] * A0313 + m[0][3] * A0213));
    out[7] = (float)(det * (m[0][0] * A2312 - m[0][2] * A0312 + m[0][3] * A0212));
    out[8] = (float)(det * (m[1][0] * A1323 - m[1][1] * A0323 + m[1][3] * A0123));
    out[9] = (float)(det * -(m[0][0] * A1323 - m[0][1] * A0323 + m[0][3] * A0123));
    out[10] = (float)(det * (m[0][0] * A1313 - m[0][1] * A0313 + m[0][3] * A0113));
    out[11] = (float)(det * -(m[0][0] * A1312 - m[0][1] * A0312 + m[0][3] * A0112));
    out[12] = (float)(det * -(m[1][0] * A1223 - m[1][1] * A0223 + m[1][2] * A0123));
    out[13] = (float)(det * (m[0][0] * A1223 - m[0][1] * A0223 + m[0][2] * A0123));
    out[14] = (float)(det * -(m[0][0] * A1213 - m[0][1] * A0213 + m[0][2] * A0113));
    out[15] = (float)(det * (m[0][0] * A1212 - m[0][1] * A0212 + m[0][2] * A0112));
}

// matrix_3x3(vec3 r) (src/matrix.cpp:70-80).  The unqualified cos/sin there are the
// C library's double versions; products are formed in double and rounded when the
// vec3 is built.
struct M3 { V3 i, j, k; };
M3 rotation_matrix(V3 r) {
    double cx = std::cos((double)r.x), sx = std::sin((double)r.x);
    double cy = std::cos((double)r.y), sy = std::sin((double)r.y);
    double cz = std::cos((double)r.z), sz = std::sin((double)r.z);
    M3 m;
    m.i = {(float)(cz * cy), (float)(sz * cy), (float)(-sy)};
    m.j = {(float)(cz * sy * sx - sz * cx), (float)(sz * sy * sx + cz * cx), (float)(cy * sx)};
    m.k = {(float)(cz * sy * cx + sz * sx), (float)(sz * sy * cx - cz * sx), (float)(cy * cx)};
    return m;
}
// vec3 * matrix_3x3 (src/matrix.h:92-95)
inline V3 vmul(const V3& v, const M3& m) { return add(add(mul(m.i, v.x), mul(m.j, v.y)), mul(m.k, v.z)); }

void frame_from_z(const V3& z, float* fx, float* fy, float* fz) {
    V3 tx = (std::fabs(z.x) > 0.99f) ? V3{0.0f, 1.0f, 0.0f} : V3{1.0f, 0.0f, 0.0f};
    V3 y = normalize(cross(z, tx));
    V3 x = cross(y, z);
    fx[0] = x.x; fx[1] = x.y; fx[2] = x.z;
    fy[0] = y.x; fy[1] = y.y; fy[2] = y.z;
    fz[0] = z.x; fz[1] = z.y; fz[2] = z.z;
}

}  // namespace

int ingest_mesh(HostMesh& out, const void* blender_mesh, unsigned nverts, unsigned ntris,
                const rc_matrix4x4& matrix, const int* material_indices, std::string& err) {
    if (!blender_mesh) { err = "null Blender mesh pointer"; return RC_E_INVALID; }
    if (!material_indices) { err = "null material index array"; return RC_E_INVALID; }
    // Mesh_blender field offsets in the 2.9x DNA layout (src/Blender_definitions.h:214-311)
    const char* base = static_cast<const char*>(blender_mesh);
    const char* mpoly; const char* mloop; const char* mvert;
    std::memcpy(&mpoly, base + 200, sizeof(void*));
    std::memcpy(&mloop, base + 208, sizeof(void*));
    std::memcpy(&mvert, base + 256, sizeof(void*));
    if (ntris && (!mpoly || !mloop)) { err = "Blender mesh has null mpoly/mloop"; return RC_E_INVALID; }
    if (nverts && !mvert) { err = "Blender mesh has null mvert"; return RC_E_INVALID; }
    out.num_tris = ntris;
    out.num_verts = nverts;
    std::memcpy(out.m, matrix.t, sizeof(out.m));
    inverse4(out.m, out.inv);
    const float* M = out.m;
    const float* I = out.inv;
    out.wpos.resize(nverts);
    out.wnrm.resize(nverts);
    par_for(nverts, [&](size_t v0, size_t v1) {
    for (size_t v = v0; v < v1; ++v) {
        const char* mv = mvert + 20 * (size_t)v;     // MVert: co f32[3] @0, no i16[3] @12
        float co[3]; int16_t no[3];
        std::memcpy(co, mv, 12);
        std::memcpy(no, mv + 12, 6);
        float x = co[0], y = co[1], z = co[2];
        // Transform::ApplyToPoint (src/Transform.cpp:3-10)
        out.wpos[v] = {M[0] * x + M[1] * y + M[2] * z + M[3],
                       M[4] * x + M[5] * y + M[6] * z + M[7],
                       M[8] * x + M[9] * y + M[10] * z + M[11]};
        // normal_short_to_float (src/Triangle.cpp:9-14) then ApplyToNormal with the
        // inverse transpose (src/Transform.cpp:21-30) and normalize
        float nx = no[0] * (1.0f / 32767.0f), ny = no[1] * (1.0f / 32767.0f), nz = no[2] * (1.0f / 32767.0f);
        V3 n = {I[0] * nx + I[4] * ny + I[8] * nz,
                I[1] * nx + I[5] * ny + I[9] * nz,
                I[2] * nx + I[6] * ny + I[10] * nz};
        out.wnrm[v] = normalize(n);
    }
    });
    out.tri.resize(3 * (size_t)ntris);
    out.mat.resize(ntris);
    std::atomic<bool> bad_index{false};
    par_for(ntris, [&](size_t t0, size_t t1) {
        for (size_t t = t0; t < t1; ++t) {
            const char* mp = mpoly + 12 * t;    // MPoly: loopstart i32 @0, mat_nr i16 @8
            int32_t ls; int16_t mat_nr;
            std::memcpy(&ls, mp, 4);
            std::memcpy(&mat_nr, mp + 8, 2);
            for (int k = 0; k < 3; ++k) {
                uint32_t vi;
                std::memcpy(&vi, mloop + 8 * ((size_t)ls + k), 4);   // MLoop: v u32 @0
                if (vi >= nverts) { bad_index = true; vi = 0; }
                out.tri[3 * t + k] = vi;
            }
            out.mat[t] = (uint32_t)material_indices[mat_nr];
        }
    });
    if (bad_index) { err = "loop vertex index out of range"; return RC_E_INVALID; }
    return RC_OK;
}

void build_mesh_bvh(HostMesh& mesh) {
    std::vector<Prim> prims(mesh.num_tris);
    for (uint32_t t = 0; t < mesh.num_tris; ++t) {
        const V3& a = mesh.wpos[mesh.tri[3 * t]];
        const V3& b = mesh.wpos[mesh.tri[3 * t + 1]];
        const V3& c = mesh.wpos[mesh.tri[3 * t + 2]];
        // Triangle::bounding_box (src/Triangle.cpp:90-106)
        Prim& p = prims[t];
        p.index = t;
        p.box.mn = {fmin_ref(fmin_ref(a.x, b.x), c.x), fmin_ref(fmin_ref(a.y, b.y), c.y), fmin_ref(fmin_ref(a.z, b.z), c.z)};
        p.box.mx = {fmax_ref(fmax_ref(a.x, b.x), c.x), fmax_ref(fmax_ref(a.y, b.y), c.y), fmax_ref(fmax_ref(a.z, b.z), c.z)};
        p.center = mul(add(p.box.mn, p.box.mx), 1 / 2.0f);
        p.cost = 0;
    }
    build_flat(prims, false, mesh.bvh.nodes, mesh.bvh.index, mesh.bvh.bounds);
    mesh.bvh.cost = cost_of_traversing(mesh.bvh, 0);
}

float cost_of_traversing(const MeshBvh& bvh, int node) {
    const BvhNode& n = bvh.nodes[node];
    if (n.w0 & 0x80000000u) return (float)(n.w0 & 0x7fffffffu);
    float a = surface_area(n.box);
    float la = surface_area(bvh.nodes[n.w0].box);
    float ra = surface_area(bvh.nodes[n.w1].box);
    return 0.16874 + (cost_of_traversing(bvh, n.w0) * la + cost_of_traversing(bvh, n.w1) * ra) / a;
}

void build_world_bvh(HostScene& scene) {
    std::vector<Prim> prims(scene.meshes.size());
    for (size_t i = 0; i < scene.meshes.size(); ++i) {
        Prim& p = prims[i];
        p.index = (uint32_t)i;
        p.box = scene.meshes[i].bvh.bounds;
        p.center = mul(add(p.box.mn, p.box.mx), 1 / 2.0f);
        p.cost = (int)scene.meshes[i].bvh.cost;
    }
    build_flat(prims, true, scene.world.nodes, scene.world.index, scene.bounds);
    // SceneRadius (src/main.cpp:166)
    V3 c = mul(add(scene.bounds.mn, scene.bounds.mx), 0.5f);
    V3 d = sub(scene.bounds.mn, c);
    scene.scene_radius = std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
}

int convert_lights(HostScene& scene, std::string& err) {
    scene.lights.clear();
    for (unsigned i = 0; i < scene.num_lights; ++i) {
        const rc_python_light& pl = scene.py_lights[i];
        DevLight L{};
        L.power = pl.power;
        V3 color = {pl.color[0], pl.color[1], pl.color[2]};
        if (pl.type == 'P') {
            // Point_Light::sample_light is a stub in the reference (src/Lights.h:78-81);
            // here it emits isotropically from the position.
            L.type = LIGHT_POINT;
            V3 c = mul(color, pl.power);
            L.cr = c.x; L.cg = c.y; L.cb = c.z;
            L.pos[0] = pl.position.x; L.pos[1] = pl.position.y; L.pos[2] = pl.position.z;
        } else if (pl.type == 'S') {
            // Sun_Light constructor (src/Lights.cpp:58-119)
            L.type = LIGHT_SUN;
            V3 c = mul(color, pl.power);
            L.cr = c.x; L.cg = c.y; L.cb = c.z;
            V3 r = {pl.rotation.x, pl.rotation.y, pl.rotation.z};
            M3 mat = rotation_matrix(r);
            // rotate_vec_rad(normal, 0, r): (v - p) * m + p, kept literally for the
            // sign of zero components
            V3 normal = add(vmul(sub(V3{0, 0, -1}, V3{0, 0, 0}), mat), V3{0, 0, 0});
            M3 inv = mat;
            inv.i = {mat.i.x, mat.j.x, mat.k.x};
            inv.j = {mat.i.y, mat.j.y, mat.k.y};
            inv.k = {mat.i.z, mat.j.z, mat.k.z};
            Box bb = scene.bounds;
            V3 diag = sub(bb.mx, bb.mn);
            float dl = std::sqrt(diag.x * diag.x + diag.y * diag.y + diag.z * diag.z);
            V3 neg = {-normal.x, -normal.y, -normal.z};
            V3 position = add(mul(neg, dl), mul(add(bb.mx, bb.mn), 0.5f));
            auto project = [&](V3 p) {
                V3 t = sub(p, position);
                float nl2 = normal.x * normal.x + normal.y * normal.y + normal.z * normal.z;
                return add(sub(t, mul(normal, dot(t, normal) / nl2)), position);
            };
            V3 pts[8] = {bb.mn, {bb.mx.x, bb.mn.y, bb.mn.z}, {bb.mn.x, bb.mx.y, bb.mn.z}, {bb.mx.x, bb.mx.y, bb.mn.z},
                         {bb.mn.x, bb.mn.y, bb.mx.z}, {bb.mx.x, bb.mn.y, bb.mx.z}, {bb.mn.x, bb.mx.y, bb.mx.z}, bb.mx};
            V3 mx = {-INFINITY, -INFINITY, 0.0f}, mn = {INFINITY, INFINITY, 0.0f};
            for (int k = 0; k < 8; ++k) {
                V3 q = vmul(sub(project(pts[k]), position), inv);
                if (q.x > mx.x) mx.x = q.x;
                if (q.y > mx.y) mx.y = q.y;
                if (q.x < mn.x) mn.x = q.x;
                if (q.y < mn.y) mn.y = q.y;
            }
            V3 br_local = {mx.x, mn.y, 0.0f}, tl_local = {mn.x, mx.y, 0.0f};
            V3 bl = add(vmul(mn, mat), position);
            V3 br = add(vmul(br_local, mat), position);
            V3 tl = add(vmul(tl_local, mat), position);
            V3 hz = sub(br, bl), vt = sub(tl, bl);
            L.bl[0] = bl.x; L.bl[1] = bl.y; L.bl[2] = bl.z;
            L.hz[0] = hz.x; L.hz[1] = hz.y; L.hz[2] = hz.z;
            L.vt[0] = vt.x; L.vt[1] = vt.y; L.vt[2] = vt.z;
            L.fz[0] = normal.x; L.fz[1] = normal.y; L.fz[2] = normal.z;
        } else {
            // Area_Light constructor (src/Lights.cpp:18-36); rotation in degrees
            L.type = LIGHT_AREA;
            V3 c = mul(color, pl.power);
            L.cr = c.x; L.cg = c.y; L.cb = c.z;
            float w = pl.width, h = pl.height;
            V3 pos = {pl.position.x, pl.position.y, pl.position.z};
            V3 bl = sub(pos, V3{w / 2.f, h / 2.f, 0.f});
            V3 hz = {w, 0.0f, 0.0f}, vt = {0.0f, h, 0.0f};
            V3 normal = {0, 0, -1};
            V3 tl = add(bl, vt), br = add(bl, hz);
            const float PI = 3.14159265359f;
            V3 rr = {pl.rotation.x * PI / 180.f, pl.rotation.y * PI / 180.f, pl.rotation.z * PI / 180.f};
            M3 rm = rotation_matrix(rr);
            bl = add(vmul(sub(bl, pos), rm), pos);
            tl = add(vmul(sub(tl, pos), rm), pos);
            br = add(vmul(sub(br, pos), rm), pos);
            normal = add(vmul(sub(normal, V3{0, 0, 0}), rm), V3{0, 0, 0});
            hz = sub(br, bl);
            vt = sub(tl, bl);
            L.bl[0] = bl.x; L.bl[1] = bl.y; L.bl[2] = bl.z;
            L.hz[0] = hz.x; L.hz[1] = hz.y; L.hz[2] = hz.z;
            L.vt[0] = vt.x; L.vt[1] = vt.y; L.vt[2] = vt.z;
            frame_from_z(normal, L.fx, L.fy, L.fz);
        }
        scene.lights.push_back(L);
    }
    if (scene.lights.empty()) { err = "scene has no lights"; return RC_E_INVALID; }
    // Lights_list::update_pdf_distribution (src/Light_list.cpp:32-45)
    size_t n = scene.lights.size();
    scene.light_cdf.assign(n + 1, 0.0f);
    for (size_t i = 1; i < n + 1; ++i) scene.light_cdf[i] = scene.light_cdf[i - 1] + scene.lights[i - 1].power;
    scene.light_integral = scene.light_cdf[n];
    if (!(scene.light_integral > 0.0f)) { err = "total light power is not positive"; return RC_E_INVALID; }
    for (size_t i = 1; i < n + 1; ++i) scene.light_cdf[i] /= scene.light_integral;
    return RC_OK;
}

void convert_materials(HostScene& scene) {
    scene.materials.clear();
    for (const rc_python_material& pm : scene.py_materials) {
        DevMaterial m{};
        float cr = pm.color[0], cg = pm.color[1], cb = pm.color[2];
        if (pm.type == 'P') {
            // Plastic_Material (src/materials.h:59-90): roughness r*r, specular s*0.08
            float rough = pm.roughness * pm.roughness;
            m.s = pm.specular * 0.08f;
            m.r = cr; m.g = cg; m.b = cb;
            if (rough < 0.01f) m.kind = BSDF_K_PLASTIC_SMOOTH;
            else { m.kind = BSDF_K_PLASTIC_GGX; m.a2 = rough * rough; }
        } else if (pm.type == 'G') {
            // Glass_Material -> Fresnel_Specular (src/materials.h:93-115); roughness ignored
            m.kind = BSDF_K_FRESNEL_SPECULAR;
            m.r = cr; m.g = cg; m.b = cb;
            m.ior = pm.ior;
        } else if (pm.type == 'M') {
            // Metal_Material (src/materials.h:117-146)
            m.r = cr; m.g = cg; m.b = cb;
            if (pm.roughness < 0.01f) m.kind = BSDF_K_SPECULAR_REFLECTION;
            else { m.kind = BSDF_K_GGX_REFLECTION; m.a2 = pm.roughness * pm.roughness; }
        } else if (pm.type == 'R') {
            // rough GGX dielectric (additive type): alpha = roughness; `specular` > 0 is
            // the per-channel IOR dispersion (R: ior - d, G: ior, B: ior + d)
            m.r = cr; m.g = cg; m.b = cb;
            m.ior = pm.ior;
            m.disp = pm.specular > 0.0f ? pm.specular : 0.0f;
            if (pm.roughness < 0.01f) m.kind = BSDF_K_FRESNEL_SPECULAR;
            else { m.kind = BSDF_K_GGX_DIELECTRIC; m.a2 = pm.roughness * pm.roughness; }
        } else {
            // default: Plastic_Material(vec3(1,1,1), 1, 0.0) (src/Scene.cpp:66)
            m.kind = BSDF_K_PLASTIC_GGX;
            m.r = 1.0f; m.g = 1.0f; m.b = 1.0f;
            m.a2 = 1.0f;
            m.s = 0.0f;
        }
        m.cont = std::max(0.05f, std::max(std::max(m.r, m.g), m.b));
        scene.materials.push_back(m);
    }
}

}  // namespace rc
