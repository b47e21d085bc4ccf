// CPU ORACLE - test infrastructure only.
//
// A restatement of RealCausticsEngine's vertex-merging path, used only by tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker; the
// product (librealcaustics.so) never links or calls it.  Each function cites the
// reference file:line (paths within "Real Caustics/src") it follows.
//
// Pinning: tests compare this restatement against the reference itself, compiled
// from its own sources by oracle/build_ref.sh (closest hits, BVH layout, KD radius
// sets, BSDF and light samples, a full reference-mode render), and against golden
// fixtures generated from it (tests/golden, tests/golden/make_golden.py) where the
// reference cannot be built (the GPU host).
//
// Two render modes:
//   reference mode - float, the reference's global xorshift stream and its hybrid
//                    Metropolis light sampler (src/Vertex_Merging.cpp:196-379)
//                    consumed in the same order, so it reproduces the reference's
//                    own image;
//   plain mode     - float or double, independent uniform light paths with the
//                    counter-based Philox primary samples the GPU kernels use (same
//                    sample layout), the estimator the GPU's plain vertex merging
//                    computes; in double it is the FP64 image oracle.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <random>
#include <string>
#include <thread>
#include <vector>
#include <cstdio>
#include <cstdlib>

namespace orc {

const float INF = std::numeric_limits<float>::infinity();
const float PIf = 3.14159265359f;
const float PI2f = 6.28318530718f;
const float INV_PIf = 0.31830988618f;
const float PI_OVER_2f = 1.57079632679f;
const float PI_OVER_4f = 0.78539816339f;
const float INV_Ef = 0.36787944117f;

// ---------------------------------------------------------------- vectors
template <class R> struct V3 {
    R x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(R a) : x(a), y(a), z(a) {}
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator*=(const V3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    V3& operator*=(R t) { x *= t; y *= t; z *= t; return *this; }
    V3& operator/=(R t) { x /= t; y /= t; z /= t; return *this; }
    V3 operator-() const { return V3(-x, -y, -z); }
    R length_squared() const { return x * x + y * y + z * z; }
    R length() const { return std::sqrt(length_squared()); }
    R Max() const { return std::max(std::max(x, y), z); }
};
template <class R> V3<R> operator+(const V3<R>& u, const V3<R>& v) { return V3<R>(u.x + v.x, u.y + v.y, u.z + v.z); }
template <class R> V3<R> operator-(const V3<R>& u, const V3<R>& v) { return V3<R>(u.x - v.x, u.y - v.y, u.z - v.z); }
template <class R> V3<R> operator*(const V3<R>& u, const V3<R>& v) { return V3<R>(u.x * v.x, u.y * v.y, u.z * v.z); }
template <class R> V3<R> operator*(const V3<R>& u, R t) { return V3<R>(u.x * t, u.y * t, u.z * t); }
template <class R> V3<R> operator*(R t, const V3<R>& u) { return u * t; }
template <class R> V3<R> operator/(const V3<R>& u, R t) { return (1 / t) * u; }   // src/vec3.h:154
template <class R> R dot(const V3<R>& u, const V3<R>& v) { return u.x * v.x + u.y * v.y + u.z * v.z; }
template <class R> R abs_dot(const V3<R>& u, const V3<R>& v) { return std::abs(u.x * v.x + u.y * v.y + u.z * v.z); }
template <class R> V3<R> cross(const V3<R>& u, const V3<R>& v) {
    return V3<R>(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
template <class R> V3<R> normalize(const V3<R>& u) { return u / u.length(); }
template <class R> V3<R> reflect(const V3<R>& v, const V3<R>& n) { return v - 2 * dot(v, n) * n; }
template <class R> bool refract(const V3<R>& wi, const V3<R>& n, R eta, V3<R>& wo) {   // src/vec3.h:185-200
    R ci = dot(n, wi);
    R s2i = std::max(R(0), R(1) - ci * ci);
    R s2t = eta * eta * s2i;
    if (s2t >= R(1)) return false;
    R ct = std::sqrt(R(1) - s2t);
    wo = eta * -wi + (eta * ci - ct) * n;
    return true;
}
template <class R, class S> V3<R> cvt(const V3<S>& v) { return V3<R>((R)v.x, (R)v.y, (R)v.z); }

template <class R> struct Frame {   // src/Frame.h
    V3<R> mX, mY, mZ;
    void set_from_z(const V3<R>& z) {
        mZ = z;
        V3<R> tx = (std::abs(z.x) > R(0.99f)) ? V3<R>(0, 1, 0) : V3<R>(1, 0, 0);
        mY = normalize(cross(z, tx));
        mX = cross(mY, z);
    }
    V3<R> to_world(const V3<R>& a) const { return mX * a.x + mY * a.y + mZ * a.z; }
    V3<R> to_local(const V3<R>& a) const { return V3<R>(dot(a, mX), dot(a, mY), dot(a, mZ)); }
};

// ---------------------------------------------------------------- scene
struct Box {
    V3<float> mn{INF, INF, INF}, mx{-INF, -INF, -INF};
};
Box unite(const Box& a, const Box& b) {
    Box r;
    r.mn = V3<float>(std::min(a.mn.x, b.mn.x), std::min(a.mn.y, b.mn.y), std::min(a.mn.z, b.mn.z));
    r.mx = V3<float>(std::max(a.mx.x, b.mx.x), std::max(a.mx.y, b.mx.y), std::max(a.mx.z, b.mx.z));
    return r;
}
Box unite(const Box& a, const V3<float>& p) {
    Box r;
    r.mn = V3<float>(std::min(a.mn.x, p.x), std::min(a.mn.y, p.y), std::min(a.mn.z, p.z));
    r.mx = V3<float>(std::max(a.mx.x, p.x), std::max(a.mx.y, p.y), std::max(a.mx.z, p.z));
    return r;
}
float area(const Box& b) { V3<float> d = b.mx - b.mn; return 2 * (d.x * d.y + d.x * d.z + d.y * d.z); }
int extent_axis(const Box& b) {
    V3<float> d = b.mx - b.mn;
    if (d.x > d.y && d.x > d.z) return 0;
    return d.y > d.z ? 1 : 2;
}
float offset(const Box& b, const V3<float>& p, int dim) {
    V3<float> o = p - b.mn;
    float v[3] = {o.x / (b.mx.x - b.mn.x), o.y / (b.mx.y - b.mn.y), o.z / (b.mx.z - b.mn.z)};
    return v[dim];
}

struct Node { Box box; uint32_t w0, w1; };
struct Bvh { std::vector<Node> nodes; std::vector<int> index; float cost = 0; Box bounds; };

struct Mesh {
    std::vector<V3<float>> wp; std::vector<V3<float>> wn;   // float world space (reference)
    std::vector<V3<double>> wpd; std::vector<V3<double>> wnd;
    std::vector<uint32_t> tri; std::vector<uint32_t> mat;
    float M[16], I[16];
    Bvh bvh;
    std::vector<Box> dbox;   // per node: boxes refitted from double vertices (rounded outward)
};

struct Light {
    int type;   // 0 area, 1 sun, 2 point
    float power;
    V3<float> color, bl, hz, vt, normal, pos;
    Frame<float> frame;
};

struct Material { char type; float ior, roughness, specular; V3<float> color; };

struct Scene {
    int samples = 1;
    float base_radius = 0, alpha = 0;
    std::vector<Mesh> meshes;
    int W = 0, H = 0;
    V3<float> cam_o, cam_bl, cam_h, cam_v;
    std::vector<unsigned char> py_lights;   // copied at init (the reference borrows them)
    unsigned num_lights = 0;
    std::vector<Material> mats;
    Bvh world;
    std::vector<Box> wdbox;   // world boxes refitted from the double mesh boxes
    Box bounds;
    float scene_radius = 0;
    std::vector<Light> lights;
    std::vector<float> cdf;
    float integral = 0;
    bool prepared = false;
};

std::unique_ptr<Scene> g;

// ---------------------------------------------------------------- BVH (src/BVH/BVH_mesh.cpp, BVH_world.cpp)
struct Prim { uint32_t index; Box box; V3<float> center; int cost; };
struct TNode { Box box; bool leaf = false; int l = -1, r = -1; std::vector<uint32_t> items; };

int recurse(std::vector<Prim>& p, int start, int end, bool world, std::vector<TNode>& pool) {
    Box bbox;
    for (int i = start; i < end; ++i) bbox = unite(bbox, p[i].box);
    int n = end - start;
    int me = (int)pool.size();
    pool.emplace_back();
    pool[me].box = bbox;
    auto leaf = [&]() { pool[me].leaf = true; for (int i = start; i < end; ++i) pool[me].items.push_back(p[i].index); return me; };
    if (n == 1) return leaf();
    Box cb;
    for (int i = start; i < end; ++i) cb = unite(cb, p[i].center);
    int dim = extent_axis(cb);
    int mid = (start + end) / 2;
    if (cb.mx[dim] == cb.mn[dim]) return leaf();
    if (n == 2) {
        if (!(p[start].center[dim] < p[end - 1].center[dim])) std::swap(p[start], p[end - 1]);
    } else {
        const int nB = 12;
        int count[nB] = {0}; Box bb[nB]; float trav[nB] = {0};
        for (int i = start; i < end; ++i) {
            int b = nB * offset(cb, p[i].center, dim);
            if (b == nB) b = nB - 1;
            count[b]++; bb[b] = unite(bb[b], p[i].box);
            if (world) trav[b] += p[i].cost;
        }
        float cost[nB - 1];
        for (int i = 0; i < nB - 1; ++i) {
            Box b0, b1; int c0 = 0, c1 = 0; int t0 = 0, t1 = 0;
            for (int j = 0; j <= i; ++j) { b0 = unite(b0, bb[j]); c0 += count[j]; t0 += trav[j]; }
            for (int j = i + 1; j < nB; ++j) { b1 = unite(b1, bb[j]); c1 += count[j]; t1 += trav[j]; }
            if (world) cost[i] = 0.16874 + (area(b0) * t0 + area(b1) * t1) / area(bbox);
            else cost[i] = 0.16874 + (c0 * area(b0) + c1 * area(b1)) / area(bbox);
        }
        float minCost = cost[0]; float minB = 0; float leaf_cost = 0;
        for (int i = 0; i < nB - 1; ++i) {
            if (world) leaf_cost += trav[i];
            if (cost[i] < minCost) { minCost = cost[i]; minB = i; }
        }
        if (!world) leaf_cost = n;
        if (minCost < leaf_cost) {
            Prim* m = std::partition(&p[start], &p[end - 1] + 1, [=](const Prim& q) {
                int b = nB * offset(cb, q.center, dim);
                if (b == nB) b = nB - 1;
                return b <= minB;
            });
            mid = (int)(m - &p[0]);
        } else {
            return leaf();
        }
    }
    int l = recurse(p, start, mid, world, pool);
    int r = recurse(p, mid, end, world, pool);
    pool[me].l = l; pool[me].r = r;
    return me;
}

void populate(const std::vector<TNode>& pool, int t, unsigned& ib, unsigned& it, Bvh& out) {
    const TNode& n = pool[t];
    unsigned cur = ib;
    out.nodes[cur].box = n.box;
    if (!n.leaf) {
        int l = ++ib; populate(pool, n.l, ib, it, out);
        int r = ++ib; populate(pool, n.r, ib, it, out);
        out.nodes[cur].w0 = l; out.nodes[cur].w1 = r;
    } else {
        out.nodes[cur].w0 = 0x80000000u | (unsigned)n.items.size();
        out.nodes[cur].w1 = it;
        for (uint32_t x : n.items) out.index[++it] = (int)x;
    }
}

void build(std::vector<Prim>& prims, bool world, Bvh& out) {
    std::vector<TNode> pool;
    int root = recurse(prims, 0, (int)prims.size(), world, pool);
    out.bounds = pool[root].box;
    size_t items = 0;
    for (auto& t : pool) items += t.items.size();
    out.nodes.assign(pool.size(), Node{});
    out.index.assign(items + 1, 0);
    unsigned ib = 0, it = 0;
    populate(pool, root, ib, it, out);
}

float traversal_cost(const Bvh& b, int i) {   // src/BVH/BVH_mesh.cpp:286-305
    const Node& n = b.nodes[i];
    if (n.w0 & 0x80000000u) return (float)(n.w0 & 0x7fffffffu);
    return 0.16874 + (traversal_cost(b, n.w0) * area(b.nodes[n.w0].box) + traversal_cost(b, n.w1) * area(b.nodes[n.w1].box)) / area(n.box);
}

// double-precision boxes for the FP64 render: exact double triangle bounds rounded
// outward to float, merged up the tree
Box refit(Mesh& m, int i) {
    const Node& n = m.bvh.nodes[i];
    Box b;
    if (n.w0 & 0x80000000u) {
        unsigned cnt = n.w0 & 0x7fffffffu;
        for (unsigned k = 0; k < cnt; ++k) {
            uint32_t t = (uint32_t)m.bvh.index[n.w1 + 1 + k];
            for (int c = 0; c < 3; ++c) {
                const V3<double>& v = m.wpd[m.tri[3 * t + c]];
                auto lo1 = [](double x) { return (float)(x - std::abs(x) * 1e-6 - 1e-30); };
                auto hi1 = [](double x) { return (float)(x + std::abs(x) * 1e-6 + 1e-30); };
                V3<float> lo(lo1(v.x), lo1(v.y), lo1(v.z));
                V3<float> hi(hi1(v.x), hi1(v.y), hi1(v.z));
                b = unite(unite(b, lo), hi);
            }
        }
    } else {
        b = unite(refit(m, n.w0), refit(m, n.w1));
    }
    m.dbox[i] = b;
    return b;
}

Box refit_world(Scene& s, int i) {
    const Node& n = s.world.nodes[i];
    Box b;
    if (n.w0 & 0x80000000u) {
        for (unsigned k = 0; k < (n.w0 & 0x7fffffffu); ++k) b = unite(b, s.meshes[s.world.index[n.w1 + 1 + k]].dbox[0]);
    } else {
        b = unite(refit_world(s, n.w0), refit_world(s, n.w1));
    }
    s.wdbox[i] = b;
    return b;
}

// ---------------------------------------------------------------- traversal (src/Scene.cpp:154-189 etc.)
template <class R> struct Hit { R t = (R)INF, u = 0, v = 0; int mesh = -1; int tri = -1; };

template <class R> bool box_hit(const Box& b, const V3<R>& o, const V3<R>& d, R tmin, R tmax) {   // src/aabb.cpp:6-41
    for (int a = 0; a < 3; ++a) {
        R invD = 1 / d[a];
        R t0 = ((R)b.mn[a] - o[a]) * invD;
        R t1 = ((R)b.mx[a] - o[a]) * invD;
        if (invD < 0) std::swap(t0, t1);
        tmin = t0 > tmin ? t0 : tmin;
        tmax = t1 < tmax ? t1 : tmax;
        if (tmax < tmin) return false;
    }
    return true;
}

template <class R> const V3<R>& wpos(const Mesh& m, uint32_t v);
template <> const V3<float>& wpos<float>(const Mesh& m, uint32_t v) { return m.wp[v]; }
template <> const V3<double>& wpos<double>(const Mesh& m, uint32_t v) { return m.wpd[v]; }
template <class R> const V3<R>& wnrm(const Mesh& m, uint32_t v);
template <> const V3<float>& wnrm<float>(const Mesh& m, uint32_t v) { return m.wn[v]; }
template <> const V3<double>& wnrm<double>(const Mesh& m, uint32_t v) { return m.wnd[v]; }

template <class R> bool tri_hit(const Mesh& m, uint32_t t, const V3<R>& o, const V3<R>& d, R tmin, R tmax, R& tt, R& uu, R& vv) {
    // src/Triangle.cpp:20-66
    const V3<R>& v0 = wpos<R>(m, m.tri[3 * t]);
    const V3<R>& v1 = wpos<R>(m, m.tri[3 * t + 1]);
    const V3<R>& v2 = wpos<R>(m, m.tri[3 * t + 2]);
    V3<R> e1 = v1 - v0, e2 = v2 - v0;
    V3<R> pvec = cross(d, e2);
    R det = dot(e1, pvec);
    if (std::abs(det) < R(0.0000001f)) return false;
    R inv = R(1.0f) / det;
    V3<R> tvec = o - v0;
    R u = dot(tvec, pvec) * inv;
    if (u < R(0) || u > R(1)) return false;
    V3<R> q = cross(tvec, e1);
    R v = dot(d, q) * inv;
    if (v < R(0) || u + v > R(1)) return false;
    R t_ = dot(e2, q) * inv;
    if (t_ > tmin && t_ < tmax) { tt = t_; uu = u; vv = v; return true; }
    return false;
}

template <class R> const Box& node_box(const Mesh& m, int i) {
    return std::is_same<R, double>::value ? m.dbox[i] : m.bvh.nodes[i].box;
}

template <class R> bool mesh_hit(const Mesh& m, int mi, const V3<R>& o, const V3<R>& d, R tmin, Hit<R>& rec) {
    int stack[64]; int sp = 0; stack[sp++] = 0;
    bool hit = false;
    while (sp) {
        int id = stack[--sp];
        const Node& n = m.bvh.nodes[id];
        if (!box_hit<R>(node_box<R>(m, id), o, d, tmin, rec.t)) continue;
        if (n.w0 & 0x80000000u) {
            unsigned cnt = n.w0 & 0x7fffffffu;
            for (unsigned k = 0; k < cnt; ++k) {
                uint32_t t = (uint32_t)m.bvh.index[n.w1 + 1 + k];
                R tt, uu, vv;
                if (tri_hit<R>(m, t, o, d, tmin, rec.t, tt, uu, vv)) {
                    rec.t = tt; rec.u = uu; rec.v = vv; rec.mesh = mi; rec.tri = (int)t; hit = true;
                }
            }
        } else {
            stack[sp++] = n.w1;
            stack[sp++] = n.w0;
        }
    }
    return hit;
}

template <class R> bool scene_hit(const Scene& s, const V3<R>& o, const V3<R>& d, R tmin, Hit<R>& out) {
    int stack[64]; int sp = 0; stack[sp++] = 0;
    bool hit = false;
    out = Hit<R>();
    while (sp) {
        int id = stack[--sp];
        const Node& n = s.world.nodes[id];
        const Box& b = std::is_same<R, double>::value ? s.wdbox[id] : n.box;
        if (!box_hit<R>(b, o, d, tmin, out.t)) continue;
        if (n.w0 & 0x80000000u) {
            Hit<R> leaf;   // fresh Isect per world leaf (src/BVH/BVH_world.cpp:269)
            bool any = false;
            for (unsigned k = 0; k < (n.w0 & 0x7fffffffu); ++k) {
                int mi = s.world.index[n.w1 + 1 + k];
                if (mesh_hit<R>(s.meshes[mi], mi, o, d, tmin, leaf)) any = true;
            }
            if (any) { out = leaf; hit = true; }
        } else {
            stack[sp++] = n.w1;
            stack[sp++] = n.w0;
        }
    }
    return hit;
}

template <class R> struct Isect {
    V3<R> ng, ns, pos, dir; R t, u, v; bool front; int mat, tri, mesh;
};

template <class R> void fill(const Scene& s, const Hit<R>& h, const V3<R>& o, const V3<R>& d, Isect<R>& is) {
    const Mesh& m = s.meshes[h.mesh];
    uint32_t a = m.tri[3 * h.tri], b = m.tri[3 * h.tri + 1], c = m.tri[3 * h.tri + 2];
    V3<R> e1 = wpos<R>(m, b) - wpos<R>(m, a), e2 = wpos<R>(m, c) - wpos<R>(m, a);
    is.t = h.t; is.u = h.u; is.v = h.v;
    is.ng = normalize(cross(e1, e2));
    is.ns = wnrm<R>(m, a) * (1 - h.u - h.v) + wnrm<R>(m, b) * h.u + wnrm<R>(m, c) * h.v;
    is.front = dot(is.ns, d) < 0;
    is.pos = o + d * h.t;
    is.dir = d;
    is.mat = (int)m.mat[h.tri];
    is.tri = h.tri;
    is.mesh = h.mesh;
}

// ---------------------------------------------------------------- sampling (src/Sampling.h, src/BXDF.*)
template <class R> V3<R> cos_hemisphere(R e0, R e1) {
    R ox = R(2.0f) * e0 - R(1.0f), oy = R(2.0f) * e1 - R(1.0f);
    R dx = 0, dy = 0;
    if (!(ox == 0 && oy == 0)) {
        R theta, r;
        if (std::abs(ox) > std::abs(oy)) { r = ox; theta = R(PI_OVER_4f) * (oy / ox); }
        else { r = oy; theta = R(PI_OVER_2f) - R(PI_OVER_4f) * (ox / oy); }
        dx = r * std::cos(theta); dy = r * std::sin(theta);
    }
    R z = std::sqrt(std::max(R(0), R(1) - dx * dx - dy * dy));
    return V3<R>(dx, dy, z);
}

template <class R> R fresnel_eta(R c, R eta) {   // src/BXDF.h:461-478
    R g = eta * eta - R(1) + c * c;
    if (g > R(0)) {
        g = std::sqrt(g);
        R A = (g - c) / (g + c);
        R B = (c * (g + c) - R(1)) / (c * (g - c) + R(1));
        return R(0.5f) * A * A * (R(1) + B * B);
    }
    return 1;
}
template <class R> R fresnel_refl(R c, R refl) {   // src/BXDF.h:480-498
    if (refl >= R(1)) return 1;
    R n = (R(1) + std::sqrt(refl)) / (R(1) - std::sqrt(refl));
    R g = n * n - 1 + c * c;
    if (g > R(0)) {
        g = std::sqrt(g);
        R A = (g - c) / (g + c);
        R B = (c * (g + c) - R(1)) / (c * (g - c) + R(1));
        return R(0.5f) * A * A * (R(1) + B * B);
    }
    return 1;
}
template <class R> R D(R nh, R a2) { R den = nh * nh * (a2 - R(1)) + R(1); return a2 / (R(PIf) * den * den); }
template <class R> R G2(R nw, R nl, R a2) {
    R A = nw * std::sqrt(a2 + (R(1) - a2) * nl * nl);
    R B = nl * std::sqrt(a2 + (R(1) - a2) * nw * nw);
    return R(2) * nl * nw / (A + B);
}
// theta from acos(sqrt(..)), then convert_from_spherical_coordinates
// (src/BXDF.cpp:311-314, src/BXDF.h:501-505).  Its unqualified sin/cos are the C
// library's double functions: sin_theta is rounded to float, and the products
// sin_theta * cos(phi) are formed in double and rounded when the vec3 is built.
template <class R> V3<R> ggx_half(R e1, R e2, R a2) {
    R theta = std::acos(std::sqrt((R(1) - e1) / (e1 * (a2 - R(1)) + R(1))));
    R phi = e2 * R(PI2f);
    R st = (R)::sin((double)theta);
    return V3<R>((R)((double)st * ::cos((double)phi)), (R)((double)st * ::sin((double)phi)), (R)::cos((double)theta));
}

enum { EV_R = 1, EV_T = 2, EV_D = 4, EV_G = 8, EV_S = 16 };
enum Kind { K_SPEC_REFL, K_FRESNEL_SPEC, K_GGX_REFL, K_PLASTIC, K_PLASTIC_SMOOTH, K_GGX_DIEL };

template <class R> struct Bsdf {
    Kind kind; V3<R> Rc; R ior = 0, a2 = 0, s = 0, contp = 0; bool radiance;
    Frame<R> fr; V3<R> wo;
    void init(const Material& m, const V3<R>& ns, const V3<R>& dir, bool rad, float ior_shift = 0.0f) {   // src/materials.h:59-146
        radiance = rad;
        Rc = cvt<R>(m.color);
        if (m.type == 'P') {
            float rough = m.roughness * m.roughness;
            s = (R)(m.specular * 0.08f);
            if (rough < 0.01f) kind = K_PLASTIC_SMOOTH;
            else { kind = K_PLASTIC; a2 = (R)(rough * rough); }
        } else if (m.type == 'G') {
            kind = K_FRESNEL_SPEC; ior = (R)m.ior;
        } else if (m.type == 'M') {
            if (m.roughness < 0.01f) kind = K_SPEC_REFL;
            else { kind = K_GGX_REFL; a2 = (R)(m.roughness * m.roughness); }
        } else if (m.type == 'R') {
            ior = (R)(m.ior + ior_shift);
            if (m.roughness < 0.01f) kind = K_FRESNEL_SPEC;
            else { kind = K_GGX_DIEL; a2 = (R)(m.roughness * m.roughness); }
        } else {
            kind = K_PLASTIC; Rc = V3<R>(1); a2 = 1; s = 0;
        }
        contp = std::max(R(0.05f), std::max(std::max(Rc.x, Rc.y), Rc.z));
        fr.set_from_z(ns);
        wo = fr.to_local(-dir);
    }
    bool valid() const { return !(std::abs(wo.z) < R(1e-6f)); }
    bool delta() const { return kind == K_SPEC_REFL || kind == K_FRESNEL_SPEC; }
    R side(const V3<R>& wi, const V3<R>& ng) const { return dot(wi, ng) * dot(fr.to_world(wo), ng); }

    struct S { V3<R> f, wi; R fwd = 0, rev = 0, cos_out = 0, cont = 0; int ev = 0; };
    S sample(R u0, R u1, R u2, const V3<R>& ng) const {
        S o;
        switch (kind) {
        case K_SPEC_REFL: {
            o.ev = EV_R | EV_G | EV_S;
            V3<R> wl(-wo.x, -wo.y, wo.z);
            o.cos_out = std::abs(wl.z);
            if (o.cos_out < R(1e-6f)) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0) return o;
            o.fwd = o.rev = 1; o.cont = contp; o.f = Rc;
            return o;
        }
        case K_FRESNEL_SPEC: {   // src/BXDF.cpp:136-205
            R eta = ior;
            if (wo.z > 0) eta = R(1.0f) / ior;
            R f = fresnel_eta<R>(std::abs(wo.z), 1 / eta);
            if (u0 < f) {
                o.ev = EV_G | EV_S | EV_R;
                V3<R> wl(-wo.x, -wo.y, wo.z);
                o.cos_out = std::abs(wl.z);
                if (o.cos_out < R(1e-6f)) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0) return o;
                o.fwd = o.rev = f; o.cont = contp; o.f = Rc;
                return o;
            }
            o.ev = EV_T | EV_G | EV_S;
            V3<R> wl;
            if (!refract<R>(wo, wo.z > 0 ? V3<R>(0, 0, 1) : V3<R>(0, 0, -1), eta, wl)) return o;
            o.cos_out = std::abs(wl.z);
            if (o.cos_out < R(1e-6f)) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) >= 0) return o;
            o.fwd = o.rev = R(1.0f) - f; o.cont = contp;
            o.f = radiance ? Rc * eta * eta : Rc;
            return o;
        }
        case K_GGX_REFL: {   // src/BXDF.cpp:302-337
            o.ev = EV_G | EV_R;
            V3<R> h = ggx_half<R>(u1, u2, a2);
            if (wo.z < 0) h.z = -h.z;
            V3<R> wl = reflect(-wo, h);
            o.cos_out = std::abs(wl.z);
            if (o.cos_out < R(1e-6f)) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0 || wl.z * wo.z <= 0) return o;
            R chn = std::abs(h.z), d = D<R>(chn, a2);
            o.fwd = o.rev = d * chn * R(0.25f) / abs_dot(h, wo);
            o.cont = contp;
            R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
            o.f = Rc * g2 * abs_dot(wo, h) / (std::abs(wo.z) * chn);
            return o;
        }
        case K_PLASTIC: {   // src/BXDF.cpp:384-489
            R f = fresnel_refl<R>(std::abs(wo.z), s);
            if (u0 < f) {
                o.ev = EV_G | EV_R;
                V3<R> h = ggx_half<R>(u1, u2, a2);
                if (wo.z < 0) h.z = -h.z;
                V3<R> wl = reflect(-wo, h);
                o.cos_out = std::abs(wl.z);
                if (o.cos_out < R(1e-6f)) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0 || wl.z * wo.z <= 0) return o;
                R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
                o.cont = std::max(R(0.05f), f);
                R fdp = std::abs(wl.z) * R(INV_PIf), rdp = std::abs(wo.z) * R(INV_PIf);
                R chn = std::abs(h.z), d = D<R>(chn, a2);
                R sp = d * chn * R(0.25f) / abs_dot(wo, h);
                if (f > 1) { o.fwd = o.rev = sp; }
                else { o.fwd = fdp * (R(1) - f) + sp * f; o.rev = rdp * (R(1) - f) + sp * f; }
                // fabs() here is the C library's double fabs: the denominator is an
                // exact double product and the quotient rounds once (src/BXDF.cpp:438)
                o.f = V3<R>((R)((double)(g2 * abs_dot(wo, h)) / ((double)std::abs(wo.z) * (double)chn)));
                return o;
            }
            o.ev = EV_D;
            V3<R> wl = cos_hemisphere<R>(u1, u2);
            o.cos_out = wl.z;
            if (o.cos_out < R(1e-6f)) return o;
            if (wo.z < 0) wl.z = -wl.z;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0 || wl.z * wo.z <= 0) return o;
            o.cont = std::max(R(0.05f), (Rc * (R)(1.0 - f)).Max());
            R fdp = std::abs(wl.z) * R(INV_PIf), rdp = std::abs(wo.z) * R(INV_PIf);
            V3<R> h = normalize(wo + wl);
            R chn = std::abs(h.z), d = D<R>(chn, a2);
            R sp = d * chn * R(0.25f) / abs_dot(wo, h);
            if (f > 1) { o.fwd = o.rev = sp; }
            else { o.fwd = fdp * (R(1) - f) + sp * f; o.rev = rdp * (R(1) - f) + sp * f; }
            o.f = Rc;
            return o;
        }
        case K_PLASTIC_SMOOTH: {   // src/BXDF.cpp:568-632
            R f = fresnel_refl<R>(std::abs(wo.z), s);
            if (u0 < f) {
                o.ev = EV_S | EV_R | EV_G;
                V3<R> wl(-wo.x, -wo.y, wo.z);
                o.cos_out = std::abs(wl.z);
                if (o.cos_out < R(1e-6f)) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0 || wl.z * wo.z <= 0) return o;
                o.fwd = o.rev = f; o.cont = std::max(R(0.05f), f); o.f = V3<R>(1);
                return o;
            }
            o.ev = EV_D;
            V3<R> wl = cos_hemisphere<R>(u1, u2);
            o.cos_out = wl.z;
            if (o.cos_out < R(1e-6f)) return o;
            if (wo.z < 0) wl.z = -wl.z;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) <= 0 || wl.z * wo.z <= 0) return o;
            o.fwd = std::abs(wl.z) * R(INV_PIf);
            o.rev = std::abs(wo.z) * R(INV_PIf);
            o.cont = std::max(R(0.05f), (Rc * (R)(1.0 - f)).Max());
            o.f = Rc;
            return o;
        }
        case K_GGX_DIEL: {   // rough dielectric (Walter et al. 2007); no reference counterpart
            R eta = (wo.z > 0) ? R(1.0f) / ior : ior;
            V3<R> m = ggx_half<R>(u1, u2, a2);
            if (wo.z < 0) m.z = -m.z;
            R c = dot(wo, m);
            if (c <= 0) return o;
            R F = fresnel_eta<R>(c, 1 / eta);
            R chn = std::abs(m.z), Dm = D<R>(chn, a2);
            V3<R> wl;
            if (u0 < F) {
                o.ev = EV_G | EV_R;
                wl = reflect(-wo, m);
                o.cos_out = std::abs(wl.z);
                if (o.cos_out < R(1e-6f)) return o;
                o.wi = fr.to_world(wl);
                if (side(o.wi, ng) <= 0 || wl.z * wo.z <= 0) return o;
                o.fwd = o.rev = F * Dm * chn * R(0.25f) / c;
                R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
                o.cont = contp;
                o.f = Rc * (g2 * c / (std::abs(wo.z) * chn));
                return o;
            }
            o.ev = EV_G | EV_T;
            if (!refract<R>(wo, m, eta, wl)) return o;
            o.cos_out = std::abs(wl.z);
            if (o.cos_out < R(1e-6f)) return o;
            o.wi = fr.to_world(wl);
            if (side(o.wi, ng) >= 0 || wl.z * wo.z >= 0) return o;
            R ci = dot(wl, m), den = eta * c + ci;
            o.fwd = (R(1) - F) * Dm * chn * std::abs(ci) / (den * den);
            R denr = ci / eta + c;
            o.rev = (R(1) - F) * Dm * chn * c / (denr * denr * eta * eta);
            R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
            o.cont = contp;
            V3<R> base = Rc * (g2 * c / (std::abs(wo.z) * chn));
            o.f = radiance ? base * eta * eta : base;
            return o;
        }
        }
        return o;
    }
    V3<R> evaluate(const V3<R>& wi, const V3<R>& ng) const {
        switch (kind) {
        case K_GGX_REFL: {
            if (side(wi, ng) <= 0) return V3<R>(0);
            V3<R> wl = fr.to_local(wi);
            if (wl.z * wo.z <= 0) return V3<R>(0);
            R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
            V3<R> h = normalize(wo + wl);
            R chn = std::abs(h.z), d = D<R>(chn, a2);
            return Rc * d * g2 * R(0.25f) / std::abs(wo.z);
        }
        case K_PLASTIC: {
            if (side(wi, ng) <= 0) return V3<R>(0);
            R f = fresnel_refl<R>(std::abs(wo.z), s);
            V3<R> wl = fr.to_local(wi);
            if (wl.z * wo.z <= 0) return V3<R>(0);
            V3<R> h = normalize(wl + wo);
            V3<R> diffuse = Rc * R(INV_PIf);
            R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
            R chn = std::abs(h.z), d = D<R>(chn, a2);
            R spec = f * d * g2 * R(0.25f) / std::abs(wo.z);
            return V3<R>(diffuse.x + spec, diffuse.y + spec, diffuse.z + spec);
        }
        case K_PLASTIC_SMOOTH:
            if (side(wi, ng) <= 0) return V3<R>(0);
            if (fr.to_local(wi).z * wo.z <= 0) return V3<R>(0);
            return Rc * R(INV_PIf);
        case K_GGX_DIEL: {
            V3<R> wl = fr.to_local(wi);
            R eta = (wo.z > 0) ? R(1.0f) / ior : ior;
            if (wl.z * wo.z > 0) {
                if (side(wi, ng) <= 0) return V3<R>(0);
                V3<R> m = normalize(wo + wl);
                R c = std::abs(dot(wo, m));
                R F = fresnel_eta<R>(c, 1 / eta);
                R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
                R d = D<R>(std::abs(m.z), a2);
                return Rc * (F * d * g2 * R(0.25f) / std::abs(wo.z));
            }
            if (side(wi, ng) >= 0) return V3<R>(0);
            V3<R> m = normalize(wo * eta + wl);
            if (dot(m, wo) < 0) m = -m;
            R c = dot(wo, m), ci = dot(wl, m);
            if (c <= 0 || ci >= 0) return V3<R>(0);
            R F = fresnel_eta<R>(c, 1 / eta);
            R g2 = G2<R>(std::abs(wo.z), std::abs(wl.z), a2);
            R d = D<R>(std::abs(m.z), a2);
            R den = eta * c + ci;
            R v = (R(1) - F) * d * g2 * c * std::abs(ci) / (std::abs(wo.z) * den * den);
            V3<R> base = Rc * v;
            return radiance ? base * eta * eta : base;
        }
        default:
            return V3<R>(0);
        }
    }
    void pdf(const V3<R>& wi, R& fwd, R& rev) const {
        switch (kind) {
        case K_GGX_REFL: {
            V3<R> wl = fr.to_local(wi);
            V3<R> h = normalize(wo + wl);
            R chn = std::abs(h.z), d = D<R>(chn, a2);
            fwd = rev = d * chn * R(0.25f) / abs_dot(h, wo);
            return;
        }
        case K_PLASTIC: {
            V3<R> wl = fr.to_local(wi);
            R fdp = std::abs(wl.z) * R(INV_PIf), rdp = std::abs(wo.z) * R(INV_PIf);
            V3<R> h = normalize(wo + wl);
            R chn = std::abs(h.z), d = D<R>(chn, a2);
            R sp = d * chn * R(0.25f) / abs_dot(h, wo);
            R f = fresnel_refl<R>(std::abs(wo.z), s);
            if (f > 1) { fwd = rev = sp; }
            else { fwd = fdp * (R(1) - f) + sp * f; rev = rdp * (R(1) - f) + sp * f; }
            return;
        }
        case K_PLASTIC_SMOOTH: {
            R f = fresnel_refl<R>(std::abs(wo.z), s);
            if (f > 1) { fwd = rev = 0; return; }
            V3<R> wl = fr.to_local(wi);
            fwd = std::abs(wl.z) * R(INV_PIf) * (R(1) - f);
            rev = std::abs(wo.z) * R(INV_PIf) * (R(1) - f);
            return;
        }
        case K_GGX_DIEL: {
            V3<R> wl = fr.to_local(wi);
            R eta = (wo.z > 0) ? R(1.0f) / ior : ior;
            fwd = rev = 0;
            if (wl.z * wo.z > 0) {
                V3<R> m = normalize(wo + wl);
                R c = std::abs(dot(wo, m));
                if (c <= 0) return;
                R F = fresnel_eta<R>(c, 1 / eta);
                R chn = std::abs(m.z);
                fwd = rev = F * D<R>(chn, a2) * chn * R(0.25f) / c;
                return;
            }
            V3<R> m = normalize(wo * eta + wl);
            if (dot(m, wo) < 0) m = -m;
            R c = dot(wo, m), ci = dot(wl, m);
            if (c <= 0 || ci >= 0) return;
            R F = fresnel_eta<R>(c, 1 / eta);
            R chn = std::abs(m.z), Dm = D<R>(chn, a2);
            R den = eta * c + ci;
            fwd = (R(1) - F) * Dm * chn * std::abs(ci) / (den * den);
            R denr = ci / eta + c;
            rev = (R(1) - F) * Dm * chn * c / (denr * denr * eta * eta);
            return;
        }
        default:
            fwd = rev = 0;
        }
    }
};

// ---------------------------------------------------------------- lights (src/Lights.cpp, src/Light_list.cpp)
struct M3 { V3<float> i, j, k; };
M3 rot(V3<float> r) {   // src/matrix.cpp:70-80 (C library double cos/sin)
    M3 m;
    m.i = V3<float>(::cos(r.z) * ::cos(r.y), ::sin(r.z) * ::cos(r.y), -::sin(r.y));
    m.j = V3<float>(::cos(r.z) * ::sin(r.y) * ::sin(r.x) - ::sin(r.z) * ::cos(r.x),
                    ::sin(r.z) * ::sin(r.y) * ::sin(r.x) + ::cos(r.z) * ::cos(r.x), ::cos(r.y) * ::sin(r.x));
    m.k = V3<float>(::cos(r.z) * ::sin(r.y) * ::cos(r.x) + ::sin(r.z) * ::sin(r.x),
                    ::sin(r.z) * ::sin(r.y) * ::cos(r.x) - ::cos(r.z) * ::sin(r.x), ::cos(r.y) * ::cos(r.x));
    return m;
}
V3<float> vm(const V3<float>& v, const M3& m) { return v.x * m.i + v.y * m.j + v.z * m.k; }

int find_interval(const std::vector<float>& cdf, float u) {   // src/utils.h:142-157
    int first = 0, len = (int)cdf.size();
    while (len > 0) {
        int half = len >> 1, middle = first + half;
        if (cdf[middle] < u) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    int v = first - 1, hi = (int)cdf.size() - 2;
    return v < 0 ? 0 : (v > hi ? hi : v);
}

template <class R> void sample_light(const Scene& s, const R* u, V3<R>& o, V3<R>& d, V3<R>& tp) {
    int idx = find_interval(s.cdf, (float)u[0]);
    const Light& L = s.lights[idx];
    R pick = (R)L.power / (R)((int)s.lights.size() * s.integral);
    if (L.type == 0) {
        o = cvt<R>(L.bl) + cvt<R>(L.hz) * u[1] + cvt<R>(L.vt) * u[2];
        V3<R> loc = cos_hemisphere<R>(u[3], u[4]);
        d = cvt<R>(L.frame.mX) * loc.x + cvt<R>(L.frame.mY) * loc.y + cvt<R>(L.frame.mZ) * loc.z;
        tp = cvt<R>(L.color) * R(PIf);
    } else if (L.type == 1) {
        o = cvt<R>(L.bl) + cvt<R>(L.hz) * u[1] + cvt<R>(L.vt) * u[2];
        d = cvt<R>(L.normal);
        tp = cvt<R>(L.color);
    } else {   // point light: isotropic (the reference's point light is a stub)
        o = cvt<R>(L.pos);
        R z = R(1.0f) - R(2.0f) * u[3];
        R r = std::sqrt(std::max(R(0), R(1) - z * z));
        R ph = R(PI2f) * u[4];
        d = V3<R>(r * std::cos(ph), r * std::sin(ph), z);
        tp = cvt<R>(L.color) * (R(4.0f) * R(PIf));
    }
    tp /= pick;
}

// ---------------------------------------------------------------- Philox (the GPU's counter RNG)
struct U4 { uint32_t a, b, c, d; };
U4 philox(U4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c.a, p1 = (uint64_t)0xCD9E8D57u * c.c;
        c = U4{(uint32_t)(p1 >> 32) ^ c.b ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.d ^ k1, (uint32_t)p0};
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return c;
}
float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }
struct PRng {
    uint32_t k0, k1, lo, hi, it;
    PRng(uint64_t seed, uint64_t path, uint32_t iter, uint32_t stream)
        : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), lo((uint32_t)path),
          hi(((uint32_t)(path >> 32) & 0xffffffu) | (stream << 24)), it(iter) {}
    U4 block(uint32_t b) const { return philox(U4{lo, hi, it, b}, k0, k1); }
};

// ---------------------------------------------------------------- KD tree (src/KD_Tree.cpp)
struct KNode { uint32_t index; float split; };
template <class R> struct Photon { V3<R> pos, dir, tp; R dVM; uint32_t path; };

// random_int11's generator is a function-local static in the reference
// (src/random_generators.h:12-17): one stream for the whole process, first used by
// the first KD build with a node of at least 500 photons.
std::mt19937 g_kd_mt{0};

struct KdRef {
    std::vector<KNode> nodes;
    std::mt19937& mt = g_kd_mt;
    struct T { const V3<float>* p; unsigned idx; };
    int axis(std::vector<T>& v, int st, int cnt) {   // src/KD_Tree.cpp:24-95, incl. the y/z typo
        V3<float> bot(INF, INF, INF), top(-INF, -INF, -INF);
        if (cnt < 500) {
            for (int i = st; i < st + cnt; ++i) {
                const V3<float>& p = *v[i].p;
                if (p.x < bot.x) bot.x = p.x;
                if (p.y < bot.y) bot.y = p.y;
                if (p.z < bot.z) bot.z = p.z;
                if (p.x > top.x) top.x = p.x;
                if (p.y > top.y) top.y = p.y;
                if (p.z > top.z) top.z = p.z;
            }
        } else {
            for (int i = 0; i < 400; ++i) {
                std::uniform_int_distribution<int> dist(st, st + cnt - 1);
                const V3<float>& p = *v[dist(mt)].p;
                if (p.x < bot.x) bot.x = p.x;
                if (p.y < bot.y) bot.y = p.y;
                if (p.z < bot.z) bot.z = p.z;
                if (p.x > top.x) top.x = p.x;
                if (p.y > top.y) top.y = p.y;
                if (p.y > top.z) top.z = p.z;
            }
        }
        float x = top.x - bot.x, y = top.y - bot.y, z = top.z - bot.z;
        float b = std::fmax(std::fmax(x, y), z);
        return b == x ? 0 : (b == y ? 1 : 2);
    }
    void rec(std::vector<T>& v, int st, int cnt, int e) {
        if (cnt < 2) { nodes[e].index = v[st].idx; return; }
        int a = axis(v, st, cnt);
        auto cmp = [a](const T& p, const T& q) { return (*p.p)[a] < (*q.p)[a]; };
        std::nth_element(v.begin() + st, v.begin() + st + cnt / 2, v.begin() + st + cnt, cmp);
        const T& m = v[st + cnt / 2];
        if (cnt & 1) {
            unsigned mask = a == 0 ? 0x90000000u : (a == 1 ? 0xb0000000u : 0xf0000000u);
            nodes[e].index = m.idx | mask;
            nodes[e].split = (*m.p)[a];
            rec(v, st, cnt / 2, 2 * e);
            rec(v, st + cnt / 2 + 1, cnt / 2, 2 * e + 1);
        } else {
            unsigned mask = a == 0 ? 0x80000000u : (a == 1 ? 0xa0000000u : 0xe0000000u);
            nodes[e].index = mask;
            nodes[e].split = (*m.p)[a] + 1.175494e-38f;
            rec(v, st, cnt / 2, 2 * e);
            rec(v, st + cnt / 2, cnt / 2, 2 * e + 1);
        }
    }
    void build(const std::vector<V3<float>>& pos) {
        nodes.clear();
        if (pos.empty()) return;
        std::vector<T> v(pos.size());
        for (size_t i = 0; i < pos.size(); ++i) v[i] = T{&pos[i], (unsigned)i};
        nodes.assign((size_t)std::pow(2, (int)(std::log2f((float)pos.size()) + 1)), KNode{0, 0.0f});
        rec(v, 0, (int)pos.size(), 1);
    }
    // find_closest_in_radius (src/KD_Tree.cpp:217-280); fn(index) in the reference's order
    template <class Fn> void find(const std::vector<V3<float>>& pos, const V3<float>& p, float r2, int e, Fn&& fn) const {
        const KNode& n = nodes[e];
        if (n.index & 0x80000000u) {
            float d;
            unsigned ax = n.index & 0x60000000u;
            if (ax == 0) d = p.x - n.split;
            else if (ax == 0x20000000u) d = p.y - n.split;
            else d = p.z - n.split;
            int nearc = d < 0 ? 2 * e : 2 * e + 1, farc = d < 0 ? 2 * e + 1 : 2 * e;
            find(pos, p, r2, nearc, fn);
            if (d * d < r2) {
                if (n.index & 0x10000000u) {
                    int i = (int)(n.index & 0xfffffffu);
                    if ((p - pos[i]).length_squared() < r2) fn(i);
                }
                find(pos, p, r2, farc, fn);
            }
        } else {
            if ((p - pos[n.index]).length_squared() < r2) fn((int)n.index);
        }
    }
};

// ---------------------------------------------------------------- the reference's global RNG (src/random_generators.h:18-50)
struct XorShift {
    uint32_t a = 132141;
    uint32_t next() { uint32_t x = a; x ^= x << 13; x ^= x >> 17; x ^= x << 5; return a = x; }
    unsigned random_int(uint32_t range) {
        uint32_t x, r;
        do { x = next(); r = x % range; } while (x - r > (~range + 1));
        return r;
    }
    float f01() { return random_int(10000000) / 9999999.f; }
};

// ---------------------------------------------------------------- prepare (src/main.cpp:150-168)
int prepare(Scene& s, std::string& err) {
    if (s.prepared) return 0;
    for (Mesh& m : s.meshes) {
        std::vector<Prim> prims(m.tri.size() / 3);
        for (size_t t = 0; t < prims.size(); ++t) {
            const V3<float>& a = m.wp[m.tri[3 * t]]; const V3<float>& b = m.wp[m.tri[3 * t + 1]]; const V3<float>& c = m.wp[m.tri[3 * t + 2]];
            Prim& p = prims[t];
            p.index = (uint32_t)t;
            p.box.mn = V3<float>(std::min(std::min(a.x, b.x), c.x), std::min(std::min(a.y, b.y), c.y), std::min(std::min(a.z, b.z), c.z));
            p.box.mx = V3<float>(std::max(std::max(a.x, b.x), c.x), std::max(std::max(a.y, b.y), c.y), std::max(std::max(a.z, b.z), c.z));
            p.center = (p.box.mn + p.box.mx) / 2.0f;
            p.cost = 0;
        }
        build(prims, false, m.bvh);
        m.bvh.cost = traversal_cost(m.bvh, 0);
        m.dbox.assign(m.bvh.nodes.size(), Box{});
        refit(m, 0);
    }
    std::vector<Prim> prims(s.meshes.size());
    for (size_t i = 0; i < s.meshes.size(); ++i) {
        prims[i].index = (uint32_t)i;
        prims[i].box = s.meshes[i].bvh.bounds;
        prims[i].center = (prims[i].box.mn + prims[i].box.mx) / 2.0f;
        prims[i].cost = (int)s.meshes[i].bvh.cost;
    }
    build(prims, true, s.world);
    s.wdbox.assign(s.world.nodes.size(), Box{});
    refit_world(s, 0);
    s.bounds = s.world.bounds;
    s.scene_radius = (s.bounds.mn - (s.bounds.mn + s.bounds.mx) * 0.5f).length();
    // lights (src/Scene.cpp:70-108, src/Lights.cpp:18-119)
    const unsigned char* pl = s.py_lights.data();
    s.lights.clear();
    for (unsigned i = 0; i < s.num_lights; ++i) {
        const unsigned char* r = pl + 64 * (size_t)i;
        char type = (char)r[0];
        float color[3], pos[3], w, h, rotv[3], power;
        std::memcpy(color, r + 4, 12); std::memcpy(pos, r + 16, 12); std::memcpy(&w, r + 28, 4);
        std::memcpy(&h, r + 32, 4); std::memcpy(rotv, r + 40, 12); std::memcpy(&power, r + 52, 4);
        Light L;
        L.power = power;
        V3<float> c(color[0], color[1], color[2]);
        L.color = c * power;
        V3<float> P(pos[0], pos[1], pos[2]);
        V3<float> rr(rotv[0], rotv[1], rotv[2]);
        if (type == 'P') {
            L.type = 2; L.pos = P;
        } else if (type == 'S') {
            L.type = 1;
            M3 m = rot(rr);
            V3<float> normal = vm(V3<float>(0, 0, -1) - V3<float>(0, 0, 0), m) + V3<float>(0, 0, 0);
            M3 inv{V3<float>(m.i.x, m.j.x, m.k.x), V3<float>(m.i.y, m.j.y, m.k.y), V3<float>(m.i.z, m.j.z, m.k.z)};
            Box bb = s.bounds;
            V3<float> position = (bb.mx - bb.mn).length() * (-normal) + ((bb.mx + bb.mn) * 0.5f);
            auto proj = [&](V3<float> p) { V3<float> t = p - position; return (t - dot(t, normal) / normal.length_squared() * normal) + position; };
            V3<float> pts[8] = {bb.mn, V3<float>(bb.mx.x, bb.mn.y, bb.mn.z), V3<float>(bb.mn.x, bb.mx.y, bb.mn.z),
                                V3<float>(bb.mx.x, bb.mx.y, bb.mn.z), V3<float>(bb.mn.x, bb.mn.y, bb.mx.z),
                                V3<float>(bb.mx.x, bb.mn.y, bb.mx.z), V3<float>(bb.mn.x, bb.mx.y, bb.mx.z), bb.mx};
            V3<float> mx(-INF, -INF, 0.0f), mn(INF, INF, 0.0f);
            for (int k = 0; k < 8; ++k) {
                V3<float> q = vm(proj(pts[k]) - position, inv);
                if (q.x > mx.x) mx.x = q.x;
                if (q.y > mx.y) mx.y = q.y;
                if (q.x < mn.x) mn.x = q.x;
                if (q.y < mn.y) mn.y = q.y;
            }
            L.bl = vm(mn, m) + position;
            V3<float> br = vm(V3<float>(mx.x, mn.y, 0.0f), m) + position;
            V3<float> tl = vm(V3<float>(mn.x, mx.y, 0.0f), m) + position;
            L.hz = br - L.bl; L.vt = tl - L.bl; L.normal = normal;
        } else {
            L.type = 0;
            V3<float> bl = P - V3<float>(w / 2.f, h / 2.f, 0.f);
            V3<float> hz(w, 0.0f, 0.0f), vt(0.0f, h, 0.0f), normal(0, 0, -1);
            V3<float> tl = bl + vt, br = bl + hz;
            M3 m = rot(V3<float>(rr.x * PIf / 180.f, rr.y * PIf / 180.f, rr.z * PIf / 180.f));
            bl = vm(bl - P, m) + P; tl = vm(tl - P, m) + P; br = vm(br - P, m) + P;
            normal = vm(normal - V3<float>(0, 0, 0), m) + V3<float>(0, 0, 0);
            L.bl = bl; L.hz = br - bl; L.vt = tl - bl; L.normal = normal;
            L.frame.set_from_z(normal);
        }
        s.lights.push_back(L);
    }
    if (s.lights.empty()) { err = "no lights"; return -2; }
    s.cdf.assign(s.lights.size() + 1, 0.0f);
    for (size_t i = 1; i <= s.lights.size(); ++i) s.cdf[i] = s.cdf[i - 1] + s.lights[i - 1].power;
    s.integral = s.cdf.back();
    for (size_t i = 1; i <= s.lights.size(); ++i) s.cdf[i] /= s.integral;
    s.base_radius *= s.scene_radius;
    s.prepared = true;
    return 0;
}

// ---------------------------------------------------------------- plain-mode iteration (uniform light paths, Philox)
template <class R> struct PlainCfg { uint64_t seed; long long paths; int maxlen; };

// Dispersion (additive, no counterpart in the reference): material 'R' with specular > 0
// has IOR ior - d, ior, ior + d for R, G, B.  A path keeps one channel c from its first
// dispersive vertex on (uniform, from Philox block 48 + bounce), throughput 3 x channel c.
inline float disp_of(const Material& m) { return (m.type == 'R' && m.specular > 0.0f) ? m.specular : 0.0f; }
template <class R> float dispersion_shift(const Material& m, int& channel, V3<R>& tp, float u) {
    const float dsp = disp_of(m);
    if (!(dsp > 0.0f)) return 0.0f;
    if (channel < 0) {
        int c = (int)(u * 3.0f);
        channel = c > 2 ? 2 : c;
        tp = V3<R>(channel == 0 ? R(3.0f) * tp.x : R(0), channel == 1 ? R(3.0f) * tp.y : R(0),
                   channel == 2 ? R(3.0f) * tp.z : R(0));
    }
    return (float)(channel - 1) * dsp;
}

template <class R> void trace_light(const Scene& s, const PlainCfg<R>& c, long long pidx, uint32_t it,
                                    std::vector<Photon<R>>& out) {
    PRng rng(c.seed, (uint64_t)pidx, it, 0u);
    U4 b0 = rng.block(0), b1 = rng.block(1);
    R u[5] = {(R)u01(b0.a), (R)u01(b0.b), (R)u01(b0.c), (R)u01(b0.d), (R)u01(b1.a)};
    V3<R> o, d, tp;
    sample_light<R>(s, u, o, d, tp);
    int diffuse = 0, last = EV_D, channel = -1;
    R dVM = 0;
    for (int len = 0;; ++len) {
        V3<R> ro = o + d * R(0.001f);
        Hit<R> h;
        if (!scene_hit<R>(s, ro, d, R(0.001f), h)) break;
        Isect<R> is; fill<R>(s, h, ro, d, is);
        const Material& mt = s.mats[is.mat];
        const float shift = disp_of(mt) > 0.0f
            ? dispersion_shift<R>(mt, channel, tp, u01(rng.block(48 + len).a)) : 0.0f;
        Bsdf<R> b; b.init(mt, is.ns, is.dir, false, shift);
        if (!b.valid()) break;
        dVM /= std::abs(std::abs(b.wo.z));
        bool stored = false;
        if (!b.delta() && (last & EV_G)) {
            out.push_back(Photon<R>{is.pos, -is.dir, tp, dVM, (uint32_t)pidx});
            stored = true;
        }
        if (len > c.maxlen || diffuse > 2) break;
        U4 bb = rng.block(2 + len);
        auto sm = b.sample((R)u01(bb.a), (R)u01(bb.b), (R)u01(bb.c), is.ng);
        if (sm.f.x == 0 && sm.f.y == 0 && sm.f.z == 0) break;
        V3<R> f = sm.f;
        if (len > 2) { if ((R)u01(bb.d) > sm.cont) break; f /= sm.cont; }
        o = is.pos; d = sm.wi;
        if (sm.ev & EV_D) diffuse++;
        tp *= f; last = sm.ev;
        if (!stored) dVM *= (sm.cos_out / sm.fwd) * sm.rev;
        else dVM = (sm.cos_out / sm.fwd) * (R(1) + sm.rev * dVM);
    }
}

template <class R> struct PhotonMap {
    std::vector<Photon<R>> ph;
    std::vector<V3<float>> posf;
    KdRef kd;
    void build() {
        posf.resize(ph.size());
        for (size_t i = 0; i < ph.size(); ++i) posf[i] = cvt<float>(ph[i].pos);
        kd.build(posf);
    }
};

// radius query in precision R: the float tree culls (|q - p| >= |q[axis] - split| holds
// for the float positions), the acceptance test runs in R on the R positions
template <class R> V3<R> contrib(const PhotonMap<R>& pm, const Isect<R>& is, const Bsdf<R>& b, R r2, R cam_dVM) {
    V3<R> color(0);
    if (pm.ph.empty()) return color;
    V3<float> qf = cvt<float>(is.pos);
    float r2f = std::is_same<R, float>::value ? (float)r2 : (float)(r2 * 1.002);
    pm.kd.find(pm.posf, qf, r2f, 1, [&](int i) {
        const Photon<R>& p = pm.ph[i];
        if (!std::is_same<R, float>::value && !((is.pos - p.pos).length_squared() < r2)) return;
        R fwd, rev;
        b.pdf(p.dir, fwd, rev);
        R w = R(1.0f) / (R(1.0f) + cam_dVM * rev + p.dVM * fwd);
        V3<R> ev = b.evaluate(p.dir, is.ng);
        color += ev * p.tp * w;
    });
    return color;
}

template <class R> V3<R> camera_path(const Scene& s, const PhotonMap<R>& pm, const PlainCfg<R>& c, long long pix,
                                     uint32_t it, R r2, R vm_norm, long long& target) {
    const int W = s.W, H = s.H;
    PRng rng(c.seed, (uint64_t)pix, it, 1u);
    U4 b1 = rng.block(1);
    const float x = (float)(int)(pix % W), y = (float)(int)(pix / W);
    const float sx = x + u01(b1.b), sy = y + u01(b1.c);
    target = -1;
    if (sx < 0 || sx >= (float)W || sy < 0 || sy >= (float)H) return V3<R>(0);
    int X = (int)sx, Y = H - (int)sy;
    if ((long long)X + (long long)Y * W > (long long)W * H - 1) return V3<R>(0);
    target = (long long)X + (long long)Y * W;
    V3<R> dir = cvt<R>(s.cam_bl) + (R)(sx / (float)W) * cvt<R>(s.cam_h) + (R)(sy / (float)H) * cvt<R>(s.cam_v);
    dir = dir - cvt<R>(s.cam_o);
    V3<R> o = cvt<R>(s.cam_o), d = normalize(dir), tp(1);
    R dVM = 0;
    V3<R> color(0);
    int channel = -1;
    for (int len = 0;; ++len) {
        V3<R> ro = o + d * R(0.001f);
        Hit<R> h;
        if (!scene_hit<R>(s, ro, d, R(0.001f), h)) break;
        Isect<R> is; fill<R>(s, h, ro, d, is);
        const Material& mt = s.mats[is.mat];
        const float shift = disp_of(mt) > 0.0f
            ? dispersion_shift<R>(mt, channel, tp, u01(rng.block(48 + len).a)) : 0.0f;
        Bsdf<R> b; b.init(mt, is.ns, is.dir, true, shift);
        if (!b.valid()) break;
        dVM /= std::abs(b.wo.z);
        if (!b.delta()) color += tp * vm_norm * contrib<R>(pm, is, b, r2, dVM);
        if (len > c.maxlen) break;
        U4 bb = rng.block(2 + len);
        auto sm = b.sample((R)u01(bb.a), (R)u01(bb.b), (R)u01(bb.c), is.ng);
        if (sm.f.x == 0 && sm.f.y == 0 && sm.f.z == 0) break;
        V3<R> f = sm.f;
        if (len > 2) { if ((R)u01(bb.d) > sm.cont) break; f /= sm.cont; }
        o = is.pos; d = sm.wi; tp *= f;
        if (sm.ev & EV_S) dVM *= (sm.cos_out / sm.fwd) * sm.rev;
        else dVM = (sm.cos_out / sm.fwd) * (R(1) + sm.rev * dVM);
    }
    return color;
}

template <class F> void parallel_for(long long n, int threads, F&& f) {
    if (threads <= 1 || n < 1024) { for (long long i = 0; i < n; ++i) f(i, 0); return; }
    std::atomic<long long> next{0};
    std::vector<std::thread> ts;
    for (int t = 0; t < threads; ++t)
        ts.emplace_back([&, t]() {
            for (;;) {
                long long b = next.fetch_add(4096);
                if (b >= n) break;
                long long e = std::min(n, b + 4096);
                for (long long i = b; i < e; ++i) f(i, t);
            }
        });
    for (auto& t : ts) t.join();
}

template <class R> void light_pass(const Scene& s, const PlainCfg<R>& c, uint32_t it, int threads, PhotonMap<R>& pm) {
    // per-thread photon lists, then concatenated in path order (deterministic)
    long long n = c.paths;
    const long long blk = 4096;
    long long nblk = (n + blk - 1) / blk;
    std::vector<std::vector<Photon<R>>> parts(nblk);
    parallel_for(nblk, threads, [&](long long b, int) {
        for (long long p = b * blk; p < std::min(n, (b + 1) * blk); ++p) trace_light<R>(s, c, p, it, parts[b]);
    });
    pm.ph.clear();
    for (auto& v : parts) pm.ph.insert(pm.ph.end(), v.begin(), v.end());
    pm.build();
}

template <class R> void plain_iteration(const Scene& s, const PlainCfg<R>& c, uint32_t it, int threads,
                                        std::vector<double>& acc, long long* stats) {
    float radius = s.base_radius;
    radius /= std::pow(float(it + 1), 0.5f * (1.0f - s.alpha));
    radius = std::max(radius, 1e-7f);
    float r2f = radius * radius;
    float vmf = 1.0f / (PIf * r2f * (float)c.paths);
    PhotonMap<R> pm;
    light_pass<R>(s, c, it, threads, pm);
    long long npix = (long long)s.W * s.H;
    std::vector<V3<R>> col(npix);
    std::vector<long long> tgt(npix);
    parallel_for(npix, threads, [&](long long p, int) {
        col[p] = camera_path<R>(s, pm, c, p, it, (R)r2f, (R)vmf, tgt[p]);
    });
    for (long long p = 0; p < npix; ++p) {
        if (tgt[p] < 0) continue;
        acc[3 * tgt[p]] += (double)col[p].x;
        acc[3 * tgt[p] + 1] += (double)col[p].y;
        acc[3 * tgt[p] + 2] += (double)col[p].z;
    }
    if (stats) { stats[0] += c.paths; stats[1] += (long long)pm.ph.size(); }
}

// ---------------------------------------------------------------- reference-mode render (src/Vertex_Merging.cpp:18-379)
struct MltSampler {   // src/MLT_Sampler.*
    struct PS { float value, back_up; };
    std::vector<PS> s; int index = 0; float mutation_size;
    MltSampler(int maxlen, float m, XorShift& rng) : mutation_size(m) {
        s.resize((maxlen + 2) * 3 + 2);
        for (auto& x : s) { float e = rng.f01(); x.value = e; x.back_up = e; }
    }
    float get() { return s[index++].value; }
    void init_uniform(XorShift& rng) { for (auto& x : s) { x.back_up = x.value; x.value = rng.f01(); } }
    void mutate(XorShift& rng) {
        for (auto& x : s) {
            x.back_up = x.value;
            float du, e = rng.f01();
            if (rng.f01() < 0.5f) du = e * powf(INV_Ef, 1.0f / mutation_size);
            else du = -e * powf(INV_Ef, 1.0f / mutation_size);
            x.value += du;
            x.value -= std::floor(x.value);
        }
    }
    void reject() { for (auto& x : s) x.value = x.back_up; }
};

void ref_trace_light(const Scene& s, MltSampler& S, XorShift& rng, int maxlen, std::vector<Photon<float>>& out, bool& visible) {
    float u[5];
    u[0] = S.get();
    int idx = find_interval(s.cdf, u[0]);
    // sample_light: Get2D (position) then Get2D or skip(2) (direction).  Get2D builds
    // vec2(Get1D(), Get1D()) and g++ evaluates those arguments right to left.
    u[2] = S.get(); u[1] = S.get(); u[4] = S.get(); u[3] = S.get();
    (void)idx;
    V3<float> o, d, tp;
    sample_light<float>(s, u, o, d, tp);
    if (s.lights[idx].type == 2) { visible = false; return; }
    int diffuse = 0, last = EV_D;
    float dVM = 0;
    for (int len = 0;; ++len) {
        V3<float> ro = o + d * 0.001f;
        Hit<float> h;
        if (!scene_hit<float>(s, ro, d, 0.001f, h)) break;
        Isect<float> is; fill<float>(s, h, ro, d, is);
        Bsdf<float> b; b.init(s.mats[is.mat], is.ns, is.dir, false);
        if (!b.valid()) break;
        dVM /= std::fabs(std::abs(b.wo.z));
        bool stored = false;
        if (!b.delta() && (last & EV_G)) {
            out.push_back(Photon<float>{is.pos, -is.dir, tp, dVM, 0});
            visible = true; stored = true;
        }
        if (len > maxlen || diffuse > 2) break;
        float u2 = S.get(), u1 = S.get(), u0 = S.get();   // Get3D, right-to-left arguments
        auto sm = b.sample(u0, u1, u2, is.ng);
        if (sm.f.x == 0 && sm.f.y == 0 && sm.f.z == 0) break;
        V3<float> f = sm.f;
        if (len > 2) { if (rng.f01() > sm.cont) break; f /= sm.cont; }
        o = is.pos; d = sm.wi;
        if (sm.ev & EV_D) diffuse++;
        tp *= f; last = sm.ev;
        if (!stored) dVM *= (sm.cos_out / sm.fwd) * sm.rev;
        else dVM = (sm.cos_out / sm.fwd) * (1.0f + sm.rev * dVM);
    }
}

void ref_render(Scene& s, std::vector<float>& img, int jitter_order) {
    const int W = s.W, H = s.H, maxlen = 6;
    img.assign(3 * (size_t)W * H, 0.0f);
    XorShift rng;
    for (int iter = 0; iter < s.samples; ++iter) {
        const float N = float(W * H);
        float radius = s.base_radius;
        radius /= std::pow(float(iter + 1), 0.5f * (1.0f - s.alpha));
        radius = std::max(radius, 1e-7f);
        float r2 = radius * radius;
        float vmn = 1.0f / (PIf * r2 * N);
        PhotonMap<float> pm;
        MltSampler S(maxlen, 1.0f, rng);
        int accepted = 1, mutated = 0, visible_uniform = 0;
        for (int p = 0; p < (int)N; ++p) {
            (void)rng.f01();   // progress report draw
            S.init_uniform(rng);
            bool vis = false;
            S.index = 0;
            ref_trace_light(s, S, rng, maxlen, pm.ph, vis);
            if (vis) { ++visible_uniform; }
            else {
                S.reject(); S.mutate(rng); mutated += 1;
                vis = false; S.index = 0;
                ref_trace_light(s, S, rng, maxlen, pm.ph, vis);
                if (vis) accepted += 1; else S.reject();
                float Rr = (float)accepted / (float)mutated;
                S.mutation_size += (Rr - 0.234f) / (float)mutated;
            }
        }
        if (getenv("ORACLE_DEBUG")) fprintf(stderr, "oracle photons %zu ratio %g vis %d acc %d mut %d\n", pm.ph.size(), pm.ph.size() / N, visible_uniform, accepted, mutated);
        float vnc = (float)visible_uniform / N;
        for (auto& ph : pm.ph) ph.tp *= vnc;
        pm.build();
        for (int p = 0; p < W * H; ++p) {
            (void)rng.f01();
            const float x = p % W, y = p / W;
            float j0, j1;
            if (jitter_order == 0) { j0 = 0 + (1 - 0) * rng.f01(); j1 = 0 + (1 - 0) * rng.f01(); }
            else { j1 = 0 + (1 - 0) * rng.f01(); j0 = 0 + (1 - 0) * rng.f01(); }
            float sx = x + j0, sy = y + j1;
            V3<float> dir = s.cam_bl + (sx / (float)W) * s.cam_h + (sy / (float)H) * s.cam_v;
            dir = dir - s.cam_o;
            V3<float> o = s.cam_o, d = normalize(dir), tp(1.0f);
            float dVM = 0;
            V3<float> color(0.0f);
            S.init_uniform(rng);
            S.index = 0;
            for (int len = 0;; ++len) {
                V3<float> ro = o + d * 0.001f;
                Hit<float> h;
                if (!scene_hit<float>(s, ro, d, 0.001f, h)) break;
                Isect<float> is; fill<float>(s, h, ro, d, is);
                Bsdf<float> b; b.init(s.mats[is.mat], is.ns, is.dir, true);
                if (!b.valid()) break;
                dVM /= std::fabs(std::abs(b.wo.z));
                if (!b.delta()) color += tp * vmn * contrib<float>(pm, is, b, r2, dVM);
                if (len > maxlen) break;
                float u2 = S.get(), u1 = S.get(), u0 = S.get();
                auto sm = b.sample(u0, u1, u2, is.ng);
                if (sm.f.x == 0 && sm.f.y == 0 && sm.f.z == 0) break;
                V3<float> f = sm.f;
                if (len > 2) { if (rng.f01() > sm.cont) break; f /= sm.cont; }
                o = is.pos; d = sm.wi; tp *= f;
                if (sm.ev & EV_S) dVM *= (sm.cos_out / sm.fwd) * sm.rev;
                else dVM = (sm.cos_out / sm.fwd) * (1.0f + sm.rev * dVM);
            }
            // Image_Buffer::add_color (src/Image_Buffer.h:24-37)
            if (sx < 0 || sx >= (float)W || sy < 0 || sy >= (float)H) continue;
            int X = (int)sx, Y = H - (int)sy;
            if ((size_t)(X + Y * W) > (size_t)W * H - 1) continue;
            img[3 * (X + Y * W)] += color.x; img[3 * (X + Y * W) + 1] += color.y; img[3 * (X + Y * W) + 2] += color.z;
        }
    }
    for (auto& v : img) v *= 1.0f / (float)s.samples;
}

std::string g_err;

}  // namespace orc

using namespace orc;

extern "C" {

struct OVec3 { float x, y, z; };
struct ODebug { int n; OVec3 d; float r, s; };

const char* oracle_last_error() { return g_err.c_str(); }

// Same argument list as the reference's init() (src/DLL.h:15-34).
void oracle_init(int samples, float base_radius, float radius_reduction, long long* meshes_pointers,
                 unsigned number_of_meshes, const float* mesh_matrices, unsigned* nverts, unsigned* ntris,
                 unsigned cam_x, unsigned cam_y, OVec3 cam_pos, OVec3 c0, OVec3 c1, OVec3 c2, OVec3 c3,
                 const unsigned char* lights, unsigned number_of_lights, const unsigned char* materials,
                 unsigned number_of_materials, int** materials_indices, int debug_test, ODebug dbg) {
    (void)debug_test; (void)dbg; (void)c0;
    g.reset(new Scene);
    g_kd_mt.seed(0);
    Scene& s = *g;
    s.samples = samples; s.base_radius = base_radius; s.alpha = radius_reduction;
    s.meshes.resize(number_of_meshes);
    for (unsigned i = 0; i < number_of_meshes; ++i) {
        Mesh& m = s.meshes[i];
        const char* base = (const char*)meshes_pointers[i];
        const char *mpoly, *mloop, *mvert;
        std::memcpy(&mpoly, base + 200, 8); std::memcpy(&mloop, base + 208, 8); std::memcpy(&mvert, base + 256, 8);
        std::memcpy(m.M, mesh_matrices + 16 * i, 64);
        // Inverse in double (src/matrix.cpp:4-63)
        double a[4][4];
        for (int r = 0; r < 4; ++r) for (int c = 0; c < 4; ++c) a[r][c] = m.M[4 * r + c];
        double A2323 = a[2][2] * a[3][3] - a[2][3] * a[3][2], A1323 = a[2][1] * a[3][3] - a[2][3] * a[3][1];
        double A1223 = a[2][1] * a[3][2] - a[2][2] * a[3][1], A0323 = a[2][0] * a[3][3] - a[2][3] * a[3][0];
        double A0223 = a[2][0] * a[3][2] - a[2][2] * a[3][0], A0123 = a[2][0] * a[3][1] - a[2][1] * a[3][0];
        double A2313 = a[1][2] * a[3][3] - a[1][3] * a[3][2], A1313 = a[1][1] * a[3][3] - a[1][3] * a[3][1];
        double A1213 = a[1][1] * a[3][2] - a[1][2] * a[3][1], A2312 = a[1][2] * a[2][3] - a[1][3] * a[2][2];
        double A1312 = a[1][1] * a[2][3] - a[1][3] * a[2][1], A1212 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
        double A0313 = a[1][0] * a[3][3] - a[1][3] * a[3][0], A0213 = a[1][0] * a[3][2] - a[1][2] * a[3][0];
        double A0312 = a[1][0] * a[2][3] - a[1][3] * a[2][0], A0212 = a[1][0] * a[2][2] - a[1][2] * a[2][0];
        double A0113 = a[1][0] * a[3][1] - a[1][1] * a[3][0], A0112 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
        double det = a[0][0] * (a[1][1] * A2323 - a[1][2] * A1323 + a[1][3] * A1223)
                   - a[0][1] * (a[1][0] * A2323 - a[1][2] * A0323 + a[1][3] * A0223)
                   + a[0][2] * (a[1][0] * A1323 - a[1][1] * A0323 + a[1][3] * A0123)
                   - a[0][3] * (a[1][0] * A1223 - a[1][1] * A0223 + a[1][2] * A0123);
        det = 1.0 / det;
        float* I = m.I;
        I[0] = (float)(det * (a[1][1] * A2323 - a[1][2] * A1323 + a[1][3] * A1223));
        I[1] = (float)(det * -(a[0][1] * A2323 - a[0][2] * A1323 + a[0][3] * A1223));
        I[2] = (float)(det * (a[0][1] * A2313 - a[0][2] * A1313 + a[0][3] * A1213));
        I[3] = (float)(det * -(a[0][1] * A2312 - a[0][2] * A1312 + a[0][3] * A1212));
        I[4] = (float)(det * -(a[1][0] * A2323 - a[1][2] * A0323 + a[1][3] * A0223));
        I[5] = (float)(det * (a[0][0] * A2323 - a[0][2] * A0323 + a[0][3] * A0223));
        I[6] = (float)(det * -(a[0][0] * A2313 - a[0][2] * A0313 + a[0][3] * A0213));
        I[7] = (float)(det * (a[0][0] * A2312 - a[0][2] * A0312 + a[0][3] * A0212));
        I[8] = (float)(det * (a[1][0] * A1323 - a[1][1] * A0323 + a[1][3] * A0123));
        I[9] = (float)(det * -(a[0][0] * A1323 - a[0][1] * A0323 + a[0][3] * A0123));
        I[10] = (float)(det * (a[0][0] * A1313 - a[0][1] * A0313 + a[0][3] * A0113));
        I[11] = (float)(det * -(a[0][0] * A1312 - a[0][1] * A0312 + a[0][3] * A0112));
        I[12] = (float)(det * -(a[1][0] * A1223 - a[1][1] * A0223 + a[1][2] * A0123));
        I[13] = (float)(det * (a[0][0] * A1223 - a[0][1] * A0223 + a[0][2] * A0123));
        I[14] = (float)(det * -(a[0][0] * A1213 - a[0][1] * A0213 + a[0][2] * A0113));
        I[15] = (float)(det * (a[0][0] * A1212 - a[0][1] * A0212 + a[0][2] * A0112));
        unsigned V = nverts[i], T = ntris[i];
        m.wp.resize(V); m.wn.resize(V); m.wpd.resize(V); m.wnd.resize(V);
        const float* M = m.M;
        for (unsigned v = 0; v < V; ++v) {
            float co[3]; int16_t no[3];
            std::memcpy(co, mvert + 20 * (size_t)v, 12); std::memcpy(no, mvert + 20 * (size_t)v + 12, 6);
            float x = co[0], y = co[1], z = co[2];
            // Transform::ApplyToPoint / ApplyToNormal (src/Transform.cpp)
            m.wp[v] = V3<float>(M[0] * x + M[1] * y + M[2] * z + M[3], M[4] * x + M[5] * y + M[6] * z + M[7],
                                M[8] * x + M[9] * y + M[10] * z + M[11]);
            float nx = no[0] * (1.0f / 32767.0f), ny = no[1] * (1.0f / 32767.0f), nz = no[2] * (1.0f / 32767.0f);
            m.wn[v] = normalize(V3<float>(I[0] * nx + I[4] * ny + I[8] * nz, I[1] * nx + I[5] * ny + I[9] * nz,
                                          I[2] * nx + I[6] * ny + I[10] * nz));
            double X = x, Y = y, Z = z;
            m.wpd[v] = V3<double>(M[0] * X + M[1] * Y + M[2] * Z + M[3], M[4] * X + M[5] * Y + M[6] * Z + M[7],
                                  M[8] * X + M[9] * Y + M[10] * Z + M[11]);
            double NX = no[0] / 32767.0, NY = no[1] / 32767.0, NZ = no[2] / 32767.0;
            m.wnd[v] = normalize(V3<double>(I[0] * NX + I[4] * NY + I[8] * NZ, I[1] * NX + I[5] * NY + I[9] * NZ,
                                            I[2] * NX + I[6] * NY + I[10] * NZ));
        }
        m.tri.resize(3 * (size_t)T); m.mat.resize(T);
        for (unsigned t = 0; t < T; ++t) {
            int32_t ls; int16_t mn;
            std::memcpy(&ls, mpoly + 12 * (size_t)t, 4); std::memcpy(&mn, mpoly + 12 * (size_t)t + 8, 2);
            for (int k = 0; k < 3; ++k) std::memcpy(&m.tri[3 * t + k], mloop + 8 * ((size_t)ls + k), 4);
            m.mat[t] = (uint32_t)materials_indices[i][mn];
        }
    }
    s.W = (int)cam_x; s.H = (int)cam_y;
    s.cam_o = V3<float>(cam_pos.x, cam_pos.y, cam_pos.z);
    s.cam_bl = V3<float>(c2.x, c2.y, c2.z);
    s.cam_h = V3<float>(c1.x, c1.y, c1.z) - s.cam_bl;
    s.cam_v = V3<float>(c3.x, c3.y, c3.z) - s.cam_bl;
    s.py_lights.assign(lights, lights + 64 * (size_t)number_of_lights);
    s.num_lights = number_of_lights;
    s.mats.clear();
    for (unsigned i = 0; i < number_of_materials; ++i) {
        const unsigned char* r = materials + 28 * (size_t)i;
        Material m; m.type = (char)r[0];
        std::memcpy(&m.ior, r + 4, 4); std::memcpy(&m.roughness, r + 8, 4); std::memcpy(&m.specular, r + 12, 4);
        float c[3]; std::memcpy(c, r + 16, 12);
        m.color = V3<float>(c[0], c[1], c[2]);
        s.mats.push_back(m);
    }
}

int oracle_prepare(float* info) {
    if (!g) { g_err = "no scene"; return -1; }
    int r = prepare(*g, g_err);
    if (r) return r;
    if (info) {
        info[0] = g->bounds.mn.x; info[1] = g->bounds.mn.y; info[2] = g->bounds.mn.z;
        info[3] = g->bounds.mx.x; info[4] = g->bounds.mx.y; info[5] = g->bounds.mx.z;
        info[6] = g->scene_radius; info[7] = g->base_radius; info[8] = (float)g->world.nodes.size();
    }
    return 0;
}

int oracle_mesh_bvh(int m, unsigned* nodes, int cap, int* tris, int tris_cap, float* cost) {
    const Bvh& b = g->meshes[m].bvh;
    int n = (int)b.nodes.size();
    for (int i = 0; i < n && i < cap; ++i) {
        float f[6] = {b.nodes[i].box.mn.x, b.nodes[i].box.mn.y, b.nodes[i].box.mn.z,
                      b.nodes[i].box.mx.x, b.nodes[i].box.mx.y, b.nodes[i].box.mx.z};
        std::memcpy(nodes + 8 * i, f, 24);
        nodes[8 * i + 6] = b.nodes[i].w0; nodes[8 * i + 7] = b.nodes[i].w1;
    }
    for (int i = 0; i < (int)b.index.size() && i < tris_cap; ++i) tris[i] = b.index[i];
    if (cost) *cost = b.cost;
    return n;
}

int oracle_world_bvh(unsigned* nodes, int cap, int* meshes, int cap2) {
    const Bvh& b = g->world;
    int n = (int)b.nodes.size();
    for (int i = 0; i < n && i < cap; ++i) {
        float f[6] = {b.nodes[i].box.mn.x, b.nodes[i].box.mn.y, b.nodes[i].box.mn.z,
                      b.nodes[i].box.mx.x, b.nodes[i].box.mx.y, b.nodes[i].box.mx.z};
        std::memcpy(nodes + 8 * i, f, 24);
        nodes[8 * i + 6] = b.nodes[i].w0; nodes[8 * i + 7] = b.nodes[i].w1;
    }
    for (int i = 0; i < (int)b.index.size() && i < cap2; ++i) meshes[i] = b.index[i];
    return n;
}

// Closest hit; out 16 floats per ray: [hit, t, u, v, Ng, Ns, pos, front, material, tri(bits)]
// tri = global triangle id in ingest order (meshes concatenated).  precision 32 or 64.
int oracle_trace(int n, const float* o, const float* d, float tmin, float* out, int precision) {
    if (!g || !g->prepared) { g_err = "not prepared"; return -1; }
    std::vector<unsigned> tri_base(g->meshes.size() + 1, 0);
    for (size_t i = 0; i < g->meshes.size(); ++i) tri_base[i + 1] = tri_base[i] + (unsigned)g->meshes[i].mat.size();
    for (int i = 0; i < n; ++i) {
        float* w = out + 16 * i;
        std::memset(w, 0, 64);
        w[14] = -1.0f;
        int tid = -1;
        if (precision == 64) {
            V3<double> ro(o[3 * i], o[3 * i + 1], o[3 * i + 2]), rd(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
            Hit<double> h;
            bool hit = scene_hit<double>(*g, ro, rd, (double)tmin, h);
            w[0] = hit; w[1] = (float)h.t; w[2] = (float)h.u; w[3] = (float)h.v;
            if (hit) {
                Isect<double> is; fill<double>(*g, h, ro, rd, is);
                w[4] = is.ng.x; w[5] = is.ng.y; w[6] = is.ng.z; w[7] = is.ns.x; w[8] = is.ns.y; w[9] = is.ns.z;
                w[10] = is.pos.x; w[11] = is.pos.y; w[12] = is.pos.z; w[13] = is.front; w[14] = is.mat;
                tid = (int)(tri_base[h.mesh] + h.tri);
            }
        } else {
            V3<float> ro(o[3 * i], o[3 * i + 1], o[3 * i + 2]), rd(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
            Hit<float> h;
            bool hit = scene_hit<float>(*g, ro, rd, tmin, h);
            w[0] = hit; w[1] = h.t; w[2] = h.u; w[3] = h.v;
            if (hit) {
                Isect<float> is; fill<float>(*g, h, ro, rd, is);
                w[4] = is.ng.x; w[5] = is.ng.y; w[6] = is.ng.z; w[7] = is.ns.x; w[8] = is.ns.y; w[9] = is.ns.z;
                w[10] = is.pos.x; w[11] = is.pos.y; w[12] = is.pos.z; w[13] = is.front; w[14] = is.mat;
                tid = (int)(tri_base[h.mesh] + h.tri);
            }
        }
        std::memcpy(&w[15], &tid, 4);
    }
    return 0;
}

// KD radius query as the reference performs it (tree built by the reference's own
// recursion with std::nth_element); indices in the reference's visiting order.
long long oracle_kd_query(int n, const float* pos, int q, const float* qpos, float r2, int* counts, int* idx, long long cap) {
    std::vector<V3<float>> p(n);
    for (int i = 0; i < n; ++i) p[i] = V3<float>(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    KdRef kd;
    kd.build(p);
    long long w = 0;
    for (int j = 0; j < q; ++j) {
        int c = 0;
        if (n > 0)
            kd.find(p, V3<float>(qpos[3 * j], qpos[3 * j + 1], qpos[3 * j + 2]), r2, 1, [&](int i) {
                if (w < cap) idx[w] = i;
                ++w; ++c;
            });
        counts[j] = c;
    }
    return w;
}

// BSDF probe (same layout as the reference harness's ref_bsdf)
int oracle_bsdf(const unsigned char* mat, const float* isect, int mode, const float* u3, const float* wi_eval, float* out) {
    Material m; m.type = (char)mat[0];
    std::memcpy(&m.ior, mat + 4, 4); std::memcpy(&m.roughness, mat + 8, 4); std::memcpy(&m.specular, mat + 12, 4);
    float c[3]; std::memcpy(c, mat + 16, 12); m.color = V3<float>(c[0], c[1], c[2]);
    Bsdf<float> b;
    V3<float> ng(isect[0], isect[1], isect[2]), ns(isect[3], isect[4], isect[5]), dir(isect[6], isect[7], isect[8]);
    b.init(m, ns, dir, mode == 0);
    std::memset(out, 0, 23 * sizeof(float));
    out[0] = b.valid(); out[1] = b.delta(); out[2] = std::abs(b.wo.z);
    // Get3D() builds vec3(Get1D(), Get1D(), Get1D()); g++ evaluates those arguments
    // right to left, so the first primary sample lands in .z
    auto sm = b.sample(u3[2], u3[1], u3[0], ng);
    out[3] = (sm.f.x == 0 && sm.f.y == 0 && sm.f.z == 0) ? 0.0f : 1.0f;
    out[4] = sm.f.x; out[5] = sm.f.y; out[6] = sm.f.z; out[7] = sm.wi.x; out[8] = sm.wi.y; out[9] = sm.wi.z;
    out[10] = sm.fwd; out[11] = sm.rev; out[12] = sm.cos_out; out[13] = sm.cont; out[14] = (float)sm.ev;
    V3<float> we(wi_eval[0], wi_eval[1], wi_eval[2]);
    V3<float> e = b.evaluate(we, ng);
    out[15] = e.x; out[16] = e.y; out[17] = e.z;
    float pf, pr; b.pdf(we, pf, pr);
    out[18] = pf; out[19] = pr;
    return 0;
}

int oracle_light_sample(const float* u, float* out) {
    if (!g || !g->prepared) return -1;
    V3<float> o, d, tp;
    sample_light<float>(*g, u, o, d, tp);
    out[0] = o.x; out[1] = o.y; out[2] = o.z; out[3] = d.x; out[4] = d.y; out[5] = d.z;
    out[6] = tp.x; out[7] = tp.y; out[8] = tp.z;
    return 0;
}

// Reference-mode render (the reference's own estimator and RNG stream).
int oracle_render_reference(float* rgb, int jitter_order) {
    if (!g) return -1;
    int r = prepare(*g, g_err);
    if (r) return r;
    std::vector<float> img;
    ref_render(*g, img, jitter_order);
    std::memcpy(rgb, img.data(), img.size() * sizeof(float));
    return 0;
}

// Debug views of the reference (src/Debug_scene.cpp:21-65 normals, :67-117 facing,
// :156-214 materials): one unjittered primary ray per pixel corner (x, y), closest hit
// with tmin 1e-4 from the camera origin, colour added through Image_Buffer::add_color
// (row 0 dropped); no averaging (src/main.cpp:170-200).  mode 2: shading normal;
// 3: (0,0,1) front / (1,0,0) back, times |dot(dir, Ns)|; 4: Fresnel reflectance with
// IOR `ior` (Debug_stuff::specular) of the view direction in the Ns frame.
int oracle_debug_view(int mode, float ior, float* rgb) {
    if (!g) return -1;
    int r = prepare(*g, g_err);
    if (r) return r;
    if (mode < 2 || mode > 4) { g_err = "debug mode must be 2, 3 or 4"; return -2; }
    const Scene& s = *g;
    const int W = s.W, H = s.H;
    std::vector<float> img(3 * (size_t)W * H, 0.0f);
    for (int p = 0; p < W * H; ++p) {
        const float x = p % W, y = p / W;
        V3<float> dir = s.cam_bl + (x / (float)W) * s.cam_h + (y / (float)H) * s.cam_v;
        dir = dir - s.cam_o;
        const V3<float> o = s.cam_o, d = normalize(dir);
        Hit<float> h;
        if (!scene_hit<float>(s, o, d, 0.0001f, h)) continue;
        Isect<float> is; fill<float>(s, h, o, d, is);
        V3<float> c;
        if (mode == 2) {
            c = is.ns;
        } else if (mode == 3) {
            const V3<float> base = is.front ? V3<float>(0, 0, 1) : V3<float>(1, 0, 0);
            c = base * std::abs(dot(d, is.ns));
        } else {
            Frame<float> fr;
            fr.set_from_z(is.ns);
            const V3<float> dl = fr.to_local(-is.dir);
            float eta = ior;
            if (dl.z > 0) eta = 1.0f / ior;
            c = V3<float>(fresnel_eta<float>((float)std::fabs((double)dl.z), eta));
        }
        int X = (int)x, Y = H - (int)y;
        if ((size_t)(X + Y * W) > (size_t)W * H - 1) continue;
        img[3 * (X + Y * W)] += c.x; img[3 * (X + Y * W) + 1] += c.y; img[3 * (X + Y * W) + 2] += c.z;
    }
    std::memcpy(rgb, img.data(), img.size() * sizeof(float));
    return 0;
}

// Plain-mode render: iterations [it0, it0 + iters) accumulated (sum, not mean) into
// acc (3*W*H doubles).  precision 32 or 64.  stats[0] += light paths, stats[1] += photons.
int oracle_render_plain(int it0, int iters, int precision, unsigned long long seed, long long paths,
                        int max_path_length, int threads, double* acc, long long* stats) {
    if (!g) return -1;
    int r = prepare(*g, g_err);
    if (r) return r;
    long long npix = (long long)g->W * g->H;
    if (paths <= 0) paths = npix;
    std::vector<double> a(acc, acc + 3 * npix);
    for (int it = it0; it < it0 + iters; ++it) {
        if (precision == 64) {
            PlainCfg<double> c{seed, paths, max_path_length};
            plain_iteration<double>(*g, c, (uint32_t)it, threads, a, stats);
        } else {
            PlainCfg<float> c{seed, paths, max_path_length};
            plain_iteration<float>(*g, c, (uint32_t)it, threads, a, stats);
        }
    }
    std::memcpy(acc, a.data(), a.size() * sizeof(double));
    return 0;
}

// Light pass only (plain mode, FP32): the photons of iteration `it` in path order.
// out: 12 floats per photon [pos xyz, dir xyz, tp xyz, dVM, path(bits), 0]
long long oracle_light_photons(int it, unsigned long long seed, long long paths, int max_path_length, float* out,
                               long long cap, int threads) {
    if (!g) return -1;
    if (prepare(*g, g_err)) return -1;
    PlainCfg<float> c{seed, paths, max_path_length};
    PhotonMap<float> pm;
    light_pass<float>(*g, c, (uint32_t)it, threads, pm);
    long long n = (long long)pm.ph.size();
    for (long long i = 0; i < n && i < cap; ++i) {
        const Photon<float>& p = pm.ph[i];
        float* w = out + 12 * i;
        w[0] = p.pos.x; w[1] = p.pos.y; w[2] = p.pos.z; w[3] = p.dir.x; w[4] = p.dir.y; w[5] = p.dir.z;
        w[6] = p.tp.x; w[7] = p.tp.y; w[8] = p.tp.z; w[9] = p.dVM;
        std::memcpy(&w[10], &p.path, 4); w[11] = 0;
    }
    return n;
}

int oracle_scene_info(int* out) {
    if (!g) return -1;
    out[0] = g->W; out[1] = g->H; out[2] = (int)g->meshes.size();
    long long t = 0;
    for (auto& m : g->meshes) t += (long long)m.mat.size();
    out[3] = (int)t;
    return 0;
}

int oracle_release() { g.reset(); return 0; }

}  // extern "C"
