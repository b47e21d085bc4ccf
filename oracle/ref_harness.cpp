// Test harness linked against the UNMODIFIED reference sources by
// oracle/build_ref.sh.  It is test infrastructure: it lets the tests and the
// fixture generator call the reference's own functions (scene build, closest
// hit, KD-tree radius query, BSDFs, light sampling, the full render) on inputs
// the tests choose.  Nothing in the product links or loads it.
//
// Reference entry points exercised (paths within "Real Caustics/src"):
//   init                                main.cpp:89-143
//   main() pre-render steps             main.cpp:150-168
//   Scene::hit                          Scene.cpp:154-189
//   KD_Tree::build_kd_tree / find_closest_in_radius   KD_Tree.cpp:178-280
//   Material::compute_scattering_functions + BxDF     materials.h:59-146, BXDF.cpp
//   Lights_list::sample_lights          Light_list.cpp:10-30
//   Vertex_Merging::run                 Vertex_Merging.cpp:367-379
#include <cstddef>
#include <cstring>
#include <vector>
#include <limits>
#include "vec3.h"
#include "ray.h"
#include "Hit_rec.h"
#include "Blender_definitions.h"
#include "matrix.h"
#include "Lights.h"
#include "Light_list.h"
#include "materials.h"
#include "BXDF.h"
#include "MLT_Sampler.h"
#include "KD_Tree.h"
#include "Path_Vertices.h"
#include "Vertex_Merging.h"
#include "Scene.h"
#include "mesh.h"
#include "BVH/BVH_mesh.h"
#include "BVH/BVH_world.h"

extern Scene* scene;
extern Python_Light* python_lights;
extern const float inf;

extern "C" {

// Layout facts of the ABI structs, as this compiler lays them out.
// out[0..2]  = offsetof(Mesh_blender, mpoly / mloop / mvert)
// out[3..5]  = sizeof(MVert), sizeof(MPoly), sizeof(MLoop)
// out[6..9]  = sizeof(Python_Light), sizeof(Python_Material),
//              sizeof(PythonMatrix4x4), sizeof(Debug_stuff)
// out[10..18]= offsetof(Python_Light, type/color/position/width/height/spread/rotation/power/angle)
// out[19]    = offsetof(Python_Light, radius)
// out[20..24]= offsetof(Python_Material, type/ior/roughness/specular/color)
// out[25..27]= offsetof(MVert, co/no/flag); out[28..30] = offsetof(MPoly, loopstart/totloop/mat_nr)
int ref_layout(long long* out)
{
    out[0] = offsetof(Mesh_blender, mpoly);
    out[1] = offsetof(Mesh_blender, mloop);
    out[2] = offsetof(Mesh_blender, mvert);
    out[3] = sizeof(MVert);
    out[4] = sizeof(MPoly);
    out[5] = sizeof(MLoop);
    out[6] = sizeof(Python_Light);
    out[7] = sizeof(Python_Material);
    out[8] = sizeof(PythonMatrix4x4);
    out[9] = sizeof(Debug_stuff);
    out[10] = offsetof(Python_Light, type);
    out[11] = offsetof(Python_Light, color);
    out[12] = offsetof(Python_Light, position);
    out[13] = offsetof(Python_Light, width);
    out[14] = offsetof(Python_Light, height);
    out[15] = offsetof(Python_Light, spread);
    out[16] = offsetof(Python_Light, rotation);
    out[17] = offsetof(Python_Light, power);
    out[18] = offsetof(Python_Light, angle);
    out[19] = offsetof(Python_Light, radius);
    out[20] = offsetof(Python_Material, type);
    out[21] = offsetof(Python_Material, ior);
    out[22] = offsetof(Python_Material, roughness);
    out[23] = offsetof(Python_Material, specular);
    out[24] = offsetof(Python_Material, color);
    out[25] = offsetof(MVert, co);
    out[26] = offsetof(MVert, no);
    out[27] = offsetof(MVert, flag);
    out[28] = offsetof(MPoly, loopstart);
    out[29] = offsetof(MPoly, totloop);
    out[30] = offsetof(MPoly, mat_nr);
    return sizeof(Mesh_blender);
}

// The pre-render half of the reference main() (main.cpp:150-168): BVH build,
// light conversion, light CDF, radius scaled by the scene radius.
// out_info: [0..5] scene bbox min/max, [6] scene radius, [7] scaled base radius,
//           [8] number of world BVH nodes
int ref_prepare(float* out_info)
{
    if (!scene) return -1;
    scene->update_bvh(1, "unused");
    scene->init_lights(python_lights);
    scene->lights.update_pdf_distribution();
    float SceneRadius = (scene->bounding_box.min - (scene->bounding_box.min + scene->bounding_box.max) * 0.5f).length();
    scene->integrator.base_radius *= SceneRadius;
    if (out_info) {
        out_info[0] = scene->bounding_box.min.x; out_info[1] = scene->bounding_box.min.y;
        out_info[2] = scene->bounding_box.min.z; out_info[3] = scene->bounding_box.max.x;
        out_info[4] = scene->bounding_box.max.y; out_info[5] = scene->bounding_box.max.z;
        out_info[6] = SceneRadius;
        out_info[7] = scene->integrator.base_radius;
        out_info[8] = (float)scene->BVH.bvh_nodes.size();
    }
    return 0;
}

// Mesh BVH of mesh m in the reference's flattened layout: nodes as 8 words
// (min xyz, max xyz as float bits, then the two union words), and the 1-based
// triangle index list.  Returns the node count; copies at most cap nodes.
int ref_mesh_bvh(int m, unsigned* nodes, int cap, int* tris, int tris_cap, float* cost)
{
    const BVH_mesh& b = scene->meshes[m].BVH;
    int n = (int)b.bvh_nodes.size();
    for (int i = 0; i < n && i < cap; ++i) {
        const CacheBVHNode_mesh& nd = b.bvh_nodes[i];
        float f[6] = {nd.bounding_box.min.x, nd.bounding_box.min.y, nd.bounding_box.min.z,
                      nd.bounding_box.max.x, nd.bounding_box.max.y, nd.bounding_box.max.z};
        std::memcpy(nodes + 8 * i, f, sizeof(f));
        nodes[8 * i + 6] = nd.u.inner.idxLeft;
        nodes[8 * i + 7] = nd.u.inner.idxRight;
    }
    int nt = (int)b.tris_indices.size();
    for (int i = 0; i < nt && i < tris_cap; ++i) tris[i] = b.tris_indices[i];
    if (cost) *cost = b.cost;
    return n;
}

int ref_world_bvh(unsigned* nodes, int cap, int* meshes, int meshes_cap)
{
    const BVH_world& b = scene->BVH;
    int n = (int)b.bvh_nodes.size();
    for (int i = 0; i < n && i < cap; ++i) {
        const CacheBVHNode_world& nd = b.bvh_nodes[i];
        float f[6] = {nd.bounding_box.min.x, nd.bounding_box.min.y, nd.bounding_box.min.z,
                      nd.bounding_box.max.x, nd.bounding_box.max.y, nd.bounding_box.max.z};
        std::memcpy(nodes + 8 * i, f, sizeof(f));
        nodes[8 * i + 6] = nd.u.inner.idxLeft;
        nodes[8 * i + 7] = nd.u.inner.idxRight;
    }
    int nm = (int)b.mesh_indices.size();
    for (int i = 0; i < nm && i < meshes_cap; ++i) meshes[i] = b.mesh_indices[i];
    return n;
}

// Scene::hit on n rays.  out: 16 floats per ray:
// [hit, t, u, v, Ng xyz, Ns xyz, position xyz, front_face, material]
int ref_trace(int n, const float* orig, const float* dir, float tmin, float* out)
{
    if (!scene) return -1;
    for (int i = 0; i < n; ++i) {
        ray r(vec3(orig[3 * i], orig[3 * i + 1], orig[3 * i + 2]),
              vec3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]));
        Isect h;
        bool hit = scene->hit(r, tmin, inf, h, 0);
        float* o = out + 16 * i;
        o[0] = hit ? 1.0f : 0.0f;
        o[1] = h.distance; o[2] = h.u; o[3] = h.v;
        o[4] = h.geometric_normal.x; o[5] = h.geometric_normal.y; o[6] = h.geometric_normal.z;
        o[7] = h.shade_normal.x; o[8] = h.shade_normal.y; o[9] = h.shade_normal.z;
        o[10] = h.position.x; o[11] = h.position.y; o[12] = h.position.z;
        o[13] = h.front_face ? 1.0f : 0.0f;
        o[14] = hit ? (float)h.material_idx : -1.0f;
        o[15] = 0.0f;
    }
    return 0;
}

// KD tree over n photon positions; photon i carries its index in throughput.x
// (the query never reads throughput).  Returns the node-array length; writes at
// most node_cap nodes as (index word, split bits).
int ref_kd_build(int n, const float* pos, unsigned* nodes, int node_cap)
{
    std::vector<Path_Vertex> pv(n);
    for (int i = 0; i < n; ++i) {
        pv[i].position = vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        float tag; std::memcpy(&tag, &i, 4);
        pv[i].throughput = vec3(tag, 0.0f, 0.0f);
    }
    KD_Tree t;
    t.build_kd_tree(pv);
    int m = (int)t.kdtree.size();
    for (int i = 0; i < m && i < node_cap; ++i) {
        nodes[2 * i] = t.kdtree[i].u.leaf.index;
        std::memcpy(&nodes[2 * i + 1], &t.kdtree[i].u.inner.split, 4);
    }
    return m;
}

// Radius query: for each of q query points, the indices of photons with
// squared distance < r2, as returned by find_closest_in_radius (tree order).
// counts[q] receives the number found; indices are packed into idx (cap total).
long long ref_kd_query(int n, const float* pos, int q, const float* qpos, float r2,
                       int* counts, int* idx, long long cap)
{
    std::vector<Path_Vertex> pv(n);
    for (int i = 0; i < n; ++i) {
        pv[i].position = vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        float tag; std::memcpy(&tag, &i, 4);
        pv[i].throughput = vec3(tag, 0.0f, 0.0f);
    }
    KD_Tree t;
    t.build_kd_tree(pv);
    long long w = 0;
    for (int j = 0; j < q; ++j) {
        std::vector<Path_Vertex> found;
        float r = r2;
        t.find_closest_in_radius(vec3(qpos[3 * j], qpos[3 * j + 1], qpos[3 * j + 2]), r, pv, found, 1);
        counts[j] = (int)found.size();
        for (const Path_Vertex& f : found) {
            int id; std::memcpy(&id, &f.throughput.x, 4);
            if (w < cap) idx[w] = id;
            ++w;
        }
    }
    return w;
}

// One BSDF built the way the integrator builds it (Isect::compute_scattering_functions),
// then sampled with the given 3 primary samples and evaluated/pdf'd at wi_eval.
// isect: [Ng xyz, Ns xyz, ray dir xyz]; mode 0 = Radiance (camera), 1 = Importance (light)
// out: [valid, delta, cos_theta_in, sample_ok, f xyz, wi xyz, fwd_pdf, rev_pdf,
//       cos_out, cont_prob, event, eval xyz, pdf_fwd, pdf_rev]  (23 floats)
int ref_bsdf(const Python_Material* mat, const float* isect, int mode, const float* u3,
             const float* wi_eval, float* out)
{
    Material* m = nullptr;
    vec3 color(mat->color.r, mat->color.g, mat->color.b);
    if (mat->type == 'P') m = new Plastic_Material(color, mat->roughness, mat->specular);
    else if (mat->type == 'G') m = new Glass_Material(color, mat->ior);
    else if (mat->type == 'M') m = new Metal_Material(color, mat->roughness);
    else m = new Plastic_Material(vec3(1, 1, 1), 1, 0.0);
    Isect h;
    h.geometric_normal = vec3(isect[0], isect[1], isect[2]);
    h.shade_normal = vec3(isect[3], isect[4], isect[5]);
    h.direction = vec3(isect[6], isect[7], isect[8]);
    h.material_idx = 0;
    BxDF* b = nullptr;
    m->compute_scattering_functions(&b, h, mode == 0 ? TransportMode::Radiance : TransportMode::Importance);
    MLT_Sampler s(6, 1.0f);
    s.samples[0].value = u3[0]; s.samples[1].value = u3[1]; s.samples[2].value = u3[2];
    s.Start_Iteration();
    vec3 wi(0.0f);
    float fwd = -1.0f, rev = -1.0f, cos_out = -1.0f, cont = -1.0f;
    BxDFType ev = BSDF_ALL;
    std::memset(out, 0, 23 * sizeof(float));
    out[0] = b->IsValid() ? 1.0f : 0.0f;
    out[1] = b->Is_delta() ? 1.0f : 0.0f;
    out[2] = b->cos_theta_in();
    vec3 f = b->sample(wi, h.geometric_normal, fwd, rev, cos_out, cont, ev, s);
    out[3] = (f.x == 0.0f && f.y == 0.0f && f.z == 0.0f) ? 0.0f : 1.0f;
    out[4] = f.x; out[5] = f.y; out[6] = f.z;
    out[7] = wi.x; out[8] = wi.y; out[9] = wi.z;
    out[10] = fwd; out[11] = rev; out[12] = cos_out; out[13] = cont; out[14] = (float)(int)ev;
    vec3 we(wi_eval[0], wi_eval[1], wi_eval[2]);
    vec3 e = b->evaluate(we, h.geometric_normal);
    out[15] = e.x; out[16] = e.y; out[17] = e.z;
    float pf = -1.0f, pr = -1.0f;
    b->pdf(we, pf, pr);
    out[18] = pf; out[19] = pr;
    out[20] = (float)s.index;
    delete b;
    delete m;
    return 0;
}

// Light emission: Lights_list::sample_lights over the scene's converted lights
// (ref_prepare must have run) with the given primary samples (5 used).
// out: [origin xyz, dir xyz, throughput xyz, samples consumed]
int ref_light_sample(const float* u, float* out)
{
    if (!scene) return -1;
    MLT_Sampler s(6, 1.0f);
    for (int i = 0; i < 8; ++i) s.samples[i].value = u[i];
    s.Start_Iteration();
    Light_Sub_Path_State st;
    st.origin = vec3(0.0f); st.direction = vec3(0.0f);
    scene->lights.sample_lights(st, s);
    out[0] = st.origin.x; out[1] = st.origin.y; out[2] = st.origin.z;
    out[3] = st.direction.x; out[4] = st.direction.y; out[5] = st.direction.z;
    out[6] = st.throughput.x; out[7] = st.throughput.y; out[8] = st.throughput.z;
    out[9] = (float)s.index;
    return 0;
}

// Full render by the reference integrator (Vertex_Merging::run) after
// ref_prepare.  Copies the accumulated image (buffer order, RGB float) and
// releases the scene as the reference main() does.
int ref_render(float* rgb)
{
    if (!scene) return -1;
    scene->integrator.run();
    const std::vector<vec3>& c = scene->integrator.image_buffer.color;
    for (size_t i = 0; i < c.size(); ++i) {
        rgb[3 * i] = c[i].x; rgb[3 * i + 1] = c[i].y; rgb[3 * i + 2] = c[i].z;
    }
    delete scene;
    scene = nullptr;
    return 0;
}

// Debug view `mode` (2 normals, 3 facing, 4 materials) by the reference's own
// Vertex_Merging::run_debug_* (src/Debug_scene.cpp) after ref_prepare; copies the
// image buffer and releases the scene.
int ref_debug(int mode, float* rgb)
{
    if (!scene) return -1;
    if (mode == 2) scene->integrator.run_debug_normals();
    else if (mode == 3) scene->integrator.run_debug_facing();
    else if (mode == 4) scene->integrator.run_debug_materials();
    else return -2;
    const std::vector<vec3>& c = scene->integrator.image_buffer.color;
    for (size_t i = 0; i < c.size(); ++i) {
        rgb[3 * i] = c[i].x; rgb[3 * i + 1] = c[i].y; rgb[3 * i + 2] = c[i].z;
    }
    delete scene;
    scene = nullptr;
    return 0;
}

// Vertex_Merging::run_debug_bvh (src/Debug_scene.cpp:284-320): OBJ files of the mesh
// BVH boxes, one per depth, written by the reference into the working directory.
int ref_debug_bvh()
{
    if (!scene) return -1;
    scene->integrator.run_debug_bvh();
    return 0;
}

int ref_release()
{
    delete scene;
    scene = nullptr;
    return 0;
}

}  // extern "C"
