// Host-side scene: ingest of the Blender meshes passed to init(), the two-level SAH
// BVH (restated from the reference so that hits are bit-identical), lights and
// materials converted to flat records the kernels read.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include "realcaustics.h"
#include "rc_device_types.h"

namespace rc {

struct V3 { float x, y, z; };

struct Box {
    V3 mn{INFINITY, INFINITY, INFINITY};
    V3 mx{-INFINITY, -INFINITY, -INFINITY};
};

// One reference BVH node (CacheBVHNode_mesh / CacheBVHNode_world,
// src/BVH/BVH_mesh.h:51-71): box + two words; word0 bit 31 marks a leaf
// (word0 = 0x80000000 | count, word1 = start in the 1-based index list).
struct BvhNode {
    Box box;
    uint32_t w0, w1;
};

struct MeshBvh {
    std::vector<BvhNode> nodes;
    std::vector<int> index;   // 1-based triangle list, slot 0 unused (src/BVH/BVH_mesh.cpp:231)
    float cost = 0.0f;        // CostOfTraversing (src/BVH/BVH_mesh.cpp:286-305)
    Box bounds;
};

struct WorldBvh {
    std::vector<BvhNode> nodes;
    std::vector<int> index;   // 1-based mesh list
};

struct HostMesh {
    uint32_t num_tris = 0, num_verts = 0;
    // world-space vertex positions, computed once with the reference's operation
    // order (Transform::ApplyToPoint, src/Transform.cpp:3-10)
    std::vector<V3> wpos;
    // normalised world-space vertex normals (src/Triangle.cpp:11-16,36-42)
    std::vector<V3> wnrm;
    std::vector<uint32_t> tri;     // 3 vertex indices per triangle
    std::vector<uint32_t> mat;     // global material index per triangle
    float m[16], inv[16];
    MeshBvh bvh;
};

struct HostCamera {
    int width = 0, height = 0;
    V3 origin{}, bottom_left{}, horizontal{}, vertical{};
};

struct HostScene {
    // init() arguments
    int samples = 1;
    float base_radius = 0.0f;
    float radius_alpha = 0.0f;
    int debug_test = 1;
    float debug_ior = 1.0f;       // Debug_stuff::specular (the materials debug view's IOR)
    std::vector<HostMesh> meshes;
    HostCamera camera;
    std::vector<rc_python_light> py_lights;      // copied at init, converted at prepare
    unsigned num_lights = 0;
    std::vector<rc_python_material> py_materials;
    // after prepare()
    WorldBvh world;
    Box bounds;
    float scene_radius = 0.0f;
    std::vector<DevLight> lights;
    std::vector<float> light_cdf;   // size n+1, Lights_list::update_pdf_distribution
    float light_integral = 0.0f;
    std::vector<DevMaterial> materials;
    bool prepared = false;
};

// Read one Blender mesh (DNA 2.9x) the way Mesh::Mesh does (src/mesh.cpp:12-27).
int ingest_mesh(HostMesh& out, const void* blender_mesh, unsigned nverts, unsigned ntris,
                const rc_matrix4x4& matrix, const int* material_indices, std::string& err);

void build_mesh_bvh(HostMesh& mesh);
void build_world_bvh(HostScene& scene);
int convert_lights(HostScene& scene, std::string& err);
void convert_materials(HostScene& scene);
float cost_of_traversing(const MeshBvh& bvh, int node);

}  // namespace rc
