// Per-mesh SAH BVH build on the device.  The node arrays, the triangle order of the
// leaves and each mesh's traversal cost are bit-identical to the host build
// (host_scene.cpp), itself the reference's recursive binned-SAH build
// (src/BVH/BVH_mesh.cpp:28-155), its depth-first flattening (:199-261) and
// CostOfTraversing (:286-305).
//
// The device build covers inputs whose triangle boxes and centroids are finite and
// contain no -0.0: box unions are then a plain min/max, independent of the order in
// which they are taken.  Any other input (and a mesh without triangles) reports
// `supported = false` and is built on the host.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "host_scene.h"

namespace rc {

struct GpuMeshSrc {
    const V3* wpos;        // world-space vertex positions
    const V3* wnrm;        // normalised world-space vertex normals
    const uint32_t* tri;   // 3 mesh-local vertex indices per triangle
    const uint32_t* mat;   // global material index per triangle
    uint32_t num_verts, num_tris;
};

class GpuBvhBuilder {
public:
    // Uploads the meshes and builds their trees.  On return with RC_OK, `supported`
    // says whether the device build applies; num_nodes() is then the node count of all
    // meshes together.
    int build(const std::vector<GpuMeshSrc>& meshes, cudaStream_t s, bool& supported, std::string& err);
    long long num_nodes() const { return num_nodes_; }
    long long num_tris() const { return num_tris_; }
    // Writes the flattened nodes (mesh after mesh, pre-order, the device format: node i
    // at nodes[2i] = (min, word0), nodes[2i+1] = (max, word1); inner word0/word1 = global
    // child indices, leaf word0 = 0x80000000 | count, word1 = first triangle slot) and
    // the triangle records in leaf order (slot j at tris[3j..3j+2] = v0 | global triangle
    // id, e1 | material, e2 | mesh; the three vertex normals in n0..n2), then fills
    // mesh_root, mesh_box and mesh_cost.
    int emit(float4* nodes, float4* tris, float4* n0, float4* n1, float4* n2, cudaStream_t s, std::string& err);
    std::vector<int> mesh_root;       // global index of each mesh's root node
    std::vector<float> mesh_box;      // 6 floats per mesh: min xyz, max xyz
    std::vector<float> mesh_cost;     // CostOfTraversing of the root
    int levels = 0;                   // level passes over segments above the warp size limit
    void release();
    ~GpuBvhBuilder() { release(); }

private:
    struct Bufs;
    Bufs* b_ = nullptr;
    long long num_nodes_ = 0, num_tris_ = 0;
    int num_meshes_ = 0;
};

}  // namespace rc
