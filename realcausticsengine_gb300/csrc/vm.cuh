// Vertex-merging iteration on the device: shared declarations of the kernels in
// vm_kernels.cu and gather.cu and the buffers they exchange.
//
// One progressive iteration (src/Vertex_Merging.cpp:196-366):
//   light pass   - light sub-paths, photons stored at non-delta vertices reached by a
//                  glossy event (Path_Vertex records)
//   KD build     - photon KD-tree over the stored photons (kdtree.cu)
//   camera pass  - one camera sub-path per pixel; every non-delta vertex becomes a
//                  merge query
//   gather       - photons within the merge radius of each query, MIS-weighted BSDF
//                  contribution, accumulated into the FP64 per-pixel running sum
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "rc_device_types.h"
#include "trace.cuh"
#include "kdtree.cuh"

namespace rc {

// Photon records (Path_Vertex, src/Path_Vertices.h:10-20), structure of arrays:
//   pos  = position.xyz | dVM          dir = direction_world.xyz | throughput.r
//   tp   = throughput.g, throughput.b  path = light path index
struct PhotonBuf {
    float4* pos;
    float4* dir;
    float2* tp;
    uint32_t* path;
    long long capacity;
    unsigned long long* count;   // device counter (may exceed capacity: overflow)
};

// Merge queries written by the camera pass (one per non-delta camera vertex):
//   q0 = position.xyz | camera dVM      q1 = shading normal.xyz | material
//   q2 = geometric normal.xyz | pixel   q3 = throughput * VM_normalization | 0
//   q4 = incoming ray direction.xyz | 0
struct QueryBuf {
    float4* q0; float4* q1; float4* q2; float4* q3; float4* q4;
    long long capacity;
    unsigned long long* count;
};

// Photon records in KD-tree order (filled after the build by launch_tree_records):
//   t0 = position.xyz | dVM   t1 = direction_world.xyz | throughput.r   t2 = throughput.gb
struct TreePhotons {
    float4* t0;
    float4* t1;
    float2* t2;
};

struct LightsView {
    const DevLight* lights;
    const float* cdf;      // n + 1 entries
    int count;
    float integral;
};

struct VMParams {
    SceneView scene;
    LightsView lights;
    const DevMaterial* materials;
    int num_materials;
    DevCamera camera;
    uint64_t seed;            // light-path samples
    uint64_t camera_seed;     // camera-path samples
    uint32_t iteration;
    long long num_light_paths;
    int max_path_length;
    float radius_sqr;
    float vm_norm;
    float merge_scale;      // gather: factor on every merge (the Metropolis samplers' visible
                            // fraction of large steps, known after the light pass; else 1)
    int* error;             // device flags: [0] stack overflow, [1] bad material
    const float4* proposal; // learned emission proposal per light path (nullptr: none)
    float* path_contrib;    // gather: per light path, sum over its merges of the squared
                            // luminance each adds to its pixel (proposal training)
    const uint32_t* photon_path;   // photon buffer index -> light path (with path_contrib)
    // tabulated learned proposal for the Metropolis samplers (proposal.cuh; nullptr: none)
    const float* proposal_table;
    int proposal_table_res;
    const uint32_t* path_order;    // light-path processing order (launch_light_order; nullptr: index order)
};

// One scene of a batch render (launch_light_pass_batch / launch_camera_pass_batch):
// its iteration parameters and the buffers its passes append to.
struct BatchScene {
    VMParams p;
    PhotonBuf ph;
    QueryBuf qb;
};

// error flag slots
enum { ERR_STACK = 0, ERR_MATERIAL = 1, ERR_PHOTON_OVERFLOW = 2, ERR_QUERY_OVERFLOW = 3, ERR_KD = 4, ERR_MLP = 5,
       ERR_GATHER = 6, ERR_COUNT = 8 };

// Metropolis light pass (RC_SAMPLER_HYBRID / RC_SAMPLER_PSSMLT), `chains` chains in one
// launch; stats[0] = visible large steps, stats[1] = large steps (HYBRID: light paths).
// The photons must be scaled by stats[0] / stats[1] (applied through VM_normalization).
constexpr int kMltMaxPathLength = 12;
// variant (PSSMLT only): 0 the chains advanced one path segment per loop iteration,
// 1 one step at a time (the same photons and counts).
void launch_mlt_pass(const VMParams& p, PhotonBuf ph, int sampler, int chains, float p_large,
                     unsigned long long* stats, cudaStream_t s, int variant = 0);
int mlt_variants();
// Processing order of the light paths (p.num_light_paths of them) for p.path_order:
// indices sorted by the 4D Morton cell (32 per axis) of their own emission samples (area
// u, v, direction u, v; with p.proposal, the proposed direction's octahedral coordinates
// for the direction), so that each warp of the persistent pass starts coherent rays.
// Every path keeps its samples and index: only the order of tracing changes.
size_t light_order_scratch_bytes(long long n);
void launch_light_order(const VMParams& p, void* scratch, uint32_t* order, cudaStream_t s);
// Exclusive scan of m counters in place; large m in three passes over 8192-counter tiles
// with tile_scratch (scan_scratch_words(m) words) for the tile totals.
size_t scan_scratch_words(long long m);
void launch_scan_counts(uint32_t* counts, long long m, uint32_t* tile_scratch, cudaStream_t s);
// next_path: device counter for the persistent kernel (nullptr: one thread per path);
// rays (optional): receives the number of closest-hit queries the pass traced.
void launch_light_pass(const VMParams& p, PhotonBuf ph, unsigned long long* next_path, cudaStream_t s, int variant = 0,
                       unsigned long long* rays = nullptr);
void launch_camera_pass(const VMParams& p, QueryBuf qb, unsigned long long* next_pixel, cudaStream_t s, int variant = 0);
// The persistent light and camera passes over n resident scenes in one launch each:
// scenes[i] (device memory) holds scene i's parameters and buffers, path_prefix
// (pixel_prefix) n + 1 device words with the first work index of each scene and the
// total at [n].  A scene's photons (queries) are the ones its own pass stores, in
// another order.  variant: the launch shapes of the single-scene passes (0-4).
void launch_light_pass_batch(const BatchScene* scenes, const long long* path_prefix, int n, long long total_paths,
                             unsigned long long* next_path, cudaStream_t s, int variant = 0);
void launch_camera_pass_batch(const BatchScene* scenes, const long long* pixel_prefix, int n, long long total_pixels,
                              unsigned long long* next_pixel, cudaStream_t s, int variant = 0);
// Debug view `mode` (2 normals, 3 facing, 4 materials with IOR `ior`) added into the
// FP64 image accumulation.
void launch_debug_view(const VMParams& p, int mode, float ior, double* accum, cudaStream_t s);
// FP32 mean image (n floats) from the FP64 running sum.
void launch_image_mean(const double* acc, float* out, long long n, double scale, cudaStream_t s);
// Photon slots [*count, capacity) get position `pad` (chosen outside the scene by more
// than any merge radius: a KD tree over the full capacity then answers the same radius
// queries as one over the stored photons), and *flag = 1 when a count overflowed its
// capacity.
void launch_pad_photons(float4* pos, const unsigned long long* count, long long capacity, float4 pad,
                        cudaStream_t s);
void launch_check_counts(const unsigned long long* photons, long long photon_cap, const unsigned long long* queries,
                         long long query_cap, int* flag, cudaStream_t s);
// shape 0: the persistent passes' traversal; 1: the wavefront pass's warp-stepped one;
// 2: pop-and-test (the reference's form).
void launch_trace_rays(const SceneView& s, int n, const float* o, const float* d, float tmin, float* out_full,
                       unsigned* out_words, int* err, cudaStream_t st, int shape = 0);
// Photon records in tree order (tp.t0/t1/t2 from ph.pos/dir/tp; only t0 when ph.dir is null).
void launch_tree_records(PhotonBuf ph, const KdTree& tree, TreePhotons tp, cudaStream_t s);
// Node bounding boxes used by the gather to prune exactly: the photons in tree order
// are cut into 2^Lc chunks of at most 32 (Lc = kd_chunk_level(n), the shallowest level
// whose nodes hold at most 31 photons: a chunk is such a node's range plus the median
// photon that may follow it); the chunk boxes carry their first position and count in
// .w, every node above has the union of its children's.  Levels [0, kd_box_levels(n)),
// arrays of 2^kd_box_levels(n) float4 each, filled from the tree's x/y/z.
int kd_chunk_level(long long n);
int kd_box_levels(long long n);
void launch_kd_boxes(const KdTree& tree, cudaStream_t s, int* launches);
// Spatial order of queries (positions at qpos + stride*i): order[] receives the query
// indices sorted by the 30-bit Morton code of their cell in a 1024^3 grid over the box
// `frame` describes (query_frame(lo, hi); positions outside are clamped), by a stable
// radix sort.  scratch: query_order_scratch_bytes(nq) bytes.
struct QueryFrame { float lo[3], scale[3]; };
QueryFrame query_frame(const float lo[3], const float hi[3]);
size_t query_order_scratch_bytes(long long nq);
void launch_query_order(const float* qpos, int stride, long long nq, const QueryFrame& frame, void* scratch,
                        uint32_t* order, int* launches, cudaStream_t s, const unsigned long long* nq_dev = nullptr);
// The gather: one fused kernel over groups of ordered queries (gather.cu).  Photon sets
// are the reference's; each accepted photon's merge (BSDF, MIS weight, throughput) is
// summed per query and added into the query's FP64 pixel.  `variant` picks the launch
// shape (gather_variant_name).  counters (optional, 4 u64 accumulated): accepted
// photon-query pairs, photon tests (chunk photons x overlapping queries), chunks
// tested, boxes tested.  With nq_dev the query count is read on the device (bounded by
// num_queries, the capacity the grid is sized for) and a non-zero *skip makes the
// launch a no-op.  Needs the boxes (launch_kd_boxes) and the tree-order records.
void launch_gather(const VMParams& p, const KdTree& tree, TreePhotons tp, QueryBuf qb, const uint32_t* order,
                   long long num_queries, double* accum, unsigned long long* counters, cudaStream_t s, int variant,
                   const unsigned long long* nq_dev = nullptr, const int* skip = nullptr);
// Parity hook: the same kernel with a sink that records each query's photon ids
// (tree.id of the accepted positions).  Without offsets it adds each query's count into
// counts[] (zeroed by the caller); with offsets it writes the ids at offsets[q] +
// cursor[q]++ (cursor zeroed by the caller).  t0: tree-order positions
// (launch_tree_records); queries at qpos + qstride*i in the order `order`.  *err is set
// if a traversal stack would overflow (cannot happen for n < 2^28).
void launch_gather_sets(const KdTree& tree, const float4* t0, const float* qpos, int qstride, const uint32_t* order,
                        long long nq, float r2, int* counts, const long long* offsets, int* cursor, int* idx,
                        int variant, unsigned long long* counters, int* err, cudaStream_t s);
int gather_variants();
int gather_default_variant();
// Wavefront light pass: the same paths and photons as launch_light_pass, one bounce of
// every live path per round, split into a closest-hit kernel and a shading kernel with
// path state and queues in `scratch` (light_wavefront_scratch_bytes(num_light_paths)).
// `tail`, if given, is recorded on s before the last launch (the few paths left after the
// rounds, which leaves most SMs idle): work that waits on it fills them.
size_t light_wavefront_scratch_bytes(long long n);
void launch_light_wavefront(const VMParams& p, PhotonBuf ph, void* scratch, cudaStream_t s,
                            cudaEvent_t tail = nullptr);
// Launch shapes of the persistent light and camera passes (block size x traversal-stack
// placement), chosen by the autotuner; 0 is the default.  The light pass has one more:
// pass_variants() is the wavefront pass.
int pass_variants();
const char* pass_variant_name(int v);
const char* gather_variant_name(int v);

}  // namespace rc
