/*
 * realcaustics.h - C ABI of librealcaustics.so, the GB300 (sm_103a) vertex-merging
 * caustics renderer.
 *
 * Two groups of entry points:
 *
 *  1. The two exports of the reference "Real Caustics.dll" that the Blender add-on
 *     binds, with unchanged names, argument lists and struct layouts:
 *        init()   replaces Real Caustics/src/DLL.h:15-34 (defined at src/main.cpp:89-143)
 *        main()   replaces Real Caustics/src/DLL.h:14    (defined at src/main.cpp:148-223)
 *     Semantics follow the reference: init() copies scalars, triangles, camera and
 *     materials and BORROWS the light array and the Blender vertex arrays until main()
 *     returns; main() builds the BVH, renders `samples` progressive iterations, writes
 *     the FP32 RGB EXR (default file name "D:\caustics.exr" in the working directory,
 *     as src/main.cpp:206) and releases the scene.  Unlike the reference, main()
 *     returns a non-zero status instead of crashing on bad input (no scene, zero
 *     photons, unsupported light), and rc_last_error() describes it.
 *
 *  2. Additive rc_* exports: configuration beyond the reference's hard-coded values,
 *     in-memory image readback, timing, and the parity hooks (closest-hit on given
 *     rays, KD-tree radius query on given photons) that tests use to compare the
 *     GPU kernels with the reference algorithms.
 *
 * All functions are synchronous and return 0 on success or a negative RC_E* code.
 * A thread that binds no context shares the process's default context, which holds one
 * scene as the reference's global `scene` does; threads that bind their own contexts
 * (rc_context_*) hold one scene each and may call concurrently.  No torch types cross
 * this ABI.
 */
#ifndef REALCAUSTICS_H
#define REALCAUSTICS_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference by-value / by-pointer structs (x86-64 and aarch64 LP64 layouts) ---- */

/* vec3: 3 x f32 (Real Caustics/src/vec3.h:13-19), passed by value */
typedef struct rc_vec3 { float x, y, z; } rc_vec3;

/* Debug_stuff (src/Vertex_Merging.h:13-19), 24 bytes, passed by value */
typedef struct rc_debug_stuff { int number_of_points; rc_vec3 direction; float roughness; float specular; } rc_debug_stuff;

/* PythonMatrix4x4 (src/matrix.h:151-170): 16 f32, row-major t00..t33 */
typedef struct rc_matrix4x4 { float t[16]; } rc_matrix4x4;

/* Python_Light (src/Lights.h:15-36), 64 bytes. type: 'S' sun, 'P' point, else area.
 * rotation is in degrees for area lights, radians for sun lights. */
typedef struct rc_python_light {
    char type; float color[3]; rc_vec3 position; float width, height, spread;
    rc_vec3 rotation; float power, angle, radius;
} rc_python_light;

/* Python_Material (src/materials.h:21-32), 28 bytes. type: 'P' plastic, 'G' glass,
 * 'M' metal, anything else a white diffuse plastic.  Additive type 'R' (rough GGX
 * dielectric: ior, roughness) has no counterpart in the reference. */
typedef struct rc_python_material { char type; float ior, roughness, specular; float color[3]; } rc_python_material;

/* Reference export `init` (src/DLL.h:15-34).  meshes_pointers[i] is the address of a
 * Blender Mesh (DNA 2.9x: mpoly at byte 200, mloop at 208, mvert at 256). */
void init(int samples, float base_radius, float radius_reduction,
          long long* meshes_pointers, unsigned int number_of_meshes,
          rc_matrix4x4* mesh_matrices, unsigned int* meshes_number_of_verts,
          unsigned int* meshes_number_of_tris, unsigned int camera_x, unsigned int camera_y,
          rc_vec3 camera_position, rc_vec3 camera_corner0, rc_vec3 camera_corner1,
          rc_vec3 camera_corner2, rc_vec3 camera_corner3,
          rc_python_light* lights, unsigned int number_of_lights,
          rc_python_material* materials, unsigned int number_of_materials,
          int** materials_indices, int debug_test, rc_debug_stuff debug_stuff);

/* Reference export `main` (src/DLL.h:14): build, render, write EXR, release. */
int main(void);

/* ---- additive exports ---- */

enum {
    RC_OK = 0,
    RC_E_NO_SCENE = -1,      /* init() was not called, or main() already released it */
    RC_E_INVALID = -2,       /* bad argument (null pointer, zero size, bad index)    */
    RC_E_CUDA = -3,          /* CUDA runtime error (message in rc_last_error)        */
    RC_E_UNSUPPORTED = -4,   /* feature this library does not provide                */
    RC_E_CAPACITY = -5,      /* a fixed-size buffer or queue would overflow          */
    RC_E_TIMEOUT = -6,       /* a bounded device-side wait expired                   */
    RC_E_IO = -7             /* output file could not be written                     */
};

/* Photon-emission sampler. */
enum { RC_SAMPLER_UNIFORM = 0,   /* plain vertex merging: independent uniform light paths */
       RC_SAMPLER_HYBRID = 1,    /* reference scheme (src/Vertex_Merging.cpp:231-276):
                                    large step, small step on an invisible path, adaptive
                                    mutation size; run as many independent chains */
       RC_SAMPLER_PSSMLT = 2 };  /* visibility-target primary-sample MLT, large-step
                                    probability `large_step_prob`, many chains */

/* Rendering configuration beyond the reference's hard-coded values.  rc_default_config
 * fills the reference values (max_path_length 6, photons per iteration = pixels,
 * hybrid sampler, all reference quirks on). */
typedef struct rc_config {
    int max_path_length;        /* src/main.cpp:112 hard-codes 6                         */
    long long photons_per_iter; /* 0 = resX*resY as src/Vertex_Merging.cpp:201           */
    int sampler;                /* RC_SAMPLER_*                                          */
    int mlt_chains;             /* chains for HYBRID/PSSMLT (0 = 65536)                  */
    float large_step_prob;      /* PSSMLT only                                           */
    unsigned long long seed;    /* counter-based RNG seed                                */
    int write_exr;              /* main(): 1 = write EXR (reference behaviour)           */
    char exr_path[256];         /* main(): output file, default "D:\\caustics.exr"       */
    int verbose;                /* 1 = print per-iteration JSON lines to stdout          */
    /* learned emission proposal (area and point lights): an MLP maps the emission
     * position to a 16-lobe von Mises-Fisher mixture over directions, used in a
     * defensive mixture with the light's own density (fraction 0.2).  It is trained
     * online on the light paths whose photons the camera merged, during the first
     * `train_iterations` iterations (`train_steps` Adam steps of 16384 samples each,
     * learning rate `learning_rate`), and guides emission from the iteration after the
     * first training round.  With the HYBRID or PSSMLT sampler the training iterations
     * are plain (uniform-sampler) iterations; the chains of the later ones draw their
     * emission from the network evaluated on a 32 x 32 grid over each light (one extra
     * primary-sample dimension picks the mixture component).  No counterpart in the
     * reference. */
    int learned_proposal;
    int train_iterations;       /* default 8                                             */
    int train_steps;            /* default 64                                            */
    float learning_rate;        /* default 1e-3                                          */
    /* seed of the camera-path samples (pixel jitter, camera BSDF choices); 0 = `seed`.
     * Two renders with the same camera_seed and different seeds share their merge
     * queries and differ only in their photons. */
    unsigned long long camera_seed;
    /* 1 (default): the first iteration of each size class times the launch shapes of
     * the light pass, the camera pass (block size x register cap) and the gather
     * (resident blocks per SM x queries per warp) and keeps the fastest for the process;
     * 0: the fixed default shapes. */
    int autotune;
    /* 1 (default): with the uniform sampler and no learned proposal, when an iteration
     * takes under 20 ms of device time, the iterations after the first of a
     * configuration are enqueued without host round trips (fixed photon and query
     * capacities from the previous counts, KD tree over the padded photon capacity) and
     * replayed as an updated CUDA graph; an iteration whose counts outgrow the
     * capacities is rendered again at the end of the call.  0: every iteration reads its
     * counts back.  2: as 1 with capacities equal to the measured counts and no time
     * limit (tests: exercises the re-render of overflowed iterations). */
    int graph_replay;
    /* 1 (default): the per-mesh BVHs (Scene::update_bvh, src/Scene.cpp:110-152) are built
     * on the device by a binned SAH build whose node arrays, triangle order and traversal
     * costs are bit-identical to the host build; meshes with non-finite or -0.0 box
     * coordinates, or without triangles, fall back to the host build.  0: host build. */
    int gpu_bvh;
} rc_config;

int rc_default_config(rc_config* cfg);
int rc_set_config(const rc_config* cfg);

/* Stage the scene: BVH build + upload + light conversion (the pre-render half of main,
 * src/main.cpp:150-168).  Called implicitly by rc_render/main. */
int rc_prepare(void);

/* Host half of rc_prepare (no GPU needed): BVH build, lights, materials, radius.
 * info (optional, 9 floats): scene bbox min/max, scene radius, scaled base radius,
 * number of world BVH nodes - the values the reference computes at src/main.cpp:150-168. */
int rc_prepare_host(float* info);

/* The host-built BVH of one mesh / of the world in the reference's flattened layout
 * (CacheBVHNode_mesh / CacheBVHNode_world, src/BVH/BVH_mesh.h:51-71): 8 words per node
 * (min xyz, max xyz as float bits, the two union words) and the 1-based index list.
 * Returns the node count (copies at most cap nodes / index_cap indices). */
int rc_host_mesh_bvh(int mesh, unsigned* nodes, int cap, int* index, int index_cap, float* cost);
int rc_host_world_bvh(unsigned* nodes, int cap, int* index, int index_cap);

/* The scene arrays as the kernels read them (after rc_prepare), for comparing the
 * device and host BVH builds.  which: 0 = mesh BVH nodes (8 words per node: min xyz |
 * word0, max xyz | word1, global indices), 1 = triangles in leaf order (24 words: v0 |
 * triangle id, e1 | material, e2 | mesh, three normals), 2 = world BVH nodes (8 words),
 * 3 = world leaf mesh list followed by each mesh's root node index.  Copies at most
 * `cap` words; *words receives the full size.  No counterpart in the reference. */
int rc_scene_dump(int which, unsigned* out, long long cap, long long* words);

/* Contexts (no counterpart in the reference, whose state is one global `scene`).  Every
 * entry point acts on the context bound to the calling thread, or on the process's
 * default context when the thread has bound none - so a caller that never binds sees
 * the reference's single global scene, from any thread.  A thread that binds its own
 * context holds its own scene, configuration, last error and device buffers (and a CUDA
 * stream): scenes in different contexts render concurrently from different threads.
 * Autotuner choices are shared by all contexts.  rc_context_bind(NULL) returns the
 * thread to the default context.  rc_context_destroy releases the context's scene and
 * device memory; it must not be bound or in use on another thread. */
typedef struct rc_context rc_context;
rc_context* rc_context_create(void);
int rc_context_bind(rc_context* ctx);
int rc_context_destroy(rc_context* ctx);

/* Batch render (no counterpart in the reference, which renders one scene per call to
 * main(): src/Vertex_Merging.cpp:367-379 is its per-scene iteration loop).  Renders
 * `iterations` more progressive iterations of each of the n scenes held by ctxs[0..n-1]
 * (distinct contexts, each with a scene from init() and the uniform sampler without the
 * learned proposal) as one launch set per iteration: one persistent light pass over all
 * scenes' light paths, one persistent camera pass over all scenes' pixels, and each
 * scene's light-path order, KD build, query order and gather as parallel branches of the
 * same CUDA graph, which is captured, updated in place and replayed per iteration.  A
 * scene that has rendered no iteration yet renders its first one alone first (it fixes
 * the photon and query capacities of the graph); an iteration whose counts outgrow
 * them is rendered again alone at the end.  Each scene's image equals what rc_render on
 * its own context gives (the same samples; FP64 sums in another order).  Synchronous; the
 * contexts must not be in use on other threads meanwhile.  Errors are reported through
 * the calling thread's context.  out (NULL or 6 doubles): [0] device ms of the batch
 * iterations, [1] batch iterations, [2] kernel launches in them, [3] iterations rendered
 * again, [4] / [5] light / camera pass ms of the last batch iteration. */
int rc_batch_render(rc_context* const* ctxs, int n, int iterations, double* out);

/* Timing of the last rc_prepare: out[0] = mesh BVH build ms (host or device, uploads
 * included), out[1] = 1 if the device built the mesh BVHs, out[2] = world BVH + light
 * + material conversion + remaining uploads ms, out[3] = mesh BVH nodes, out[4] = device
 * level passes (segments above the per-warp size).  Returns the number written. */
int rc_prepare_stats(double* out, int n);

/* Render `iterations` more progressive iterations into the FP64 running mean. */
int rc_render(int iterations);

/* rc_render timed on the device: CUDA events on the library's stream around all
 * `iterations`.  out[0] = elapsed ms, out[1] = mean gather-kernel ms per iteration,
 * out[2] = gather algorithmic bytes per iteration (40 B per stored photon + 64 B per
 * merge query + 48 B FP64 RGB read/write per pixel), out[3] = kernel launches. */
int rc_render_timed(int iterations, double* out);

/* Copy the current image (mean over rendered iterations) as FP32 RGB, rows in the
 * reference's buffer order (the order SaveEXR receives, src/main.cpp:192-206). */
int rc_read_image(float* rgb, int width, int height);

/* Release the scene (what main() does at its end). */
int rc_release(void);

/* Last error message (static storage, valid until the next call). */
const char* rc_last_error(void);

/* Per-iteration statistics of the last rc_render call.
 * out[0] light paths, [1] stored photons, [2] merge queries, [3] photons merged,
 * [4] light-pass ms, [5] KD-build ms, [6] camera-pass ms, [7] gather ms,
 * [8] accumulate ms, [9] total device ms, [10] iterations rendered so far,
 * [11] scene radius, [12] current merge radius, [13] kernel launches,
 * [14] photon-query distance tests in the gather, [15] photon chunks (of at most 32)
 * tested by the gather's query groups, [16] closest-hit queries (rays) the light pass
 * traced (persistent launch shapes; 0 for the wavefront pass, the Metropolis samplers
 * and a batch render).
 * With the learned proposal, [8] is the proposal inference + training time.
 * With uniformly sampled light paths the camera pass runs on
 * a second stream beside the light pass and the KD build: its window [6] opens with the
 * light pass, and [9] counts the overlapped span once. */
int rc_get_stats(double* out, int n);

/* Checkpoint / resume of a progressive render (no counterpart in the reference, whose
 * BVH/KD file caches are commented out: src/KD_Tree.cpp:192-214, src/Scene.cpp:137-150).
 * rc_save_state writes the FP64 image sum, the iteration count, the sampling settings
 * (seeds, photons per iteration, depth, sampler) and the learned proposal's network and
 * Adam moments.  rc_load_state, after init() of the same scene, restores them; further
 * rc_render calls continue with the next iteration's counter-based samples, so the
 * result equals an uninterrupted render up to FP64 summation order.  A state saved for
 * another scene (fingerprint of geometry, camera, lights, materials, radius) is
 * RC_E_INVALID. */
int rc_save_state(const char* path);
int rc_load_state(const char* path);

/* Debug view of the reference's debug_test modes (src/Debug_scene.cpp, dispatched by
 * src/main.cpp:172-186): mode 2 shading normals, 3 front/back facing, 4 Fresnel
 * reflectance with the IOR of Debug_stuff::specular (one unjittered primary ray per
 * pixel; replaces the image, which rc_read_image returns); mode 5 the boxes of every
 * mesh BVH as OBJ files, one per mesh and depth, named "<dir>bvh<sep>Mesh_<k>_<depth>.obj"
 * after the EXR path's directory <dir> and separator <sep> ("D:\bvh\Mesh_..." by
 * default, as src/Debug_scene.cpp:284-320; the directory must exist), with no image
 * (host only: needs no GPU).  main() runs the same view when init() got debug_test 2-5. */
int rc_render_debug(int mode);

/* Learned-proposal state (no counterpart in the reference): for the first n light
 * paths of the last rendered iteration, prop4 = [direction xyz, p_light / q] as drawn
 * with those paths' samples from the network's current 32 x 32-cell table (the draw the
 * light pass makes; zeros before the network has been trained once), and contrib = the
 * sum over the path's merges of the squared luminance each adds to its pixel (recorded
 * during training iterations only).  Either output may be NULL. */
int rc_proposal_state(long long n, float* prop4, float* contrib);

/* ---- parity hooks (device kernels on caller-chosen inputs) ---- */

/* Closest hit of n rays (origins/directions: 3 floats each, host memory) through the
 * prepared scene, by the GPU traversal kernel (Scene::hit, src/Scene.cpp:154-189,
 * including its world-leaf overwrite).  out: 8 words per ray:
 * [hit(0/1), t, u, v (float bits), triangle id (global, ingest order), material,
 *  mesh index, reserved]. */
int rc_trace_rays(int n, const float* origins, const float* directions, float tmin, unsigned* out);

/* Same closest hit, with the full hit record as floats (16 per ray, same layout as the
 * oracle): [hit, t, u, v, Ng xyz, Ns xyz, position xyz, front_face, material, tri]. */
int rc_trace_rays_full(int n, const float* origins, const float* directions, float tmin, float* out);

/* rc_trace_rays_full through a chosen traversal: 0 the persistent passes' (one lane per
 * ray, both children's boxes tested at the parent), 1 the wavefront pass's (the same
 * tests, a warp's lanes stepping one node at a time together), 2 the reference's own
 * form (pop a node, test its box).  All visit the reference's nodes in its order and
 * return its hits.  RC_E_INVALID for any other shape. */
int rc_trace_rays_shape(int n, const float* origins, const float* directions, float tmin, float* out, int shape);

/* One light pass (iteration `iteration`, current config) on the GPU; copies the stored
 * photons (Path_Vertex records, src/Path_Vertices.h:10-20), in storage order, as 12
 * floats each: [position xyz, direction_world xyz, throughput rgb, dVM, light path index
 * (u32 bits), 0].  *count receives the number stored (may exceed cap). */
int rc_light_photons(int iteration, float* out, long long cap, long long* count);

/* One Metropolis light pass (the configured sampler, iteration `iteration`); the stored
 * photons as rc_light_photons writes them, large_steps (NULL or 2) = visible large
 * steps, large steps.  PSSMLT variant 0: the render's chains, advanced one path segment
 * per loop iteration; 1: the same chains one step at a time.  Both store the same
 * photons (in another order) and count the same steps; HYBRID ignores the variant.  No
 * counterpart in the reference (its sampler is src/Vertex_Merging.cpp:218-274). */
int rc_mlt_photons(int variant, int iteration, float* out, long long cap, long long* count,
                   unsigned long long* large_steps);

/* rc_light_photons with the light pass in launch shape `shape` (0 .. 5: the persistent
 * pass's block/register shapes, 6 = the wavefront pass), for comparing them; the
 * photons of every shape are the same, only their storage order differs. */
int rc_light_photons_shape(int shape, int iteration, float* out, long long cap, long long* count);

/* One camera pass (iteration `iteration`, current config) on the GPU; copies the merge
 * queries it writes (one per non-delta camera vertex, Vertex_Merging.cpp:309-362), in
 * storage order, as 4 floats each: [position xyz, camera dVM].  *count receives the
 * number written (may exceed cap). */
int rc_camera_queries(int iteration, float* out, long long cap, long long* count);

/* Build the photon KD-tree on the GPU over n photon positions (3 floats each) and
 * answer q radius queries (squared radius r2): counts[j] = number of photons with
 * ((dx*dx + dy*dy) + dz*dz) < r2 (KD_Tree::find_closest_in_radius, src/KD_Tree.cpp:217-280),
 * indices (photon ids, unordered within a query) packed in query order into idx
 * (capacity cap).  *total receives the total count (may exceed cap). */
int rc_kd_query(int n, const float* positions, int q, const float* queries, float r2,
                int* counts, int* idx, long long cap, long long* total);

/* The same radius query run by the render's own gather kernel (KD_Tree::find_closest_in_radius,
 * src/KD_Tree.cpp:217-280, as the gather of Path_Vertices::get_contrib, src/Path_Vertices.h:46-68,
 * calls it): the tree's chunk boxes, the KD-cell query order, `variant`'s launch shape
 * (0 .. rc_gather_variants()-1, -1 = the default; the autotuner picks among the same
 * shapes) and the pending-pair lists, with a sink that records photon ids where the
 * render evaluates merges.  rc_kd_query is this call with variant -1. */
int rc_gather_query(int variant, int n, const float* positions, int q, const float* queries, float r2,
                    int* counts, int* idx, long long cap, long long* total);
int rc_gather_variants(void);

/* PCI bus id ("domain:bus:device.function") of the CUDA device the calling thread
 * uses, for tools that address GPUs by bus id (nvidia-smi numbers GPUs physically and
 * ignores CUDA_VISIBLE_DEVICES).  len >= 13. */
int rc_device_bus_id(char* out, int len);

/* The GPU-built tree in the reference's node format (8-byte KDTreeNode, heap order,
 * root at 1, src/KD_Tree.h:13-32) for n photon positions; returns the node count in
 * *num_nodes and copies up to cap nodes as (index word, split bits) pairs. */
int rc_kd_build_nodes(int n, const float* positions, unsigned* nodes, long long cap, long long* num_nodes);

/* Tensor-core self-checks (no counterpart in the reference).  rc_tc_gemm_selftest:
 * D (128 x N, FP32) = A (128 x K, BF16 bits, row-major) * B (N x K, BF16 bits,
 * row-major)^T by the tcgen05 primitive the MLP kernels use (K, N multiples of 16,
 * K <= 128, N <= 256).  rc_tc_wait_selftest: a kernel that allocates TMEM and waits,
 * `tries` polls at most (1 to 65536), on an mbarrier that nothing completes; the
 * bounded wait must expire, free the TMEM and return RC_E_TIMEOUT, leaving the context
 * usable. */
int rc_tc_gemm_selftest(int K, int N, const unsigned short* A, const unsigned short* B, float* D);
int rc_tc_wait_selftest(unsigned tries);

/* KD-tree build that allocates no GPU memory, for callers that cannot allocate at
 * the point they need a photon tree (a host application that hands this library only
 * pre-allocated device buffers, or forbids foreign allocations in its context).  No
 * counterpart in the reference.  Same tree as rc_kd_build_nodes.  All pointers are
 * device memory owned by the caller: positions4 = n float4 (xyz used), nodes =
 * node_cap entries of 2 words (node_cap >= the node-array length of rc_kd_build_nodes
 * for n), x/y/z/ids = n entries each (photons in tree order).  Working memory is one
 * fixed array inside the library (held by every device that loads it), so n is
 * limited to 524288 photons (RC_E_CAPACITY beyond).  The first call on a device looks
 * up that array's address.  Calls share the array: calls that overlap on the GPU race.
 * Runs on `stream` (a cudaStream_t, NULL = legacy default stream) and synchronises it
 * before returning, so it must not be called while that stream is being captured;
 * on error the message is in rc_kd_noalloc_last_error(). */
int rc_kd_build_noalloc(const float* positions4, long long n, unsigned* nodes, long long node_cap,
                        float* x, float* y, float* z, unsigned* ids, void* stream);
const char* rc_kd_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* REALCAUSTICS_H */
