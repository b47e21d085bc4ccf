// C ABI of librealcaustics.so: the reference's init()/main() plus the additive rc_*
// entry points, over the host scene (host_scene.cpp) and the sm_103a kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "host_scene.h"
#include "mlp.cuh"
#include "proposal.cuh"
#include "realcaustics.h"
#include "vm.cuh"

namespace rc {

namespace {


#define RC_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            ctx().err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
            return RC_E_CUDA;                                                           \
        }                                                                               \
    } while (0)

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    // Grows with 1/16 headroom: per-iteration counts fluctuate, and each reallocation
    // (cudaFree synchronises the device) would stall an iteration.
    cudaError_t reserve(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr; n = 0;
        const size_t want = std::max<size_t>(count + count / 16, 1);
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

struct DeviceState {
    bool ready = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    // the camera pass's stream, beside the light pass and the KD build: fork and join
    // events (timing disabled)
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    // scene
    DevBuf<float4> nodes, wnode_lo, wnode_hi, tris, tri_n0, tri_n1, tri_n2;   // layouts: trace.cuh SceneView
    long long num_mesh_nodes = 0, num_tris = 0;
    DevBuf<int> world_mesh, mesh_root;
    DevBuf<DevLight> lights;
    DevBuf<float> cdf;
    DevBuf<DevMaterial> materials;
    SceneView view{};
    // iteration buffers
    DevBuf<float4> ph_pos, ph_dir;
    DevBuf<float2> ph_tp;
    DevBuf<uint32_t> ph_path;
    DevBuf<float4> q0, q1, q2, q3, q4;
    DevBuf<unsigned long long> counters;   // [0] photons, [1] queries
    DevBuf<int> errors;
    DevBuf<uint2> kd_nodes;
    DevBuf<float> kd_x, kd_y, kd_z;
    DevBuf<uint32_t> kd_id;
    DevBuf<unsigned char> kd_scratch;
    DevBuf<float4> tp0, tp1, box_lo, box_hi;
    DevBuf<float2> tp2;
    DevBuf<uint32_t> qorder;
    DevBuf<unsigned char> qscratch;
    DevBuf<double> accum;
    DevBuf<float> image;          // FP32 mean for readback
    // light-path processing order (launch_light_order) and its scratch
    DevBuf<uint32_t> path_order;
    DevBuf<unsigned char> order_scratch;
    DevBuf<unsigned char> wf_scratch;   // wavefront light pass: path state and queues
    // learned emission proposal
    std::unique_ptr<MlpStore> mlp;
    DevBuf<float4> prop, train_pos, train_dir;
    DevBuf<float> prop_table;   // tabulated proposal for the Metropolis samplers
    DevBuf<float> contrib, train_wsum;
    DevBuf<unsigned> train_count;
    cudaEvent_t evm[2] = {};
    cudaEvent_t evg[2] = {};    // around the gather kernel alone
    DevBuf<double> tune_accum;
    // asynchronous iterations (graph replay): fixed capacities, launch shapes and a
    // per-iteration overflow flag; the instantiated graph is updated in place
    long long async_pcap = 0, async_qcap = 0;
    int async_lvar = 0, async_cvar = 0, async_gvar = 1;
    DevBuf<int> async_flags;
    cudaGraphExec_t graph_exec = nullptr;
    unsigned long long last_photons = 0, last_queries = 0;
    int mlp_rounds = 0;          // training rounds done (the proposal is used after the first)
    double mlp_last_rows = 0;    // training samples collected in the last round
    int iterations_done = 0;
    double stats[17] = {};
    double last_nodes = 0;
    float stats_mlt_visible = 0.0f;
    // accumulated over a timed render call
    double acc_gather_ms = 0, acc_gather_bytes = 0, acc_launches = 0;
    int acc_iters = 0, acc_async = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;

    void release() {
        DevBuf<float4>* f4[] = {&nodes, &wnode_lo, &wnode_hi, &tris, &tri_n0,
                                &tri_n1, &tri_n2, &ph_pos, &ph_dir, &q0, &q1, &q2, &q3, &q4};
        for (auto* b : f4) b->release();
        world_mesh.release(); mesh_root.release(); lights.release(); cdf.release(); materials.release();
        ph_tp.release(); ph_path.release(); counters.release(); errors.release();
        kd_nodes.release(); kd_x.release(); kd_y.release(); kd_z.release(); kd_id.release(); kd_scratch.release();
        tp0.release(); tp1.release(); tp2.release(); qorder.release(); qscratch.release();
        box_lo.release(); box_hi.release();
        accum.release();
        image.release();
        path_order.release(); order_scratch.release(); wf_scratch.release();
        mlp.reset();
        prop.release(); train_pos.release(); train_dir.release(); contrib.release(); train_wsum.release();
        prop_table.release();
        train_count.release();
        mlp_rounds = 0;
        mlp_last_rows = 0;
        tune_accum.release();   // the chosen shapes stay: they are kept for the process
        async_flags.release();
        if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
        async_pcap = async_qcap = 0;
        for (auto& e : evm) if (e) { cudaEventDestroy(e); e = nullptr; }
        for (auto& e : evg) if (e) { cudaEventDestroy(e); e = nullptr; }
        for (auto& e : ev) if (e) { cudaEventDestroy(e); e = nullptr; }
        if (t0) { cudaEventDestroy(t0); t0 = nullptr; }
        if (t1) { cudaEventDestroy(t1); t1 = nullptr; }
        if (fork) { cudaEventDestroy(fork); fork = nullptr; }
        if (join) { cudaEventDestroy(join); join = nullptr; }
        if (side) { cudaStreamDestroy(side); side = nullptr; }
        if (stream) { cudaStreamDestroy(stream); stream = nullptr; }
        ready = false;
        iterations_done = 0;
    }
};

// Autotuner choices: launch variant per size class (log2 of light paths, pixels or
// queries), -1 = untuned.  Kept for the process and shared by every context (a new
// scene, or a scene in another context, reuses them).
struct TuneTables {
    std::atomic<int> light[64], camera[64], gather[64];
    TuneTables() {
        for (int i = 0; i < 64; ++i) { light[i] = -1; camera[i] = -1; gather[i] = -1; }
    }
};
TuneTables g_tune;

// Everything one scene needs: the reference's global `scene` plus the device state.
// Entry points act on the context bound to the calling thread (rc_context_bind), or on
// the process's default context when none is bound.
struct Context {
    std::string err;
    std::unique_ptr<HostScene> scene;
    rc_config cfg;
    bool cfg_set = false;
    DeviceState dev;
    bool host_ready = false;
    double prep[5] = {};                   // rc_prepare_stats
    std::unique_ptr<GpuBvhBuilder> bvh;    // device BVH scratch, kept for the context (grow-only)
};

Context& default_ctx() {
    static Context* c = new Context();   // never destroyed: no device frees at exit
    return *c;
}
thread_local Context* t_bound = nullptr;
Context& ctx() { return t_bound ? *t_bound : default_ctx(); }

void default_config(rc_config* c) {
    std::memset(c, 0, sizeof(*c));
    c->max_path_length = 6;
    c->photons_per_iter = 0;
    c->sampler = RC_SAMPLER_UNIFORM;
    c->mlt_chains = 65536;
    c->large_step_prob = 0.3f;
    c->seed = 0;
    c->write_exr = 1;
    std::snprintf(c->exr_path, sizeof(c->exr_path), "%s", "D:\\caustics.exr");
    c->verbose = 0;
    c->learned_proposal = 0;
    c->train_iterations = 8;
    c->train_steps = 64;
    c->learning_rate = 1e-3f;
    c->autotune = 1;
    c->graph_replay = 1;
    c->gpu_bvh = 1;
}

const rc_config& cfg() {
    if (!ctx().cfg_set) { default_config(&ctx().cfg); ctx().cfg_set = true; }
    return ctx().cfg;
}

template <class T>
int upload(DevBuf<T>& b, const std::vector<T>& v, cudaStream_t s) {
    RC_CUDA(b.reserve(v.size()));
    if (!v.empty()) RC_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return RC_OK;
}

inline float4 f4(float x, float y, float z, uint32_t w) {
    float wf;
    std::memcpy(&wf, &w, 4);
    return make_float4(x, y, z, wf);
}

// Stream, events and the process-lifetime autotuner tables.
int ensure_device() {
    DeviceState& d = ctx().dev;
    if (!d.stream) {
        RC_CUDA(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
        for (auto& e : d.ev) RC_CUDA(cudaEventCreate(&e));
        for (auto& e : d.evm) RC_CUDA(cudaEventCreate(&e));
        for (auto& e : d.evg) RC_CUDA(cudaEventCreate(&e));
        RC_CUDA(cudaEventCreate(&d.t0));
        RC_CUDA(cudaEventCreate(&d.t1));
        RC_CUDA(cudaStreamCreateWithFlags(&d.side, cudaStreamNonBlocking));
        RC_CUDA(cudaEventCreateWithFlags(&d.fork, cudaEventDisableTiming));
        RC_CUDA(cudaEventCreateWithFlags(&d.join, cudaEventDisableTiming));
    }
    return RC_OK;
}

// Mesh BVH nodes and triangle records from the host build, packed and uploaded.
int upload_meshes_host(HostScene& sc, std::vector<int>& mesh_root) {
    DeviceState& d = ctx().dev;
    std::vector<float4> nod, trs, n0, n1, n2;
    mesh_root.clear();
    uint32_t node_base = 0, tri_base = 0, tri_global = 0;
    for (size_t m = 0; m < sc.meshes.size(); ++m) {
        HostMesh& hm = sc.meshes[m];
        mesh_root.push_back((int)node_base);
        for (const BvhNode& nd : hm.bvh.nodes) {
            uint32_t w0 = nd.w0, w1 = nd.w1;
            if (w0 & 0x80000000u) w1 = tri_base + w1;
            else { w0 += node_base; w1 += node_base; }
            nod.push_back(f4(nd.box.mn.x, nd.box.mn.y, nd.box.mn.z, w0));
            nod.push_back(f4(nd.box.mx.x, nd.box.mx.y, nd.box.mx.z, w1));
        }
        for (size_t k = 1; k < hm.bvh.index.size(); ++k) {
            uint32_t t = (uint32_t)hm.bvh.index[k];
            const V3& a = hm.wpos[hm.tri[3 * t]];
            const V3& b = hm.wpos[hm.tri[3 * t + 1]];
            const V3& c = hm.wpos[hm.tri[3 * t + 2]];
            trs.push_back(f4(a.x, a.y, a.z, tri_global + t));
            trs.push_back(f4(b.x - a.x, b.y - a.y, b.z - a.z, hm.mat[t]));
            trs.push_back(f4(c.x - a.x, c.y - a.y, c.z - a.z, (uint32_t)m));
            const V3& na = hm.wnrm[hm.tri[3 * t]];
            const V3& nb = hm.wnrm[hm.tri[3 * t + 1]];
            const V3& nc = hm.wnrm[hm.tri[3 * t + 2]];
            n0.push_back(make_float4(na.x, na.y, na.z, 0.0f));
            n1.push_back(make_float4(nb.x, nb.y, nb.z, 0.0f));
            n2.push_back(make_float4(nc.x, nc.y, nc.z, 0.0f));
        }
        node_base += (uint32_t)hm.bvh.nodes.size();
        tri_base += (uint32_t)(hm.bvh.index.size() - 1);
        tri_global += hm.num_tris;
    }
    cudaStream_t s = d.stream;
    int r;
    if ((r = upload(d.nodes, nod, s)) || (r = upload(d.tris, trs, s)) || (r = upload(d.tri_n0, n0, s)) ||
        (r = upload(d.tri_n1, n1, s)) || (r = upload(d.tri_n2, n2, s)))
        return r;
    d.num_mesh_nodes = (long long)nod.size() / 2;
    d.num_tris = (long long)n0.size();
    return RC_OK;
}

// World BVH, mesh roots, lights and materials; the scene view the kernels read.
int upload_scene_rest(HostScene& sc, const std::vector<int>& mesh_root) {
    DeviceState& d = ctx().dev;
    std::vector<float4> wlo, whi;
    for (const BvhNode& nd : sc.world.nodes) {
        wlo.push_back(f4(nd.box.mn.x, nd.box.mn.y, nd.box.mn.z, nd.w0));
        whi.push_back(f4(nd.box.mx.x, nd.box.mx.y, nd.box.mx.z, nd.w1));
    }
    std::vector<int> wm(sc.world.index.begin() + 1, sc.world.index.end());
    cudaStream_t s = d.stream;
    int r;
    if ((r = upload(d.wnode_lo, wlo, s)) || (r = upload(d.wnode_hi, whi, s)) ||
        (r = upload(d.world_mesh, wm, s)) || (r = upload(d.mesh_root, mesh_root, s)) ||
        (r = upload(d.lights, sc.lights, s)) || (r = upload(d.cdf, sc.light_cdf, s)) ||
        (r = upload(d.materials, sc.materials, s)))
        return r;
    RC_CUDA(d.counters.reserve(10));   // [8] closest-hit queries of the persistent light pass
    RC_CUDA(d.errors.reserve(ERR_COUNT));
    RC_CUDA(cudaMemsetAsync(d.errors.p, 0, sizeof(int) * ERR_COUNT, s));
    RC_CUDA(cudaStreamSynchronize(s));
    SceneView& v = d.view;
    v.nodes = d.nodes.p;
    v.wnode_lo = d.wnode_lo.p; v.wnode_hi = d.wnode_hi.p;
    v.world_mesh = d.world_mesh.p; v.mesh_root = d.mesh_root.p;
    v.tris = d.tris.p;
    v.tri_n0 = d.tri_n0.p; v.tri_n1 = d.tri_n1.p; v.tri_n2 = d.tri_n2.p;
    v.num_world_nodes = (int)sc.world.nodes.size();
    v.num_meshes = (int)sc.meshes.size();
    d.ready = true;
    return RC_OK;
}


// The host steps of main() after the mesh BVHs (src/main.cpp:150-168).
int finish_host(HostScene& sc) {
    build_world_bvh(sc);
    // init_lights + update_pdf_distribution (src/main.cpp:160-163)
    int r = convert_lights(sc, ctx().err);
    if (r) return r;
    convert_materials(sc);
    // base_radius *= SceneRadius (src/main.cpp:166-168)
    sc.base_radius *= sc.scene_radius;
    ctx().host_ready = true;
    return RC_OK;
}

// Host half of the pre-render steps of main() (src/main.cpp:150-168).
int prepare_host() {
    if (!ctx().scene) { ctx().err = "no scene: init() was not called"; return RC_E_NO_SCENE; }
    HostScene& sc = *ctx().scene;
    if (ctx().host_ready) return RC_OK;
    if (sc.meshes.empty()) { ctx().err = "scene has no meshes"; return RC_E_INVALID; }
    // Scene::update_bvh (src/Scene.cpp:110-152)
    for (HostMesh& m : sc.meshes) build_mesh_bvh(m);
    return finish_host(sc);
}

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Mesh BVHs built on the device (bvh_build.cu) straight into the scene arrays.  Leaves
// sc.prepared false when the input needs the host build.
int prepare_device_bvh(HostScene& sc) {
    DeviceState& d = ctx().dev;
    if (sc.meshes.empty()) return RC_OK;
    const auto t0 = std::chrono::steady_clock::now();
    int r = ensure_device();
    if (r) return r;
    std::vector<GpuMeshSrc> src;
    for (const HostMesh& hm : sc.meshes)
        src.push_back({hm.wpos.data(), hm.wnrm.data(), hm.tri.data(), hm.mat.data(), hm.num_verts, hm.num_tris});
    // scratch kept for the context (grow-only): a batch of scenes loaded one after the
    // other into one context allocates it once
    if (!ctx().bvh) ctx().bvh = std::make_unique<GpuBvhBuilder>();
    GpuBvhBuilder& bld = *ctx().bvh;
    bool supported = false;
    std::string err;
    r = bld.build(src, d.stream, supported, err);
    if (r) { ctx().err = err; return r; }
    if (!supported) return RC_OK;
    RC_CUDA(d.nodes.reserve(2 * bld.num_nodes()));
    RC_CUDA(d.tris.reserve(3 * bld.num_tris()));
    DevBuf<float4>* tb[] = {&d.tri_n0, &d.tri_n1, &d.tri_n2};
    for (auto* b : tb) RC_CUDA(b->reserve(bld.num_tris()));
    r = bld.emit(d.nodes.p, d.tris.p, d.tri_n0.p, d.tri_n1.p, d.tri_n2.p,
                 d.stream, err);
    if (r) { ctx().err = err; return r; }
    d.num_mesh_nodes = bld.num_nodes();
    d.num_tris = bld.num_tris();
    for (size_t m = 0; m < sc.meshes.size(); ++m) {
        MeshBvh& b = sc.meshes[m].bvh;
        const float* f = &bld.mesh_box[6 * m];
        b.bounds.mn = {f[0], f[1], f[2]};
        b.bounds.mx = {f[3], f[4], f[5]};
        b.cost = bld.mesh_cost[m];
        b.nodes.clear();   // the host copy is built on demand (rc_host_mesh_bvh)
        b.index.clear();
    }
    const std::vector<int> roots = bld.mesh_root;
    const int levels = bld.levels;
    ctx().prep[0] = ms_since(t0);
    ctx().prep[1] = 1.0;
    ctx().prep[3] = (double)d.num_mesh_nodes;
    ctx().prep[4] = levels;
    const auto t1 = std::chrono::steady_clock::now();
    r = finish_host(sc);
    if (r) return r;
    r = upload_scene_rest(sc, roots);
    if (r) return r;
    ctx().prep[2] = ms_since(t1);
    sc.prepared = true;
    return RC_OK;
}

int prepare() {
    if (!ctx().scene) { ctx().err = "no scene: init() was not called"; return RC_E_NO_SCENE; }
    HostScene& sc = *ctx().scene;
    if (sc.prepared) return RC_OK;
    if (cfg().gpu_bvh && !ctx().host_ready) {
        int r = prepare_device_bvh(sc);
        if (r) return r;
        if (sc.prepared) return RC_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const bool built_here = !ctx().host_ready;
    int r = prepare_host();
    if (r) return r;
    r = ensure_device();
    if (r) return r;
    std::vector<int> roots;
    r = upload_meshes_host(sc, roots);
    if (r) return r;
    ctx().prep[0] = built_here ? ms_since(t0) : 0.0;
    ctx().prep[1] = 0.0;
    ctx().prep[3] = (double)ctx().dev.num_mesh_nodes;
    ctx().prep[4] = 0.0;
    const auto t1 = std::chrono::steady_clock::now();
    r = upload_scene_rest(sc, roots);
    if (r) return r;
    ctx().prep[2] = ms_since(t1);
    sc.prepared = true;
    return RC_OK;
}

// Frame of the merge queries' Morton order: the scene's bounding box (every camera
// vertex lies on a scene surface).
QueryFrame scene_query_frame(const HostScene& sc) {
    const float lo[3] = {sc.bounds.mn.x, sc.bounds.mn.y, sc.bounds.mn.z};
    const float hi[3] = {sc.bounds.mx.x, sc.bounds.mx.y, sc.bounds.mx.z};
    return query_frame(lo, hi);
}

int check_errors() {
    int h[ERR_COUNT];
    RC_CUDA(cudaMemcpy(h, ctx().dev.errors.p, sizeof(h), cudaMemcpyDeviceToHost));
    if (h[ERR_STACK]) { ctx().err = "BVH traversal stack overflow (depth > 64)"; return RC_E_CAPACITY; }
    if (h[ERR_MATERIAL]) { ctx().err = "triangle material index out of range"; return RC_E_INVALID; }
    if (h[ERR_KD]) { ctx().err = "KD-tree build found inconsistent counts"; return RC_E_INVALID; }
    if (h[ERR_MLP]) { ctx().err = "tensor-core pipeline wait timed out in the MLP"; return RC_E_CUDA; }
    if (h[ERR_GATHER]) { ctx().err = "gather traversal stack overflow"; return RC_E_CAPACITY; }
    return RC_OK;
}

VMParams make_params(const HostScene& sc, int iteration) {
    VMParams p{};
    p.scene = ctx().dev.view;
    p.lights = LightsView{ctx().dev.lights.p, ctx().dev.cdf.p, (int)sc.lights.size(), sc.light_integral};
    p.materials = ctx().dev.materials.p;
    p.num_materials = (int)sc.materials.size();
    const HostCamera& c = sc.camera;
    p.camera.width = c.width; p.camera.height = c.height;
    float* dst[4] = {p.camera.origin, p.camera.bottom_left, p.camera.horizontal, p.camera.vertical};
    const V3* src[4] = {&c.origin, &c.bottom_left, &c.horizontal, &c.vertical};
    for (int k = 0; k < 4; ++k) { dst[k][0] = src[k]->x; dst[k][1] = src[k]->y; dst[k][2] = src[k]->z; }
    p.seed = cfg().seed;
    p.camera_seed = cfg().camera_seed ? cfg().camera_seed : cfg().seed;
    p.iteration = (uint32_t)iteration;
    long long npix = (long long)c.width * c.height;
    p.num_light_paths = cfg().photons_per_iter > 0 ? cfg().photons_per_iter : npix;
    p.max_path_length = cfg().max_path_length;
    // src/Vertex_Merging.cpp:201-212
    const float PI = 3.14159265359f;
    float light_paths_count = (float)p.num_light_paths;
    float radius = sc.base_radius;
    radius /= std::pow(float(iteration + 1), 0.5f * (1.0f - sc.radius_alpha));
    radius = std::max(radius, 1e-7f);
    float radius_sqr = radius * radius;
    p.radius_sqr = radius_sqr;
    p.vm_norm = 1.0f / (PI * radius_sqr * light_paths_count);
    p.merge_scale = 1.0f;
    p.error = ctx().dev.errors.p;
    return p;
}

float ms_between(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();   // a timing that is not available is reported as 0
        ms = 0.0f;
    }
    return ms;
}

// Event record usable for timing both in eager and in recorded (graph) iterations:
// during stream capture it becomes an external event node, which records the event
// like an ordinary record each time the graph runs.
cudaError_t record(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cs);
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal)
                                               : cudaEventRecord(e, s);
}

// Device time from the light pass's start to the later of the KD build's end and the
// camera pass's end, for an iteration whose camera pass ran on the side stream (its
// events ev[4], ev[5] overlap the light pass and the KD build).
double overlapped_ms(const DeviceState& d) {
    return std::max(ms_between(d.ev[0], d.ev[3]), ms_between(d.ev[0], d.ev[5]));
}

ProposalCtx proposal_ctx(const HostScene& sc, const VMParams& p) {
    ProposalCtx c{};
    c.lights = p.lights;
    const float mn[3] = {sc.bounds.mn.x, sc.bounds.mn.y, sc.bounds.mn.z};
    const float mx[3] = {sc.bounds.mx.x, sc.bounds.mx.y, sc.bounds.mx.z};
    for (int k = 0; k < 3; ++k) {
        const float ext = mx[k] - mn[k];
        c.bmin[k] = mn[k];
        c.binv[k] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    c.seed = p.seed;
    c.iteration = p.iteration;
    return c;
}

constexpr int kTrainBatchRows = 16384;
constexpr int kTrainCapacity = 1 << 20;

// Before the light pass: make sure the network exists and, once it has been trained,
// write every light path's proposed emission direction and weight.
int proposal_before(const HostScene& sc, VMParams& p, bool train) {
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    const long long n = p.num_light_paths;
    if (!d.mlp) {
        d.mlp = std::make_unique<MlpStore>();
        if (!d.mlp->setup(kTrainBatchRows)) { ctx().err = "MLP allocation failed"; return RC_E_CUDA; }
        if (mlp_init(d.mlp->p, cfg().seed ^ 0x9E3779B97F4A7C15ull, s)) { ctx().err = "MLP init failed"; return RC_E_CUDA; }
        RC_CUDA(d.train_pos.reserve(kTrainCapacity)); RC_CUDA(d.train_dir.reserve(kTrainCapacity));
        RC_CUDA(d.train_count.reserve(1)); RC_CUDA(d.train_wsum.reserve(1));
    }
    if (d.mlp_rounds > 0) {
        // the network on every light's 32 x 32 area cells (tensor cores); the light pass
        // draws each path's emission from that table
        RC_CUDA(d.prop_table.reserve((size_t)sc.lights.size() * kProposalRes * kProposalRes * kProposalCellFloats));
        if (mlp_proposal_table(d.mlp->p, proposal_ctx(sc, p), kProposalRes, d.prop_table.p, s, d.errors.p + ERR_MLP)) {
            ctx().err = "proposal table launch failed"; return RC_E_CUDA;
        }
        // (the draw itself follows the light-path order, render_iteration)
        p.proposal_table = d.prop_table.p;
        p.proposal_table_res = kProposalRes;
        RC_CUDA(d.prop.reserve(std::max<long long>(n, 1)));
    }
    if (train) {
        RC_CUDA(d.contrib.reserve(std::max<long long>(n, 1)));
        RC_CUDA(cudaMemsetAsync(d.contrib.p, 0, sizeof(float) * std::max<long long>(n, 1), s));
        p.path_contrib = d.contrib.p;
        p.photon_path = d.ph_path.p;
    }
    return RC_OK;
}

// After the gather: collect (position, direction, weight) of the paths that reached the
// image and take Adam steps on them.
int proposal_train(const HostScene& sc, const VMParams& p) {
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    unsigned rows = 0;
    mlp_collect(proposal_ctx(sc, p), p.num_light_paths, d.contrib.p, p.proposal, kTrainCapacity, d.train_pos.p,
                d.train_dir.p, d.train_count.p, d.train_wsum.p, s);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaMemcpyAsync(&rows, d.train_count.p, sizeof(rows), cudaMemcpyDeviceToHost, s));
    RC_CUDA(cudaStreamSynchronize(s));
    const int total = (int)std::min<unsigned>(rows, (unsigned)kTrainCapacity);
    d.mlp_last_rows = total;
    if (total < 256) return RC_OK;   // too few merged paths to learn from in this pass
    mlp_normalize_weights(d.train_dir.p, total, d.train_wsum.p, s);
    if (mlp_train(d.mlp->p, d.mlp->b, d.train_pos.p, d.train_dir.p, total, cfg().train_steps, cfg().learning_rate, s,
                  d.errors.p + ERR_MLP)) {
        ctx().err = "MLP training launch failed"; return RC_E_CUDA;
    }
    RC_CUDA(cudaGetLastError());
    d.mlp_rounds++;
    return RC_OK;
}

// Autotuner: time each launch variant of a pass (warm-up launch, then one timed launch;
// `run(v)` must reset whatever the pass appends to) and return the fastest.
template <class Run>
int autotune_variants(int nvariants, Run&& run, const char* what, long long size) {
    DeviceState& d = ctx().dev;
    float best = 1e30f;
    int best_v = 0;
    for (int v = 0; v < nvariants; ++v) {
        run(v);
        cudaEventRecord(d.evm[0], d.stream);
        run(v);
        cudaEventRecord(d.evm[1], d.stream);
        cudaEventSynchronize(d.evm[1]);
        const float ms = ms_between(d.evm[0], d.evm[1]);
        if (cfg().verbose) std::printf("{\"autotune_shape\": \"%s\", \"variant\": %d, \"ms\": %.3f}\n", what, v, ms);
        if (ms < best) { best = ms; best_v = v; }
    }
    if (cfg().verbose)
        std::printf("{\"autotune\": \"%s\", \"size\": %lld, \"variant\": %d, \"ms\": %.3f}\n", what, size, best_v,
                    best);
    return best_v;
}

int size_class(long long n) { return n > 0 ? 63 - __builtin_clzll((unsigned long long)n) : 0; }

// The light pass in launch shape v: the persistent pass's shapes, or (v ==
// pass_variants()) the wavefront pass with its path state in the context's scratch.
// `tail`, if given, is recorded where work forked from it can fill the slots the pass
// stops using: before the wavefront pass's last launch, before a persistent pass.
int light_pass(const VMParams& p, PhotonBuf ph, cudaStream_t s, int v, cudaEvent_t tail = nullptr) {
    DeviceState& d = ctx().dev;
    if (v == pass_variants()) {
        RC_CUDA(d.wf_scratch.reserve(light_wavefront_scratch_bytes(p.num_light_paths)));
        RC_CUDA(cudaMemsetAsync(d.counters.p + 8, 0, sizeof(unsigned long long), s));   // (not counted)
        launch_light_wavefront(p, ph, d.wf_scratch.p, s, tail);
        return RC_OK;
    }
    // (the persistent pass holds every block slot until its pool drains: work forked
    // before it takes the slots its tail frees; measured 20.62 -> 20.53 ms per water-pool
    // iteration against forking after it)
    if (tail) RC_CUDA(cudaEventRecord(tail, s));
    launch_light_pass(p, ph, d.counters.p + 6, s, v, d.counters.p + 8);
    return RC_OK;
}

// Debug view 5 (Vertex_Merging::run_debug_bvh, src/Debug_scene.cpp:284-320): for every
// mesh of every world leaf, in world-node order, one OBJ file per depth of the mesh's
// BVH, "<dir>bvh<sep>Mesh_<k>_<depth>.obj" (k counts the meshes written, from 1; <dir>
// and <sep> from the EXR path, the reference's "D:\bvh\" by default), holding the boxes
// of that depth's nodes: 8 vertices and 6 quads each, numbered per file
// (write_bvh / write_bounding_box, src/Debug_scene.cpp:217-262), numbers printed as an
// ostream prints a float (%g).  The reference also walks inner world nodes as if they
// were leaves (their child words read as a mesh range, past the end of the mesh list
// when the world BVH has inner nodes); only leaves are walked here.
int debug_bvh_obj(HostScene& sc) {
    const std::string exr = cfg().exr_path;
    const size_t cut = exr.find_last_of("/\\");
    const std::string dir = cut == std::string::npos ? std::string() : exr.substr(0, cut + 1);
    const char sep = cut == std::string::npos ? '\\' : exr[cut];
    const std::string prefix = dir + "bvh" + sep + "Mesh_";
    const std::vector<BvhNode>& wn = sc.world.nodes;
    int written = 0;
    for (size_t w = 0; w < wn.size(); ++w) {
        if (!(wn[w].w0 & 0x80000000u)) continue;
        const uint32_t cnt = wn[w].w0 & 0x7fffffffu;
        for (uint32_t k = 0; k < cnt; ++k) {
            const int mesh = sc.world.index[wn[w].w1 + 1 + k];
            HostMesh& hm = sc.meshes[mesh];
            if (hm.bvh.nodes.empty()) build_mesh_bvh(hm);   // the device built this scene's meshes
            const std::vector<BvhNode>& nodes = hm.bvh.nodes;
            // depth of every node (root 1), children after their parent in the array
            std::vector<int> depth(nodes.size(), 0);
            int max_depth = 0;
            std::vector<std::pair<int, int>> stack{{0, 1}};
            std::vector<int> order;   // pre-order: the reference's write_bvh recursion
            while (!stack.empty()) {
                const auto [i, dpt] = stack.back();
                stack.pop_back();
                depth[i] = dpt;
                order.push_back(i);
                if (nodes[i].w0 & 0x80000000u) { max_depth = std::max(max_depth, dpt); continue; }
                stack.push_back({(int)nodes[i].w1, dpt + 1});
                stack.push_back({(int)nodes[i].w0, dpt + 1});
            }
            ++written;
            std::vector<FILE*> files((size_t)max_depth, nullptr);
            for (int dpt = 1; dpt <= max_depth; ++dpt) {
                const std::string name = prefix + std::to_string(written) + "_" + std::to_string(dpt) + ".obj";
                files[dpt - 1] = std::fopen(name.c_str(), "w");
                if (!files[dpt - 1]) {
                    for (FILE* f : files) if (f) std::fclose(f);
                    ctx().err = "cannot write " + name;
                    return RC_E_IO;
                }
            }
            std::vector<int> base((size_t)max_depth, 0);
            for (int i : order) {
                FILE* f = files[depth[i] - 1];
                const Box& b = nodes[i].box;
                const float cx[2] = {b.mx.x, b.mn.x}, cy[2] = {b.mx.y, b.mn.y}, cz[2] = {b.mx.z, b.mn.z};
                for (int v = 0; v < 8; ++v)
                    std::fprintf(f, "v %g %g %g\n", (double)cx[v >> 2], (double)cy[(v >> 1) & 1], (double)cz[v & 1]);
                static const int quad[6][4] = {{1, 5, 7, 3}, {4, 3, 7, 8}, {8, 7, 5, 6}, {6, 2, 4, 8}, {2, 1, 3, 4}, {6, 5, 1, 2}};
                const int o = base[depth[i] - 1];
                for (const auto& q : quad)
                    std::fprintf(f, "f %d/ %d/ %d/ %d/\n", q[0] + o, q[1] + o, q[2] + o, q[3] + o);
                base[depth[i] - 1] += 8;
            }
            for (FILE* f : files) std::fclose(f);
        }
    }
    return RC_OK;
}

// One progressive iteration with host round trips (counts read back, buffers grown on
// overflow).  redo_iteration >= 0 renders that iteration index again without counting
// it (an iteration an asynchronous replay had to skip).
int render_iteration(HostScene& sc, int redo_iteration = -1) {
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    int r0 = RC_OK;
    const int it = redo_iteration >= 0 ? redo_iteration : d.iterations_done;
    VMParams p = make_params(sc, it);
    // With a Metropolis sampler and the learned proposal, the first train_iterations
    // iterations are plain ones that train the network; the chains of the later ones
    // draw their emission from the network's table (proposal.cuh).
    const bool train_phase = cfg().learned_proposal && it < cfg().train_iterations;
    const int sampler = (cfg().sampler != RC_SAMPLER_UNIFORM && train_phase) ? RC_SAMPLER_UNIFORM : cfg().sampler;
    const bool learned = cfg().learned_proposal && sampler == RC_SAMPLER_UNIFORM;
    const bool train = learned && it < cfg().train_iterations;
    const bool tabulated = cfg().learned_proposal && sampler != RC_SAMPLER_UNIFORM && d.mlp && d.mlp_rounds > 0;
    float t_mlp = 0.0f;
    const long long npix = (long long)sc.camera.width * sc.camera.height;
    if (d.accum.n < (size_t)(3 * npix)) {
        RC_CUDA(d.accum.reserve(3 * npix));
        RC_CUDA(cudaMemsetAsync(d.accum.p, 0, sizeof(double) * 3 * npix, s));
    }
    // photon buffer: grow and re-trace the iteration if it overflowed (the RNG is
    // counter based, so the re-trace produces the same photons)
    long long cap = (long long)d.ph_pos.n;
    if (cap < p.num_light_paths * 2) cap = p.num_light_paths * 2;
    unsigned long long nph = 0, rays = 0;
    unsigned long long mlt[2] = {0, 0};
    float t_light = 0.0f;
    if (tabulated) {
        RC_CUDA(cudaEventRecord(d.evm[0], s));
        RC_CUDA(d.prop_table.reserve((size_t)sc.lights.size() * kProposalRes * kProposalRes * kProposalCellFloats));
        if (mlp_proposal_table(d.mlp->p, proposal_ctx(sc, p), kProposalRes, d.prop_table.p, s, d.errors.p + ERR_MLP)) {
            ctx().err = "proposal table launch failed";
            return RC_E_CUDA;
        }
        RC_CUDA(cudaEventRecord(d.evm[1], s));
        p.proposal_table = d.prop_table.p;
        p.proposal_table_res = kProposalRes;
    }
    // The camera pass reads nothing that the light pass writes (the Metropolis samplers'
    // visibility factor, known only after the light pass, is applied by the gather).
    // Once its launch shape is tuned it then runs on the side stream: with uniformly
    // sampled light paths issued right before the light pass, so that its blocks take
    // the SMs that the light pass's tail frees and run through the host's read-back of
    // the photon count and the KD build's launches; with a Metropolis sampler issued
    // before the chains, whose one thread per chain leaves room on every SM.  It joins
    // the main stream before the query order.  (With the learned proposal the network's
    // inference ends before the fork and its training starts after the join: no
    // tensor-core kernel runs beside it.)
    long long qcap = std::max<long long>((long long)d.q0.n, npix * 2);
    unsigned long long nq = 0;
    float t_cam = 0.0f;
    // (Metropolis samplers: only when the chains are long enough for the camera pass to
    // hide beside them - 512 steps per chain on the 4K gem cluster: 50 ms of camera pass
    // hidden; 8 per chain at 960x540: 4.75 ms per iteration serial against 5.28 beside)
    const bool mlt_long = (long long)cfg().mlt_chains * 64 <= p.num_light_paths;
    const bool cam_side = (sampler == RC_SAMPLER_UNIFORM || mlt_long) &&
                          (!cfg().autotune || g_tune.camera[size_class(npix)].load() >= 0);
    const int cam_var = cfg().autotune ? std::max(g_tune.camera[size_class(npix)].load(), 0) : 0;
    if (cam_side) {
        RC_CUDA(d.q0.reserve(qcap)); RC_CUDA(d.q1.reserve(qcap)); RC_CUDA(d.q2.reserve(qcap));
        RC_CUDA(d.q3.reserve(qcap)); RC_CUDA(d.q4.reserve(qcap));
    }
    for (int attempt = 0; attempt < 3; ++attempt) {
        RC_CUDA(d.ph_pos.reserve(cap)); RC_CUDA(d.ph_dir.reserve(cap));
        RC_CUDA(d.ph_tp.reserve(cap)); RC_CUDA(d.ph_path.reserve(cap));
        RC_CUDA(cudaMemsetAsync(d.counters.p, 0, sizeof(unsigned long long), s));
        PhotonBuf ph{d.ph_pos.p, d.ph_dir.p, d.ph_tp.p, d.ph_path.p, cap, d.counters.p};
        if (learned) {
            RC_CUDA(cudaEventRecord(d.evm[0], s));
            int r = proposal_before(sc, p, train);
            if (r) return r;
            RC_CUDA(cudaEventRecord(d.evm[1], s));
        }
        RC_CUDA(cudaEventRecord(d.ev[0], s));
        if (sampler == RC_SAMPLER_UNIFORM && attempt == 0) {
            // coherent processing order of the light paths (their samples unchanged)
            RC_CUDA(d.path_order.reserve(std::max<long long>(p.num_light_paths, 1)));
            RC_CUDA(d.order_scratch.reserve(light_order_scratch_bytes(p.num_light_paths)));
            launch_light_order(p, d.order_scratch.p, d.path_order.p, s);
            p.path_order = d.path_order.p;
        }
        if (learned && p.proposal_table) {
            // every path's emission drawn from the network's table, in the light-path
            // order (neighbouring threads read the same cells); the light pass and the
            // training collection read the draws
            if (mlp_proposal_draw(proposal_ctx(sc, p), kProposalRes, p.proposal_table, p.num_light_paths, p.path_order,
                                  d.prop.p, s)) {
                ctx().err = "proposal draw launch failed"; return RC_E_CUDA;
            }
            p.proposal = d.prop.p;
            p.proposal_table = nullptr;
        }
        int lvar = 0;
        if (sampler == RC_SAMPLER_UNIFORM && cfg().autotune) {
            std::atomic<int>& slot = g_tune.light[size_class(p.num_light_paths)];
            if (slot.load() < 0)
                slot = autotune_variants(pass_variants() + 1, [&](int v) {
                    cudaMemsetAsync(d.counters.p, 0, sizeof(unsigned long long), s);
                    light_pass(p, ph, s, v);
                }, "light pass", p.num_light_paths);
            lvar = slot.load();
            RC_CUDA(cudaMemsetAsync(d.counters.p, 0, sizeof(unsigned long long), s));
        }
        // the camera pass forks where the light pass stops filling the GPU
        const bool fork = cam_side && attempt == 0;
        if (sampler == RC_SAMPLER_UNIFORM) {
            r0 = light_pass(p, ph, s, lvar, fork ? d.fork : nullptr);
            if (r0) return r0;
        }
        else {
            if (fork) RC_CUDA(cudaEventRecord(d.fork, s));
            RC_CUDA(cudaMemsetAsync(d.counters.p + 8, 0, sizeof(unsigned long long), s));   // (not counted)
            launch_mlt_pass(p, ph, sampler, cfg().mlt_chains, cfg().large_step_prob, d.counters.p + 2, s);
        }
        RC_CUDA(cudaGetLastError());
        RC_CUDA(cudaEventRecord(d.ev[1], s));
        if (fork) {
            // (its count is read at the join: a read into pageable memory would wait here)
            RC_CUDA(cudaStreamWaitEvent(d.side, d.fork, 0));
            RC_CUDA(cudaMemsetAsync(d.counters.p + 1, 0, sizeof(unsigned long long), d.side));
            QueryBuf qb{d.q0.p, d.q1.p, d.q2.p, d.q3.p, d.q4.p, qcap, d.counters.p + 1};
            RC_CUDA(cudaEventRecord(d.ev[4], d.side));
            launch_camera_pass(p, qb, d.counters.p + 7, d.side, cam_var);
            RC_CUDA(cudaGetLastError());
            RC_CUDA(cudaEventRecord(d.ev[5], d.side));
            RC_CUDA(cudaEventRecord(d.join, d.side));
        }
        RC_CUDA(cudaMemcpyAsync(&nph, d.counters.p, sizeof(nph), cudaMemcpyDeviceToHost, s));
        RC_CUDA(cudaMemcpyAsync(&rays, d.counters.p + 8, sizeof(rays), cudaMemcpyDeviceToHost, s));
        if (sampler != RC_SAMPLER_UNIFORM)
            RC_CUDA(cudaMemcpyAsync(mlt, d.counters.p + 2, sizeof(mlt), cudaMemcpyDeviceToHost, s));
        RC_CUDA(cudaStreamSynchronize(s));
        t_light = ms_between(d.ev[0], d.ev[1]);
        if (learned || tabulated) t_mlp = ms_between(d.evm[0], d.evm[1]);
        if ((long long)nph <= cap) break;
        cap = (long long)nph + nph / 8 + 1024;
        if (attempt == 2) { ctx().err = "photon buffer overflow"; return RC_E_CAPACITY; }
    }
    if (nph >= (1ull << 28)) {
        // the KD node word holds a photon index in 28 bits (src/KD_Tree.h:13-32)
        ctx().err = "more than 2^28 photons stored in one iteration";
        return RC_E_CAPACITY;
    }
    int r = check_errors();
    if (r) return r;
    if (sampler != RC_SAMPLER_UNIFORM) {
        // visibility normalisation of the Metropolis samplers (src/Vertex_Merging.cpp:277-282)
        const float vis = mlt[1] ? (float)mlt[0] / (float)mlt[1] : 0.0f;
        p.merge_scale = vis;
        d.stats_mlt_visible = vis;
    }
    // KD tree over the stored photons
    long long n = (long long)nph;
    long long nn = kd_node_array_len(n);
    RC_CUDA(d.kd_nodes.reserve(std::max<long long>(nn, 2)));
    RC_CUDA(d.kd_x.reserve(std::max<long long>(n, 1))); RC_CUDA(d.kd_y.reserve(std::max<long long>(n, 1)));
    RC_CUDA(d.kd_z.reserve(std::max<long long>(n, 1))); RC_CUDA(d.kd_id.reserve(std::max<long long>(n, 1)));
    size_t sb = kd_scratch_bytes(n);
    RC_CUDA(d.kd_scratch.reserve(sb));
    KdTree tree;
    tree.nodes = d.kd_nodes.p; tree.x = d.kd_x.p; tree.y = d.kd_y.p; tree.z = d.kd_z.p; tree.id = d.kd_id.p;
    int kd_launches = 0;
    RC_CUDA(cudaEventRecord(d.ev[2], s));
    if (kd_build(d.ph_pos.p, n, tree, d.kd_scratch.p, d.kd_scratch.n, s, &kd_launches, d.errors.p + ERR_KD)) {
        ctx().err = "KD scratch too small"; return RC_E_CAPACITY;
    }
    RC_CUDA(cudaGetLastError());
    RC_CUDA(d.tp0.reserve(std::max<long long>(n, 1))); RC_CUDA(d.tp1.reserve(std::max<long long>(n, 1)));
    RC_CUDA(d.tp2.reserve(std::max<long long>(n, 1)));
    TreePhotons tph{d.tp0.p, d.tp1.p, d.tp2.p};
    tree.box_levels = kd_box_levels(n);
    if (tree.box_levels > 0) {
        RC_CUDA(d.box_lo.reserve((size_t)1 << tree.box_levels));
        RC_CUDA(d.box_hi.reserve((size_t)1 << tree.box_levels));
        tree.box_lo = d.box_lo.p; tree.box_hi = d.box_hi.p;
        launch_kd_boxes(tree, s, &kd_launches);
        RC_CUDA(cudaGetLastError());
    }
    {
        PhotonBuf phb{d.ph_pos.p, d.ph_dir.p, d.ph_tp.p, d.ph_path.p, (long long)d.ph_pos.n, d.counters.p};
        launch_tree_records(phb, tree, tph, s);
        RC_CUDA(cudaGetLastError());
    }
    RC_CUDA(cudaEventRecord(d.ev[3], s));
    // camera pass -> merge queries (joined from the side stream, or run here: untuned
    // launch shape, a Metropolis sampler, or a query overflow)
    bool cam_done = false;
    if (cam_side) {
        RC_CUDA(cudaMemcpyAsync(&nq, d.counters.p + 1, sizeof(nq), cudaMemcpyDeviceToHost, d.side));
        RC_CUDA(cudaStreamSynchronize(d.side));
        RC_CUDA(cudaStreamWaitEvent(s, d.join, 0));
        t_cam = ms_between(d.ev[4], d.ev[5]);
        cam_done = (long long)nq <= qcap;
        if (!cam_done) qcap = (long long)nq + nq / 8 + 1024;
    }
    // a side-stream camera pass of an earlier iteration that returned an error may
    // still be writing the query buffers (a wait before the event's first record is void)
    if (!cam_side) RC_CUDA(cudaStreamWaitEvent(s, d.join, 0));
    for (int attempt = 0; attempt < 3 && !cam_done; ++attempt) {
        RC_CUDA(d.q0.reserve(qcap)); RC_CUDA(d.q1.reserve(qcap)); RC_CUDA(d.q2.reserve(qcap));
        RC_CUDA(d.q3.reserve(qcap)); RC_CUDA(d.q4.reserve(qcap));
        RC_CUDA(cudaMemsetAsync(d.counters.p + 1, 0, sizeof(unsigned long long), s));
        QueryBuf qb{d.q0.p, d.q1.p, d.q2.p, d.q3.p, d.q4.p, qcap, d.counters.p + 1};
        int cvar = 0;
        if (cfg().autotune) {
            std::atomic<int>& slot = g_tune.camera[size_class(npix)];
            if (slot.load() < 0)
                slot = autotune_variants(pass_variants(), [&](int v) {
                    cudaMemsetAsync(d.counters.p + 1, 0, sizeof(unsigned long long), s);
                    launch_camera_pass(p, qb, d.counters.p + 7, s, v);
                }, "camera pass", npix);
            cvar = slot.load();
            RC_CUDA(cudaMemsetAsync(d.counters.p + 1, 0, sizeof(unsigned long long), s));
        }
        RC_CUDA(cudaEventRecord(d.ev[4], s));
        launch_camera_pass(p, qb, d.counters.p + 7, s, cvar);
        RC_CUDA(cudaGetLastError());
        RC_CUDA(cudaEventRecord(d.ev[5], s));
        RC_CUDA(cudaMemcpyAsync(&nq, d.counters.p + 1, sizeof(nq), cudaMemcpyDeviceToHost, s));
        RC_CUDA(cudaStreamSynchronize(s));
        t_cam = ms_between(d.ev[4], d.ev[5]);
        if ((long long)nq <= qcap) break;
        qcap = (long long)nq + nq / 8 + 1024;
        if (attempt == 2) { ctx().err = "query buffer overflow"; return RC_E_CAPACITY; }
    }
    r = check_errors();
    if (r) return r;
    QueryBuf qb{d.q0.p, d.q1.p, d.q2.p, d.q3.p, d.q4.p, (long long)d.q0.n, d.counters.p + 1};
    RC_CUDA(d.qorder.reserve(std::max<unsigned long long>(nq, 1)));
    RC_CUDA(d.qscratch.reserve(query_order_scratch_bytes((long long)nq)));
    RC_CUDA(cudaEventRecord(d.ev[6], s));
    int qlaunch = 0;
    launch_query_order(reinterpret_cast<const float*>(d.q0.p), 4, (long long)nq, scene_query_frame(sc), d.qscratch.p,
                       d.qorder.p, &qlaunch, s);
    int variant = gather_default_variant();
    if (cfg().autotune && nq > 0) {
        const int cls = 63 - __builtin_clzll((unsigned long long)nq);
        if (g_tune.gather[cls].load() < 0) {
            // time every launch shape on this iteration's queries into a scratch image
            // (warm-up launch first: the first launch of a shape loads its code)
            RC_CUDA(d.tune_accum.reserve(std::max<long long>(3 * npix, 1)));
            float best = 1e30f;
            int best_v = variant;
            for (int v = 0; v < gather_variants(); ++v) {
                launch_gather(p, tree, tph, qb, d.qorder.p, (long long)nq, d.tune_accum.p, nullptr, s, v);
                RC_CUDA(cudaEventRecord(d.evm[0], s));
                launch_gather(p, tree, tph, qb, d.qorder.p, (long long)nq, d.tune_accum.p, nullptr, s, v);
                RC_CUDA(cudaEventRecord(d.evm[1], s));
                RC_CUDA(cudaEventSynchronize(d.evm[1]));
                const float ms = ms_between(d.evm[0], d.evm[1]);
                if (cfg().verbose) std::printf("{\"gather_shape\": %d, \"ms\": %.4f}\n", v, ms);
                if (ms < best) { best = ms; best_v = v; }
            }
            g_tune.gather[cls] = best_v;
            if (cfg().verbose)
                std::printf("{\"autotune\": \"gather\", \"queries\": %llu, \"variant\": \"%s\", \"ms\": %.3f}\n",
                            nq, gather_variant_name(best_v), best);
        }
        variant = g_tune.gather[cls].load();
    }
    unsigned long long gc[4] = {0, 0, 0, 0};
    RC_CUDA(cudaMemsetAsync(d.counters.p + 2, 0, 4 * sizeof(unsigned long long), s));
    RC_CUDA(cudaEventRecord(d.evg[0], s));
    launch_gather(p, tree, tph, qb, d.qorder.p, (long long)nq, d.accum.p, d.counters.p + 2, s, variant);
    RC_CUDA(cudaEventRecord(d.evg[1], s));
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaEventRecord(d.ev[7], s));
    RC_CUDA(cudaMemcpyAsync(gc, d.counters.p + 2, sizeof(gc), cudaMemcpyDeviceToHost, s));
    RC_CUDA(cudaStreamSynchronize(s));
    r = check_errors();
    if (r) return r;
    if (train) {
        RC_CUDA(cudaEventRecord(d.evm[0], s));
        r = proposal_train(sc, p);
        if (r) return r;
        RC_CUDA(cudaEventRecord(d.evm[1], s));
        RC_CUDA(cudaEventSynchronize(d.evm[1]));
        t_mlp += ms_between(d.evm[0], d.evm[1]);
        r = check_errors();
        if (r) return r;
    }
    if (redo_iteration < 0) d.iterations_done++;
    d.last_photons = nph;
    d.last_queries = nq;
    double* st = d.stats;
    st[0] = (double)p.num_light_paths;
    st[1] = (double)nph;
    st[2] = (double)nq;
    st[3] = (double)gc[0];   // accepted photon-query pairs
    st[14] = (double)gc[1];  // photon tests
    st[15] = (double)gc[2];  // photon chunks tested (per group)
    st[16] = (double)rays;   // closest-hit queries of the light pass (persistent shapes)
    d.last_nodes = (double)gc[3];
    st[4] = t_light;
    st[5] = ms_between(d.ev[2], d.ev[3]);
    st[6] = t_cam;
    st[7] = ms_between(d.ev[6], d.ev[7]);
    st[8] = t_mlp;           // proposal inference + training
    st[9] = (cam_side ? overlapped_ms(d) : st[4] + st[5] + st[6]) + st[7] + st[8];
    st[10] = d.iterations_done;
    st[11] = sc.scene_radius;
    st[12] = std::sqrt(p.radius_sqr);
    st[13] = kd_launches + 3 + qlaunch;
    d.acc_gather_ms += ms_between(d.evg[0], d.evg[1]);   // the gather kernel alone
    // gather algorithmic bytes: each photon record read once (40 B), each query record
    // read once (64 B), each pixel's FP64 RGB sum read and written once (48 B)
    d.acc_gather_bytes += 40.0 * (double)nph + 64.0 * (double)nq + 48.0 * (double)npix;
    d.acc_launches += st[13];
    d.acc_iters += 1;
    if (cfg().verbose)
        std::printf("{\"iteration\": %d, \"light_paths\": %lld, \"photons\": %llu, \"queries\": %llu, "
                    "\"merged\": %llu, \"tests\": %llu, \"chunks\": %llu, \"boxes\": %llu, "
                    "\"light_ms\": %.3f, \"kd_ms\": %.3f, \"camera_ms\": %.3f, \"gather_ms\": %.3f}\n",
                    it, p.num_light_paths, nph, nq, gc[0], gc[1], gc[2], gc[3], st[4], st[5], st[6], st[7]);
    return RC_OK;
}

// ---------------------------------------------------------------- asynchronous iterations
// After one iteration with host round trips has fixed the sizes, further iterations of
// the uniform sampler are enqueued without any: photon and query capacities are fixed
// (the KD tree is built over the whole photon capacity, unused slots padded far away,
// which leaves every radius query's answer unchanged), the query order and the gather
// read the query count on the device, and a per-iteration flag records a count that
// overflowed its capacity (that iteration's gather is skipped and the iteration is
// rendered again with host round trips at the end).  Each iteration is captured as a
// CUDA graph; the instantiated graph is updated in place with the next iteration's
// parameters and replayed.
constexpr double kReplayMaxIterationMs = 20.0;

bool async_eligible() {
    return cfg().graph_replay && cfg().sampler == RC_SAMPLER_UNIFORM && !cfg().learned_proposal;
}

int async_setup(const HostScene& sc) {
    DeviceState& d = ctx().dev;
    const long long npix = (long long)sc.camera.width * sc.camera.height;
    // capacities: the last measured counts with a 2% + 4096 margin, 1024-aligned (the
    // counts of a configuration vary by ~0.1% between iterations)
    // (graph_replay 2, for tests: the counts themselves, so that iterations that store
    // more photons or queries than the measured one overflow and are rendered again)
    const bool tight = cfg().graph_replay == 2;
    auto capacity = [tight](unsigned long long c) {
        return tight ? (long long)c : (long long)(((c + c / 50 + 4096) + 1023) / 1024 * 1024);
    };
    d.async_pcap = std::min<long long>(capacity(d.last_photons), (1ll << 28) - 1);   // 28-bit photon index
    d.async_qcap = capacity(d.last_queries);
    RC_CUDA(d.ph_pos.reserve(d.async_pcap)); RC_CUDA(d.ph_dir.reserve(d.async_pcap));
    RC_CUDA(d.ph_tp.reserve(d.async_pcap)); RC_CUDA(d.ph_path.reserve(d.async_pcap));
    {
        const long long paths = cfg().photons_per_iter > 0 ? cfg().photons_per_iter : npix;
        RC_CUDA(d.path_order.reserve(std::max<long long>(paths, 1)));
        RC_CUDA(d.order_scratch.reserve(light_order_scratch_bytes(paths)));
    }
    RC_CUDA(d.q0.reserve(d.async_qcap)); RC_CUDA(d.q1.reserve(d.async_qcap)); RC_CUDA(d.q2.reserve(d.async_qcap));
    RC_CUDA(d.q3.reserve(d.async_qcap)); RC_CUDA(d.q4.reserve(d.async_qcap));
    const long long n = d.async_pcap;
    RC_CUDA(d.kd_nodes.reserve(std::max<long long>(kd_node_array_len(n), 2)));
    RC_CUDA(d.kd_x.reserve(n)); RC_CUDA(d.kd_y.reserve(n)); RC_CUDA(d.kd_z.reserve(n)); RC_CUDA(d.kd_id.reserve(n));
    RC_CUDA(d.kd_scratch.reserve(kd_scratch_bytes(n)));
    RC_CUDA(d.tp0.reserve(n)); RC_CUDA(d.tp1.reserve(n)); RC_CUDA(d.tp2.reserve(n));
    const int bl = kd_box_levels(n);
    if (bl > 0) { RC_CUDA(d.box_lo.reserve((size_t)1 << bl)); RC_CUDA(d.box_hi.reserve((size_t)1 << bl)); }
    RC_CUDA(d.qorder.reserve(d.async_qcap));
    RC_CUDA(d.qscratch.reserve(query_order_scratch_bytes(d.async_qcap)));
    RC_CUDA(d.accum.reserve(3 * npix));
    auto var = [](int v, int dflt) { return v >= 0 ? v : dflt; };
    d.async_lvar = var(g_tune.light[size_class(cfg().photons_per_iter > 0 ? cfg().photons_per_iter : npix)].load(), 0);
    d.async_cvar = var(g_tune.camera[size_class(npix)].load(), 0);
    d.async_gvar = var(g_tune.gather[size_class((long long)d.last_queries)].load(), gather_default_variant());
    if (!cfg().autotune) d.async_lvar = d.async_cvar = 0, d.async_gvar = gather_default_variant();
    if (d.async_lvar == pass_variants()) {   // the wavefront pass's state: reserved before any capture
        const long long paths = cfg().photons_per_iter > 0 ? cfg().photons_per_iter : npix;
        RC_CUDA(d.wf_scratch.reserve(light_wavefront_scratch_bytes(paths)));
    }
    return RC_OK;
}

// The two ends of an asynchronous iteration (no host synchronisation), shared by the
// single-scene replay and the batch (batch_render).  async_head, on s: the iteration's
// photon and query counters reset, the light-path order.
int async_head(VMParams& p, cudaStream_t s) {
    DeviceState& d = ctx().dev;
    RC_CUDA(cudaMemsetAsync(d.counters.p, 0, sizeof(unsigned long long) * 2, s));
    RC_CUDA(record(d.ev[0], s));
    launch_light_order(p, d.order_scratch.p, d.path_order.p, s);
    p.path_order = d.path_order.p;
    return RC_OK;
}

// async_tail, on s after the light pass: the photon capacity padded, the KD tree and its
// boxes, the tree-order records; then, once the camera pass has recorded `camera_done`,
// the count check (`flag` = 1 on an overflow), the query order and the gather.
int async_tail(HostScene& sc, const VMParams& p, cudaStream_t s, cudaEvent_t camera_done, int* flag) {
    DeviceState& d = ctx().dev;
    const long long pc = d.async_pcap, qc = d.async_qcap;
    QueryBuf qb{d.q0.p, d.q1.p, d.q2.p, d.q3.p, d.q4.p, qc, d.counters.p + 1};
    // pads one scene extent (plus four base radii) beyond the scene's +x face: outside
    // every merge radius, and close enough that the KD build's largest-extent rule
    // separates them from the stored photons along x within a few levels
    const float ext = std::max(std::max(sc.bounds.mx.x - sc.bounds.mn.x, sc.bounds.mx.y - sc.bounds.mn.y),
                               sc.bounds.mx.z - sc.bounds.mn.z);
    const float4 pad = make_float4(sc.bounds.mx.x + ext + 4.0f * sc.base_radius + 1.0f,
                                   0.5f * (sc.bounds.mn.y + sc.bounds.mx.y), 0.5f * (sc.bounds.mn.z + sc.bounds.mx.z),
                                   0.0f);
    launch_pad_photons(d.ph_pos.p, d.counters.p, pc, pad, s);
    KdTree tree{};
    tree.nodes = d.kd_nodes.p; tree.x = d.kd_x.p; tree.y = d.kd_y.p; tree.z = d.kd_z.p; tree.id = d.kd_id.p;
    RC_CUDA(record(d.ev[2], s));
    int kl = 0;
    if (kd_build(d.ph_pos.p, pc, tree, d.kd_scratch.p, d.kd_scratch.n, s, &kl, d.errors.p + ERR_KD)) {
        ctx().err = "KD scratch too small"; return RC_E_CAPACITY;
    }
    TreePhotons tph{d.tp0.p, d.tp1.p, d.tp2.p};
    tree.box_levels = kd_box_levels(pc);
    if (tree.box_levels > 0) {
        tree.box_lo = d.box_lo.p; tree.box_hi = d.box_hi.p;
        launch_kd_boxes(tree, s, nullptr);
    }
    launch_tree_records(PhotonBuf{d.ph_pos.p, d.ph_dir.p, d.ph_tp.p, d.ph_path.p, pc, d.counters.p}, tree, tph, s);
    RC_CUDA(record(d.ev[3], s));
    RC_CUDA(cudaStreamWaitEvent(s, camera_done, 0));
    launch_check_counts(d.counters.p, pc, d.counters.p + 1, qc, flag, s);
    RC_CUDA(record(d.ev[6], s));
    launch_query_order(reinterpret_cast<const float*>(d.q0.p), 4, qc, scene_query_frame(sc), d.qscratch.p, d.qorder.p,
                       nullptr, s, d.counters.p + 1);
    RC_CUDA(cudaMemsetAsync(d.counters.p + 2, 0, 4 * sizeof(unsigned long long), s));
    RC_CUDA(record(d.evg[0], s));
    launch_gather(p, tree, tph, qb, d.qorder.p, qc, d.accum.p, d.counters.p + 2, s, d.async_gvar, d.counters.p + 1,
                  flag);
    RC_CUDA(record(d.evg[1], s));
    RC_CUDA(record(d.ev[7], s));
    return RC_OK;
}

// Enqueue iteration `it` (no host synchronisation); `flag` receives the overflow flag.
int enqueue_async_iteration(HostScene& sc, int it, int* flag) {
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    VMParams p = make_params(sc, it);
    const long long pc = d.async_pcap, qc = d.async_qcap;
    PhotonBuf ph{d.ph_pos.p, d.ph_dir.p, d.ph_tp.p, d.ph_path.p, pc, d.counters.p};
    QueryBuf qb{d.q0.p, d.q1.p, d.q2.p, d.q3.p, d.q4.p, qc, d.counters.p + 1};
    int r = async_head(p, s);
    if (r) return r;
    // the camera pass on a branch of its own beside the light pass's tail and the KD
    // build (it reads nothing they write), joined before the count check
    r = light_pass(p, ph, s, d.async_lvar, d.fork);   // the camera branch forks where
    if (r) return r;                                   // the light pass stops filling the GPU
    RC_CUDA(record(d.ev[1], s));
    RC_CUDA(cudaStreamWaitEvent(d.side, d.fork, 0));
    RC_CUDA(record(d.ev[4], d.side));
    launch_camera_pass(p, qb, d.counters.p + 7, d.side, d.async_cvar);
    RC_CUDA(record(d.ev[5], d.side));
    RC_CUDA(cudaEventRecord(d.join, d.side));
    return async_tail(sc, p, s, d.join, flag);
}

// Capture iteration `it` as a graph, update the instantiated graph with it (or
// instantiate it) and launch it.
int launch_async_iteration(HostScene& sc, int it, int* flag) {
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    int r = enqueue_async_iteration(sc, it, flag);
    const cudaError_t le = cudaGetLastError();   // launch errors recorded during capture
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (r) { if (graph) cudaGraphDestroy(graph); return r; }
    if (le != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        ctx().err = std::string("kernel launch while recording an iteration: ") + cudaGetErrorString(le);
        return RC_E_CUDA;
    }
    if (e != cudaSuccess) { ctx().err = std::string("graph capture: ") + cudaGetErrorString(e); return RC_E_CUDA; }
    if (d.graph_exec) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(d.graph_exec, graph, &info) != cudaSuccess) {
            cudaGetLastError();
            cudaGraphExecDestroy(d.graph_exec);
            d.graph_exec = nullptr;
        }
    }
    if (!d.graph_exec) {
        e = cudaGraphInstantiate(&d.graph_exec, graph, 0);
        if (e != cudaSuccess) { cudaGraphDestroy(graph); ctx().err = std::string("graph instantiate: ") + cudaGetErrorString(e); return RC_E_CUDA; }
    }
    cudaGraphDestroy(graph);
    RC_CUDA(cudaGraphLaunch(d.graph_exec, s));
    RC_CUDA(cudaGetLastError());
    return RC_OK;
}

// After n_async asynchronous iterations from first_it were enqueued: their overflow
// flags read back (synchronising the context's stream), the statistics of the last one,
// every flagged iteration rendered again with host round trips, and the capacities sized
// again if any overflowed.  `windows`: the light and camera passes' event windows
// belong to this scene (not in a batch, whose passes cover every scene at once).
int async_finish(HostScene& sc, int first_it, int n_async, bool windows) {
    DeviceState& d = ctx().dev;
    int r = RC_OK;
    std::vector<int> flags(n_async, 0);
    RC_CUDA(cudaMemcpyAsync(flags.data(), d.async_flags.p, sizeof(int) * n_async, cudaMemcpyDeviceToHost, d.stream));
    RC_CUDA(cudaStreamSynchronize(d.stream));
    r = check_errors();
    if (r) return r;
    // stats of the last replayed iteration
    unsigned long long cnt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    RC_CUDA(cudaMemcpy(cnt, d.counters.p, sizeof(cnt), cudaMemcpyDeviceToHost));
    VMParams p = make_params(sc, d.iterations_done - 1);
    double* st = d.stats;
    st[0] = (double)p.num_light_paths;
    st[1] = (double)cnt[0];
    st[2] = (double)cnt[1];
    st[3] = (double)cnt[2];
    st[14] = (double)cnt[3];
    st[15] = (double)cnt[4];
    st[16] = windows ? (double)cnt[8] : 0.0;
    st[4] = windows ? ms_between(d.ev[0], d.ev[1]) : 0.0;
    st[5] = ms_between(d.ev[2], d.ev[3]);
    st[6] = windows ? ms_between(d.ev[4], d.ev[5]) : 0.0;
    st[7] = ms_between(d.ev[6], d.ev[7]);
    st[8] = 0.0;
    st[9] = windows ? overlapped_ms(d) + st[7] : ms_between(d.ev[2], d.ev[7]);
    st[10] = d.iterations_done;
    st[11] = sc.scene_radius;
    st[12] = std::sqrt(p.radius_sqr);
    const double gms = ms_between(d.evg[0], d.evg[1]);
    d.acc_gather_ms += gms * n_async;    // the last replay's gather time stands for each
    d.acc_gather_bytes += (40.0 * (double)cnt[0] + 64.0 * (double)cnt[1] +
                           48.0 * (double)sc.camera.width * sc.camera.height) * n_async;
    d.acc_iters += n_async;
    d.acc_async += n_async;
    d.acc_launches += (d.stats[13] + 2.0) * n_async;   // an eager iteration's kernels + pad + check
    bool regrow = false;
    for (int k = 0; k < n_async; ++k) {
        if (!flags[k]) continue;
        regrow = true;
        r = render_iteration(sc, first_it + k);   // the skipped iteration, with round trips
        if (r) return r;
    }
    if (regrow) {
        // counts outgrew the capacities: size them again from the last measured counts
        if (d.graph_exec) { cudaGraphExecDestroy(d.graph_exec); d.graph_exec = nullptr; }
        r = async_setup(sc);
        if (r) return r;
    }
    if (cfg().verbose)
        std::printf("{\"replayed_iterations\": %d, \"redone\": %d, \"photon_capacity\": %lld, \"query_capacity\": %lld}\n",
                    n_async, (int)std::count(flags.begin(), flags.end(), 1), d.async_pcap, d.async_qcap);
    return RC_OK;
}


// `iterations` progressive iterations: the first with host round trips, the rest
// replayed asynchronously when eligible; overflowed iterations are rendered again.
int render_iterations(HostScene& sc, int iterations) {
    DeviceState& d = ctx().dev;
    int r = RC_OK;
    int i = 0;
    if (!async_eligible()) {
        for (; i < iterations && !r; ++i) r = render_iteration(sc);
        return r;
    }
    if (d.async_pcap == 0 && i < iterations) {
        r = render_iteration(sc);
        ++i;
        if (r) return r;
        // Replay pays where host round trips and launch gaps are a visible share of an
        // iteration; for long iterations the KD tree over the padded capacity costs more
        // than it saves (measured: 64-scene batch +6%, 37 ms water-pool iterations -2%).
        if (d.stats[9] > kReplayMaxIterationMs && cfg().graph_replay != 2) d.async_pcap = -1;
        else {
            r = async_setup(sc);
            if (r) return r;
        }
    }
    if (d.async_pcap < 0) {
        for (; i < iterations && !r; ++i) r = render_iteration(sc);
        return r;
    }
    const int n_async = iterations - i;
    if (n_async <= 0) return RC_OK;
    // the replayed iterations' camera branch writes the query buffers that an eager
    // iteration's side-stream camera pass may still be writing (after an error return)
    RC_CUDA(cudaStreamSynchronize(d.side));
    RC_CUDA(d.async_flags.reserve(n_async));
    const int first_it = d.iterations_done;
    for (int k = 0; k < n_async; ++k) {
        r = launch_async_iteration(sc, first_it + k, d.async_flags.p + k);
        if (r) return r;
        d.iterations_done++;
    }
    return async_finish(sc, first_it, n_async, true);
}

// ---------------------------------------------------------------- batch of scenes
// Several resident scenes (one context each) rendered as one launch set per iteration:
// one persistent light pass over every scene's light paths and one persistent camera
// pass over every scene's pixels (scene index found per work item), and per scene its
// light-path order, KD build, query order and gather on a branch of its own; the whole
// iteration is captured as one CUDA graph, updated in place and replayed per iteration.
// Capacities are each scene's asynchronous ones (async_setup: fixed from a first
// iteration with host round trips), so the graph holds no host round trip, whatever
// an iteration's length; overflowed iterations are rendered again afterwards.

// Launch shapes of the batch passes, tuned on the first batch (-1: untuned).
std::atomic<int> g_batch_light{-1}, g_batch_camera{-1};

struct BatchRun {
    cudaStream_t main = nullptr, side = nullptr;
    std::vector<cudaStream_t> branch;
    cudaEvent_t start = nullptr, light = nullptr, camera = nullptr, join = nullptr, t0 = nullptr, t1 = nullptr;
    cudaEvent_t cam_fork = nullptr;
    cudaEvent_t light_start = nullptr, light_end = nullptr, camera_start = nullptr, camera_end = nullptr;
    DevBuf<BatchScene> scenes;          // per graph iteration: its scenes' entries, end to end
    DevBuf<long long> prefix;           // per graph iteration: path prefix (m + 1), pixel prefix (m + 1)
    DevBuf<unsigned long long> next;    // [0] next light path, [1] next pixel
    cudaGraphExec_t exec = nullptr;
    ~BatchRun() {
        if (exec) cudaGraphExecDestroy(exec);
        scenes.release(); prefix.release(); next.release();
        for (cudaEvent_t e : {start, light, camera, join, cam_fork, t0, t1, light_start, light_end, camera_start,
                              camera_end})
            if (e) cudaEventDestroy(e);
        for (cudaStream_t b : branch) if (b) cudaStreamDestroy(b);
        if (side) cudaStreamDestroy(side);
        if (main) cudaStreamDestroy(main);
    }
};

struct BindGuard {
    Context* prev = t_bound;
    ~BindGuard() { t_bound = prev; }
};

int batch_render(Context* const* cs, int n, int iterations, double* out) {
    BindGuard guard;
    Context* caller = &ctx();
    caller->err.clear();
    auto fail = [&](int code, const std::string& msg) { caller->err = msg; return code; };
    auto scene_fail = [&](int i, int code) {
        caller->err = "batch scene " + std::to_string(i) + ": " + cs[i]->err;
        return code;
    };
    // 1. every scene prepared, with its asynchronous capacities (a first iteration with
    //    host round trips where none has been rendered yet)
    std::vector<int> remaining(n, iterations), first_it(n, 0), pcap_was(n, 0);
    for (int i = 0; i < n; ++i)
        if (!cs[i]) return fail(RC_E_INVALID, "rc_batch_render: null context " + std::to_string(i));
    {
        std::vector<std::pair<const Context*, int>> seen(n);
        for (int i = 0; i < n; ++i) seen[i] = {cs[i], i};
        std::sort(seen.begin(), seen.end());
        for (int i = 1; i < n; ++i)
            if (seen[i].first == seen[i - 1].first)
                return fail(RC_E_INVALID, "rc_batch_render: context " +
                                              std::to_string(std::max(seen[i].second, seen[i - 1].second)) +
                                              " repeated");
    }
    for (int i = 0; i < n; ++i) {
        t_bound = cs[i];
        if (!ctx().scene) return fail(RC_E_NO_SCENE, "rc_batch_render: scene " + std::to_string(i) + " has no scene");
        if (cfg().sampler != RC_SAMPLER_UNIFORM || cfg().learned_proposal)
            return fail(RC_E_INVALID, "rc_batch_render: scene " + std::to_string(i) +
                                          " uses a Metropolis sampler or the learned proposal (uniform sampler only)");
    }
    for (int i = 0; i < n; ++i) {
        t_bound = cs[i];
        int r = prepare();
        if (r) return scene_fail(i, r);
        HostScene& sc = *ctx().scene;
        DeviceState& d = ctx().dev;
        pcap_was[i] = d.async_pcap < 0 ? -1 : 0;
        if (d.async_pcap <= 0) {
            if (d.iterations_done == 0 && remaining[i] > 0) {
                r = render_iteration(sc);
                if (r) return scene_fail(i, r);
                remaining[i]--;
            }
            if (d.iterations_done > 0) {
                r = async_setup(sc);
                if (r) return scene_fail(i, r);
            } else {
                remaining[i] = 0;
            }
        }
        if (remaining[i] > 0) {
            // an eager iteration's side-stream camera pass (error return) may still write
            // the query buffers the graph's camera pass writes
            if (cudaStreamSynchronize(d.side) != cudaSuccess || cudaStreamSynchronize(d.stream) != cudaSuccess)
                return fail(RC_E_CUDA, std::string("rc_batch_render: ") + cudaGetErrorString(cudaGetLastError()));
            if (d.async_flags.reserve(remaining[i]) != cudaSuccess) return fail(RC_E_CUDA, "batch flag allocation failed");
        }
        first_it[i] = d.iterations_done;
    }
    const int K = n > 0 ? *std::max_element(remaining.begin(), remaining.end()) : 0;
    t_bound = caller;
    if (out) for (int k = 0; k < 6; ++k) out[k] = 0.0;
    if (K <= 0) return RC_OK;
    // 2. per graph iteration: the scenes still rendering, their entries and prefixes
    std::vector<std::vector<int>> active(K);
    std::vector<BatchScene> entries;
    std::vector<long long> prefix;
    std::vector<size_t> entry_at(K), prefix_at(K);
    std::vector<long long> total_paths(K), total_pixels(K);
    for (int j = 0; j < K; ++j) {
        for (int i = 0; i < n; ++i) if (remaining[i] > j) active[j].push_back(i);
        entry_at[j] = entries.size();
        prefix_at[j] = prefix.size();
        const int m = (int)active[j].size();
        prefix.resize(prefix.size() + 2 * (m + 1));
        long long* pp = prefix.data() + prefix_at[j];
        long long* px = pp + m + 1;
        pp[0] = px[0] = 0;
        for (int a = 0; a < m; ++a) {
            const int i = active[j][a];
            t_bound = cs[i];
            DeviceState& d = ctx().dev;
            BatchScene b{};
            b.p = make_params(*ctx().scene, first_it[i] + j);
            b.p.path_order = d.path_order.p;
            b.ph = PhotonBuf{d.ph_pos.p, d.ph_dir.p, d.ph_tp.p, d.ph_path.p, d.async_pcap, d.counters.p};
            b.qb = QueryBuf{d.q0.p, d.q1.p, d.q2.p, d.q3.p, d.q4.p, d.async_qcap, d.counters.p + 1};
            entries.push_back(b);
            pp[a + 1] = pp[a] + b.p.num_light_paths;
            px[a + 1] = px[a] + (long long)b.p.camera.width * b.p.camera.height;
        }
        total_paths[j] = pp[m];
        total_pixels[j] = px[m];
    }
    t_bound = caller;
    BatchRun B;
    RC_CUDA(B.scenes.reserve(entries.size()));
    RC_CUDA(B.prefix.reserve(prefix.size()));
    RC_CUDA(B.next.reserve(2));
    RC_CUDA(cudaMemcpy(B.scenes.p, entries.data(), entries.size() * sizeof(BatchScene), cudaMemcpyHostToDevice));
    RC_CUDA(cudaMemcpy(B.prefix.p, prefix.data(), prefix.size() * sizeof(long long), cudaMemcpyHostToDevice));
    RC_CUDA(cudaStreamCreateWithFlags(&B.main, cudaStreamNonBlocking));
    RC_CUDA(cudaStreamCreateWithFlags(&B.side, cudaStreamNonBlocking));
    // one capture stream per scene branch, at most kBatchStreams (scenes beyond share them
    // in turn: their branches then follow one another in the graph)
    constexpr int kBatchStreams = 64;
    B.branch.assign(std::min(n, kBatchStreams), nullptr);
    for (cudaStream_t& b : B.branch) RC_CUDA(cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking));
    auto branch = [&](int i) { return B.branch[(size_t)i % B.branch.size()]; };
    for (cudaEvent_t* e : {&B.start, &B.light, &B.camera, &B.join, &B.cam_fork})
        RC_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    for (cudaEvent_t* e : {&B.t0, &B.t1, &B.light_start, &B.light_end, &B.camera_start, &B.camera_end})
        RC_CUDA(cudaEventCreate(e));
    // 3. launch shapes of the batch passes, timed once per process on the first
    //    iteration's scenes (warm-up launch, then a timed one; the graph resets every
    //    counter the passes append to)
    if (g_batch_light.load() < 0 || g_batch_camera.load() < 0) {
        const int m = (int)active[0].size();
        const BatchScene* sc0 = B.scenes.p + entry_at[0];
        const long long* pp = B.prefix.p + prefix_at[0];
        for (int a = 0; a < m; ++a) {
            t_bound = cs[active[0][a]];
            VMParams p = entries[entry_at[0] + a].p;
            launch_light_order(p, ctx().dev.order_scratch.p, ctx().dev.path_order.p, B.main);
        }
        t_bound = caller;
        auto reset = [&](int which) {
            for (int a = 0; a < m; ++a)
                cudaMemsetAsync(cs[active[0][a]]->dev.counters.p + which, 0, sizeof(unsigned long long), B.main);
        };
        auto tune = [&](auto&& run) {
            float best = 1e30f;
            int best_v = 0;
            for (int v = 0; v < pass_variants(); ++v) {
                run(v);
                cudaEventRecord(B.t0, B.main);
                run(v);
                cudaEventRecord(B.t1, B.main);
                cudaEventSynchronize(B.t1);
                const float ms = ms_between(B.t0, B.t1);
                if (ms < best) { best = ms; best_v = v; }
            }
            return best_v;
        };
        g_batch_light = tune([&](int v) {
            reset(0);
            launch_light_pass_batch(sc0, pp, m, total_paths[0], B.next.p, B.main, v);
        });
        g_batch_camera = tune([&](int v) {
            reset(1);
            launch_camera_pass_batch(sc0, pp + m + 1, m, total_pixels[0], B.next.p + 1, B.main, v);
        });
        RC_CUDA(cudaStreamSynchronize(B.main));
        RC_CUDA(cudaGetLastError());
        if (caller->cfg_set && caller->cfg.verbose)
            std::printf("{\"autotune\": \"batch passes\", \"light\": %d, \"camera\": %d}\n", g_batch_light.load(),
                        g_batch_camera.load());
    }
    const int lvar = g_batch_light.load(), cvar = g_batch_camera.load();
    // 4. one graph per iteration: captured, the executable graph updated in place (or
    //    instantiated) and launched
    double kernels = 0;
    RC_CUDA(cudaEventRecord(B.t0, B.main));
    for (int j = 0; j < K; ++j) {
        const int m = (int)active[j].size();
        RC_CUDA(cudaStreamBeginCapture(B.main, cudaStreamCaptureModeRelaxed));
        int r = RC_OK;
        auto enqueue = [&]() -> int {
            RC_CUDA(cudaEventRecord(B.start, B.main));
            for (int a = 0; a < m; ++a) {
                const int i = active[j][a];
                t_bound = cs[i];
                VMParams p = entries[entry_at[j] + a].p;
                RC_CUDA(cudaStreamWaitEvent(branch(i), B.start, 0));
                int rr = async_head(p, branch(i));
                if (rr) return scene_fail(i, rr);
                RC_CUDA(cudaEventRecord(B.join, branch(i)));
                RC_CUDA(cudaStreamWaitEvent(B.main, B.join, 0));
            }
            t_bound = caller;
            // the camera pass forks before the light pass: its blocks take the slots the
            // persistent light pass's tail frees
            RC_CUDA(cudaEventRecord(B.cam_fork, B.main));
            RC_CUDA(record(B.light_start, B.main));
            launch_light_pass_batch(B.scenes.p + entry_at[j], B.prefix.p + prefix_at[j], m, total_paths[j], B.next.p,
                                    B.main, lvar);
            RC_CUDA(record(B.light_end, B.main));
            RC_CUDA(cudaEventRecord(B.light, B.main));
            RC_CUDA(cudaStreamWaitEvent(B.side, B.cam_fork, 0));
            RC_CUDA(record(B.camera_start, B.side));
            launch_camera_pass_batch(B.scenes.p + entry_at[j], B.prefix.p + prefix_at[j] + m + 1, m, total_pixels[j],
                                     B.next.p + 1, B.side, cvar);
            RC_CUDA(record(B.camera_end, B.side));
            RC_CUDA(cudaEventRecord(B.camera, B.side));
            for (int a = 0; a < m; ++a) {
                const int i = active[j][a];
                t_bound = cs[i];
                RC_CUDA(cudaStreamWaitEvent(branch(i), B.light, 0));
                int rr = async_tail(*ctx().scene, entries[entry_at[j] + a].p, branch(i), B.camera,
                                    ctx().dev.async_flags.p + j);
                if (rr) return scene_fail(i, rr);
                RC_CUDA(cudaEventRecord(B.join, branch(i)));
                RC_CUDA(cudaStreamWaitEvent(B.main, B.join, 0));
            }
            t_bound = caller;
            RC_CUDA(cudaStreamWaitEvent(B.main, B.camera, 0));
            return RC_OK;
        };
        r = enqueue();
        Context* at = t_bound;
        t_bound = caller;
        if (r && caller->err.empty())
            caller->err = "batch graph capture: " + (at && at != caller ? at->err : std::string("failed"));
        const cudaError_t le = cudaGetLastError();
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(B.main, &graph);
        if (r) { if (graph) cudaGraphDestroy(graph); return r; }
        if (le != cudaSuccess || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(RC_E_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(le != cudaSuccess ? le : e));
        }
        {
            size_t nodes = 0;
            cudaGraphGetNodes(graph, nullptr, &nodes);
            std::vector<cudaGraphNode_t> list(nodes);
            if (nodes) cudaGraphGetNodes(graph, list.data(), &nodes);
            for (cudaGraphNode_t g : list) {
                cudaGraphNodeType t;
                if (cudaGraphNodeGetType(g, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) kernels += 1;
            }
        }
        if (B.exec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(B.exec, graph, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(B.exec);
                B.exec = nullptr;
            }
        }
        if (!B.exec) {
            const cudaError_t ie = cudaGraphInstantiate(&B.exec, graph, 0);
            if (ie != cudaSuccess) {
                cudaGraphDestroy(graph);
                return fail(RC_E_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(ie));
            }
        }
        cudaGraphDestroy(graph);
        RC_CUDA(cudaGraphLaunch(B.exec, B.main));
    }
    RC_CUDA(cudaEventRecord(B.t1, B.main));
    RC_CUDA(cudaStreamSynchronize(B.main));
    const double batch_ms = ms_between(B.t0, B.t1);
    // 5. per scene: flags, statistics of its last iteration, overflowed iterations again
    int redone = 0;
    for (int i = 0; i < n; ++i) {
        if (remaining[i] <= 0) continue;
        t_bound = cs[i];
        DeviceState& d = ctx().dev;
        d.iterations_done += remaining[i];
        d.acc_gather_ms = d.acc_gather_bytes = d.acc_launches = 0;
        d.acc_iters = d.acc_async = 0;
        std::vector<int> fl(remaining[i], 0);
        RC_CUDA(cudaMemcpy(fl.data(), d.async_flags.p, sizeof(int) * remaining[i], cudaMemcpyDeviceToHost));
        redone += (int)std::count(fl.begin(), fl.end(), 1);
        const int r = async_finish(*ctx().scene, first_it[i], remaining[i], false);
        if (r) return scene_fail(i, r);
        if (pcap_was[i] < 0) d.async_pcap = -1;   // single-scene renders keep their round trips
    }
    t_bound = caller;
    if (out) {
        out[0] = batch_ms;
        out[1] = K;
        out[2] = kernels;
        out[3] = redone;
        out[4] = ms_between(B.light_start, B.light_end);
        out[5] = ms_between(B.camera_start, B.camera_end);
    }
    return RC_OK;
}

// Debug view `mode` (2-4) into the image accumulation, counted as one iteration.
int render_debug(HostScene& sc, int mode) {
    if (mode < 2 || mode > 4) { ctx().err = "debug view must be 2 (normals), 3 (facing) or 4 (materials)"; return RC_E_INVALID; }
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    VMParams p = make_params(sc, 0);
    const long long npix = (long long)sc.camera.width * sc.camera.height;
    RC_CUDA(d.accum.reserve(std::max<long long>(3 * npix, 1)));
    RC_CUDA(cudaMemsetAsync(d.accum.p, 0, sizeof(double) * std::max<long long>(3 * npix, 1), s));
    launch_debug_view(p, mode, sc.debug_ior, d.accum.p, s);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaStreamSynchronize(s));
    int r = check_errors();
    if (r) return r;
    d.iterations_done = 1;
    return RC_OK;
}

// ---------------------------------------------------------------- progressive state
// Checkpoint of a progressive render: the FP64 image sum, the iteration index (the
// counter RNG continues from it, so a resumed render draws the same samples as an
// uninterrupted one), the sampling configuration, and the learned proposal's network
// and Adam state.  The scene itself is not stored; a fingerprint of the prepared scene
// (triangles, vertices, camera, lights, materials, radius) must match on load.
constexpr char kStateMagic[8] = {'R', 'C', 'S', 'T', 'A', 'T', 'E', '1'};

uint64_t fnv1a(uint64_t h, const void* data, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
    return h;
}

uint64_t scene_fingerprint(const HostScene& sc) {
    uint64_t h = 14695981039346656037ull;
    for (const HostMesh& m : sc.meshes) {
        h = fnv1a(h, m.wpos.data(), m.wpos.size() * sizeof(V3));
        h = fnv1a(h, m.tri.data(), m.tri.size() * sizeof(uint32_t));
        h = fnv1a(h, m.mat.data(), m.mat.size() * sizeof(uint32_t));
    }
    h = fnv1a(h, &sc.camera, sizeof(sc.camera));
    h = fnv1a(h, sc.lights.data(), sc.lights.size() * sizeof(DevLight));
    h = fnv1a(h, sc.materials.data(), sc.materials.size() * sizeof(DevMaterial));
    h = fnv1a(h, &sc.base_radius, sizeof(float));
    h = fnv1a(h, &sc.radius_alpha, sizeof(float));
    return h;
}

struct StateHeader {
    char magic[8];
    int32_t width, height, iterations_done, max_path_length;
    uint64_t seed, camera_seed, fingerprint;
    int64_t photons_per_iter;
    int32_t sampler, learned, mlp_rounds, adam_step;
    uint64_t accum_doubles, mlp_floats;
};

int save_state(const char* path) {
    if (!ctx().scene || !ctx().scene->prepared) { ctx().err = "save_state: no prepared scene"; return RC_E_NO_SCENE; }
    if (!path) { ctx().err = "save_state: null path"; return RC_E_INVALID; }
    const HostScene& sc = *ctx().scene;
    DeviceState& d = ctx().dev;
    const size_t npix = (size_t)sc.camera.width * sc.camera.height;
    StateHeader h{};
    std::memcpy(h.magic, kStateMagic, 8);
    h.width = sc.camera.width; h.height = sc.camera.height;
    h.iterations_done = d.iterations_done;
    h.max_path_length = cfg().max_path_length;
    h.seed = cfg().seed;
    h.camera_seed = cfg().camera_seed ? cfg().camera_seed : cfg().seed;
    h.fingerprint = scene_fingerprint(sc);
    h.photons_per_iter = cfg().photons_per_iter;
    h.sampler = cfg().sampler;
    h.learned = cfg().learned_proposal;
    h.mlp_rounds = d.mlp_rounds;
    h.adam_step = d.mlp ? d.mlp->p.adam_step : 0;
    h.accum_doubles = 3 * npix;
    h.mlp_floats = d.mlp ? mlp_state_floats() : 0;
    std::vector<double> acc(3 * npix, 0.0);
    if (d.accum.p && d.accum.n >= 3 * npix)
        RC_CUDA(cudaMemcpy(acc.data(), d.accum.p, acc.size() * sizeof(double), cudaMemcpyDeviceToHost));
    std::vector<float> ml(h.mlp_floats);
    if (h.mlp_floats && mlp_export(d.mlp->p, ml.data())) { ctx().err = "save_state: MLP read-back failed"; return RC_E_CUDA; }
    FILE* f = std::fopen(path, "wb");
    if (!f) { ctx().err = std::string("cannot open ") + path; return RC_E_IO; }
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
              std::fwrite(acc.data(), sizeof(double), acc.size(), f) == acc.size() &&
              std::fwrite(ml.data(), sizeof(float), ml.size(), f) == ml.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) { ctx().err = std::string("write failed: ") + path; return RC_E_IO; }
    return RC_OK;
}

int load_state(const char* path) {
    int r = prepare();
    if (r) return r;
    if (!path) { ctx().err = "load_state: null path"; return RC_E_INVALID; }
    const HostScene& sc = *ctx().scene;
    DeviceState& d = ctx().dev;
    FILE* f = std::fopen(path, "rb");
    if (!f) { ctx().err = std::string("cannot open ") + path; return RC_E_IO; }
    StateHeader h{};
    const size_t npix = (size_t)sc.camera.width * sc.camera.height;
    bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, kStateMagic, 8) == 0;
    if (ok && (h.width != sc.camera.width || h.height != sc.camera.height || h.fingerprint != scene_fingerprint(sc) ||
               h.accum_doubles != 3 * npix || (h.mlp_floats && h.mlp_floats != mlp_state_floats()) ||
               h.iterations_done < 0)) {
        std::fclose(f);
        ctx().err = "load_state: the state was saved for another scene";
        return RC_E_INVALID;
    }
    std::vector<double> acc(ok ? h.accum_doubles : 0);
    std::vector<float> ml(ok ? h.mlp_floats : 0);
    ok = ok && std::fread(acc.data(), sizeof(double), acc.size(), f) == acc.size() &&
         std::fread(ml.data(), sizeof(float), ml.size(), f) == ml.size();
    std::fclose(f);
    if (!ok) { ctx().err = std::string("load_state: unreadable or truncated state file ") + path; return RC_E_IO; }
    // sampling configuration continues as saved
    rc_config c = cfg();
    c.seed = h.seed;
    c.camera_seed = h.camera_seed;
    c.photons_per_iter = h.photons_per_iter;
    c.max_path_length = h.max_path_length;
    c.sampler = h.sampler;
    c.learned_proposal = h.learned;
    ctx().cfg = c;
    RC_CUDA(d.accum.reserve(std::max<size_t>(acc.size(), 1)));
    RC_CUDA(cudaMemcpy(d.accum.p, acc.data(), acc.size() * sizeof(double), cudaMemcpyHostToDevice));
    d.iterations_done = h.iterations_done;
    d.mlp_rounds = 0;
    if (h.mlp_floats) {
        if (!d.mlp) {
            d.mlp = std::make_unique<MlpStore>();
            if (!d.mlp->setup(kTrainBatchRows)) { ctx().err = "MLP allocation failed"; return RC_E_CUDA; }
            RC_CUDA(d.train_pos.reserve(kTrainCapacity)); RC_CUDA(d.train_dir.reserve(kTrainCapacity));
            RC_CUDA(d.train_count.reserve(1)); RC_CUDA(d.train_wsum.reserve(1));
        }
        if (mlp_import(d.mlp->p, ml.data(), h.adam_step, d.stream)) { ctx().err = "MLP upload failed"; return RC_E_CUDA; }
        d.mlp_rounds = h.mlp_rounds;
    }
    return RC_OK;
}

// Minimal single-part scanline OpenEXR writer: FP32 RGB, no compression.
int write_exr(const char* path, const float* rgb, int w, int h) {
    FILE* f = std::fopen(path, "wb");
    if (!f) { ctx().err = std::string("cannot open ") + path; return RC_E_IO; }
    std::vector<unsigned char> hdr;
    auto put = [&](const void* p, size_t n) { const unsigned char* c = (const unsigned char*)p; hdr.insert(hdr.end(), c, c + n); };
    auto put_i32 = [&](int32_t v) { put(&v, 4); };
    auto put_str = [&](const char* s) { put(s, std::strlen(s) + 1); };
    auto attr = [&](const char* name, const char* type, int32_t size) { put_str(name); put_str(type); put_i32(size); };
    const uint32_t magic = 20000630u;
    put(&magic, 4);
    put_i32(2);
    attr("channels", "chlist", 3 * (2 + 16) + 1);
    for (const char* ch : {"B", "G", "R"}) {
        put_str(ch);
        put_i32(2);                       // FLOAT
        unsigned char lin[4] = {0, 0, 0, 0};
        put(lin, 4);
        put_i32(1); put_i32(1);           // sampling
    }
    unsigned char z = 0;
    put(&z, 1);
    attr("compression", "compression", 1); put(&z, 1);
    attr("dataWindow", "box2i", 16); put_i32(0); put_i32(0); put_i32(w - 1); put_i32(h - 1);
    attr("displayWindow", "box2i", 16); put_i32(0); put_i32(0); put_i32(w - 1); put_i32(h - 1);
    attr("lineOrder", "lineOrder", 1); put(&z, 1);
    float one = 1.0f, zero = 0.0f;
    attr("pixelAspectRatio", "float", 4); put(&one, 4);
    attr("screenWindowCenter", "v2f", 8); put(&zero, 4); put(&zero, 4);
    attr("screenWindowWidth", "float", 4); put(&one, 4);
    put(&z, 1);
    const uint64_t line_bytes = 8 + 12ull * (uint64_t)w;
    uint64_t off = hdr.size() + 8ull * (uint64_t)h;
    for (int y = 0; y < h; ++y) { put(&off, 8); off += line_bytes; }
    bool ok = std::fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
    std::vector<float> line(3 * (size_t)w);
    for (int y = 0; y < h && ok; ++y) {
        int32_t yy = y, sz = 12 * w;
        for (int x = 0; x < w; ++x) {
            line[x] = rgb[3 * ((size_t)y * w + x) + 2];
            line[w + x] = rgb[3 * ((size_t)y * w + x) + 1];
            line[2 * w + x] = rgb[3 * ((size_t)y * w + x) + 0];
        }
        ok = std::fwrite(&yy, 4, 1, f) == 1 && std::fwrite(&sz, 4, 1, f) == 1 &&
             std::fwrite(line.data(), 4, line.size(), f) == line.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) { ctx().err = std::string("write failed: ") + path; return RC_E_IO; }
    return RC_OK;
}

int read_image(float* rgb, int w, int h) {
    if (!ctx().scene) { ctx().err = "no scene"; return RC_E_NO_SCENE; }
    if (!rgb || w != ctx().scene->camera.width || h != ctx().scene->camera.height) { ctx().err = "bad image buffer"; return RC_E_INVALID; }
    size_t n = 3 * (size_t)w * h;
    DeviceState& d = ctx().dev;
    if (!d.accum.p || d.accum.n < n || !d.stream) {
        std::memset(rgb, 0, n * sizeof(float));
        return RC_OK;
    }
    // mean on the device, then one FP32 copy (half the bytes of the FP64 sum)
    const int it = d.iterations_done;
    const double sc = it > 0 ? 1.0 / it : 0.0;
    RC_CUDA(d.image.reserve(n));
    launch_image_mean(d.accum.p, d.image.p, (long long)n, sc, d.stream);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaMemcpyAsync(rgb, d.image.p, n * sizeof(float), cudaMemcpyDeviceToHost, d.stream));
    RC_CUDA(cudaStreamSynchronize(d.stream));
    return RC_OK;
}

void release_all() {
    ctx().dev.release();
    ctx().scene.reset();
    ctx().host_ready = false;
}

int dump_bvh(const std::vector<BvhNode>& nodes, const std::vector<int>& index, unsigned* out, int cap, int* idx, int idx_cap) {
    int n = (int)nodes.size();
    for (int i = 0; i < n && i < cap; ++i) {
        float f[6] = {nodes[i].box.mn.x, nodes[i].box.mn.y, nodes[i].box.mn.z, nodes[i].box.mx.x, nodes[i].box.mx.y, nodes[i].box.mx.z};
        std::memcpy(out + 8 * i, f, 24);
        out[8 * i + 6] = nodes[i].w0;
        out[8 * i + 7] = nodes[i].w1;
    }
    for (int i = 0; i < (int)index.size() && i < idx_cap; ++i) idx[i] = index[i];
    return n;
}

}  // namespace
}  // namespace rc

using namespace rc;

extern "C" {

void init(int samples, float base_radius, float radius_reduction, long long* meshes_pointers,
          unsigned int number_of_meshes, rc_matrix4x4* mesh_matrices, unsigned int* meshes_number_of_verts,
          unsigned int* meshes_number_of_tris, unsigned int camera_x, unsigned int camera_y, rc_vec3 camera_position,
          rc_vec3 camera_corner0, rc_vec3 camera_corner1, rc_vec3 camera_corner2, rc_vec3 camera_corner3,
          rc_python_light* lights, unsigned int number_of_lights, rc_python_material* materials,
          unsigned int number_of_materials, int** materials_indices, int debug_test, rc_debug_stuff debug_stuff) {
    release_all();
    ctx().err.clear();
    auto sc = std::make_unique<HostScene>();
    sc->samples = samples;
    sc->base_radius = base_radius;
    sc->radius_alpha = radius_reduction;
    sc->debug_test = debug_test;
    sc->debug_ior = debug_stuff.specular;   // src/main.cpp:116 (read by run_debug_materials)
    if (number_of_meshes && (!meshes_pointers || !mesh_matrices || !meshes_number_of_verts ||
                             !meshes_number_of_tris || !materials_indices)) {
        ctx().err = "init: null mesh arrays";
        return;
    }
    sc->meshes.resize(number_of_meshes);
    for (unsigned i = 0; i < number_of_meshes; ++i) {
        int r = ingest_mesh(sc->meshes[i], (const void*)meshes_pointers[i], meshes_number_of_verts[i],
                            meshes_number_of_tris[i], mesh_matrices[i], materials_indices[i], ctx().err);
        if (r) return;
    }
    for (unsigned i = 0; i < number_of_meshes; ++i)
        for (uint32_t m : sc->meshes[i].mat)
            if (m >= number_of_materials) { ctx().err = "init: material index out of range"; return; }
    // Camera(camera_x, camera_y, position, corners...) (src/Camera.h:21-26)
    HostCamera& c = sc->camera;
    c.width = (int)camera_x;
    c.height = (int)camera_y;
    c.origin = {camera_position.x, camera_position.y, camera_position.z};
    c.bottom_left = {camera_corner2.x, camera_corner2.y, camera_corner2.z};
    c.horizontal = {camera_corner1.x - camera_corner2.x, camera_corner1.y - camera_corner2.y, camera_corner1.z - camera_corner2.z};
    c.vertical = {camera_corner3.x - camera_corner2.x, camera_corner3.y - camera_corner2.y, camera_corner3.z - camera_corner2.z};
    // The reference keeps the caller's light array and converts it in main()
    // (src/main.cpp:134,163); the records are copied here so that the caller may free
    // them after init (converted at prepare time all the same).
    if (number_of_lights && !lights) { ctx().err = "init: null lights"; return; }
    sc->py_lights.assign(lights, lights + number_of_lights);
    sc->num_lights = number_of_lights;
    if (number_of_materials && !materials) { ctx().err = "init: null materials"; return; }
    sc->py_materials.assign(materials, materials + number_of_materials);
    ctx().scene = std::move(sc);
}

int main(void) {
    if (!ctx().scene) { ctx().err = "main: no scene (init was not called or failed: " + ctx().err + ")"; return RC_E_NO_SCENE; }
    // src/main.cpp:170-186: 1 = vertex merging, 2-4 = debug views (one pass, no
    // averaging), 5 = the mesh BVHs' boxes as OBJ files (host only, no image)
    const int mode = ctx().scene->debug_test;
    int r = mode == 5 ? prepare_host() : prepare();
    if (!r) {
        if (mode == 1) {
            r = render_iterations(*ctx().scene, ctx().scene->samples);
        } else if (mode >= 2 && mode <= 4) {
            r = render_debug(*ctx().scene, mode);
        } else if (mode == 5) {
            r = debug_bvh_obj(*ctx().scene);
        } else {
            ctx().err = "debug_test must be 1 (render), 2-4 (debug views) or 5 (BVH boxes as OBJ files)";
            r = RC_E_UNSUPPORTED;
        }
    }
    if (!r && cfg().write_exr && mode != 5) {
        int w = ctx().scene->camera.width, h = ctx().scene->camera.height;
        std::vector<float> img(3 * (size_t)w * h);
        r = read_image(img.data(), w, h);
        if (!r) r = write_exr(cfg().exr_path, img.data(), w, h);
    }
    std::string keep = ctx().err;
    release_all();
    ctx().err = keep;
    return r;
}

int rc_default_config(rc_config* c) {
    if (!c) return RC_E_INVALID;
    default_config(c);
    return RC_OK;
}

int rc_set_config(const rc_config* c) {
    if (!c) { ctx().err = "null config"; return RC_E_INVALID; }
    if (c->max_path_length < 0 || c->max_path_length > 30) { ctx().err = "max_path_length out of range [0, 30]"; return RC_E_INVALID; }
    if (c->photons_per_iter < 0) { ctx().err = "photons_per_iter < 0"; return RC_E_INVALID; }
    if (c->sampler != RC_SAMPLER_UNIFORM && c->sampler != RC_SAMPLER_HYBRID && c->sampler != RC_SAMPLER_PSSMLT) {
        ctx().err = "unknown sampler"; return RC_E_INVALID;
    }
    if (c->learned_proposal) {
        if (c->train_iterations < 0 || c->train_steps < 0 || !(c->learning_rate > 0.0f && c->learning_rate < 1.0f)) {
            ctx().err = "learned proposal: train_iterations/train_steps >= 0, learning_rate in (0, 1)"; return RC_E_INVALID;
        }
    }
    if (c->sampler != RC_SAMPLER_UNIFORM) {
        if (c->mlt_chains <= 0) { ctx().err = "mlt_chains must be positive"; return RC_E_INVALID; }
        if (c->max_path_length > kMltMaxPathLength) { ctx().err = "Metropolis samplers support max_path_length <= 12"; return RC_E_UNSUPPORTED; }
        if (c->sampler == RC_SAMPLER_PSSMLT && !(c->large_step_prob > 0.0f && c->large_step_prob <= 1.0f)) {
            ctx().err = "large_step_prob must be in (0, 1]"; return RC_E_INVALID;
        }
    }
    if (c->graph_replay < 0 || c->graph_replay > 2) { ctx().err = "graph_replay must be 0, 1 or 2"; return RC_E_INVALID; }
    if (c->gpu_bvh < 0 || c->gpu_bvh > 1) { ctx().err = "gpu_bvh must be 0 or 1"; return RC_E_INVALID; }
    ctx().cfg = *c;
    ctx().cfg.exr_path[sizeof(ctx().cfg.exr_path) - 1] = 0;
    ctx().cfg_set = true;
    // sizes and shapes of asynchronous iterations are re-derived under the new settings
    ctx().dev.async_pcap = ctx().dev.async_qcap = 0;
    if (ctx().dev.graph_exec) { cudaGraphExecDestroy(ctx().dev.graph_exec); ctx().dev.graph_exec = nullptr; }
    return RC_OK;
}

int rc_prepare(void) { return prepare(); }

int rc_prepare_host(float* info) {
    int r = prepare_host();
    if (r) return r;
    const HostScene& sc = *ctx().scene;
    if (info) {
        info[0] = sc.bounds.mn.x; info[1] = sc.bounds.mn.y; info[2] = sc.bounds.mn.z;
        info[3] = sc.bounds.mx.x; info[4] = sc.bounds.mx.y; info[5] = sc.bounds.mx.z;
        info[6] = sc.scene_radius; info[7] = sc.base_radius; info[8] = (float)sc.world.nodes.size();
    }
    return RC_OK;
}

int rc_host_mesh_bvh(int mesh, unsigned* nodes, int cap, int* index, int index_cap, float* cost) {
    int r = prepare_host();
    if (r) return r;
    if (mesh < 0 || mesh >= (int)ctx().scene->meshes.size() || !nodes || !index) { ctx().err = "bad mesh index"; return RC_E_INVALID; }
    HostMesh& hm = ctx().scene->meshes[mesh];
    if (hm.bvh.nodes.empty()) build_mesh_bvh(hm);   // the device built this scene's meshes
    const MeshBvh& b = hm.bvh;
    if (cost) *cost = b.cost;
    return dump_bvh(b.nodes, b.index, nodes, cap, index, index_cap);
}

int rc_host_world_bvh(unsigned* nodes, int cap, int* index, int index_cap) {
    int r = prepare_host();
    if (r) return r;
    if (!nodes || !index) { ctx().err = "null output"; return RC_E_INVALID; }
    return dump_bvh(ctx().scene->world.nodes, ctx().scene->world.index, nodes, cap, index, index_cap);
}

int rc_scene_dump(int which, unsigned* out, long long cap, long long* words) {
    if (!ctx().scene || !ctx().scene->prepared) { ctx().err = "rc_scene_dump: scene not prepared"; return RC_E_NO_SCENE; }
    if (!words || (cap > 0 && !out) || cap < 0) { ctx().err = "rc_scene_dump: bad arguments"; return RC_E_INVALID; }
    DeviceState& d = ctx().dev;
    struct Part { const void* p; long long words; int width; };   // width: words per item
    std::vector<Part> parts;
    const long long wn = d.view.num_world_nodes;
    const long long nm = (long long)ctx().scene->meshes.size();
    const long long nw = (long long)ctx().scene->world.index.size() - 1;
    switch (which) {
        case 0: parts = {{d.nodes.p, 8 * d.num_mesh_nodes, 8}}; break;
        case 1:
            parts = {{d.tris.p, 12 * d.num_tris, 12}, {d.tri_n0.p, 4 * d.num_tris, 4}, {d.tri_n1.p, 4 * d.num_tris, 4},
                     {d.tri_n2.p, 4 * d.num_tris, 4}};
            break;
        case 2: parts = {{d.wnode_lo.p, 4 * wn, 4}, {d.wnode_hi.p, 4 * wn, 4}}; break;
        case 3: parts = {{d.world_mesh.p, nw, 0}, {d.mesh_root.p, nm, 0}}; break;
        default: ctx().err = "rc_scene_dump: which must be 0..3"; return RC_E_INVALID;
    }
    // 0 and 2 per node as (lo, hi); 1 per triangle as (v0, e1, e2, n0, n1, n2); 3 the
    // two lists one after the other
    long long total = 0;
    for (const Part& q : parts) total += q.words;
    *words = total;
    std::vector<unsigned> host((size_t)total);
    long long off = 0;
    for (const Part& q : parts) {
        if (q.words) RC_CUDA(cudaMemcpy(host.data() + off, q.p, 4 * (size_t)q.words, cudaMemcpyDeviceToHost));
        off += q.words;
    }
    if (parts[0].width > 0 && parts.size() > 1) {
        int stride = 0;
        for (const Part& q : parts) stride += q.width;
        const long long items = total / stride;
        std::vector<unsigned> il((size_t)total);
        long long src = 0;
        int col = 0;
        for (const Part& q : parts) {
            for (long long i = 0; i < items; ++i)
                std::memcpy(&il[(size_t)(i * stride + col)], &host[(size_t)(src + i * q.width)], 4 * (size_t)q.width);
            src += q.words;
            col += q.width;
        }
        host.swap(il);
    }
    if (cap > 0) std::memcpy(out, host.data(), 4 * (size_t)std::min(cap, total));
    return RC_OK;
}

rc_context* rc_context_create(void) { return reinterpret_cast<rc_context*>(new (std::nothrow) Context()); }

int rc_context_bind(rc_context* c) {
    t_bound = reinterpret_cast<Context*>(c);
    return RC_OK;
}

int rc_context_destroy(rc_context* c) {
    if (!c) { ctx().err = "rc_context_destroy: null context"; return RC_E_INVALID; }
    Context* x = reinterpret_cast<Context*>(c);
    Context* prev = t_bound;
    t_bound = x;
    release_all();   // the scene and its device buffers
    x->bvh.reset();
    t_bound = prev == x ? nullptr : prev;
    delete x;
    return RC_OK;
}

int rc_prepare_stats(double* out, int n) {
    if (!out || n < 0) { ctx().err = "rc_prepare_stats: bad arguments"; return RC_E_INVALID; }
    const int k = std::min(n, 5);
    for (int i = 0; i < k; ++i) out[i] = ctx().prep[i];
    return k;
}

int rc_render(int iterations) {
    if (iterations < 0) { ctx().err = "iterations < 0"; return RC_E_INVALID; }
    int r = prepare();
    if (!r) r = render_iterations(*ctx().scene, iterations);
    return r;
}

int rc_save_state(const char* path) { return save_state(path); }
int rc_load_state(const char* path) { return load_state(path); }

int rc_render_debug(int mode) {
    if (mode == 5) {
        int r = prepare_host();
        if (r) return r;
        return debug_bvh_obj(*ctx().scene);
    }
    int r = prepare();
    if (r) return r;
    return render_debug(*ctx().scene, mode);
}

int rc_batch_render(rc_context* const* ctxs, int n, int iterations, double* out) {
    if (!ctxs || n < 1 || iterations < 0) { ctx().err = "rc_batch_render: bad arguments"; return RC_E_INVALID; }
    return batch_render(reinterpret_cast<Context* const*>(ctxs), n, iterations, out);
}

int rc_render_timed(int iterations, double* out) {
    if (iterations < 0 || !out) { ctx().err = "bad arguments"; return RC_E_INVALID; }
    int r = prepare();
    if (r) return r;
    DeviceState& d = ctx().dev;
    d.acc_gather_ms = d.acc_gather_bytes = d.acc_launches = 0;
    d.acc_iters = 0;
    d.acc_async = 0;
    RC_CUDA(cudaStreamSynchronize(d.stream));
    RC_CUDA(cudaEventRecord(d.t0, d.stream));
    r = render_iterations(*ctx().scene, iterations);
    if (r) return r;
    RC_CUDA(cudaEventRecord(d.t1, d.stream));
    RC_CUDA(cudaEventSynchronize(d.t1));
    float ms = 0.0f;
    RC_CUDA(cudaEventElapsedTime(&ms, d.t0, d.t1));
    int n = std::max(d.acc_iters, 1);
    out[0] = ms;
    out[1] = d.acc_gather_ms / n;
    out[2] = d.acc_gather_bytes / n;
    out[3] = d.acc_launches;
    return RC_OK;
}

int rc_read_image(float* rgb, int width, int height) { return read_image(rgb, width, height); }

int rc_release(void) {
    release_all();
    return RC_OK;
}

const char* rc_last_error(void) { return ctx().err.c_str(); }

int rc_get_stats(double* out, int n) {
    if (!out || n < 0) return RC_E_INVALID;
    for (int i = 0; i < n && i < 17; ++i) out[i] = ctx().dev.stats[i];
    return RC_OK;
}

int rc_proposal_state(long long n, float* prop4, float* contrib) {
    if (n < 0) { ctx().err = "n < 0"; return RC_E_INVALID; }
    DeviceState& d = ctx().dev;
    if (prop4) {
        std::memset(prop4, 0, sizeof(float) * 4 * (size_t)n);
        if (d.mlp && d.mlp_rounds > 0 && n > 0 && ctx().scene && d.iterations_done > 0) {
            // the last rendered iteration's draws, recomputed from the network's table with
            // the paths' own samples (the light pass draws the same ones)
            const HostScene& sc = *ctx().scene;
            const VMParams p = make_params(sc, d.iterations_done - 1);
            const long long m = std::min<long long>(n, p.num_light_paths);
            RC_CUDA(d.prop.reserve(std::max<long long>(m, 1)));
            RC_CUDA(d.prop_table.reserve((size_t)sc.lights.size() * kProposalRes * kProposalRes * kProposalCellFloats));
            if (mlp_proposal(d.mlp->p, proposal_ctx(sc, p), kProposalRes, d.prop_table.p, m, d.prop.p, d.stream,
                             d.errors.p + ERR_MLP)) {
                ctx().err = "proposal launch failed"; return RC_E_CUDA;
            }
            RC_CUDA(cudaMemcpyAsync(prop4, d.prop.p, sizeof(float4) * m, cudaMemcpyDeviceToHost, d.stream));
            RC_CUDA(cudaStreamSynchronize(d.stream));
        }
    }
    if (contrib) {
        std::memset(contrib, 0, sizeof(float) * (size_t)n);
        const long long m = std::min<long long>(n, (long long)d.contrib.n);
        if (m > 0) RC_CUDA(cudaMemcpy(contrib, d.contrib.p, sizeof(float) * m, cudaMemcpyDeviceToHost));
    }
    return RC_OK;
}

int rc_camera_queries(int iteration, float* out, long long cap, long long* count) {
    int r = prepare();
    if (r) return r;
    if (iteration < 0 || (cap > 0 && !out)) { ctx().err = "bad query output"; return RC_E_INVALID; }
    HostScene& sc = *ctx().scene;
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    VMParams p = make_params(sc, iteration);
    const long long npix = (long long)sc.camera.width * sc.camera.height;
    long long qcap = std::max<long long>(npix * 2, 1024);
    unsigned long long nq = 0;
    for (int attempt = 0; attempt < 3; ++attempt) {
        RC_CUDA(d.q0.reserve(qcap)); RC_CUDA(d.q1.reserve(qcap)); RC_CUDA(d.q2.reserve(qcap));
        RC_CUDA(d.q3.reserve(qcap)); RC_CUDA(d.q4.reserve(qcap));
        RC_CUDA(d.counters.reserve(10));
        RC_CUDA(cudaMemsetAsync(d.counters.p + 1, 0, sizeof(unsigned long long), s));
        QueryBuf qb{d.q0.p, d.q1.p, d.q2.p, d.q3.p, d.q4.p, (long long)d.q0.n, d.counters.p + 1};
        launch_camera_pass(p, qb, d.counters.p + 7, s);
        RC_CUDA(cudaGetLastError());
        RC_CUDA(cudaMemcpyAsync(&nq, d.counters.p + 1, sizeof(nq), cudaMemcpyDeviceToHost, s));
        RC_CUDA(cudaStreamSynchronize(s));
        if ((long long)nq <= (long long)d.q0.n) break;
        qcap = (long long)nq + 1024;
    }
    r = check_errors();
    if (r) return r;
    if (count) *count = (long long)nq;
    const long long n = std::min<long long>((long long)nq, cap);
    if (n > 0) RC_CUDA(cudaMemcpy(out, d.q0.p, 16 * (size_t)n, cudaMemcpyDeviceToHost));
    return RC_OK;
}

int rc_light_photons(int iteration, float* out, long long cap, long long* count) {
    return rc_light_photons_shape(0, iteration, out, cap, count);
}

int rc_light_photons_shape(int shape, int iteration, float* out, long long cap, long long* count) {
    int r = prepare();
    if (r) return r;
    if (iteration < 0 || (cap > 0 && !out)) { ctx().err = "bad photon output"; return RC_E_INVALID; }
    if (shape < 0 || shape > pass_variants()) { ctx().err = "light pass shape out of range"; return RC_E_INVALID; }
    HostScene& sc = *ctx().scene;
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    VMParams p = make_params(sc, iteration);
    long long pcap = std::max<long long>(p.num_light_paths * 2, 1024);
    unsigned long long nph = 0;
    for (int attempt = 0; attempt < 3; ++attempt) {
        RC_CUDA(d.ph_pos.reserve(pcap)); RC_CUDA(d.ph_dir.reserve(pcap));
        RC_CUDA(d.ph_tp.reserve(pcap)); RC_CUDA(d.ph_path.reserve(pcap));
        RC_CUDA(d.counters.reserve(10));
        RC_CUDA(cudaMemsetAsync(d.counters.p, 0, sizeof(unsigned long long), s));
        PhotonBuf ph{d.ph_pos.p, d.ph_dir.p, d.ph_tp.p, d.ph_path.p, (long long)d.ph_pos.n, d.counters.p};
        r = light_pass(p, ph, s, shape);
        if (r) return r;
        RC_CUDA(cudaGetLastError());
        RC_CUDA(cudaMemcpyAsync(&nph, d.counters.p, sizeof(nph), cudaMemcpyDeviceToHost, s));
        RC_CUDA(cudaStreamSynchronize(s));
        if ((long long)nph <= (long long)d.ph_pos.n) break;
        pcap = (long long)nph + 1024;
    }
    r = check_errors();
    if (r) return r;
    if (count) *count = (long long)nph;
    long long n = std::min<long long>((long long)nph, cap);
    if (n > 0) {
        std::vector<float4> pos(n), dir(n);
        std::vector<float2> tp(n);
        std::vector<uint32_t> path(n);
        RC_CUDA(cudaMemcpy(pos.data(), d.ph_pos.p, 16 * n, cudaMemcpyDeviceToHost));
        RC_CUDA(cudaMemcpy(dir.data(), d.ph_dir.p, 16 * n, cudaMemcpyDeviceToHost));
        RC_CUDA(cudaMemcpy(tp.data(), d.ph_tp.p, 8 * n, cudaMemcpyDeviceToHost));
        RC_CUDA(cudaMemcpy(path.data(), d.ph_path.p, 4 * n, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < n; ++i) {
            float* w = out + 12 * i;
            w[0] = pos[i].x; w[1] = pos[i].y; w[2] = pos[i].z;
            w[3] = dir[i].x; w[4] = dir[i].y; w[5] = dir[i].z;
            w[6] = dir[i].w; w[7] = tp[i].x; w[8] = tp[i].y; w[9] = pos[i].w;
            std::memcpy(&w[10], &path[i], 4);
            w[11] = 0.0f;
        }
    }
    return RC_OK;
}

int rc_mlt_photons(int variant, int iteration, float* out, long long cap, long long* count,
                   unsigned long long* large_steps) {
    if (iteration < 0 || (cap > 0 && !out)) { ctx().err = "bad photon output"; return RC_E_INVALID; }
    if (variant < 0 || variant >= mlt_variants()) { ctx().err = "Metropolis pass shape out of range"; return RC_E_INVALID; }
    if (cfg().sampler == RC_SAMPLER_UNIFORM) { ctx().err = "the configuration has no Metropolis sampler"; return RC_E_INVALID; }
    int r = prepare();
    if (r) return r;
    HostScene& sc = *ctx().scene;
    DeviceState& d = ctx().dev;
    cudaStream_t s = d.stream;
    VMParams p = make_params(sc, iteration);
    long long pcap = std::max<long long>(p.num_light_paths * 2, 1024);
    unsigned long long nph = 0, st[2] = {0, 0};
    for (int attempt = 0; attempt < 3; ++attempt) {
        RC_CUDA(d.ph_pos.reserve(pcap)); RC_CUDA(d.ph_dir.reserve(pcap));
        RC_CUDA(d.ph_tp.reserve(pcap)); RC_CUDA(d.ph_path.reserve(pcap));
        RC_CUDA(cudaMemsetAsync(d.counters.p, 0, sizeof(unsigned long long), s));
        PhotonBuf ph{d.ph_pos.p, d.ph_dir.p, d.ph_tp.p, d.ph_path.p, (long long)d.ph_pos.n, d.counters.p};
        launch_mlt_pass(p, ph, cfg().sampler, cfg().mlt_chains, cfg().large_step_prob, d.counters.p + 2, s, variant);
        RC_CUDA(cudaGetLastError());
        RC_CUDA(cudaMemcpyAsync(&nph, d.counters.p, sizeof(nph), cudaMemcpyDeviceToHost, s));
        RC_CUDA(cudaMemcpyAsync(st, d.counters.p + 2, sizeof(st), cudaMemcpyDeviceToHost, s));
        RC_CUDA(cudaStreamSynchronize(s));
        if ((long long)nph <= (long long)d.ph_pos.n) break;
        pcap = (long long)nph + 1024;
    }
    r = check_errors();
    if (r) return r;
    if (count) *count = (long long)nph;
    if (large_steps) { large_steps[0] = st[0]; large_steps[1] = st[1]; }
    long long n = std::min<long long>((long long)nph, cap);
    if (n > 0) {
        std::vector<float4> pos(n), dir(n);
        std::vector<float2> tp(n);
        std::vector<uint32_t> path(n);
        RC_CUDA(cudaMemcpy(pos.data(), d.ph_pos.p, 16 * n, cudaMemcpyDeviceToHost));
        RC_CUDA(cudaMemcpy(dir.data(), d.ph_dir.p, 16 * n, cudaMemcpyDeviceToHost));
        RC_CUDA(cudaMemcpy(tp.data(), d.ph_tp.p, 8 * n, cudaMemcpyDeviceToHost));
        RC_CUDA(cudaMemcpy(path.data(), d.ph_path.p, 4 * n, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < n; ++i) {
            float* w = out + 12 * i;
            w[0] = pos[i].x; w[1] = pos[i].y; w[2] = pos[i].z;
            w[3] = dir[i].x; w[4] = dir[i].y; w[5] = dir[i].z;
            w[6] = dir[i].w; w[7] = tp[i].x; w[8] = tp[i].y; w[9] = pos[i].w;
            std::memcpy(&w[10], &path[i], 4);
            w[11] = 0.0f;
        }
    }
    return RC_OK;
}

int rc_trace_rays(int n, const float* origins, const float* directions, float tmin, unsigned* out) {
    int r = prepare();
    if (r) return r;
    if (n < 0 || (n > 0 && (!origins || !directions || !out))) { ctx().err = "bad ray arrays"; return RC_E_INVALID; }
    if (n == 0) return RC_OK;
    cudaStream_t s = ctx().dev.stream;
    DevBuf<float> o, d;
    DevBuf<unsigned> w;
    RC_CUDA(o.reserve(3 * (size_t)n)); RC_CUDA(d.reserve(3 * (size_t)n)); RC_CUDA(w.reserve(8 * (size_t)n));
    RC_CUDA(cudaMemcpyAsync(o.p, origins, 12 * (size_t)n, cudaMemcpyHostToDevice, s));
    RC_CUDA(cudaMemcpyAsync(d.p, directions, 12 * (size_t)n, cudaMemcpyHostToDevice, s));
    launch_trace_rays(ctx().dev.view, n, o.p, d.p, tmin, nullptr, w.p, ctx().dev.errors.p, s);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaMemcpyAsync(out, w.p, 32 * (size_t)n, cudaMemcpyDeviceToHost, s));
    RC_CUDA(cudaStreamSynchronize(s));
    o.release(); d.release(); w.release();
    return check_errors();
}

int rc_trace_rays_full(int n, const float* origins, const float* directions, float tmin, float* out) {
    return rc_trace_rays_shape(n, origins, directions, tmin, out, 0);
}

int rc_trace_rays_shape(int n, const float* origins, const float* directions, float tmin, float* out, int shape) {
    if (shape < 0 || shape > 2) { ctx().err = "traversal shape must be 0, 1 or 2"; return RC_E_INVALID; }
    int r = prepare();
    if (r) return r;
    if (n < 0 || (n > 0 && (!origins || !directions || !out))) { ctx().err = "bad ray arrays"; return RC_E_INVALID; }
    if (n == 0) return RC_OK;
    cudaStream_t s = ctx().dev.stream;
    DevBuf<float> o, d, f;
    RC_CUDA(o.reserve(3 * (size_t)n)); RC_CUDA(d.reserve(3 * (size_t)n)); RC_CUDA(f.reserve(16 * (size_t)n));
    RC_CUDA(cudaMemcpyAsync(o.p, origins, 12 * (size_t)n, cudaMemcpyHostToDevice, s));
    RC_CUDA(cudaMemcpyAsync(d.p, directions, 12 * (size_t)n, cudaMemcpyHostToDevice, s));
    launch_trace_rays(ctx().dev.view, n, o.p, d.p, tmin, f.p, nullptr, ctx().dev.errors.p, s, shape);
    RC_CUDA(cudaGetLastError());
    RC_CUDA(cudaMemcpyAsync(out, f.p, 64 * (size_t)n, cudaMemcpyDeviceToHost, s));
    RC_CUDA(cudaStreamSynchronize(s));
    o.release(); d.release(); f.release();
    return check_errors();
}

static int kd_build_host(int n, const float* positions, DevBuf<float4>& pos, DevBuf<uint2>& nodes, DevBuf<float>& x,
                         DevBuf<float>& y, DevBuf<float>& z, DevBuf<uint32_t>& id, DevBuf<unsigned char>& scratch,
                         DevBuf<float4>& boxes, DevBuf<float4>& t0, KdTree& tree, cudaStream_t s) {
    DevBuf<int> err;
    RC_CUDA(err.reserve(1));
    RC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    std::vector<float4> p4((size_t)n);
    for (int i = 0; i < n; ++i) p4[i] = make_float4(positions[3 * i], positions[3 * i + 1], positions[3 * i + 2], 0.0f);
    RC_CUDA(pos.reserve(std::max(n, 1)));
    if (n) RC_CUDA(cudaMemcpyAsync(pos.p, p4.data(), 16 * (size_t)n, cudaMemcpyHostToDevice, s));
    long long nn = kd_node_array_len(n);
    RC_CUDA(nodes.reserve(std::max<long long>(nn, 2)));
    RC_CUDA(x.reserve(std::max(n, 1))); RC_CUDA(y.reserve(std::max(n, 1)));
    RC_CUDA(z.reserve(std::max(n, 1))); RC_CUDA(id.reserve(std::max(n, 1)));
    RC_CUDA(scratch.reserve(kd_scratch_bytes(n)));
    tree.nodes = nodes.p; tree.x = x.p; tree.y = y.p; tree.z = z.p; tree.id = id.p;
    if (kd_build(pos.p, n, tree, scratch.p, scratch.n, s, nullptr, err.p)) { ctx().err = "KD scratch"; return RC_E_CAPACITY; }
    RC_CUDA(cudaGetLastError());
    tree.box_levels = kd_box_levels(n);
    if (tree.box_levels > 0) {
        RC_CUDA(boxes.reserve((size_t)2 << tree.box_levels));
        tree.box_lo = boxes.p;
        tree.box_hi = boxes.p + ((size_t)1 << tree.box_levels);
        launch_kd_boxes(tree, s, nullptr);
        RC_CUDA(cudaGetLastError());
        RC_CUDA(t0.reserve(std::max(n, 1)));
        launch_tree_records(PhotonBuf{pos.p, nullptr, nullptr, nullptr, n, nullptr}, tree, TreePhotons{t0.p, nullptr, nullptr},
                            s);
        RC_CUDA(cudaGetLastError());
    }
    int h = 0;
    RC_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    RC_CUDA(cudaStreamSynchronize(s));
    err.release();
    if (h) { ctx().err = "KD-tree build found inconsistent counts"; return RC_E_INVALID; }
    return RC_OK;
}

int rc_gather_variants(void) { return gather_variants(); }

int rc_device_bus_id(char* out, int len) {
    if (!out || len < 13) { ctx().err = "bus id buffer too small"; return RC_E_INVALID; }
    int dev = 0;
    RC_CUDA(cudaGetDevice(&dev));
    RC_CUDA(cudaDeviceGetPCIBusId(out, len, dev));
    return RC_OK;
}

int rc_gather_query(int variant, int n, const float* positions, int q, const float* queries, float r2, int* counts,
                    int* idx, long long cap, long long* total) {
    if (n < 0 || q < 0 || (n > 0 && !positions) || (q > 0 && (!queries || !counts))) { ctx().err = "bad KD arrays"; return RC_E_INVALID; }
    if (variant < -1 || variant >= gather_variants()) { ctx().err = "gather variant out of range"; return RC_E_INVALID; }
    if (variant < 0) variant = gather_default_variant();
    cudaStream_t s = nullptr;
    RC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    DevBuf<float4> pos, boxes, t0; DevBuf<uint2> nodes; DevBuf<float> x, y, z, qp; DevBuf<uint32_t> id, ord;
    DevBuf<unsigned char> scratch, osc; DevBuf<int> cnt, cur, out, err; DevBuf<long long> off;
    KdTree tree;
    int r = kd_build_host(n, positions, pos, nodes, x, y, z, id, scratch, boxes, t0, tree, s);
    if (!r && total) *total = 0;
    if (!r && q > 0) {
        r = [&]() -> int {
            RC_CUDA(qp.reserve(3 * (size_t)q)); RC_CUDA(cnt.reserve(q)); RC_CUDA(cur.reserve(q)); RC_CUDA(off.reserve(q));
            RC_CUDA(err.reserve(1)); RC_CUDA(ord.reserve(q));
            RC_CUDA(osc.reserve(query_order_scratch_bytes(q)));
            RC_CUDA(cudaMemcpyAsync(qp.p, queries, 12 * (size_t)q, cudaMemcpyHostToDevice, s));
            RC_CUDA(cudaMemsetAsync(cnt.p, 0, 4 * (size_t)q, s));
            RC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int j = 0; j < q; ++j)
                for (int k = 0; k < 3; ++k) {
                    lo[k] = std::min(lo[k], queries[3 * j + k]);
                    hi[k] = std::max(hi[k], queries[3 * j + k]);
                }
            launch_query_order(qp.p, 3, q, query_frame(lo, hi), osc.p, ord.p, nullptr, s);
            launch_gather_sets(tree, t0.p, qp.p, 3, ord.p, q, r2, cnt.p, nullptr, nullptr, nullptr, variant, nullptr,
                               err.p, s);
            RC_CUDA(cudaGetLastError());
            int h = 0;
            RC_CUDA(cudaMemcpyAsync(counts, cnt.p, 4 * (size_t)q, cudaMemcpyDeviceToHost, s));
            RC_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
            RC_CUDA(cudaStreamSynchronize(s));
            if (h) { ctx().err = "gather traversal stack overflow"; return RC_E_CAPACITY; }
            std::vector<long long> offs(q);
            long long t = 0;
            for (int j = 0; j < q; ++j) { offs[j] = t; t += counts[j]; }
            if (total) *total = t;
            if (idx && t > 0 && t <= cap) {
                RC_CUDA(out.reserve(t));
                RC_CUDA(cudaMemcpyAsync(off.p, offs.data(), 8 * (size_t)q, cudaMemcpyHostToDevice, s));
                RC_CUDA(cudaMemsetAsync(cur.p, 0, 4 * (size_t)q, s));
                launch_gather_sets(tree, t0.p, qp.p, 3, ord.p, q, r2, nullptr, off.p, cur.p, out.p, variant, nullptr,
                                   err.p, s);
                RC_CUDA(cudaGetLastError());
                RC_CUDA(cudaMemcpyAsync(idx, out.p, 4 * (size_t)t, cudaMemcpyDeviceToHost, s));
                RC_CUDA(cudaStreamSynchronize(s));
            }
            return RC_OK;
        }();
    }
    pos.release(); nodes.release(); x.release(); y.release(); z.release(); id.release(); scratch.release();
    cnt.release(); cur.release(); out.release(); off.release(); qp.release(); ord.release(); osc.release();
    boxes.release(); t0.release(); err.release();
    cudaStreamDestroy(s);
    return r;
}

int rc_kd_query(int n, const float* positions, int q, const float* queries, float r2, int* counts, int* idx,
                long long cap, long long* total) {
    return rc_gather_query(-1, n, positions, q, queries, r2, counts, idx, cap, total);
}

int rc_kd_build_nodes(int n, const float* positions, unsigned* nodes_out, long long cap, long long* num_nodes) {
    if (n < 0 || (n > 0 && !positions)) { ctx().err = "bad KD arrays"; return RC_E_INVALID; }
    cudaStream_t s = nullptr;
    RC_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    DevBuf<float4> pos; DevBuf<uint2> nodes; DevBuf<float> x, y, z; DevBuf<uint32_t> id; DevBuf<unsigned char> scratch;
    KdTree tree;
    DevBuf<float4> boxes, t0;
    int r = kd_build_host(n, positions, pos, nodes, x, y, z, id, scratch, boxes, t0, tree, s);
    if (!r) {
        long long nn = kd_node_array_len(n);
        if (num_nodes) *num_nodes = nn;
        if (nodes_out && nn > 0) {
            long long m = std::min(nn, cap);
            cudaError_t e = cudaMemcpyAsync(nodes_out, nodes.p, 8 * (size_t)m, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) { ctx().err = cudaGetErrorString(e); r = RC_E_CUDA; }
        }
    }
    pos.release(); nodes.release(); x.release(); y.release(); z.release(); id.release(); scratch.release();
    boxes.release(); t0.release();
    cudaStreamDestroy(s);
    return r;
}

}  // extern "C"
