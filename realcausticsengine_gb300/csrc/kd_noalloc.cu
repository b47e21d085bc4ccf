// Photon KD-tree build for callers that cannot allocate GPU memory.
//
// Some hosts of this library cannot call cudaMalloc at the moment they want a photon
// tree: a renderer running inside another application's frame loop that hands the
// library only pre-allocated device buffers, an allocator-owned context (a memory
// pool whose owner forbids foreign allocations), or code that must not block on the
// allocator's implicit synchronisation.  For them rc_kd_build_noalloc builds the same
// tree as rc_kd_build_nodes / the renderer, with its working memory taken from one
// fixed array compiled into this library instead of allocated per call.
//
// The array (`g_kd_scratch`) is a file-scope __device__ object: every GPU that loads
// the library holds it until the process exits.  Host code cannot use its name as a
// device address, so the first call on each device, with that device current, looks
// the address up with cudaGetSymbolAddress and caches it.  Every call reads an error
// flag back and synchronises its stream before returning, so no call may be issued
// while that stream is being captured into a CUDA graph.  All calls share the array
// and it keeps the previous call's contents; the build clears every part it reads
// before using it.  Calls whose work overlaps on the GPU (concurrent streams, or
// threads sharing a device) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "kdtree.cuh"
#include "realcaustics.h"

namespace rc {

namespace {

// Largest photon count the fixed scratch holds (sized by kd_scratch_bytes).
constexpr long long kNoAllocMaxPhotons = 1LL << 19;
constexpr size_t kNoAllocScratchBytes = 16u * (size_t)kNoAllocMaxPhotons + (1u << 20);

static __device__ __align__(256) unsigned char g_kd_scratch[kNoAllocScratchBytes];
static __device__ __align__(16) int g_kd_error;

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
int* g_error_ptr[kMaxDevices] = {};
std::mutex g_setup_mutex;
thread_local char g_noalloc_err[256];

int fail(int code, const char* msg) {
    snprintf(g_noalloc_err, sizeof(g_noalloc_err), "%s", msg);
    return code;
}

}  // namespace

}  // namespace rc

extern "C" const char* rc_kd_noalloc_last_error(void) { return rc::g_noalloc_err; }

extern "C" int rc_kd_build_noalloc(const float* positions4, long long n, unsigned* nodes, long long node_cap,
                                   float* x, float* y, float* z, unsigned* ids, void* stream) {
    using namespace rc;
    g_noalloc_err[0] = 0;
    if (n < 0 || n > kNoAllocMaxPhotons) return fail(RC_E_CAPACITY, "photon count outside [0, 524288]");
    if (n > 0 && (!positions4 || !nodes || !x || !y || !z || !ids)) return fail(RC_E_INVALID, "null device buffer");
    long long need = kd_node_array_len(n);
    if (node_cap < need) return fail(RC_E_CAPACITY, "node buffer smaller than the tree's node array");
    if (kd_scratch_bytes(n) > kNoAllocScratchBytes) return fail(RC_E_CAPACITY, "scratch too small for this count");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(RC_E_CUDA, "cudaGetDevice failed");
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {
            void* s = nullptr;
            void* e = nullptr;
            cudaError_t r1 = cudaGetSymbolAddress(&s, g_kd_scratch);
            cudaError_t r2 = cudaGetSymbolAddress(&e, g_kd_error);
            if (r1 != cudaSuccess || r2 != cudaSuccess || !s || !e)
                return fail(RC_E_CUDA, "cudaGetSymbolAddress of the fixed scratch failed");
            g_scratch_ptr[dev] = s;
            g_error_ptr[dev] = static_cast<int*>(e);
        }
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int* err = g_error_ptr[dev];
    // a launch error left by an earlier, unrelated call would otherwise be reported as
    // this call's
    (void)cudaGetLastError();
    if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return fail(RC_E_CUDA, "cudaMemsetAsync failed");
    KdTree tree;
    tree.nodes = reinterpret_cast<uint2*>(nodes);
    tree.x = x; tree.y = y; tree.z = z; tree.id = ids;
    if (kd_build(reinterpret_cast<const float4*>(positions4), n, tree, g_scratch_ptr[dev], kNoAllocScratchBytes, st,
                 nullptr, err))
        return fail(RC_E_CAPACITY, "scratch too small");
    if (cudaGetLastError() != cudaSuccess) return fail(RC_E_CUDA, "kernel launch failed");
    int h = 0;
    if (cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(RC_E_CUDA, "synchronisation failed");
    if (h) return fail(RC_E_INVALID, "KD-tree build found inconsistent counts");
    return RC_OK;
}
