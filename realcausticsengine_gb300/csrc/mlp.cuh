// Learned photon-emission proposal: a small MLP (BF16 weights and activations, FP32
// accumulation on the tcgen05 tensor cores) maps an emission position to a mixture
// of 16 von Mises-Fisher lobes over emission directions.
//
// Input: the emission position normalised to the scene box, each coordinate encoded as
// (c, sin(2^k pi c), cos(2^k pi c)) for k = 0..11: 3 x 25 = 75 values, padded to 80.
// Layers 80 -> 64 -> 64 -> 64 -> 80 with ReLU between.  Output per lobe k:
// (logit, mu_raw xyz, kappa_raw) -> weight softmax(logit), mean mu_raw/|mu_raw|,
// concentration 0.1 + softplus(kappa_raw) (at most 2000).
// Proposal density: q(w) = a * p_light(w) + (1 - a) * sum_k pi_k vMF(w; mu_k, kappa_k)
// with the defensive fraction a = 0.2 of the light's own emission density.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "vm.cuh"

namespace rc {

constexpr int kMlpIn = 80, kMlpInReal = 75, kMlpHid = 64, kMlpOut = 80, kMlpLobes = 16, kMlpFreqs = 12;
constexpr int kMlpLayers = 4;
constexpr float kMlpDefensive = 0.2f;

__host__ __device__ constexpr int mlp_in_dim(int l) { return l == 0 ? kMlpIn : kMlpHid; }
__host__ __device__ constexpr int mlp_out_dim(int l) { return l == 3 ? kMlpOut : kMlpHid; }

struct MlpParams {
    __nv_bfloat16* w[kMlpLayers];   // out x in, row-major (the forward weights)
    float* b[kMlpLayers];
    float* wm[kMlpLayers];          // FP32 master weights
    float* gw[kMlpLayers];          // gradients
    float* gb[kMlpLayers];
    float* mw[kMlpLayers];          // Adam moments
    float* vw[kMlpLayers];
    float* mb[kMlpLayers];
    float* vb[kMlpLayers];
    int adam_step;
};

// Training batch buffers (n rows).
struct MlpBatch {
    float4* pos;                    // normalised position (xyz)
    float4* dir;                    // sampled direction (xyz) | weight f / q_old
    float* out;                     // n x 80 network outputs (forward test)
    float* loss;                    // weighted loss of the last step (1 float)
    float* part;                    // per-CTA partial gradients (part_rows x parameters)
    int part_rows;
    int n;
};

// Owns the device buffers of one network (weights, gradients, Adam moments) and one
// training batch of `n` rows.
struct MlpStore {
    MlpParams p{};
    MlpBatch b{};
    std::vector<void*> allocs;
    void* alloc_bytes(size_t bytes);
    template <class T>
    T* alloc(size_t n) { return static_cast<T*>(alloc_bytes(std::max<size_t>(n, 1) * sizeof(T))); }
    bool setup(int n);
    void release();
    MlpStore() = default;
    MlpStore(const MlpStore&) = delete;
    MlpStore& operator=(const MlpStore&) = delete;
    ~MlpStore() { release(); }
};

// Emission proposal for the light pass: per light path index, the emission position
// from the path's own primary samples, the MLP's mixture, a direction sample and the
// throughput factor p_light / q.
struct ProposalCtx {
    LightsView lights;
    float bmin[3], binv[3];   // scene box: normalised position = (p - bmin) * binv
    uint64_t seed;
    uint32_t iteration;
};

size_t mlp_param_floats();
// The tabulated proposal (proposal.cuh): the mixture at the centres of res x res cells
// per light, written to cells (lights x res x res x 80 floats) by the tensor-core forward
// kernel.  The Metropolis samplers draw from it directly.
int mlp_proposal_table(const MlpParams& p, const ProposalCtx& c, int res, float* cells, cudaStream_t s, int* err);
// Emission of n uniformly sampled light paths from the same tabulated proposal: the
// table (into cells), then per path prop[i] = (direction, p_light / q) drawn with the
// path's own samples; the light pass, the light-path order and the training collection
// read prop.
int mlp_proposal(const MlpParams& p, const ProposalCtx& c, int res, float* cells, long long n, float4* prop,
                 cudaStream_t s, int* err);
// The per-path draw alone, from a table already in cells, over the paths in `order`
// (nullptr: index order).
int mlp_proposal_draw(const ProposalCtx& c, int res, const float* cells, long long n, const uint32_t* order,
                      float4* prop, cudaStream_t s);
// Training samples from the light paths that contributed to the image (contrib > 0,
// contrib = the gather's per-path sum of squared per-merge luminance):
// pos4 = (normalised emission position, p_light(dir)), dir4 = (dir, sqrt(contrib)),
// *wsum = the sum of the weights.  *count (device) receives the number of contributing
// paths (may exceed cap; rows beyond cap are dropped).
void mlp_collect(const ProposalCtx& c, long long n, const float* contrib, const float4* prop, int cap,
                 float4* pos4, float4* dir4, unsigned* count, float* wsum, cudaStream_t s);
void mlp_normalize_weights(float4* dir4, int n, const float* wsum, cudaStream_t s);
// `steps` Adam steps on minibatches of b.n rows taken from (pos4, dir4)[0, total).
int mlp_train(MlpParams& p, MlpBatch& b, const float4* pos4, const float4* dir4, int total, int steps, float lr,
              cudaStream_t s, int* err);
// Training state as host floats (per layer: FP32 master weights, biases, the four Adam
// moments) for checkpoints; mlp_import restores it and refreshes the BF16 weights.
size_t mlp_state_floats();
int mlp_export(const MlpParams& p, float* out);
int mlp_import(MlpParams& p, const float* in, int adam_step, cudaStream_t s);
// Initialise weights (seeded), zero Adam state.
int mlp_init(MlpParams& p, uint64_t seed, cudaStream_t s);
// Forward on b.n normalised positions (b.pos) -> b.out (n x 80 FP32).
int mlp_forward_batch(const MlpParams& p, MlpBatch& b, cudaStream_t s, int* err);
// One training step on rows (pos4, dir4)[0, n): forward, loss gradient and backward
// fused in one tensor-core kernel (weight gradients accumulated in TMEM per CTA), then
// the partial sums reduced into gw/gb and, when `apply`, one Adam step (learning rate lr).
// *b.loss receives the step's loss.
int mlp_train_step(MlpParams& p, MlpBatch& b, const float4* pos4, const float4* dir4, int n, float lr, bool apply,
                   cudaStream_t s, int* err);

}  // namespace rc
