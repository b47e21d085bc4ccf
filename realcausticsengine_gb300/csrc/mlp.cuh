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
#include <cstdint>
#include <cuda_runtime.h>

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
    __nv_bfloat16* x;               // n x 80 encoded inputs
    __nv_bfloat16* h[3];            // n x 64 post-ReLU activations
    float* out;                     // n x 80 network outputs
    __nv_bfloat16* dy[kMlpLayers];  // n x out_dim(l) gradients w.r.t. pre-activations
    float* loss;                    // accumulated weighted loss (1 float)
    int n;
};

// Proposal context for the light pass.
struct ProposalView {
    const float4* prop;             // per light path: direction xyz | p_light / q
    int enabled;
};

size_t mlp_param_floats();
// Initialise weights (seeded), zero Adam state.
int mlp_init(MlpParams& p, uint64_t seed, cudaStream_t s);
// Forward on `n` normalised positions -> outputs (n x 80 FP32); saves activations when
// the batch buffers are given.
int mlp_forward_batch(const MlpParams& p, MlpBatch& b, cudaStream_t s, int* err);
// Loss and its gradient w.r.t. the outputs, backward through the layers, weight and
// bias gradients (zeroed first).  Tensor-core GEMMs for all matrix products.
int mlp_backward_batch(const MlpParams& p, MlpBatch& b, cudaStream_t s, int* err);
void mlp_adam(MlpParams& p, float lr, cudaStream_t s);

}  // namespace rc
