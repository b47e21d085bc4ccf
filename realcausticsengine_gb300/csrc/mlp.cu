// MLP emission proposal: tcgen05 forward / backward kernels, loss, Adam.
#include "mlp.cuh"
#include "lights.cuh"
#include "proposal.cuh"
#include "tc_gemm.cuh"
#include "rng.cuh"
#include "dev_once.h"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

namespace rc {

namespace {

constexpr uint32_t kWait = 1u << 22;

// sin/cos(2^k pi c) for k = 0..11: sincospi at k = 0, then the double-angle identities
// sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a (rounding error doubles per step:
// below 3e-4 at k = 11, under the BF16 rounding of the network input).
__device__ __forceinline__ void encode(float px, float py, float pz, float* x) {
    const float c[3] = {px, py, pz};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float sn, cs;
        sincospif(c[i], &sn, &cs);
        x[25 * i] = c[i];
#pragma unroll
        for (int k = 0; k < kMlpFreqs; ++k) {
            x[25 * i + 1 + 2 * k] = sn;
            x[25 * i + 2 + 2 * k] = cs;
            const float s2 = 2.0f * sn * cs;
            cs = 1.0f - 2.0f * sn * sn;
            sn = s2;
        }
    }
#pragma unroll
    for (int o = 3 * (1 + 2 * kMlpFreqs); o < kMlpIn; ++o) x[o] = 0.0f;
}

__device__ __forceinline__ float softplus(float v) { return v > 20.0f ? v : log1pf(expf(v)); }
__device__ __forceinline__ float sigmoid(float v) { return 1.0f / (1.0f + expf(-v)); }

// Mixture parameters from the 80 network outputs.
struct Lobes {
    float pi[kMlpLobes], mx[kMlpLobes], my[kMlpLobes], mz[kMlpLobes], kappa[kMlpLobes], rlen[kMlpLobes];
};

__device__ __forceinline__ void lobes_from(const float* o, Lobes& L) {
    float mxl = -INFINITY;
    for (int k = 0; k < kMlpLobes; ++k) mxl = fmaxf(mxl, o[5 * k]);
    float sum = 0.0f;
    for (int k = 0; k < kMlpLobes; ++k) { L.pi[k] = expf(o[5 * k] - mxl); sum += L.pi[k]; }
    for (int k = 0; k < kMlpLobes; ++k) {
        L.pi[k] /= sum;
        float x = o[5 * k + 1], y = o[5 * k + 2], z = o[5 * k + 3];
        float len = sqrtf(x * x + y * y + z * z);
        len = fmaxf(len, 1e-6f);
        L.rlen[k] = len;
        L.mx[k] = x / len; L.my[k] = y / len; L.mz[k] = z / len;
        L.kappa[k] = fminf(kKappaMin + softplus(o[5 * k + 4]), kKappaMax);
    }
}

__device__ __forceinline__ float vmf_pdf(float kappa, float cosang) {
    return kappa / (2.0f * 3.14159265f * (1.0f - expf(-2.0f * kappa))) * expf(kappa * (cosang - 1.0f));
}

// ----------------------------------------------------------------------------- fused forward
struct SmemFwd {
    static constexpr int w0 = 0;                                  // 64 x 80
    static constexpr int w1 = w0 + 64 * 80 * 2;                   // 64 x 64
    static constexpr int w2 = w1 + 64 * 64 * 2;
    static constexpr int w3 = w2 + 64 * 64 * 2;                   // 80 x 64
    static constexpr int act = w3 + 80 * 64 * 2;                  // 128 x 80 activations, in place
    static constexpr int bias = act + 128 * 80 * 2;               // 272 floats
    static constexpr int total = bias + 272 * 4;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 t = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&t);
}

__device__ __forceinline__ void store_row_bf16(unsigned char* base, int row, const float* v, int K) {
#pragma unroll
    for (int k = 0; k < K; k += 8) {
        const uint4 t = make_uint4(pack_bf16x2(v[k], v[k + 1]), pack_bf16x2(v[k + 2], v[k + 3]),
                                   pack_bf16x2(v[k + 4], v[k + 5]), pack_bf16x2(v[k + 6], v[k + 7]));
        *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, k, K)) = t;
    }
}

// One layer of the fused forward: product on the tensor cores, bias (+ ReLU for the
// hidden layers) in the epilogue; hidden activations go back to the activation tile,
// the output layer's 80 values stay in v.  False if the product did not complete.
template <int L>
__device__ __forceinline__ bool fwd_layer(uint32_t tm, uint32_t lane_base, unsigned char* Act,
                                          const unsigned char* W, const float* bias, float* v, uint64_t* mbar,
                                          uint32_t& phase, int* err) {
    constexpr int K = mlp_in_dim(L), N = mlp_out_dim(L);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc::fence_after_sync();
        tc::gemm_issue(tm, Act, W, K, N, false, mbar);
    }
    const bool ok = tc::mbar_wait(mbar, phase, kWait);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(err, 1);
        return false;
    }
    tc::fence_after_sync();
#pragma unroll
    for (int c = 0; c < N; c += 16) tc::tmem_ld16(tm + lane_base + (uint32_t)c, v + c);
    const float* bl = bias + 64 * L;
    if (L < 3) {
#pragma unroll
        for (int c = 0; c < N; ++c) v[c] = fmaxf(v[c] + bl[c], 0.0f);
        store_row_bf16(Act, threadIdx.x, v, N);
    } else {
#pragma unroll
        for (int c = 0; c < N; ++c) v[c] += bl[c];
    }
    return true;
}

template <class IO>
__global__ void __launch_bounds__(128) k_mlp_forward(const MlpParams P, IO io, long long n, int* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights into the K-major core layout, biases
    unsigned char* Ws[4] = {sm + SmemFwd::w0, sm + SmemFwd::w1, sm + SmemFwd::w2, sm + SmemFwd::w3};
    for (int l = 0; l < 4; ++l) {
        const int in = mlp_in_dim(l), out = mlp_out_dim(l);
        for (int i = tid; i < in * out; i += 128) {
            int r = i / in, c = i % in;
            *reinterpret_cast<__nv_bfloat16*>(Ws[l] + tc::kmajor_offset(r, c, in)) = P.w[l][i];
        }
    }
    float* bias = reinterpret_cast<float*>(sm + SmemFwd::bias);
    for (int i = tid; i < 272; i += 128) {
        int l = i < 64 ? 0 : (i < 128 ? 1 : (i < 192 ? 2 : 3));
        int off = l * 64;
        bias[i] = P.b[l][i - off];
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    // one activation tile: each layer's product is complete (waited on) before its
    // epilogue overwrites the tile with the next layer's input, and every thread's TMEM
    // reads are done (barrier) before the next product reuses TMEM columns 0..79
    unsigned char* Act = sm + SmemFwd::act;
    uint32_t phase = 0;
    bool failed = false;
    for (long long tile = blockIdx.x; tile * 128 < n && !failed; tile += gridDim.x) {
        const long long row = tile * 128 + tid;
        const bool valid = row < n;
        typename IO::State st;
        {
            float x[kMlpIn];
            io.input(row, valid, x, st);
            store_row_bf16(Act, tid, x, kMlpIn);
        }
        float v[kMlpOut];
        failed = !fwd_layer<0>(tm, lane_base, Act, Ws[0], bias, v, &mbar, phase, err) ||
                 !fwd_layer<1>(tm, lane_base, Act, Ws[1], bias, v, &mbar, phase, err) ||
                 !fwd_layer<2>(tm, lane_base, Act, Ws[2], bias, v, &mbar, phase, err) ||
                 !fwd_layer<3>(tm, lane_base, Act, Ws[3], bias, v, &mbar, phase, err);
        if (!failed) io.output(row, valid, v, st);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, 128);
}

struct BatchIO {
    struct State {};
    const float4* pos;
    float* out;
    __device__ __forceinline__ void input(long long row, bool valid, float* x_out, State&) const {
        if (!valid) {
#pragma unroll
            for (int i = 0; i < kMlpIn; ++i) x_out[i] = 0.0f;
            return;
        }
        float4 p = pos[row];
        encode(p.x, p.y, p.z, x_out);
    }
    __device__ __forceinline__ void output(long long row, bool valid, const float* o, const State&) const {
        if (!valid) return;
#pragma unroll
        for (int i = 0; i < kMlpOut; ++i) out[row * kMlpOut + i] = o[i];
    }
};

// ----------------------------------------------------------------------------- proposal

// The tabulated proposal (proposal.cuh): one row per (light, cell); the cell centre's
// position in, the mixture (cumulative lobe weights, unit means, concentrations) out.
struct TableIO {
    struct State {};
    ProposalCtx c;
    int res;
    float* cells;
    __device__ __forceinline__ void input(long long row, bool valid, float* x, State&) const {
        if (!valid) {
#pragma unroll
            for (int i = 0; i < kMlpIn; ++i) x[i] = 0.0f;
            return;
        }
        const int cells_per_light = res * res;
        const int li = (int)(row / cells_per_light), cell = (int)(row % cells_per_light);
        const DevLight& l = c.lights.lights[li];
        const float u1 = ((cell % res) + 0.5f) / (float)res, u2 = ((cell / res) + 0.5f) / (float)res;
        F3 o;
        if (l.type == LIGHT_POINT) o = ld3(l.pos);
        else o = ld3(l.bl) + ld3(l.hz) * u1 + ld3(l.vt) * u2;   // light_position's area/sun mapping
        encode((o.x - c.bmin[0]) * c.binv[0], (o.y - c.bmin[1]) * c.binv[1], (o.z - c.bmin[2]) * c.binv[2], x);
    }
    __device__ __forceinline__ void output(long long row, bool valid, const float* o, const State&) const {
        if (!valid) return;
        float mxl = -INFINITY;
#pragma unroll
        for (int k = 0; k < kMlpLobes; ++k) mxl = fmaxf(mxl, o[5 * k]);
        float e[kMlpLobes], sum = 0.0f;
#pragma unroll
        for (int k = 0; k < kMlpLobes; ++k) { e[k] = __expf(o[5 * k] - mxl); sum += e[k]; }
        float* out = cells + (size_t)row * kProposalCellFloats;
        float cum = 0.0f;
#pragma unroll
        for (int k = 0; k < kMlpLobes; ++k) {
            cum += e[k];
            const float x = o[5 * k + 1], y = o[5 * k + 2], z = o[5 * k + 3];
            const float len = fmaxf(sqrtf(x * x + y * y + z * z), 1e-6f);
            out[5 * k + 0] = k == kMlpLobes - 1 ? 1.0f : cum / sum;   // sampling and density agree
            out[5 * k + 1] = x / len;
            out[5 * k + 2] = y / len;
            out[5 * k + 3] = z / len;
            out[5 * k + 4] = kappa_of(o[5 * k + 4]);
        }
    }
};

__global__ void k_collect(const ProposalCtx c, long long n, const float* __restrict__ contrib,
                          const float4* __restrict__ prop, int cap, float4* pos4, float4* dir4, unsigned* count,
                          float* wsum) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float f = contrib[p];
    if (!(f > 0.0f)) return;
    PathRng g;
    g.init(c.seed, (uint64_t)p, c.iteration, STREAM_LIGHT);
    const U4 b0 = g.block(0), b1 = g.block(1);
    const LightSample ls = light_position(c.lights, u01(b0.a), u01(b0.b), u01(b0.c));
    const DevLight& l = c.lights.lights[ls.idx];
    if (l.type == LIGHT_SUN) return;
    F3 w;
    float q_old, pl;
    if (prop) {
        const float4 pr = prop[p];
        w = f3(pr.x, pr.y, pr.z);
        pl = light_direction_pdf(l, w);
        q_old = pr.w > 0.0f ? pl / pr.w : 0.0f;
    } else {
        w = light_direction(l, u01(b0.d), u01(b1.a));
        pl = light_direction_pdf(l, w);
        q_old = pl;
    }
    if (!(q_old > 0.0f)) return;
    const unsigned slot = atomicAdd(count, 1u);
    if (slot >= (unsigned)cap) return;
    // Per-pixel image variance, summed over pixels, is (1/N) sum_j int F_j(w)^2 / q(w) dw
    // minus a constant (F_j: the path's contribution to pixel j as a function of its
    // emission direction), minimised by q proportional to sqrt(sum_j F_j^2).  The path's
    // throughput already holds p_light / q_old, so the gather's sum of squared per-merge
    // contributions is sum_j (F_j / q_old)^2 and its square root is the importance weight
    // of this direction sample for that target.
    const float wt = sqrtf(f);
    pos4[slot] = make_float4((ls.o.x - c.bmin[0]) * c.binv[0], (ls.o.y - c.bmin[1]) * c.binv[1],
                             (ls.o.z - c.bmin[2]) * c.binv[2], pl);
    dir4[slot] = make_float4(w.x, w.y, w.z, wt);
    atomicAdd(wsum, wt);
}

__global__ void k_norm_weights(float4* dir4, int n, const float* wsum) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float mean = *wsum / (float)n;
    if (mean > 0.0f) dir4[i].w /= mean;
}

// ----------------------------------------------------------------------------- loss gradient
// Per row: L = -w log q(dir) with q = a p_light + (1 - a) sum_k pi_k vMF_k (w = dir.w,
// the light's own density at dir = pl).  g = dL/d(outputs) * inv_n; returns L * inv_n.
__device__ float loss_grad_row(const float* o, float4 d, float pl, float inv_n, float* g) {
    Lobes L;
    lobes_from(o, L);
    const float w = d.w;
    float s[kMlpLobes], ca[kMlpLobes];
    float S = 0.0f;
#pragma unroll
    for (int k = 0; k < kMlpLobes; ++k) {
        ca[k] = L.mx[k] * d.x + L.my[k] * d.y + L.mz[k] * d.z;
        s[k] = L.pi[k] * vmf_pdf(L.kappa[k], ca[k]);
        S += s[k];
    }
    const float q = fmaxf(kMlpDefensive * pl + (1.0f - kMlpDefensive) * S, 1e-20f);
    const float c = -(1.0f - kMlpDefensive) * w * inv_n / q;
#pragma unroll
    for (int k = 0; k < kMlpLobes; ++k) {
        g[5 * k] = c * (s[k] - L.pi[k] * S);
        const float kap = L.kappa[k];
        const float gm = c * s[k] * kap / L.rlen[k];
        g[5 * k + 1] = gm * (d.x - ca[k] * L.mx[k]);
        g[5 * k + 2] = gm * (d.y - ca[k] * L.my[k]);
        g[5 * k + 3] = gm * (d.z - ca[k] * L.mz[k]);
        const float e2 = expf(-2.0f * kap);
        const float dlog = 1.0f / kap - 2.0f * e2 / (1.0f - e2) + (ca[k] - 1.0f);
        const float dk = (kap >= kKappaMax) ? 0.0f : sigmoid(o[5 * k + 4]);
        g[5 * k + 4] = c * s[k] * dlog * dk;
    }
    return -w * logf(q) * inv_n;
}

// ----------------------------------------------------------------------------- fused training step
// One CTA of 128 threads takes 128-row tiles of the batch (thread = row) and runs, per
// tile, the forward pass, the loss gradient and the backward pass on the tensor cores:
//   dW_l += dY_l^T . In_l        (M = 128 (out rows, zero-padded), N = in,  K = 128 rows)
//   db_l += dY_l^T . 1           (N = 16 columns of ones)
//   dX_l  = dY_l . W_l           (M = 128 rows, N = in, K = out), dY_{l-1} = dX_l * relu'(In_l)
// The weight and bias gradients accumulate in TMEM across the CTA's tiles and are
// written once per CTA as a partial sum; k_reduce_adam adds the partials.
// Operands with the batch rows as the reduction dimension (In_l^T, dY_l^T) are written
// transposed by the epilogues: element (feature i, row r) at kmajor_offset(i, r, 128).
struct SmemTrain {
    static constexpr int wf0 = 0;                       // forward weights (out x in), K-major over in
    static constexpr int wf1 = wf0 + 64 * 80 * 2;
    static constexpr int wf2 = wf1 + 64 * 64 * 2;
    static constexpr int wf3 = wf2 + 64 * 64 * 2;
    static constexpr int wt1 = wf3 + 80 * 64 * 2;       // W_l^T (in x out), K-major over out
    static constexpr int wt2 = wt1 + 64 * 64 * 2;
    static constexpr int wt3 = wt2 + 64 * 64 * 2;
    static constexpr int act = wt3 + 64 * 80 * 2;       // 128 x 80 activations (forward A operand)
    static constexpr int xt = act + 128 * 80 * 2;       // X^T 80 x 128
    static constexpr int ht0 = xt + 80 * 128 * 2;       // H_l^T 64 x 128
    static constexpr int ht1 = ht0 + 64 * 128 * 2;
    static constexpr int ht2 = ht1 + 64 * 128 * 2;
    static constexpr int dy = ht2 + 64 * 128 * 2;       // 128 x out output gradients
    static constexpr int dyt = dy + 128 * 80 * 2;       // dY^T 128 x 128, rows >= out zero
    static constexpr int ones = dyt + 128 * 128 * 2;    // 16 x 128 ones
    static constexpr int bias = ones + 16 * 128 * 2;    // 272 floats
    static constexpr int total = bias + 272 * 4;
};
static_assert(SmemTrain::total <= 227 * 1024, "training step shared memory");

// TMEM columns: dW_l accumulators (N = in_l) at 0, 80, 144, 208; db_l (N = 16) at
// 272 + 16 l; per-tile products (N <= 80) at 336.
__device__ __forceinline__ uint32_t col_w(int l) { return l == 0 ? 0u : 16u + 64u * (uint32_t)l; }
__device__ __forceinline__ uint32_t col_b(int l) { return 272u + 16u * (uint32_t)l; }
constexpr uint32_t kColT = 336;

__device__ __forceinline__ void store_col_bf16(unsigned char* base, int r, const float* v, int cnt) {
#pragma unroll
    for (int i = 0; i < cnt; ++i)
        *reinterpret_cast<__nv_bfloat16*>(base + tc::kmajor_offset(i, r, 128)) = __float2bfloat16_rn(v[i]);
}

// MMAs of one K extent without the completion commit (several products share one).
__device__ __forceinline__ void gemm_issue_nc(uint32_t d_tmem, const void* a_smem, const void* b_smem, int K, int N,
                                              bool accumulate) {
    const uint32_t idesc = tc::idesc_bf16_f32(128, N);
    const uint32_t a0 = tc::smem_u32(a_smem), b0 = tc::smem_u32(b_smem);
    const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
    for (int k = 0; k < K; k += 16) {
        const uint64_t ad = tc::smem_desc(a0 + (uint32_t)(k >> 3) * 128u, 128u, sbo);
        const uint64_t bd = tc::smem_desc(b0 + (uint32_t)(k >> 3) * 128u, 128u, sbo);
        tc::mma_bf16(d_tmem, ad, bd, idesc, accumulate || k > 0);
    }
}

__device__ __forceinline__ bool cta_sync_wait(uint64_t* mbar, uint32_t& phase, int* err, int code) {
    const bool ok = tc::mbar_wait(mbar, phase, kWait);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(err, code);
        return false;
    }
    tc::fence_after_sync();
    return true;
}

__device__ __forceinline__ void publish_smem() {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
}

__global__ void __launch_bounds__(128, 1) k_mlp_train(const MlpParams P, const float4* __restrict__ pos,
                                                       const float4* __restrict__ dir, int n, float inv_n,
                                                       float* __restrict__ part, int part_stride,
                                                       float* __restrict__ loss, int* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    unsigned char* Wf[4] = {sm + SmemTrain::wf0, sm + SmemTrain::wf1, sm + SmemTrain::wf2, sm + SmemTrain::wf3};
    unsigned char* Wt[4] = {nullptr, sm + SmemTrain::wt1, sm + SmemTrain::wt2, sm + SmemTrain::wt3};
    unsigned char* InT[4] = {sm + SmemTrain::xt, sm + SmemTrain::ht0, sm + SmemTrain::ht1, sm + SmemTrain::ht2};
    unsigned char* Act = sm + SmemTrain::act;
    unsigned char* Dy = sm + SmemTrain::dy;
    unsigned char* DyT = sm + SmemTrain::dyt;
    unsigned char* Ones = sm + SmemTrain::ones;
    for (int l = 0; l < 4; ++l) {
        const int in = mlp_in_dim(l), out = mlp_out_dim(l);
        for (int i = tid; i < in * out; i += 128) {
            const int o = i / in, c = i % in;
            const __nv_bfloat16 v = P.w[l][i];
            *reinterpret_cast<__nv_bfloat16*>(Wf[l] + tc::kmajor_offset(o, c, in)) = v;
            if (l > 0) *reinterpret_cast<__nv_bfloat16*>(Wt[l] + tc::kmajor_offset(c, o, out)) = v;
        }
    }
    for (int i = tid; i < 128 * 128 * 2 / 16; i += 128) reinterpret_cast<uint4*>(DyT)[i] = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < 16 * 128 * 2 / 16; i += 128)
        reinterpret_cast<uint4*>(Ones)[i] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    float* bias = reinterpret_cast<float*>(sm + SmemTrain::bias);
    for (int i = tid; i < 272; i += 128) {
        const int l = i < 64 ? 0 : (i < 128 ? 1 : (i < 192 ? 2 : 3));
        bias[i] = P.b[l][i - 64 * l];
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
    publish_smem();
    tc::fence_after_sync();
    const uint32_t tm = tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    uint32_t phase = 0;
    bool failed = false, first = true;
    float loss_acc = 0.0f;
    for (long long tile = blockIdx.x; tile * 128 < n && !failed; tile += gridDim.x) {
        const long long row = tile * 128 + tid;
        const bool valid = row < n;
        const float4 pd = valid ? pos[row] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float4 dd = valid ? dir[row] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float v[kMlpOut];
        {
            float x[kMlpIn];
            if (valid) encode(pd.x, pd.y, pd.z, x);
            else for (int i = 0; i < kMlpIn; ++i) x[i] = 0.0f;
            store_row_bf16(Act, tid, x, kMlpIn);
            store_col_bf16(InT[0], tid, x, kMlpIn);
        }
        for (int l = 0; l < 4 && !failed; ++l) {
            const int K = mlp_in_dim(l), N = mlp_out_dim(l);
            publish_smem();
            if (tid == 0) {
                tc::fence_after_sync();
                tc::gemm_issue(tm + kColT, Act, Wf[l], K, N, false, &mbar);
            }
            if (!cta_sync_wait(&mbar, phase, err, 4)) { failed = true; break; }
#pragma unroll
            for (int c = 0; c < N; c += 16) tc::tmem_ld16(tm + lane_base + kColT + (uint32_t)c, v + c);
            const float* bl = bias + 64 * l;
            if (l < 3) {
#pragma unroll
                for (int c = 0; c < N; ++c) v[c] = fmaxf(v[c] + bl[c], 0.0f);
                store_row_bf16(Act, tid, v, N);
                store_col_bf16(InT[l + 1], tid, v, N);
            } else {
#pragma unroll
                for (int c = 0; c < N; ++c) v[c] += bl[c];
            }
        }
        if (failed) break;
        {
            float g[kMlpOut];
            if (valid) loss_acc += loss_grad_row(v, dd, pd.w, inv_n, g);
            else for (int i = 0; i < kMlpOut; ++i) g[i] = 0.0f;
            store_row_bf16(Dy, tid, g, kMlpOut);
            store_col_bf16(DyT, tid, g, kMlpOut);
        }
        for (int l = 3; l >= 0 && !failed; --l) {
            const int in = mlp_in_dim(l), out = mlp_out_dim(l);
            publish_smem();
            if (tid == 0) {
                tc::fence_after_sync();
                gemm_issue_nc(tm + col_w(l), DyT, InT[l], 128, in, !first);
                gemm_issue_nc(tm + col_b(l), DyT, Ones, 128, 16, !first);
                if (l > 0) gemm_issue_nc(tm + kColT, Dy, Wt[l], out, in, false);
                tc::mma_commit(&mbar);
            }
            if (!cta_sync_wait(&mbar, phase, err, 8)) { failed = true; break; }
            if (l == 3) {
                // rows 64..79 of dY^T held the output layer's extra gradients
                uint4* z = reinterpret_cast<uint4*>(DyT + tc::kmajor_offset(64, 0, 128));
                for (int i = tid; i < 16 * 128 * 2 / 16; i += 128) z[i] = make_uint4(0, 0, 0, 0);
            }
            if (l > 0) {
                float g[kMlpHid];
#pragma unroll
                for (int c = 0; c < in; c += 16) tc::tmem_ld16(tm + lane_base + kColT + (uint32_t)c, g + c);
#pragma unroll
                for (int i = 0; i < in; ++i) {
                    const float h = __bfloat162float(
                        *reinterpret_cast<const __nv_bfloat16*>(InT[l] + tc::kmajor_offset(i, tid, 128)));
                    if (!(h > 0.0f)) g[i] = 0.0f;
                }
                store_row_bf16(Dy, tid, g, in);
                store_col_bf16(DyT, tid, g, in);
            }
        }
        first = false;
    }
    for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if ((tid & 31) == 0 && loss_acc != 0.0f) atomicAdd(loss, loss_acc);
    if (!failed && !first) {
        // this CTA's gradient sums, packed like the parameters (per layer: W out x in, b)
        float* mine = part + (size_t)blockIdx.x * part_stride;
        int off = 0;
        for (int l = 0; l < 4; ++l) {
            const int in = mlp_in_dim(l), out = mlp_out_dim(l);
            float t[16];
#pragma unroll
            for (int c = 0; c < in; c += 16) {
                tc::tmem_ld16(tm + lane_base + col_w(l) + (uint32_t)c, t);
                if (tid < out)
                    for (int j = 0; j < 16; ++j) mine[off + tid * in + c + j] = t[j];
            }
            tc::tmem_ld16(tm + lane_base + col_b(l), t);
            if (tid < out) mine[off + out * in + tid] = t[0];
            off += out * in + out;
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, 512);
}

// Sum of the per-CTA partial gradients into gw/gb, then (apply) one Adam step.
__global__ void k_reduce_adam(const MlpParams P, const float* __restrict__ part, int nparts, int total, int apply,
                              float lr, float b1t, float b2t) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= total) return;
    float g = 0.0f;
    for (int b = 0; b < nparts; ++b) g += part[(size_t)b * total + j];
    int l = 0, idx = j;
    for (; l < 3; ++l) {
        const int sz = mlp_in_dim(l) * mlp_out_dim(l) + mlp_out_dim(l);
        if (idx < sz) break;
        idx -= sz;
    }
    const int nw = mlp_in_dim(l) * mlp_out_dim(l);
    const bool is_w = idx < nw;
    const int i = is_w ? idx : idx - nw;
    float* w = is_w ? P.wm[l] : P.b[l];
    float* m = is_w ? P.mw[l] : P.mb[l];
    float* v = is_w ? P.vw[l] : P.vb[l];
    (is_w ? P.gw[l] : P.gb[l])[i] = g;
    if (!apply) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / (1.0f - b1t)) / (sqrtf(vi / (1.0f - b2t)) + eps);
    w[i] = wi;
    if (is_w) P.w[l][i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(const float* w, __nv_bfloat16* wb, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

int sm_count() {
    static const int sms = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n;
    }();
    return sms;
}

// Persistent forward grid: 3 CTAs per SM (58 KB of shared memory and 128 TMEM columns
// each), so one CTA's tensor-core products overlap the others' epilogues.
int forward_blocks() { return 3 * sm_count(); }

}  // namespace

size_t mlp_param_floats() {
    size_t t = 0;
    for (int l = 0; l < kMlpLayers; ++l) t += (size_t)mlp_in_dim(l) * mlp_out_dim(l) + mlp_out_dim(l);
    return t;
}

size_t mlp_state_floats() { return 3 * mlp_param_floats(); }

int mlp_export(const MlpParams& p, float* out) {
    size_t o = 0;
    for (int l = 0; l < kMlpLayers; ++l) {
        const size_t nw = (size_t)mlp_in_dim(l) * mlp_out_dim(l), nb = mlp_out_dim(l);
        const float* src[6] = {p.wm[l], p.b[l], p.mw[l], p.vw[l], p.mb[l], p.vb[l]};
        const size_t cnt[6] = {nw, nb, nw, nw, nb, nb};
        for (int k = 0; k < 6; ++k) {
            if (cudaMemcpy(out + o, src[k], 4 * cnt[k], cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
            o += cnt[k];
        }
    }
    return 0;
}

int mlp_import(MlpParams& p, const float* in, int adam_step, cudaStream_t s) {
    size_t o = 0;
    for (int l = 0; l < kMlpLayers; ++l) {
        const size_t nw = (size_t)mlp_in_dim(l) * mlp_out_dim(l), nb = mlp_out_dim(l);
        float* dst[6] = {p.wm[l], p.b[l], p.mw[l], p.vw[l], p.mb[l], p.vb[l]};
        const size_t cnt[6] = {nw, nb, nw, nw, nb, nb};
        for (int k = 0; k < 6; ++k) {
            if (cudaMemcpyAsync(dst[k], in + o, 4 * cnt[k], cudaMemcpyHostToDevice, s) != cudaSuccess) return -1;
            o += cnt[k];
        }
        k_to_bf16<<<(unsigned)((nw + 255) / 256), 256, 0, s>>>(p.wm[l], p.w[l], (int)nw);
    }
    p.adam_step = adam_step;
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -1;
}

int mlp_init(MlpParams& p, uint64_t seed, cudaStream_t s) {
    // Xavier-uniform weights from a seeded host generator (Philox over the index);
    // biases zero; the output layer's concentrations start broad.
    for (int l = 0; l < kMlpLayers; ++l) {
        const int in = mlp_in_dim(l), out = mlp_out_dim(l);
        const int real_in = l == 0 ? kMlpInReal : in;
        std::vector<float> w((size_t)in * out, 0.0f), b(out, 0.0f);
        const float a = std::sqrt(6.0f / (float)(real_in + out));
        for (int r = 0; r < out; ++r)
            for (int c = 0; c < real_in; ++c) {
                U4 u = philox4x32_10(U4{(uint32_t)(r * in + c), (uint32_t)l, 0x6d6c70u, 0u}, (uint32_t)seed,
                                     (uint32_t)(seed >> 32));
                w[(size_t)r * in + c] = a * (2.0f * u01(u.a) - 1.0f);
            }
        if (l == 3)
            for (int k = 0; k < kMlpLobes; ++k) b[5 * k + 4] = 1.0f;
        if (cudaMemcpyAsync(p.wm[l], w.data(), 4 * w.size(), cudaMemcpyHostToDevice, s) ||
            cudaMemcpyAsync(p.b[l], b.data(), 4 * b.size(), cudaMemcpyHostToDevice, s))
            return -1;
        cudaMemsetAsync(p.mw[l], 0, 4 * w.size(), s);
        cudaMemsetAsync(p.vw[l], 0, 4 * w.size(), s);
        cudaMemsetAsync(p.mb[l], 0, 4 * b.size(), s);
        cudaMemsetAsync(p.vb[l], 0, 4 * b.size(), s);
        k_to_bf16<<<(unsigned)((w.size() + 255) / 256), 256, 0, s>>>(p.wm[l], p.w[l], (int)w.size());
    }
    p.adam_step = 0;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int mlp_forward_batch(const MlpParams& p, MlpBatch& b, cudaStream_t s, int* err) {
    if (b.n <= 0) return 0;
    BatchIO io{b.pos, b.out};
    const size_t smem = SmemFwd::total;
    static std::once_flag attr[kOnceDevices];   // once per device (contexts on several threads launch)
    once_per_device(attr, [&] { cudaFuncSetAttribute(k_mlp_forward<BatchIO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); });
    const long long tiles = (b.n + 127) / 128;
    const int grid = (int)(tiles < forward_blocks() ? tiles : forward_blocks());
    k_mlp_forward<BatchIO><<<grid, 128, smem, s>>>(p, io, b.n, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Per light path, the tabulated proposal's direction and weight p_light / q, from the
// path's own Philox samples: light and area coordinates from block 0 (a, b, c), the
// direction samples the plain path uses (block 0 d, block 1 a) and a sample the plain
// path leaves unused (block 1 b) for the mixture component.  Paths are taken in
// `order` (when given), so that neighbouring threads read the same table cells.
__global__ void k_table_proposal(const ProposalCtx c, const float* __restrict__ cells, int res, long long n,
                                 const uint32_t* __restrict__ order, float4* __restrict__ prop) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const long long i = order ? (long long)__ldg(&order[t]) : t;
    PathRng g;
    g.init(c.seed, (uint64_t)i, c.iteration, STREAM_LIGHT);
    const U4 b0 = g.block(0), b1 = g.block(1);
    const LightSample ls = light_position(c.lights, u01(b0.a), u01(b0.b), u01(b0.c));
    const DevLight& l = c.lights.lights[ls.idx];
    if (l.type == LIGHT_SUN) { prop[i] = make_float4(l.fz[0], l.fz[1], l.fz[2], 1.0f); return; }
    F3 w;
    const float ratio = table_direction(ProposalTable{cells, res}, l, ls.idx, u01(b0.b), u01(b0.c), u01(b0.d),
                                        u01(b1.a), u01(b1.b), w);
    prop[i] = make_float4(w.x, w.y, w.z, ratio);
}

int mlp_proposal(const MlpParams& p, const ProposalCtx& c, int res, float* cells, long long n, float4* prop,
                 cudaStream_t s, int* err) {
    if (n <= 0) return 0;
    if (mlp_proposal_table(p, c, res, cells, s, err)) return -1;
    return mlp_proposal_draw(c, res, cells, n, nullptr, prop, s);
}

int mlp_proposal_draw(const ProposalCtx& c, int res, const float* cells, long long n, const uint32_t* order,
                      float4* prop, cudaStream_t s) {
    if (n <= 0) return 0;
    k_table_proposal<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c, cells, res, n, order, prop);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int mlp_proposal_table(const MlpParams& p, const ProposalCtx& c, int res, float* cells, cudaStream_t s, int* err) {
    const long long n = (long long)c.lights.count * res * res;
    if (n <= 0) return 0;
    TableIO io{c, res, cells};
    const size_t smem = SmemFwd::total;
    static std::once_flag attr[kOnceDevices];   // once per device (contexts on several threads launch)
    once_per_device(attr, [&] { cudaFuncSetAttribute(k_mlp_forward<TableIO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); });
    const long long tiles = (n + 127) / 128;
    const int grid = (int)(tiles < forward_blocks() ? tiles : forward_blocks());
    k_mlp_forward<TableIO><<<grid, 128, smem, s>>>(p, io, n, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void mlp_collect(const ProposalCtx& c, long long n, const float* contrib, const float4* prop, int cap, float4* pos4,
                 float4* dir4, unsigned* count, float* wsum, cudaStream_t s) {
    if (n <= 0) return;
    cudaMemsetAsync(count, 0, sizeof(unsigned), s);
    cudaMemsetAsync(wsum, 0, sizeof(float), s);
    k_collect<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c, n, contrib, prop, cap, pos4, dir4, count, wsum);
}

void mlp_normalize_weights(float4* dir4, int n, const float* wsum, cudaStream_t s) {
    if (n <= 0) return;
    k_norm_weights<<<(n + 255) / 256, 256, 0, s>>>(dir4, n, wsum);
}

int mlp_train_step(MlpParams& p, MlpBatch& b, const float4* pos4, const float4* dir4, int n, float lr, bool apply,
                   cudaStream_t s, int* err) {
    if (n <= 0) return 0;
    const size_t smem = SmemTrain::total;
    static std::once_flag attr[kOnceDevices];   // once per device (contexts on several threads launch)
    once_per_device(attr, [&] { cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); });
    const int total = (int)mlp_param_floats();
    const int tiles = (n + 127) / 128;
    const int grid = std::min(std::min(tiles, sm_count()), b.part_rows);
    cudaMemsetAsync(b.loss, 0, sizeof(float), s);
    k_mlp_train<<<grid, 128, smem, s>>>(p, pos4, dir4, n, 1.0f / (float)n, b.part, total, b.loss, err);
    if (apply) p.adam_step++;
    const float b1t = std::pow(0.9f, (float)std::max(p.adam_step, 1));
    const float b2t = std::pow(0.999f, (float)std::max(p.adam_step, 1));
    k_reduce_adam<<<(total + 255) / 256, 256, 0, s>>>(p, b.part, grid, total, apply ? 1 : 0, lr, b1t, b2t);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int mlp_train(MlpParams& p, MlpBatch& b, const float4* pos4, const float4* dir4, int total, int steps, float lr,
              cudaStream_t s, int* err) {
    if (total <= 0 || steps <= 0) return 0;
    const int bn = b.n < total ? b.n : total;
    for (int i = 0; i < steps; ++i) {
        const int span = total - bn;
        const int off = span > 0 ? (int)(((long long)i * 7919 * bn) % (span + 1)) : 0;
        if (mlp_train_step(p, b, pos4 + off, dir4 + off, bn, lr, true, s, err)) return -1;
    }
    return 0;
}

void* MlpStore::alloc_bytes(size_t bytes) {
    void* ptr = nullptr;
    if (cudaMalloc(&ptr, bytes) != cudaSuccess) return nullptr;
    cudaMemset(ptr, 0, bytes);
    allocs.push_back(ptr);
    return ptr;
}

bool MlpStore::setup(int n) {
    release();
    for (int l = 0; l < kMlpLayers; ++l) {
        const size_t nw = (size_t)mlp_in_dim(l) * mlp_out_dim(l), nb = mlp_out_dim(l);
        p.w[l] = alloc<__nv_bfloat16>(nw); p.b[l] = alloc<float>(nb); p.wm[l] = alloc<float>(nw);
        p.gw[l] = alloc<float>(nw); p.gb[l] = alloc<float>(nb); p.mw[l] = alloc<float>(nw);
        p.vw[l] = alloc<float>(nw); p.mb[l] = alloc<float>(nb); p.vb[l] = alloc<float>(nb);
    }
    b.n = n;
    b.pos = alloc<float4>(n); b.dir = alloc<float4>(n);
    b.out = alloc<float>((size_t)n * kMlpOut);
    b.loss = alloc<float>(1);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    b.part_rows = std::max(sms, 1);
    b.part = alloc<float>((size_t)b.part_rows * mlp_param_floats());
    for (void* a : allocs) if (!a) return false;
    return true;
}

void MlpStore::release() {
    for (void* a : allocs) if (a) cudaFree(a);
    allocs.clear();
    p = MlpParams{};
    b = MlpBatch{};
}

}  // namespace rc

// ----------------------------------------------------------------------------- test hooks
namespace rc {
namespace {

struct HostMlp : MlpStore {
    void set_weights(const float* packed) {
        size_t o = 0;
        for (int l = 0; l < kMlpLayers; ++l) {
            const size_t nw = (size_t)mlp_in_dim(l) * mlp_out_dim(l), nb = mlp_out_dim(l);
            cudaMemcpy(p.wm[l], packed + o, 4 * nw, cudaMemcpyHostToDevice); o += nw;
            cudaMemcpy(p.b[l], packed + o, 4 * nb, cudaMemcpyHostToDevice); o += nb;
            k_to_bf16<<<(unsigned)((nw + 255) / 256), 256>>>(p.wm[l], p.w[l], (int)nw);
        }
    }
    void get(float* const* src_w, float* const* src_b, float* packed) {
        size_t o = 0;
        for (int l = 0; l < kMlpLayers; ++l) {
            const size_t nw = (size_t)mlp_in_dim(l) * mlp_out_dim(l), nb = mlp_out_dim(l);
            cudaMemcpy(packed + o, src_w[l], 4 * nw, cudaMemcpyDeviceToHost); o += nw;
            cudaMemcpy(packed + o, src_b[l], 4 * nb, cudaMemcpyDeviceToHost); o += nb;
        }
    }
};

}  // namespace
}  // namespace rc

// Test hooks (no counterpart in the reference).  Parameters are packed per layer as
// W (out x in, row-major; layer 0 in = 80 with columns 75..79 unused) then b.
extern "C" int rc_mlp_param_count(void) { return (int)rc::mlp_param_floats(); }

// Forward pass on the tensor cores: pos4 (n x 4 floats, xyz normalised) -> out (n x 80).
extern "C" int rc_mlp_forward_test(int n, const float* params, const float* pos4, float* out) {
    using namespace rc;
    if (n <= 0 || !params || !pos4 || !out) return -2;
    HostMlp m;
    if (!m.setup(n)) return -3;
    m.set_weights(params);
    cudaMemcpy(m.b.pos, pos4, 16 * (size_t)n, cudaMemcpyHostToDevice);
    int* err = m.alloc<int>(1);
    if (mlp_forward_batch(m.p, m.b, 0, err)) return -3;
    int h = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) return -3;
    cudaMemcpy(&h, err, 4, cudaMemcpyDeviceToHost);
    if (h) return -6;
    cudaMemcpy(out, m.b.out, 4 * (size_t)n * kMlpOut, cudaMemcpyDeviceToHost);
    return 0;
}

// Loss and gradients (the fused training step without the Adam update): pos4 (xyz,
// w = light density at dir), dir4 (xyz, w = sample weight); grads packed like params;
// *loss = mean weighted negative log-likelihood.
extern "C" int rc_mlp_grad_test(int n, const float* params, const float* pos4, const float* dir4, float* grads,
                                float* loss) {
    using namespace rc;
    if (n <= 0 || !params || !pos4 || !dir4 || !grads || !loss) return -2;
    HostMlp m;
    if (!m.setup(n)) return -3;
    m.set_weights(params);
    cudaMemcpy(m.b.pos, pos4, 16 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(m.b.dir, dir4, 16 * (size_t)n, cudaMemcpyHostToDevice);
    int* err = m.alloc<int>(1);
    if (mlp_train_step(m.p, m.b, m.b.pos, m.b.dir, n, 0.0f, false, 0, err)) return -3;
    if (cudaDeviceSynchronize() != cudaSuccess) return -3;
    int h = 0;
    cudaMemcpy(&h, err, 4, cudaMemcpyDeviceToHost);
    if (h) return -6;
    m.get(m.p.gw, m.p.gb, grads);
    cudaMemcpy(loss, m.b.loss, 4, cudaMemcpyDeviceToHost);
    return 0;
}

// `steps` Adam steps (learning rate lr) on one fixed batch; losses[i] = loss before step i.
extern "C" int rc_mlp_train_test(int n, const float* params, const float* pos4, const float* dir4, int steps,
                                 float lr, float* losses, float* params_out) {
    using namespace rc;
    if (n <= 0 || steps <= 0 || !params || !pos4 || !dir4 || !losses) return -2;
    HostMlp m;
    if (!m.setup(n)) return -3;
    m.set_weights(params);
    cudaMemcpy(m.b.pos, pos4, 16 * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemcpy(m.b.dir, dir4, 16 * (size_t)n, cudaMemcpyHostToDevice);
    int* err = m.alloc<int>(1);
    for (int i = 0; i < steps; ++i) {
        if (mlp_train_step(m.p, m.b, m.b.pos, m.b.dir, n, lr, true, 0, err)) return -3;
        cudaMemcpy(&losses[i], m.b.loss, 4, cudaMemcpyDeviceToHost);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return -3;
    int h = 0;
    cudaMemcpy(&h, err, 4, cudaMemcpyDeviceToHost);
    if (h) return -6;
    if (params_out) m.get(m.p.wm, m.p.b, params_out);
    return 0;
}
