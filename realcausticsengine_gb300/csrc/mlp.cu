// MLP emission proposal: tcgen05 forward / backward kernels, loss, Adam.
#include "mlp.cuh"
#include "tc_gemm.cuh"
#include "rng.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace rc {

namespace {

constexpr uint32_t kWait = 1u << 22;
constexpr float kKappaMin = 0.1f, kKappaMax = 2000.0f;

__device__ __forceinline__ void encode(float px, float py, float pz, float* x) {
    const float c[3] = {px, py, pz};
    int o = 0;
    for (int i = 0; i < 3; ++i) {
        x[o++] = c[i];
        float f = 1.0f;
        for (int k = 0; k < kMlpFreqs; ++k) {
            float s, co;
            sincospif(f * c[i], &s, &co);
            x[o++] = s;
            x[o++] = co;
            f *= 2.0f;
        }
    }
    for (; o < kMlpIn; ++o) x[o] = 0.0f;
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
    static constexpr int x = w3 + 80 * 64 * 2;                    // 128 x 80
    static constexpr int h0 = x + 128 * 80 * 2;                   // 128 x 64
    static constexpr int h1 = h0 + 128 * 64 * 2;
    static constexpr int bias = h1 + 128 * 64 * 2;                // 272 floats
    static constexpr int total = bias + 272 * 4;
};

__device__ __forceinline__ void store_row_bf16(unsigned char* base, int row, const float* v, int K) {
    for (int k = 0; k < K; k += 8) {
        __align__(16) __nv_bfloat16 t[8];
        for (int j = 0; j < 8; ++j) t[j] = __float2bfloat16_rn(v[k + j]);
        *reinterpret_cast<uint4*>(base + tc::kmajor_offset(row, k, K)) = *reinterpret_cast<const uint4*>(t);
    }
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
    if (warp == 0) tc::tmem_alloc(&tmem_base, 256);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    unsigned char* Xs = sm + SmemFwd::x;
    unsigned char* H[2] = {sm + SmemFwd::h0, sm + SmemFwd::h1};
    uint32_t phase = 0;
    bool failed = false;
    for (long long tile = blockIdx.x; tile * 128 < n && !failed; tile += gridDim.x) {
        const long long row = tile * 128 + tid;
        const bool valid = row < n;
        {
            float x[kMlpIn];
            io.input(row, valid, x);
            store_row_bf16(Xs, tid, x, kMlpIn);
        }
        const unsigned char* a_in = Xs;
        for (int l = 0; l < 4 && !failed; ++l) {
            const int K = mlp_in_dim(l), N = mlp_out_dim(l);
            const uint32_t dcol = (l == 3) ? 128u : ((l & 1) ? 64u : 0u);
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                tc::gemm_issue(tm + dcol, a_in, Ws[l], K, N, false, &mbar);
            }
            bool ok = tc::mbar_wait(&mbar, phase, kWait);
            phase ^= 1u;
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicOr(err, 1);
                failed = true;
                break;
            }
            tc::fence_after_sync();
            float v[kMlpOut];
            for (int c = 0; c < N; c += 16) tc::tmem_ld16(tm + lane_base + dcol + (uint32_t)c, v + c);
            const float* bl = bias + 64 * l;
            if (l < 3) {
                for (int c = 0; c < N; ++c) v[c] = fmaxf(v[c] + bl[c], 0.0f);
                io.save_hidden(l, row, valid, v);
                store_row_bf16(H[l & 1], tid, v, N);
                a_in = H[l & 1];
            } else {
                for (int c = 0; c < N; ++c) v[c] += bl[c];
                io.output(row, valid, v);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, 256);
}

struct BatchIO {
    const float4* pos;
    __nv_bfloat16* x;
    __nv_bfloat16* h0; __nv_bfloat16* h1; __nv_bfloat16* h2;
    float* out;
    __device__ void input(long long row, bool valid, float* x_out) const {
        if (!valid) { for (int i = 0; i < kMlpIn; ++i) x_out[i] = 0.0f; return; }
        float4 p = pos[row];
        encode(p.x, p.y, p.z, x_out);
        if (x) for (int i = 0; i < kMlpIn; ++i) x[row * kMlpIn + i] = __float2bfloat16_rn(x_out[i]);
    }
    __device__ void save_hidden(int l, long long row, bool valid, const float* h) const {
        __nv_bfloat16* dst = l == 0 ? h0 : (l == 1 ? h1 : h2);
        if (!valid || !dst) return;
        for (int i = 0; i < kMlpHid; ++i) dst[row * kMlpHid + i] = __float2bfloat16_rn(h[i]);
    }
    __device__ void output(long long row, bool valid, const float* o) const {
        if (!valid) return;
        for (int i = 0; i < kMlpOut; ++i) out[row * kMlpOut + i] = o[i];
    }
};

// ----------------------------------------------------------------------------- generic GEMM
// D[m][n] = sum_k A(m, k) B(n, k); A(m, k) = A[m*sam + k*sak], B(n, k) = B[n*sbn + k*sbk].
// One CTA: 128 rows of D, a K range [k0, k1) staged 128 at a time.
// mode 0: out[m*N + n] = D; 1: atomicAdd(out[m*N + n], D); 2: outb[m*N + n] = bf16(D if mask[m*N+n] > 0 else 0)
struct GemmArgs {
    const __nv_bfloat16* A; long long sam, sak;
    const __nv_bfloat16* B; long long sbn, sbk;
    long long M, K;
    int N;
    int mode;
    float* out;
    __nv_bfloat16* outb;
    const __nv_bfloat16* mask;
    long long kchunk;
};

__global__ void __launch_bounds__(128) k_tc_gemm(const GemmArgs g, int* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    unsigned char* As = sm;                 // 128 x 128
    unsigned char* Bs = sm + 128 * 128 * 2; // N x 128
    const long long m0 = (long long)blockIdx.x * 128;
    const long long k0 = (long long)blockIdx.y * g.kchunk;
    const long long k1 = k0 + g.kchunk < g.K ? k0 + g.kchunk : g.K;
    if (tid == 0) tc::mbar_init(&mbar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = tmem_base;
    uint32_t phase = 0;
    bool failed = false, any = false;
    for (long long ks = k0; ks < k1; ks += 128) {
        const int kk = (int)((k1 - ks) < 128 ? (k1 - ks) : 128);
        const int KS = (kk + 15) & ~15;
        for (int i = tid; i < 128 * KS; i += 128) {
            const int r = i / KS, c = i % KS;
            const long long m = m0 + r, k = ks + c;
            __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
            if (m < g.M && c < kk) v = g.A[m * g.sam + k * g.sak];
            *reinterpret_cast<__nv_bfloat16*>(As + tc::kmajor_offset(r, c, KS)) = v;
        }
        for (int i = tid; i < g.N * KS; i += 128) {
            const int r = i / KS, c = i % KS;
            const long long k = ks + c;
            __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
            if (c < kk) v = g.B[(long long)r * g.sbn + k * g.sbk];
            *reinterpret_cast<__nv_bfloat16*>(Bs + tc::kmajor_offset(r, c, KS)) = v;
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            tc::gemm_issue(tm, As, Bs, KS, g.N, any, &mbar);
        }
        bool ok = tc::mbar_wait(&mbar, phase, kWait);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(err, 2);
            failed = true;
            break;
        }
        tc::fence_after_sync();
        any = true;
    }
    if (!failed && any) {
        const long long m = m0 + tid;
        float v[128];
        for (int c = 0; c < g.N; c += 16) tc::tmem_ld16(tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v + c);
        if (m < g.M) {
            for (int c = 0; c < g.N; ++c) {
                const long long o = m * g.N + c;
                if (g.mode == 0) g.out[o] = v[c];
                else if (g.mode == 1) atomicAdd(&g.out[o], v[c]);
                else g.outb[o] = __float2bfloat16_rn(__bfloat162float(g.mask[o]) > 0.0f ? v[c] : 0.0f);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, 128);
}

// ----------------------------------------------------------------------------- loss, biases, Adam
// L = -w log q(dir) with q = a p_light + (1 - a) sum_k pi_k vMF_k (w = dir.w, the
// light's own density p_light at dir = pos.w).  Gradient w.r.t. the 80 outputs, / n.
__global__ void k_loss_grad(const float* __restrict__ out, const float4* __restrict__ dir,
                            const float4* __restrict__ pos, int n, __nv_bfloat16* __restrict__ dy,
                            float* __restrict__ loss) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    const float* o = out + (long long)row * kMlpOut;
    Lobes L;
    lobes_from(o, L);
    const float4 d = dir[row];
    const float w = d.w;
    float s[kMlpLobes], ca[kMlpLobes];
    float S = 0.0f;
    for (int k = 0; k < kMlpLobes; ++k) {
        ca[k] = L.mx[k] * d.x + L.my[k] * d.y + L.mz[k] * d.z;
        s[k] = L.pi[k] * vmf_pdf(L.kappa[k], ca[k]);
        S += s[k];
    }
    const float pl = pos[row].w;   // the light's own emission density at dir
    const float q = fmaxf(kMlpDefensive * pl + (1.0f - kMlpDefensive) * S, 1e-20f);
    atomicAdd(loss, -w * logf(q) / n);
    const float c = -(1.0f - kMlpDefensive) * w / (q * n);
    for (int k = 0; k < kMlpLobes; ++k) {
        float g[5];
        g[0] = c * (s[k] - L.pi[k] * S);
        const float kap = L.kappa[k];
        const float gm = c * s[k] * kap / L.rlen[k];
        g[1] = gm * (d.x - ca[k] * L.mx[k]);
        g[2] = gm * (d.y - ca[k] * L.my[k]);
        g[3] = gm * (d.z - ca[k] * L.mz[k]);
        const float e2 = expf(-2.0f * kap);
        const float dlog = 1.0f / kap - 2.0f * e2 / (1.0f - e2) + (ca[k] - 1.0f);
        const float raw = o[5 * k + 4];
        const float dk = (kap >= kKappaMax) ? 0.0f : sigmoid(raw);
        g[4] = c * s[k] * dlog * dk;
        for (int j = 0; j < 5; ++j) dy[(long long)row * kMlpOut + 5 * k + j] = __float2bfloat16_rn(g[j]);
    }
}

__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dy, int n, int cols, float* __restrict__ gb) {
    const int c = blockIdx.x;
    float acc = 0.0f;
    for (int r = threadIdx.x; r < n; r += blockDim.x) acc += __bfloat162float(dy[(long long)r * cols + c]);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ float ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += ws[i];
        gb[c] = t;
    }
}

__global__ void k_adam(float* w, float* m, float* v, const float* g, __nv_bfloat16* wb, int n, float lr, float b1t,
                       float b2t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float gi = g[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi; v[i] = vi;
    float mh = mi / (1.0f - b1t), vh = vi / (1.0f - b2t);
    float wi = w[i] - lr * mh / (sqrtf(vh) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(const float* w, __nv_bfloat16* wb, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

int forward_blocks() {
    static int blocks = 0;
    if (!blocks) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        blocks = 2 * sms;
    }
    return blocks;
}

int launch_gemm(const GemmArgs& g, cudaStream_t s, int* err) {
    const unsigned gx = (unsigned)((g.M + 127) / 128);
    const unsigned gy = (unsigned)((g.K + g.kchunk - 1) / g.kchunk);
    const size_t smem = 128 * 128 * 2 + 128 * 128 * 2;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    k_tc_gemm<<<dim3(gx, gy), 128, smem, s>>>(g, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

size_t mlp_param_floats() {
    size_t t = 0;
    for (int l = 0; l < kMlpLayers; ++l) t += (size_t)mlp_in_dim(l) * mlp_out_dim(l) + mlp_out_dim(l);
    return t;
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
    BatchIO io{b.pos, b.x, b.h[0], b.h[1], b.h[2], b.out};
    const size_t smem = SmemFwd::total;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_mlp_forward<BatchIO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    const long long tiles = (b.n + 127) / 128;
    const int grid = (int)(tiles < forward_blocks() ? tiles : forward_blocks());
    k_mlp_forward<BatchIO><<<grid, 128, smem, s>>>(p, io, b.n, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int mlp_backward_batch(const MlpParams& p, MlpBatch& b, cudaStream_t s, int* err) {
    const int n = b.n;
    if (n <= 0) return 0;
    for (int l = 0; l < kMlpLayers; ++l) {
        cudaMemsetAsync(p.gw[l], 0, 4 * (size_t)mlp_in_dim(l) * mlp_out_dim(l), s);
        cudaMemsetAsync(p.gb[l], 0, 4 * (size_t)mlp_out_dim(l), s);
    }
    cudaMemsetAsync(b.loss, 0, sizeof(float), s);
    k_loss_grad<<<(n + 127) / 128, 128, 0, s>>>(b.out, b.dir, b.pos, n, b.dy[3], b.loss);
    // activation gradients: dy[l] = (dy[l+1] . W[l+1]) * relu'(h[l])
    for (int l = 2; l >= 0; --l) {
        GemmArgs g{};
        const int out_next = mlp_out_dim(l + 1), in_next = mlp_in_dim(l + 1);
        g.A = b.dy[l + 1]; g.sam = out_next; g.sak = 1;
        g.B = p.w[l + 1]; g.sbn = 1; g.sbk = in_next;
        g.M = n; g.K = out_next; g.N = in_next; g.mode = 2;
        g.outb = b.dy[l]; g.mask = b.h[l]; g.kchunk = 128;
        if (launch_gemm(g, s, err)) return -1;
    }
    // weight gradients: gw[l] (out x in) = sum_rows dy[l]^T . in[l]
    for (int l = 0; l < kMlpLayers; ++l) {
        GemmArgs g{};
        const int out = mlp_out_dim(l), in = mlp_in_dim(l);
        g.A = b.dy[l]; g.sam = 1; g.sak = out;
        g.B = l == 0 ? b.x : b.h[l - 1]; g.sbn = 1; g.sbk = in;
        g.M = out; g.K = n; g.N = in; g.mode = 1; g.out = p.gw[l]; g.kchunk = 1024;
        if (launch_gemm(g, s, err)) return -1;
        k_bias_grad<<<out, 256, 0, s>>>(b.dy[l], n, out, p.gb[l]);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

void mlp_adam(MlpParams& p, float lr, cudaStream_t s) {
    p.adam_step++;
    const float b1t = std::pow(0.9f, (float)p.adam_step), b2t = std::pow(0.999f, (float)p.adam_step);
    for (int l = 0; l < kMlpLayers; ++l) {
        const int nw = mlp_in_dim(l) * mlp_out_dim(l), nb = mlp_out_dim(l);
        k_adam<<<(nw + 255) / 256, 256, 0, s>>>(p.wm[l], p.mw[l], p.vw[l], p.gw[l], p.w[l], nw, lr, b1t, b2t);
        k_adam<<<(nb + 255) / 256, 256, 0, s>>>(p.b[l], p.mb[l], p.vb[l], p.gb[l], nullptr, nb, lr, b1t, b2t);
    }
}

}  // namespace rc

// ----------------------------------------------------------------------------- test hooks
namespace rc {
namespace {

struct HostMlp {
    MlpParams p{};
    MlpBatch b{};
    std::vector<void*> allocs;
    template <class T> T* alloc(size_t n) {
        void* ptr = nullptr;
        if (cudaMalloc(&ptr, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        cudaMemset(ptr, 0, std::max<size_t>(n, 1) * sizeof(T));
        allocs.push_back(ptr);
        return static_cast<T*>(ptr);
    }
    bool setup(int n) {
        for (int l = 0; l < kMlpLayers; ++l) {
            const size_t nw = (size_t)mlp_in_dim(l) * mlp_out_dim(l), nb = mlp_out_dim(l);
            p.w[l] = alloc<__nv_bfloat16>(nw); p.b[l] = alloc<float>(nb); p.wm[l] = alloc<float>(nw);
            p.gw[l] = alloc<float>(nw); p.gb[l] = alloc<float>(nb); p.mw[l] = alloc<float>(nw);
            p.vw[l] = alloc<float>(nw); p.mb[l] = alloc<float>(nb); p.vb[l] = alloc<float>(nb);
        }
        b.n = n;
        b.pos = alloc<float4>(n); b.dir = alloc<float4>(n); b.x = alloc<__nv_bfloat16>((size_t)n * kMlpIn);
        for (int i = 0; i < 3; ++i) b.h[i] = alloc<__nv_bfloat16>((size_t)n * kMlpHid);
        b.out = alloc<float>((size_t)n * kMlpOut);
        for (int l = 0; l < kMlpLayers; ++l) b.dy[l] = alloc<__nv_bfloat16>((size_t)n * mlp_out_dim(l));
        b.loss = alloc<float>(1);
        for (void* a : allocs) if (!a) return false;
        return true;
    }
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
    ~HostMlp() { for (void* a : allocs) cudaFree(a); }
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

// Loss and gradients: pos4 (xyz, w = light density at dir), dir4 (xyz, w = sample
// weight); grads packed like params; *loss = mean weighted negative log-likelihood.
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
    if (mlp_forward_batch(m.p, m.b, 0, err) || mlp_backward_batch(m.p, m.b, 0, err)) return -3;
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
        if (mlp_forward_batch(m.p, m.b, 0, err) || mlp_backward_batch(m.p, m.b, 0, err)) return -3;
        cudaMemcpy(&losses[i], m.b.loss, 4, cudaMemcpyDeviceToHost);
        mlp_adam(m.p, lr, 0);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return -3;
    int h = 0;
    cudaMemcpy(&h, err, 4, cudaMemcpyDeviceToHost);
    if (h) return -6;
    if (params_out) m.get(m.p.wm, m.p.b, params_out);
    return 0;
}
