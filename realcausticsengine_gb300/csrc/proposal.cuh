// Sampling from the learned emission proposal: von Mises-Fisher lobes, and the
// tabulated proposal the Metropolis samplers draw from.
//
// The proposal depends only on the emission position, and for area and sun lights the
// position is an affine function of the light's area coordinates (u1, u2) (a point light
// has one position).  The table holds, per light and per cell of a kProposalRes x
// kProposalRes grid over (u1, u2), the network's mixture at the cell centre (evaluated by
// the tensor-core forward kernel); a path emitted from a cell samples that mixture and is
// weighted by p_light / q with q the same mixture's density, so the table defines a
// proposal of its own and the estimator stays consistent.
#pragma once
#include "lights.cuh"
#include "mlp.cuh"

namespace rc {

constexpr float kKappaMin = 0.1f, kKappaMax = 2000.0f;
constexpr int kProposalRes = 32;                    // cells per light side
constexpr int kProposalCellFloats = 5 * kMlpLobes;  // per lobe: cumulative weight, mean xyz, kappa

// Cells of the table: light l, cell (ix, iy) at cells + ((l * res + iy) * res + ix) * 80.
struct ProposalTable {
    const float* cells;   // nullptr: no tabulated proposal
    int res;
};

__device__ __forceinline__ F3 sample_vmf(F3 mu, float kappa, float u1, float u2) {
    u1 = fmaxf(u1, 1e-7f);
    const float w = 1.0f + logf(u1 + (1.0f - u1) * expf(-2.0f * kappa)) / kappa;
    const float st = sqrtf(fmaxf(0.0f, 1.0f - w * w));
    Frame f;
    f.set_from_z(mu);
    float sp, cp;
    sincosf(kPI2 * u2, &sp, &cp);
    return f.x * (st * cp) + f.y * (st * sp) + mu * w;
}

// Fast-intrinsic vMF density for the proposal weights (relative error ~1e-6 against
// the sampler's own density: a bias of that order in p_light / q).
__device__ __forceinline__ float vmf_pdf_fast(float kappa, float cosang) {
    return kappa * __expf(kappa * (cosang - 1.0f)) / (kPI2 * (1.0f - __expf(-2.0f * kappa)));
}
__device__ __forceinline__ float kappa_of(float raw) {
    const float sp = raw > 20.0f ? raw : __logf(1.0f + __expf(raw));
    return fminf(kKappaMin + sp, kKappaMax);
}

// Emission direction of light `l` (index li, not a sun) at area coordinates (u1, u2)
// from the tabulated proposal: with probability kMlpDefensive (xi below it) the light's
// own density with (u3, u4), else a lobe picked by xi and a vMF sample with (u3, u4).
// Returns p_light(w) / q(w) (0 when the light does not emit along w).
__device__ __forceinline__ float table_direction(const ProposalTable& T, const DevLight& l, int li, float u1, float u2,
                                                 float u3, float u4, float xi, F3& w) {
    const int res = T.res;
    int ix = 0, iy = 0;
    if (l.type != LIGHT_POINT) {
        ix = min(max((int)(u1 * res), 0), res - 1);
        iy = min(max((int)(u2 * res), 0), res - 1);
    }
    const float* c = T.cells + ((size_t)(li * res + iy) * res + ix) * kProposalCellFloats;
    if (xi < kMlpDefensive) {
        w = light_direction(l, u3, u4);
    } else {
        const float t = (xi - kMlpDefensive) / (1.0f - kMlpDefensive);
        int k = 0;
        while (k < kMlpLobes - 1 && !(t < __ldg(&c[5 * k]))) ++k;
        w = sample_vmf(f3(__ldg(&c[5 * k + 1]), __ldg(&c[5 * k + 2]), __ldg(&c[5 * k + 3])), __ldg(&c[5 * k + 4]), u3,
                       u4);
    }
    const float pl = light_direction_pdf(l, w);
    float S = 0.0f, prev = 0.0f;
    for (int k = 0; k < kMlpLobes; ++k) {
        const float cdf = __ldg(&c[5 * k]);
        const F3 mu = f3(__ldg(&c[5 * k + 1]), __ldg(&c[5 * k + 2]), __ldg(&c[5 * k + 3]));
        S += (cdf - prev) * vmf_pdf_fast(__ldg(&c[5 * k + 4]), dot(mu, w));
        prev = cdf;
    }
    const float q = kMlpDefensive * pl + (1.0f - kMlpDefensive) * S;
    return (pl > 0.0f && q > 0.0f) ? pl / q : 0.0f;
}

}  // namespace rc
