// Parameter activation of a GStex training step (the reference demo's
// per-step preprocessing, example.py:126-143, and the opacity sigmoid of
// example.py:155-171), shared by the standalone preprocess kernels and the
// batched projection, which activates each Gaussian as it projects it:
//
//   scales[:, :2] = exp(raw_scales[:, :2]); scales[:, 2] = 1e-5 * mean(scales[:, :2])
//   quats         = raw_quats / |raw_quats|
//   uv0           = mapping[..., 0:2]
//   umap          = exp(mapping[..., 2]) * ( ax1 cos(theta) + ax2 sin(theta))
//   vmap          = exp(mapping[..., 2]) * (-ax1 sin(theta) + ax2 cos(theta)),  theta = mapping[..., 3]
//   opacity       = sigmoid(raw_opacity)
#pragma once

#include "common.cuh"

namespace gstex {

// Raw trainer parameters of N Gaussians with P charts each, and where their
// activated values go.  raw_scales == nullptr means "already activated".
struct RawParams {
    const float* raw_scales;   // [N, 3] log-scales (first two used)
    const float4* raw_quats;   // [N, 4] wxyz, any norm
    const float4* mapping;     // [N, P, 4] uv0 x, uv0 y, log uv-scale, theta
    const float* raw_opacity;  // [N] logits, or null (opacity left as it is)
    int P;
    float* scales;             // [N, 3]
    float4* quats;             // [N, 4]
    float2* uv0;               // [N, P, 2]
    float* umap;               // [N, P, 3]
    float* vmap;               // [N, P, 3]
    float* opacity;            // [N]
};

__device__ __forceinline__ float sigmoidf(float x) { return 1.f / (1.f + expf(-x)); }

// Activates Gaussian i, writes its activated parameters and returns the two
// scales and the unit quaternion.
__device__ __forceinline__ void activate(const RawParams& r, int i, float& s0, float& s1, float4& q) {
    s0 = expf(r.raw_scales[3 * i]);
    s1 = expf(r.raw_scales[3 * i + 1]);
    r.scales[3 * i] = s0;
    r.scales[3 * i + 1] = s1;
    r.scales[3 * i + 2] = 1e-5f * (0.5f * (s0 + s1));
    const float4 w = r.raw_quats[i];
    const float in = 1.f / sqrtf(w.x * w.x + w.y * w.y + w.z * w.z + w.w * w.w);
    q = make_float4(w.x * in, w.y * in, w.z * in, w.w * in);
    r.quats[i] = q;
    const Axes A = quat_axes(q);
    for (int p = 0; p < r.P; p++) {
        const size_t k = (size_t)i * r.P + p;
        const float4 m = r.mapping[k];
        r.uv0[k] = make_float2(m.x, m.y);
        const float us = expf(m.z);
        float sn, cs;
        sincosf(m.w, &sn, &cs);
        const float3 u = us * (cs * A.a1 + sn * A.a2);
        const float3 v = us * (cs * A.a2 - sn * A.a1);
        r.umap[3 * k] = u.x; r.umap[3 * k + 1] = u.y; r.umap[3 * k + 2] = u.z;
        r.vmap[3 * k] = v.x; r.vmap[3 * k + 1] = v.y; r.vmap[3 * k + 2] = v.z;
    }
    if (r.raw_opacity) r.opacity[i] = sigmoidf(r.raw_opacity[i]);
}

}  // namespace gstex
