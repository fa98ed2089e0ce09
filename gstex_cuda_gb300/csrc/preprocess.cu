// Per-step parameter activation of a GStex training loop on the device: the
// preprocessing of the reference's demo trainer (example.py:126-143 and the
// sigmoids of example.py:155-171) as one forward and one backward kernel;
// the formulas are in preprocess.cuh.  One thread per Gaussian; P charts per
// Gaussian.
#include "preprocess.cuh"

namespace gstex {

__global__ void preprocess_fwd_kernel(int N, RawParams r) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float s0, s1;
    float4 q;
    activate(r, i, s0, s1, q);
}

__global__ void preprocess_bwd_kernel(int N, int P, const float* __restrict__ raw_scales,
                                      const float4* __restrict__ raw_quats, const float4* __restrict__ mapping,
                                      const float* __restrict__ raw_opacity, const float* __restrict__ v_scales,
                                      const float4* __restrict__ v_quats, const float2* __restrict__ v_uv0,
                                      const float* __restrict__ v_umap, const float* __restrict__ v_vmap,
                                      const float* __restrict__ v_opacity, float* __restrict__ v_raw_scales,
                                      float4* __restrict__ v_raw_quats, float4* __restrict__ v_mapping,
                                      float* __restrict__ v_raw_opacity) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    // exp: d scale / d raw = scale; the third scale is detached in the trainer
    v_raw_scales[3 * i] = v_scales ? v_scales[3 * i] * expf(raw_scales[3 * i]) : 0.f;
    v_raw_scales[3 * i + 1] = v_scales ? v_scales[3 * i + 1] * expf(raw_scales[3 * i + 1]) : 0.f;
    v_raw_scales[3 * i + 2] = 0.f;
    const float4 r = raw_quats[i];
    const float in = 1.f / sqrtf(r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w);
    const float4 q = make_float4(r.x * in, r.y * in, r.z * in, r.w * in);
    const Axes A = quat_axes(q);
    float3 g1 = make_float3(0.f, 0.f, 0.f), g2 = make_float3(0.f, 0.f, 0.f);
    for (int p = 0; p < P; p++) {
        const size_t k = (size_t)i * P + p;
        const float4 m = mapping[k];
        const float us = expf(m.z);
        float sn, cs;
        sincosf(m.w, &sn, &cs);
        const float3 vu = v_umap ? make_float3(v_umap[3 * k], v_umap[3 * k + 1], v_umap[3 * k + 2])
                                 : make_float3(0.f, 0.f, 0.f);
        const float3 vv = v_vmap ? make_float3(v_vmap[3 * k], v_vmap[3 * k + 1], v_vmap[3 * k + 2])
                                 : make_float3(0.f, 0.f, 0.f);
        const float3 u = us * (cs * A.a1 + sn * A.a2);
        const float3 v = us * (cs * A.a2 - sn * A.a1);
        // umap, vmap are linear in (ax1, ax2); d/d log-scale gives themselves,
        // d/d theta turns umap into vmap and vmap into -umap
        g1 = g1 + us * (cs * vu - sn * vv);
        g2 = g2 + us * (sn * vu + cs * vv);
        const float2 vo = v_uv0 ? v_uv0[k] : make_float2(0.f, 0.f);
        v_mapping[k] = make_float4(vo.x, vo.y, dot3(vu, u) + dot3(vv, v), dot3(vu, v) - dot3(vv, u));
    }
    float4 vq = quat_axes_vjp(q, g1, g2, make_float3(0.f, 0.f, 0.f));
    if (v_quats) {
        const float4 d = v_quats[i];
        vq.x += d.x; vq.y += d.y; vq.z += d.z; vq.w += d.w;
    }
    // normalisation: d q / d r = (I - q q^T) / |r|
    const float qv = q.x * vq.x + q.y * vq.y + q.z * vq.z + q.w * vq.w;
    v_raw_quats[i] = make_float4((vq.x - q.x * qv) * in, (vq.y - q.y * qv) * in, (vq.z - q.z * qv) * in,
                                 (vq.w - q.w * qv) * in);
    if (raw_opacity && v_raw_opacity) {
        const float o = sigmoidf(raw_opacity[i]);
        v_raw_opacity[i] = v_opacity ? v_opacity[i] * o * (1.f - o) : 0.f;
    }
}

}  // namespace gstex

using namespace gstex;

extern "C" int gstex_preprocess_forward(int N, int P, const float* raw_scales, const float* raw_quats,
                                        const float* mapping, const float* raw_opacity, float* scales, float* quats,
                                        float* uv0, float* umap, float* vmap, float* opacity, gstex_stream_t s) {
    GSTEX_REQUIRE(N >= 0 && P >= 0);
    if (N == 0) return GSTEX_OK;
    GSTEX_REQUIRE(raw_scales && raw_quats && scales && quats);
    if (P > 0) GSTEX_REQUIRE(mapping && uv0 && umap && vmap);
    if (raw_opacity) GSTEX_REQUIRE(opacity);
    const RawParams r{ raw_scales, (const float4*)raw_quats, (const float4*)mapping, raw_opacity, P, scales,
                       (float4*)quats, (float2*)uv0, umap, vmap, opacity };
    preprocess_fwd_kernel<<<ceil_div(N, 256), 256, 0, (cudaStream_t)s>>>(N, r);
    return check_launch("preprocess_forward");
}

extern "C" int gstex_preprocess_backward(int N, int P, const float* raw_scales, const float* raw_quats,
                                         const float* mapping, const float* raw_opacity, const float* v_scales,
                                         const float* v_quats, const float* v_uv0, const float* v_umap,
                                         const float* v_vmap, const float* v_opacity, float* v_raw_scales,
                                         float* v_raw_quats, float* v_mapping, float* v_raw_opacity,
                                         gstex_stream_t s) {
    GSTEX_REQUIRE(N >= 0 && P >= 0);
    if (N == 0) return GSTEX_OK;
    GSTEX_REQUIRE(raw_scales && raw_quats && v_raw_scales && v_raw_quats);
    if (P > 0) GSTEX_REQUIRE(mapping && v_mapping);
    if (raw_opacity) GSTEX_REQUIRE(v_raw_opacity);
    preprocess_bwd_kernel<<<ceil_div(N, 256), 256, 0, (cudaStream_t)s>>>(
        N, P, raw_scales, (const float4*)raw_quats, (const float4*)mapping, raw_opacity, v_scales,
        (const float4*)v_quats, (const float2*)v_uv0, v_umap, v_vmap, v_opacity, v_raw_scales, (float4*)v_raw_quats,
        (float4*)v_mapping, v_raw_opacity);
    return check_launch("preprocess_backward");
}
