// texture_sample: bilinear lookups of arbitrary queries in jagged charts.
//
// Reference: csrc/texture_sample.cu:11-36 (forward) with the [0,1] uv clamp
// of gstex_cuda/_torch_impl.py:149-194 and of the documented Python API
// (gstex_cuda/texture_sample.py:24-26).  The backward returns the texel and
// uv gradients of that lookup (the reference's backward kernel,
// texture_sample.cu:38-70, reads its upstream gradient from the output buffer
// and its autograd function returns no gradients).
#include "common.cuh"

namespace gstex {

__global__ void sample_fwd_kernel(int nq, int C, const int3* __restrict__ dims, const float2* __restrict__ uvs,
                                  const float* __restrict__ tex, float* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int3 d = dims[q];
    const float2 uv = uvs[q];
    const Bilerp B = bilerp(d.x, d.y, d.z, clamp01(uv.x), clamp01(uv.y), true);
    for (int ch = 0; ch < C; ch++) {
        out[(size_t)q * C + ch] = B.w00 * tex[(size_t)B.i00 * C + ch] + B.w01 * tex[(size_t)B.i01 * C + ch] +
                                  B.w10 * tex[(size_t)B.i10 * C + ch] + B.w11 * tex[(size_t)B.i11 * C + ch];
    }
}

__global__ void sample_bwd_kernel(int nq, int C, const int3* __restrict__ dims, const float2* __restrict__ uvs,
                                  const float* __restrict__ tex, const float* __restrict__ v_out,
                                  float* __restrict__ v_tex, float2* __restrict__ v_uvs) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int3 d = dims[q];
    const float2 uv = uvs[q];
    const Bilerp B = bilerp(d.x, d.y, d.z, clamp01(uv.x), clamp01(uv.y), true);
    float gu = 0.f, gv = 0.f;
    for (int ch = 0; ch < C; ch++) {
        const float g = v_out[(size_t)q * C + ch];
        const float c00 = tex[(size_t)B.i00 * C + ch], c01 = tex[(size_t)B.i01 * C + ch];
        const float c10 = tex[(size_t)B.i10 * C + ch], c11 = tex[(size_t)B.i11 * C + ch];
        atomicAdd(v_tex + (size_t)B.i00 * C + ch, B.w00 * g);
        atomicAdd(v_tex + (size_t)B.i01 * C + ch, B.w01 * g);
        atomicAdd(v_tex + (size_t)B.i10 * C + ch, B.w10 * g);
        atomicAdd(v_tex + (size_t)B.i11 * C + ch, B.w11 * g);
        gu += g * (-(1.f - B.fy) * c00 - B.fy * c01 + (1.f - B.fy) * c10 + B.fy * c11) * (float)d.x;
        gv += g * (-(1.f - B.fx) * c00 + (1.f - B.fx) * c01 - B.fx * c10 + B.fx * c11) * (float)d.y;
    }
    if (v_uvs) {
        // a clamp passes the gradient only inside [0,1]
        v_uvs[q] = make_float2((uv.x >= 0.f && uv.x <= 1.f) ? gu : 0.f, (uv.y >= 0.f && uv.y <= 1.f) ? gv : 0.f);
    }
}

}  // namespace gstex

using namespace gstex;

extern "C" int gstex_texture_sample_forward(int nq, int C, const int32_t* dims, const float* uvs, const float* tex,
                                            float* out, gstex_stream_t s) {
    GSTEX_REQUIRE(nq >= 0 && C >= 0);
    if (nq == 0 || C == 0) return GSTEX_OK;
    GSTEX_REQUIRE(dims && uvs && tex && out);
    sample_fwd_kernel<<<ceil_div(nq, 256), 256, 0, (cudaStream_t)s>>>(nq, C, (const int3*)dims, (const float2*)uvs,
                                                                       tex, out);
    return check_launch("texture_sample_forward");
}

extern "C" int gstex_texture_sample_backward(int nq, int C, const int32_t* dims, const float* uvs, const float* tex,
                                             const float* v_out, float* v_tex, float* v_uvs, gstex_stream_t s) {
    GSTEX_REQUIRE(nq >= 0 && C >= 0);
    if (nq == 0) return GSTEX_OK;
    GSTEX_REQUIRE(dims && uvs && tex && v_out && v_tex);
    sample_bwd_kernel<<<ceil_div(nq, 256), 256, 0, (cudaStream_t)s>>>(nq, C, (const int3*)dims, (const float2*)uvs,
                                                                       tex, v_out, v_tex, (float2*)v_uvs);
    return check_launch("texture_sample_backward");
}
