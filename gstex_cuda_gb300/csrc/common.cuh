// Shared device code of the gstex_gb300 library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/gstex_gb300.h"

namespace gstex {

constexpr int kMaxChannels = 64;
constexpr int kMaxBlockWidth = 16;

// Reference float constants (csrc/texture.cu:198, 213-217; texture_helpers.cuh:305)
constexpr float kTNear = 0.01f;
constexpr float kTFar = 1000.0f;
constexpr float kAlphaMax = 0.99f;
constexpr float kAlphaMin = 1.f / 255.f;
constexpr float kTDone = 1e-4f;
constexpr float kDenomEps = 1e-6f;
constexpr float kBlurFsq = 2.0f;

// Host-side status helpers (defined in status.cu).
int check_launch(const char* what, int launches = 1);
void set_cuda_error(cudaError_t e, const char* what);

#define GSTEX_REQUIRE(cond)                         \
    do {                                            \
        if (!(cond)) return GSTEX_ERR_INVALID_ARGUMENT; \
    } while (0)

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// quaternion (w, x, y, z) -> columns ax1, ax2, ax3 of the rotation
// (reference csrc/helpers.cuh:166-185)
// ---------------------------------------------------------------------------
struct Axes {
    float3 a1, a2, a3;
};

__device__ __forceinline__ Axes quat_axes(float4 q) {
    const float w = q.x, x = q.y, y = q.z, z = q.w;
    Axes A;
    A.a1 = make_float3(1.f - 2.f * (y * y + z * z), 2.f * (x * y + w * z), 2.f * (x * z - w * y));
    A.a2 = make_float3(2.f * (x * y - w * z), 1.f - 2.f * (x * x + z * z), 2.f * (y * z + w * x));
    A.a3 = make_float3(2.f * (x * z + w * y), 2.f * (y * z - w * x), 1.f - 2.f * (x * x + y * y));
    return A;
}

// d(R(q)) adjoint for gradients vR = columns (v_a1, v_a2, v_a3)
// (reference csrc/helpers.cuh:187-228)
__device__ __forceinline__ float4 quat_axes_vjp(float4 q, float3 c0, float3 c1, float3 c2) {
    const float w = q.x, x = q.y, y = q.z, z = q.w;
    const float r00 = c0.x, r01 = c0.y, r02 = c0.z;
    const float r10 = c1.x, r11 = c1.y, r12 = c1.z;
    const float r20 = c2.x, r21 = c2.y, r22 = c2.z;
    float4 o;
    o.x = 2.f * (x * (r12 - r21) + y * (r20 - r02) + z * (r01 - r10));
    o.y = 2.f * (-2.f * x * (r11 + r22) + y * (r01 + r10) + z * (r02 + r20) + w * (r12 - r21));
    o.z = 2.f * (x * (r01 + r10) - 2.f * y * (r00 + r22) + z * (r12 + r21) + w * (r20 - r02));
    o.w = 2.f * (x * (r02 + r20) + y * (r12 + r21) - 2.f * z * (r00 + r11) + w * (r01 - r10));
    return o;
}

__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }

// World->camera view transform (row-major 4x4, first 12 entries used).
struct View {
    float r[9];
    float t[3];
    float fx, fy, cx, cy;
    __device__ __forceinline__ float3 rot(float3 p) const {
        return make_float3(r[0] * p.x + r[1] * p.y + r[2] * p.z, r[3] * p.x + r[4] * p.y + r[5] * p.z,
                           r[6] * p.x + r[7] * p.y + r[8] * p.z);
    }
    __device__ __forceinline__ float3 rot_t(float3 p) const {
        return make_float3(r[0] * p.x + r[3] * p.y + r[6] * p.z, r[1] * p.x + r[4] * p.y + r[7] * p.z,
                           r[2] * p.x + r[5] * p.y + r[8] * p.z);
    }
    __device__ __forceinline__ float3 xform(float3 p) const {
        return make_float3(r[0] * p.x + r[1] * p.y + r[2] * p.z + t[0], r[3] * p.x + r[4] * p.y + r[5] * p.z + t[1],
                           r[6] * p.x + r[7] * p.y + r[8] * p.z + t[2]);
    }
};

__device__ __forceinline__ View load_view(const float* viewmat, float fx, float fy, float cx, float cy) {
    View v;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        v.r[3 * i + 0] = viewmat[4 * i + 0];
        v.r[3 * i + 1] = viewmat[4 * i + 1];
        v.r[3 * i + 2] = viewmat[4 * i + 2];
        v.t[i] = viewmat[4 * i + 3];
    }
    v.fx = fx; v.fy = fy; v.cx = cx; v.cy = cy;
    return v;
}

// ---------------------------------------------------------------------------
// Per-view, per-Gaussian record staged in shared memory by the compositor.
//
// The reference intersects every pixel ray with the splat plane in world
// space (texture_helpers.cuh:302-313 then texture.cu:171-181).  Here the same
// intersection is evaluated in camera space relative to the projected centre
// d0 = mu_c / mu_c.z: for a pixel direction d = d0 + e (e = (du/fx, dv/fy, 0))
//   den   = n_c . d                 = g + nu*du + nv*dv
//   t_cam = (n_c . mu_c) / den      = tvn / den         (camera z of the hit)
//   delta = t_cam d - mu_c          = mu_z (g e - (n_c.e) d0) / den
//   l_k   = a_k . delta             = (Pku*du + Pkv*dv) / den
// which has no cancellation between the camera distance and the splat size.
// Gaussians with mu_z <= 0.01 (only reachable through the reference's
// zero-slot entries) and pixels whose ray is within the reference's 1e-6
// denominator clamp use the direct camera-space form instead.
// ---------------------------------------------------------------------------
struct GaussRec {
    float px0, py0;        // projected centre, pixels
    float g, nu, nv;       // den = g + nu*du + nv*dv
    float tvn;             // n_c . mu_c
    float p1u, p1v, p2u, p2v;  // plane coordinates l1, l2 numerators (unscaled)
    float is1, is2;        // 1 / (scale * glob_scale)
    float opac;
    float3 color;
    float3 mu_c;           // camera-space mean (direct form)
    float3 a1c, a2c, nc;   // camera-space axes
    float uu, uv_, vu, vv; // texture uv numerators: u = uv0.x + (uu*du + uv_*dv)/den
    float uv0x, uv0y;
    float3 umc, vmc;       // camera-space umap / vmap (direct form, backward)
    float3 nw;             // world-space normal (axis 3)
    float bx, by;          // reference projected centre (helpers.cuh:145-152), for the blur term
    int h, w, start;       // texture chart
    int gid;
    int flags;             // bit 0: direct form only
};

__device__ __forceinline__ void make_record(GaussRec& R, int gid, const View& V, const float3 mean,
                                            const float4 quat, const float2 scale, float glob_scale, float opac,
                                            float3 color, float2 uv0, float3 umap, float3 vmap, int3 dims) {
    const Axes A = quat_axes(quat);
    const float3 mc = V.xform(mean);
    const float3 a1c = V.rot(A.a1), a2c = V.rot(A.a2), nc = V.rot(A.a3);
    const float3 umc = V.rot(umap), vmc = V.rot(vmap);
    R.gid = gid;
    R.mu_c = mc; R.a1c = a1c; R.a2c = a2c; R.nc = nc; R.umc = umc; R.vmc = vmc;
    R.nw = A.a3;
    R.is1 = 1.f / (scale.x * glob_scale);
    R.is2 = 1.f / (scale.y * glob_scale);
    R.opac = opac;
    R.color = color;
    R.uv0x = uv0.x; R.uv0y = uv0.y;
    R.h = dims.x; R.w = dims.y; R.start = dims.z;
    // blur centre exactly as the reference projects it
    {
        const float rw = 1.f / (mc.z + 1e-6f);
        R.bx = mc.x * rw * V.fx + V.cx;
        R.by = mc.y * rw * V.fy + V.cy;
    }
    R.tvn = dot3(nc, mc);
    if (!(mc.z > kTNear)) {
        R.flags = 1;
        R.px0 = V.cx; R.py0 = V.cy;
        R.g = R.nu = R.nv = 0.f;
        R.p1u = R.p1v = R.p2u = R.p2v = 0.f;
        R.uu = R.uv_ = R.vu = R.vv = 0.f;
        return;
    }
    R.flags = 0;
    // Near edge-on splats: the coefficient algebra runs in double.
    const float u0f = mc.x / mc.z, v0f = mc.y / mc.z;
    const float gf = nc.x * u0f + nc.y * v0f + nc.z;
    if (fabsf(gf) < 0.05f) {
        const double mz = mc.z, u0 = (double)mc.x / mz, v0 = (double)mc.y / mz;
        const double g = (double)nc.x * u0 + (double)nc.y * v0 + nc.z;
        const double ifx = 1.0 / V.fx, ify = 1.0 / V.fy;
        const double a1d = a1c.x * u0 + a1c.y * v0 + a1c.z, a2d = a2c.x * u0 + a2c.y * v0 + a2c.z;
        const double umd = umc.x * u0 + umc.y * v0 + umc.z, vmd = vmc.x * u0 + vmc.y * v0 + vmc.z;
        R.px0 = (float)(V.fx * u0 + V.cx);
        R.py0 = (float)(V.fy * v0 + V.cy);
        R.g = (float)g;
        R.nu = (float)(nc.x * ifx);
        R.nv = (float)(nc.y * ify);
        R.p1u = (float)(mz * (g * a1c.x - a1d * nc.x) * ifx);
        R.p1v = (float)(mz * (g * a1c.y - a1d * nc.y) * ify);
        R.p2u = (float)(mz * (g * a2c.x - a2d * nc.x) * ifx);
        R.p2v = (float)(mz * (g * a2c.y - a2d * nc.y) * ify);
        R.uu = (float)(mz * (g * umc.x - umd * nc.x) * ifx);
        R.uv_ = (float)(mz * (g * umc.y - umd * nc.y) * ify);
        R.vu = (float)(mz * (g * vmc.x - vmd * nc.x) * ifx);
        R.vv = (float)(mz * (g * vmc.y - vmd * nc.y) * ify);
        return;
    }
    const float mz = mc.z, ifx = 1.f / V.fx, ify = 1.f / V.fy;
    const float a1d = a1c.x * u0f + a1c.y * v0f + a1c.z, a2d = a2c.x * u0f + a2c.y * v0f + a2c.z;
    const float umd = umc.x * u0f + umc.y * v0f + umc.z, vmd = vmc.x * u0f + vmc.y * v0f + vmc.z;
    R.px0 = V.fx * u0f + V.cx;
    R.py0 = V.fy * v0f + V.cy;
    R.g = gf;
    R.nu = nc.x * ifx;
    R.nv = nc.y * ify;
    R.p1u = mz * (gf * a1c.x - a1d * nc.x) * ifx;
    R.p1v = mz * (gf * a1c.y - a1d * nc.y) * ify;
    R.p2u = mz * (gf * a2c.x - a2d * nc.x) * ifx;
    R.p2v = mz * (gf * a2c.y - a2d * nc.y) * ify;
    R.uu = mz * (gf * umc.x - umd * nc.x) * ifx;
    R.uv_ = mz * (gf * umc.y - umd * nc.y) * ify;
    R.vu = mz * (gf * vmc.x - vmd * nc.x) * ifx;
    R.vv = mz * (gf * vmc.y - vmd * nc.y) * ify;
}

// Per-pixel constants: pixel centre, camera direction d = (u, v, 1), |d|.
struct PixelRay {
    float px, py;
    float u, v;
    float dn;    // |d|
    float idn;   // 1/|d| = the reference's view_depth
};

__device__ __forceinline__ PixelRay make_pixel(const View& V, int i, int j) {
    PixelRay P;
    P.px = (float)j + 0.5f;
    P.py = (float)i + 0.5f;
    P.u = (P.px - V.cx) / V.fx;
    P.v = (P.py - V.cy) / V.fy;
    P.dn = sqrtf(P.u * P.u + P.v * P.v + 1.f);
    P.idn = 1.f / P.dn;
    return P;
}

// Intersection of a pixel ray with a staged splat.
struct Hit {
    float t;       // ray parameter along the unit ray (reference t)
    float tcam;    // camera z of the hit (reference t * view_depth)
    float l1, l2;  // plane coordinates
    float du, dv;  // pixel offset from the projected centre
    float inv;     // 1 / den (pixel-direction denominator, unnormalised)
    float tu, tv;  // texture uv before clamping
};

__device__ __forceinline__ float clamp_denom(float d) {
    if (0.f <= d && d < kDenomEps) return kDenomEps;
    if (-kDenomEps < d && d <= 0.f) return -kDenomEps;
    return d;
}

__device__ __forceinline__ Hit intersect(const GaussRec& R, const PixelRay& P) {
    Hit H;
    H.du = P.px - R.px0;
    H.dv = P.py - R.py0;
    const float den = R.g + R.nu * H.du + R.nv * H.dv;
    if (!R.flags && fabsf(den) >= kDenomEps * P.dn) {
        const float inv = __frcp_rn(den);
        H.inv = inv;
        H.tcam = R.tvn * inv;
        H.t = H.tcam * P.dn;
        H.l1 = (R.p1u * H.du + R.p1v * H.dv) * inv;
        H.l2 = (R.p2u * H.du + R.p2v * H.dv) * inv;
        H.tu = R.uv0x + (R.uu * H.du + R.uv_ * H.dv) * inv;
        H.tv = R.uv0y + (R.vu * H.du + R.vv * H.dv) * inv;
        return H;
    }
    // direct camera-space form (with the reference's denominator clamp)
    const float3 d = make_float3(P.u, P.v, 1.f);
    const float dref = clamp_denom(dot3(R.nc, d) * P.idn);
    const float t = R.tvn / dref;
    const float3 r = P.idn * d;
    const float3 delta = t * r - R.mu_c;
    H.inv = P.idn / dref;
    H.t = t;
    H.tcam = t * P.idn;
    H.l1 = dot3(R.a1c, delta);
    H.l2 = dot3(R.a2c, delta);
    H.tu = R.uv0x + dot3(R.umc, delta);
    H.tv = R.uv0y + dot3(R.vmc, delta);
    return H;
}

__device__ __forceinline__ float clamp01(float x) {
    // texture_helpers.cuh:37-51
    if (x <= 0.f) x = 0.f;
    if (x >= 1.f) x = 1.f;
    return x;
}

// Bilinear corner indices (texel rows) and weights inside chart (h, w, start)
// (texture_helpers.cuh:162-215).  Indices are texel rows, not element offsets.
struct Bilerp {
    int i00, i01, i10, i11;
    float w00, w01, w10, w11;
    float fx, fy;  // fractional parts (for the uv gradient)
};

__device__ __forceinline__ Bilerp bilerp(int h, int w, int start, float u, float v, bool bilinear) {
    Bilerp B;
    const float tcx = (float)h * u, tcy = (float)w * v;
    int iix = __float2int_rz(tcx), iiy = __float2int_rz(tcy);
    const int jjx = min(iix + 1, h - 1), jjy = min(iiy + 1, w - 1);
    const float wx = tcx - (float)iix, wy = tcy - (float)iiy;
    iix = min(iix, h - 1);
    iiy = min(iiy, w - 1);
    B.fx = wx; B.fy = wy;
    const float w00 = (1.f - wx) * (1.f - wy), w01 = (1.f - wx) * wy, w10 = wx * (1.f - wy), w11 = wx * wy;
    B.i00 = start + iix * w + iiy;
    B.i01 = start + iix * w + jjy;
    B.i10 = start + jjx * w + iiy;
    B.i11 = start + jjx * w + jjy;
    if (bilinear) {
        B.w00 = w00; B.w01 = w01; B.w10 = w10; B.w11 = w11;
    } else {
        B.w00 = B.w01 = B.w10 = B.w11 = 0.f;
        if (w00 >= w01 && w00 >= w10 && w00 >= w11) B.w00 = 1.f;
        else if (w01 >= w00 && w01 >= w10 && w01 >= w11) B.w01 = 1.f;
        else if (w10 >= w00 && w10 >= w01 && w10 >= w11) B.w10 = 1.f;
        else B.w11 = 1.f;
    }
    return B;
}

}  // namespace gstex
