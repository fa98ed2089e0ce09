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
//
// The record also carries a conservative screen box of the region where the
// splat can reach alpha >= 1/255: sigma <= ln(255 * opacity) is an ellipse
// in the splat plane, inside the rectangle +-a*s1*ax1 +-a*s2*ax2 with
// a = sqrt(2 ln(255 opacity)) (inflated slightly); when all four corners are
// in front of the camera the projected rectangle, hence the box of its
// projected corners, contains every pixel whose ray meets the ellipse.  A
// pixel outside the box is a pixel the reference skips (alpha < 1/255).
//
// Fields are grouped by how often the per-pixel loop reads them.
// ---------------------------------------------------------------------------
struct RecHot {   // every (pixel, Gaussian) pair
    float4 box;   // screen box of alpha >= 1/255: x0, x1, y0, y1 (one load for the per-visit test)
    float4 org;   // px0, py0, g, tvn
    float4 lc;    // p1u, p1v, p2u, p2v (scaled by 1 / (scale * glob_scale))
    float4 nop;   // nu, nv, opacity, flags (int bits; bit 0: direct form only)
};
struct RecWarm {  // pairs that pass the alpha test
    float4 uvm;   // uu, uv_, vu, vv: texture uv numerators
    float4 uvs;   // uv0.x, uv0.y, blur centre x, blur centre y
    float4 col;   // colour rgb, 1 / (scale_x * glob_scale)
    float4 nrm;   // world normal (axis 3), 1 / (scale_y * glob_scale)
    int4 tex;     // chart h, w, start, Gaussian id
};
struct RecCold {  // the backward's ray terms and the blur adjoint
    float4 mu;    // camera-space mean, a1 . mean
    float4 dt;    // a2 . mean, umap . mean, vmap . mean (camera space), unused
};
constexpr int kRecBytes = sizeof(RecHot) + sizeof(RecWarm) + sizeof(RecCold);

// The four edges of the projected alpha >= 1/255 rectangle (a convex quad
// inside the screen box): a pixel centre (x, y) can only meet the splat where
// A.k x + B.k y + C.k >= 0 for every edge k (pixel units, with a margin).
// Used by the backward's candidate lists; all-pass (A = B = 0, C = 1) where
// the box is infinite, with blur, or for a degenerate edge.
struct RecEdge {
    float4 A, B, C;
};
constexpr int kEdgeBytes = sizeof(RecEdge);

// One (view, Gaussian) record as the batched path stores it in device memory:
// built once per view by the record kernel (where the near-edge-on solve runs
// in double), then copied into shared memory by every tile the splat touches.
struct __align__(16) RecAll {
    RecHot h;
    RecWarm w;
    RecCold c;
    RecEdge e;
};
static_assert(sizeof(RecAll) == kRecBytes + kEdgeBytes, "record layout");

struct Recs {
    RecHot* hot;
    RecWarm* warm;
    RecCold* cold;
    RecEdge* edge;  // null when the kernel does not stage edges
    __device__ __forceinline__ static Recs carve(unsigned char* smem, int n, bool with_edges) {
        Recs r;
        r.hot = reinterpret_cast<RecHot*>(smem);
        r.warm = reinterpret_cast<RecWarm*>(smem + sizeof(RecHot) * n);
        r.cold = reinterpret_cast<RecCold*>(smem + (sizeof(RecHot) + sizeof(RecWarm)) * n);
        r.edge = with_edges ? reinterpret_cast<RecEdge*>(smem + (size_t)kRecBytes * n) : nullptr;
        return r;
    }
};

__device__ __forceinline__ float4 f4(float3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }

// Pairs of fp32 values in one instruction (the f32x2 add / mul / fma of this
// GPU): each half is the IEEE fp32 operation, rounded to nearest; fma2 is a
// fused multiply-add per half.
__device__ __forceinline__ unsigned long long pack2(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long r) {
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)), "l"(pack2(c)));
    return unpack2(r);
}
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }

// Near-edge-on splats (|n_c . d0| < kEdgeOn): the plane coefficients in
// double.  Writes H.org, H.nop.x/.y, H.lc and Wm.uvm.
constexpr float kEdgeOn = 0.05f;
__device__ __forceinline__ void edge_on_solve(RecHot& H, RecWarm& Wm, const View& V, float3 mc, float3 a1c,
                                              float3 a2c, float3 nc, float3 umc, float3 vmc, float is1, float is2,
                                              float tvn) {
    const double mz = mc.z, imz = 1.0 / mz;
    const double u0 = (double)mc.x * imz, v0 = (double)mc.y * imz;
    const double g = (double)nc.x * u0 + (double)nc.y * v0 + nc.z;
    const double ifx = 1.0 / V.fx, ify = 1.0 / V.fy;
    const double a1d = a1c.x * u0 + a1c.y * v0 + a1c.z, a2d = a2c.x * u0 + a2c.y * v0 + a2c.z;
    const double umd = umc.x * u0 + umc.y * v0 + umc.z, vmd = vmc.x * u0 + vmc.y * v0 + vmc.z;
    H.org = make_float4((float)(V.fx * u0 + V.cx), (float)(V.fy * v0 + V.cy), (float)g, tvn);
    H.nop.x = (float)(nc.x * ifx);
    H.nop.y = (float)(nc.y * ify);
    H.lc = make_float4((float)(mz * (g * a1c.x - a1d * nc.x) * ifx * is1),
                      (float)(mz * (g * a1c.y - a1d * nc.y) * ify * is1),
                      (float)(mz * (g * a2c.x - a2d * nc.x) * ifx * is2),
                      (float)(mz * (g * a2c.y - a2d * nc.y) * ify * is2));
    Wm.uvm = make_float4((float)(mz * (g * umc.x - umd * nc.x) * ifx), (float)(mz * (g * umc.y - umd * nc.y) * ify),
                         (float)(mz * (g * vmc.x - vmd * nc.x) * ifx), (float)(mz * (g * vmc.y - vmd * nc.y) * ify));
}

// Edges of the convex quad with corners k = 0 (+,+), 1 (-,+), 3 (-,-), 2 (+,-)
// in cyclic order, oriented so that the quad's centroid is inside, normalised
// to pixel distances and widened by a margin; a degenerate edge passes all.
__device__ __forceinline__ void quad_edges(const float (&qx)[4], const float (&qy)[4], RecEdge& E) {
    const int cyc[5] = { 0, 1, 3, 2, 0 };
    const float gx = 0.25f * (qx[0] + qx[1] + qx[2] + qx[3]), gy = 0.25f * (qy[0] + qy[1] + qy[2] + qy[3]);
    const float margin = 0.05f + 1e-5f * (fabsf(gx) + fabsf(gy));
    float A[4], B[4], C[4];
    float side = 0.f;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int i = cyc[e], j = cyc[e + 1];
        const float ax = -(qy[j] - qy[i]), by = qx[j] - qx[i];
        const float len = sqrtf(ax * ax + by * by);
        if (len > 1e-3f) {
            const float il = 1.f / len;
            A[e] = ax * il;
            B[e] = by * il;
            C[e] = -(A[e] * qx[i] + B[e] * qy[i]);
            side += A[e] * gx + B[e] * gy + C[e];
        } else {
            A[e] = B[e] = 0.f;
            C[e] = 1.f;
        }
    }
    if (fabsf(side) < 1e-3f) {  // a quad of (near) zero width: no usable orientation
        E.A = E.B = make_float4(0.f, 0.f, 0.f, 0.f);
        E.C = make_float4(1.f, 1.f, 1.f, 1.f);
        return;
    }
    const float sg = side < 0.f ? -1.f : 1.f;
    // a flipped edge keeps C = 1 for the degenerate (all-pass) case
#pragma unroll
    for (int e = 0; e < 4; e++) {
        if (A[e] != 0.f || B[e] != 0.f) {
            A[e] *= sg;
            B[e] *= sg;
            C[e] = C[e] * sg + margin;
        }
    }
    E.A = make_float4(A[0], A[1], A[2], A[3]);
    E.B = make_float4(B[0], B[1], B[2], B[3]);
    E.C = make_float4(C[0], C[1], C[2], C[3]);
}

__device__ __forceinline__ bool make_record(RecHot& H, RecWarm& Wm, RecCold& Cd, int gid, const View& V,
                                            const float3 mean, const float4 quat, const float2 scale,
                                            float glob_scale, float opac, float3 color, float2 uv0, float3 umap,
                                            float3 vmap, int3 dims, bool use_blur, bool allow_double = true,
                                            RecEdge* E = nullptr, bool cull = true) {
    const Axes A = quat_axes(quat);
    const float3 mc = V.xform(mean);
    const float3 a1c = V.rot(A.a1), a2c = V.rot(A.a2), nc = V.rot(A.a3);
    const float3 umc = V.rot(umap), vmc = V.rot(vmap);
    const float is1 = 1.f / (scale.x * glob_scale), is2 = 1.f / (scale.y * glob_scale);
    const float tvn = dot3(nc, mc);
    // blur centre exactly as the reference projects it (helpers.cuh:145-152)
    const float rwb = 1.f / (mc.z + 1e-6f);
    const float bx = mc.x * rwb * V.fx + V.cx, by = mc.y * rwb * V.fy + V.cy;
    Cd.mu = f4(mc, dot3(a1c, mc));
    Cd.dt = make_float4(dot3(a2c, mc), dot3(umc, mc), dot3(vmc, mc), 0.f);
    Wm.uvs = make_float4(uv0.x, uv0.y, bx, by);
    Wm.col = f4(color, is1);
    Wm.nrm = f4(A.a3, is2);
    Wm.tex = make_int4(dims.x, dims.y, dims.z, gid);

    // screen box of alpha >= 1/255 (empty when the splat can never reach it)
    float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
    const float smax = __logf(255.f * opac);
    int flags = 0;
    if (!(mc.z > kTNear)) flags = 1;
    if (E) {
        E->A = E->B = make_float4(0.f, 0.f, 0.f, 0.f);
        E->C = make_float4(1.f, 1.f, 1.f, 1.f);
    }
    if (smax > 0.f) {
        const float a = sqrtf(2.f * smax + 1e-3f) * 1.002f;
        const float e1 = a / is1, e2 = a / is2;
        bool front = !flags;
        float qx[4], qy[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float s1 = (k & 1) ? -e1 : e1, s2 = (k & 2) ? -e2 : e2;
            const float3 c = make_float3(mc.x + s1 * a1c.x + s2 * a2c.x, mc.y + s1 * a1c.y + s2 * a2c.y,
                                         mc.z + s1 * a1c.z + s2 * a2c.z);
            front = front && c.z > 1e-3f;
            const float iz = 1.f / c.z;
            const float px = V.fx * c.x * iz + V.cx, py = V.fy * c.y * iz + V.cy;
            qx[k] = px;
            qy[k] = py;
            x0 = fminf(x0, px); x1 = fmaxf(x1, px);
            y0 = fminf(y0, py); y1 = fmaxf(y1, py);
        }
        if (front) {
            const float mx = 1e-2f + 1e-5f * (fabsf(x0) + fabsf(x1)), my = 1e-2f + 1e-5f * (fabsf(y0) + fabsf(y1));
            x0 -= mx; x1 += mx; y0 -= my; y1 += my;
            if (E && !use_blur) quad_edges(qx, qy, *E);
        } else {
            x0 = y0 = -INFINITY;
            x1 = y1 = INFINITY;
        }
        if (use_blur) {
            const float r = sqrtf(smax) * 1.002f + 1e-2f;
            x0 = fminf(x0, bx - r); x1 = fmaxf(x1, bx + r);
            y0 = fminf(y0, by - r); y1 = fmaxf(y1, by + r);
        }
    } else if (opac != opac) {
        // a NaN opacity gives alpha = fminf(0.99, NaN) = 0.99 in the reference: never cull it
        x0 = y0 = -INFINITY;
        x1 = y1 = INFINITY;
    }
    if (!cull) {
        // alpha-visualisation mode sets alpha without the opacity: no box
        x0 = y0 = -INFINITY;
        x1 = y1 = INFINITY;
        if (E) {
            E->A = E->B = make_float4(0.f, 0.f, 0.f, 0.f);
            E->C = make_float4(1.f, 1.f, 1.f, 1.f);
        }
    }

    H.box = make_float4(x0, x1, y0, y1);
    if (flags) {
        H.org = make_float4(V.cx, V.cy, 0.f, tvn);
        H.lc = make_float4(0.f, 0.f, 0.f, 0.f);
        H.nop = make_float4(0.f, 0.f, opac, __int_as_float(flags));
        Wm.uvm = make_float4(0.f, 0.f, 0.f, 0.f);
        return false;
    }
    const float u0f = mc.x / mc.z, v0f = mc.y / mc.z;
    const float gf = nc.x * u0f + nc.y * v0f + nc.z;
    const bool edge_on = fabsf(gf) < kEdgeOn;
    if (edge_on && allow_double) {
        edge_on_solve(H, Wm, V, mc, a1c, a2c, nc, umc, vmc, is1, is2, tvn);
    } else {
        const float mz = mc.z, ifx = 1.f / V.fx, ify = 1.f / V.fy;
        const float a1d = a1c.x * u0f + a1c.y * v0f + a1c.z, a2d = a2c.x * u0f + a2c.y * v0f + a2c.z;
        const float umd = umc.x * u0f + umc.y * v0f + umc.z, vmd = vmc.x * u0f + vmc.y * v0f + vmc.z;
        H.org = make_float4(V.fx * u0f + V.cx, V.fy * v0f + V.cy, gf, tvn);
        H.nop.x = nc.x * ifx;
        H.nop.y = nc.y * ify;
        H.lc = make_float4(mz * (gf * a1c.x - a1d * nc.x) * ifx * is1, mz * (gf * a1c.y - a1d * nc.y) * ify * is1,
                          mz * (gf * a2c.x - a2d * nc.x) * ifx * is2, mz * (gf * a2c.y - a2d * nc.y) * ify * is2);
        Wm.uvm = make_float4(mz * (gf * umc.x - umd * nc.x) * ifx, mz * (gf * umc.y - umd * nc.y) * ify,
                             mz * (gf * vmc.x - vmd * nc.x) * ifx, mz * (gf * vmc.y - vmd * nc.y) * ify);
    }
    H.nop.z = opac;
    H.nop.w = __int_as_float(flags);
    return edge_on && !allow_double;
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

__device__ __forceinline__ bool outside_box(const RecHot& H, const PixelRay& P) {
    return P.px < H.box.x || P.px > H.box.y || P.py < H.box.z || P.py > H.box.w;
}

// Intersection of a pixel ray with a staged splat.
struct Hit {
    float t;         // ray parameter along the unit ray (reference t)
    float tcam;      // camera z of the hit (reference t * view_depth)
    float l1s, l2s;  // plane coordinates divided by the scales
    float du, dv;    // pixel offset from the projected centre (fast form)
    float inv;       // d t_cam / d tvn: 1 / den (fast form), idn / den_ref (direct form)
    float nd;        // n_c . d, the sign of ray . normal
    float tu, tv;    // texture uv before clamping (direct form only)
    bool direct;
};

__device__ __forceinline__ float clamp_denom(float d) {
    if (0.f <= d && d < kDenomEps) return kDenomEps;
    if (-kDenomEps < d && d <= 0.f) return -kDenomEps;
    return d;
}

// Fast form of the intersection; sets H.direct when the pixel needs the
// direct form (computed by the caller from the Gaussian's parameters).
__device__ __forceinline__ Hit intersect(const RecHot& Hr, const PixelRay& P) {
    Hit H;
    const float2 d = sub2(make_float2(P.px, P.py), make_float2(Hr.org.x, Hr.org.y));
    H.du = d.x;
    H.dv = d.y;
    const float den = Hr.org.z + Hr.nop.x * H.du + Hr.nop.y * H.dv;
    H.nd = den;
    H.direct = __float_as_int(Hr.nop.w) != 0 || !(fabsf(den) >= kDenomEps * P.dn);
    const float inv = __fdividef(1.f, den);
    H.inv = inv;
    H.tcam = Hr.org.w * inv;
    H.t = H.tcam * P.dn;
    const float2 l = mul2(fma2(make_float2(Hr.lc.y, Hr.lc.w), dup2(H.dv),
                               mul2(make_float2(Hr.lc.x, Hr.lc.z), dup2(H.du))), dup2(inv));
    H.l1s = l.x;
    H.l2s = l.y;
    return H;
}

// Direct camera-space form with the reference's denominator clamp, from the
// camera-space frame of the Gaussian.
__device__ __forceinline__ void intersect_direct(Hit& H, const PixelRay& P, float tvn, float3 mc, float3 a1c,
                                                 float3 a2c, float3 nc, float3 umc, float3 vmc, float is1, float is2,
                                                 float uv0x, float uv0y) {
    const float3 d = make_float3(P.u, P.v, 1.f);
    H.nd = dot3(nc, d);
    const float dref = clamp_denom(H.nd * P.idn);
    const float t = tvn / dref;
    const float3 delta = t * (P.idn * d) - mc;
    H.inv = P.idn / dref;
    H.t = t;
    H.tcam = t * P.idn;
    H.l1s = dot3(a1c, delta) * is1;
    H.l2s = dot3(a2c, delta) * is2;
    H.tu = uv0x + dot3(umc, delta);
    H.tv = uv0y + dot3(vmc, delta);
}

// Texture coordinates of the hit (before clamping).
__device__ __forceinline__ float2 hit_uv(const Hit& H, const RecWarm& Wm) {
    if (!H.direct) {
        const float2 t = fma2(make_float2(Wm.uvm.y, Wm.uvm.w), dup2(H.dv),
                              mul2(make_float2(Wm.uvm.x, Wm.uvm.z), dup2(H.du)));
        return fma2(t, dup2(H.inv), make_float2(Wm.uvs.x, Wm.uvs.y));
    }
    return make_float2(H.tu, H.tv);
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
    const float2 tc = mul2(make_float2((float)h, (float)w), make_float2(u, v));
    const float tcx = tc.x, tcy = tc.y;
    int iix = __float2int_rz(tcx), iiy = __float2int_rz(tcy);
    const int jjx = min(iix + 1, h - 1), jjy = min(iiy + 1, w - 1);
    const float wx = tcx - (float)iix, wy = tcy - (float)iiy;
    iix = min(iix, h - 1);
    iiy = min(iiy, w - 1);
    B.fx = wx; B.fy = wy;
    const float2 wyy = make_float2(1.f - wy, wy);
    const float2 w0 = mul2(dup2(1.f - wx), wyy), w1 = mul2(dup2(wx), wyy);
    const float w00 = w0.x, w01 = w0.y, w10 = w1.x, w11 = w1.y;
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
