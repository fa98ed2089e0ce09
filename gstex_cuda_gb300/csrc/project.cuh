// Projection helpers shared by the per-view and the batched entry points.
// Both are compiled with -fmad=false and IEEE division, so a splat's screen
// box, tile count and emitted tiles agree bit for bit between the two paths
// and with a CPU restatement of the same operations.
#pragma once

#include "common.cuh"

namespace gstex {

// helpers.cuh:145-152
__device__ __forceinline__ float2 project_pix(float fx, float fy, float3 p, float cx, float cy) {
    const float rw = 1.f / (p.z + 1e-6f);
    return make_float2(p.x * rw * fx + cx, p.y * rw * fy + cy);
}

// Screen AABB of the +-3 sigma rectangle; reference csrc/get_aabb_2d.cu:11-89.
// m: first 12 entries of the row-major world->camera matrix.  zv receives the
// camera-space depth of the mean.
__device__ __forceinline__ void aabb_2d(const float* m, float fx, float fy, float cx, float cy, float3 p, float4 quat,
                                        float sx, float sy, float glob_scale, float2& center, float2& extent,
                                        float& zv) {
    auto xf = [&](float3 q) {
        return make_float3(m[0] * q.x + m[1] * q.y + m[2] * q.z + m[3], m[4] * q.x + m[5] * q.y + m[6] * q.z + m[7],
                           m[8] * q.x + m[9] * q.y + m[10] * q.z + m[11]);
    };
    const float3 pv = xf(p);
    zv = pv.z;
    const bool clipped = pv.z <= kTNear;
    const float2 xy = project_pix(fx, fy, pv, cx, cy);
    const Axes A = quat_axes(quat);
    const float ell = 3.0f * glob_scale;
    const float e1 = ell * sx, e2 = ell * sy;
    float2 pix[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const bool s1 = k < 2, s2 = (k % 2) == 0;
        float3 c;
        c.x = s1 ? p.x + e1 * A.a1.x : p.x - e1 * A.a1.x;
        c.x = s2 ? c.x + e2 * A.a2.x : c.x - e2 * A.a2.x;
        c.y = s1 ? p.y + e1 * A.a1.y : p.y - e1 * A.a1.y;
        c.y = s2 ? c.y + e2 * A.a2.y : c.y - e2 * A.a2.y;
        c.z = s1 ? p.z + e1 * A.a1.z : p.z - e1 * A.a1.z;
        c.z = s2 ? c.z + e2 * A.a2.z : c.z - e2 * A.a2.z;
        float3 cv = xf(c);
        cv.z = fmaxf(cv.z, kTNear);
        pix[k] = project_pix(fx, fy, cv, cx, cy);
    }
    const float mxx = fmaxf(fmaxf(pix[0].x, pix[1].x), fmaxf(pix[2].x, pix[3].x));
    const float mxy = fmaxf(fmaxf(pix[0].y, pix[1].y), fmaxf(pix[2].y, pix[3].y));
    const float mnx = fminf(fminf(pix[0].x, pix[1].x), fminf(pix[2].x, pix[3].x));
    const float mny = fminf(fminf(pix[0].y, pix[1].y), fminf(pix[2].y, pix[3].y));
    if (clipped) {
        center = xy;
        extent = make_float2(0.f, 0.f);
    } else {
        center = make_float2(0.5f * (mxx + mnx), 0.5f * (mxy + mny));
        extent = make_float2(0.5f * (mxx - mnx), 0.5f * (mxy - mny));
    }
}

// Tile count of gstex_cuda/get_aabb_2d.py:70-91 (float32 floor formula).
__device__ __forceinline__ int tiles_hit(float2 c, float2 e, int tiles_x, int tiles_y, float fbw) {
    const int x0 = min(max(__float2int_rz(floorf(__fdiv_rn(c.x - e.x, fbw))), 0), tiles_x);
    const int y0 = min(max(__float2int_rz(floorf(__fdiv_rn(c.y - e.y, fbw))), 0), tiles_y);
    const int x1 = min(max(__float2int_rz(floorf(__fdiv_rn(c.x + e.x, fbw) + 1.0f)), 0), tiles_x);
    const int y1 = min(max(__float2int_rz(floorf(__fdiv_rn(c.y + e.y, fbw) + 1.0f)), 0), tiles_y);
    return (x1 - x0) * (y1 - y0);
}

// Tile rectangle enumerated by the emission kernel (helpers.cuh:37-92).
__device__ __forceinline__ void tile_rect(float2 c, float2 e, int tiles_x, int tiles_y, int bw, int& x0, int& y0,
                                          int& x1, int& y1) {
    const float fbw = (float)bw;
    const float tcx = __fdiv_rn(c.x, fbw), tcy = __fdiv_rn(c.y, fbw);
    const float tex = __fdiv_rn(e.x, fbw), tey = __fdiv_rn(e.y, fbw);
    x0 = min(max(0, __float2int_rz(__fsub_rn(tcx, tex))), tiles_x);
    x1 = min(max(0, __float2int_rz(__fadd_rn(__fadd_rn(tcx, tex), 1.0f))), tiles_x);
    y0 = min(max(0, __float2int_rz(__fsub_rn(tcy, tey))), tiles_y);
    y1 = min(max(0, __float2int_rz(__fadd_rn(__fadd_rn(tcy, tey), 1.0f))), tiles_y);
}

// Spherical-harmonic basis (csrc/sh.cuh:46-118; gstex_cuda/_torch_impl.py:62-113).
__device__ __forceinline__ int sh_bases(int deg) { return deg <= 0 ? 1 : deg == 1 ? 4 : deg == 2 ? 9 : deg == 3 ? 16 : 25; }

__device__ __forceinline__ int sh_basis(int deg, float3 dir, float* Y) {
    Y[0] = 0.28209479177387814f;
    if (deg < 1) return 1;
    const float nrm = sqrtf(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
    const float x = dir.x / nrm, y = dir.y / nrm, z = dir.z / nrm;
    const float xx = x * x, xy = x * y, xz = x * z, yy = y * y, yz = y * z, zz = z * z;
    Y[1] = -0.4886025119029199f * y;
    Y[2] = 0.4886025119029199f * z;
    Y[3] = -0.4886025119029199f * x;
    if (deg < 2) return 4;
    Y[4] = 1.0925484305920792f * xy;
    Y[5] = -1.0925484305920792f * yz;
    Y[6] = 0.31539156525252005f * (2.f * zz - xx - yy);
    Y[7] = -1.0925484305920792f * xz;
    Y[8] = 0.5462742152960396f * (xx - yy);
    if (deg < 3) return 9;
    Y[9] = -0.5900435899266435f * y * (3.f * xx - yy);
    Y[10] = 2.890611442640554f * xy * z;
    Y[11] = -0.4570457994644658f * y * (4.f * zz - xx - yy);
    Y[12] = 0.3731763325901154f * z * (2.f * zz - 3.f * xx - 3.f * yy);
    Y[13] = -0.4570457994644658f * x * (4.f * zz - xx - yy);
    Y[14] = 1.445305721320277f * z * (xx - yy);
    Y[15] = -0.5900435899266435f * x * (xx - 3.f * yy);
    if (deg < 4) return 16;
    Y[16] = 2.5033429417967046f * xy * (xx - yy);
    Y[17] = -1.7701307697799304f * yz * (3.f * xx - yy);
    Y[18] = 0.9461746957575601f * xy * (7.f * zz - 1.f);
    Y[19] = -0.6690465435572892f * yz * (7.f * zz - 3.f);
    Y[20] = 0.10578554691520431f * (zz * (35.f * zz - 30.f) + 3.f);
    Y[21] = -0.6690465435572892f * xz * (7.f * zz - 3.f);
    Y[22] = 0.47308734787878004f * (xx - yy) * (7.f * zz - 1.f);
    Y[23] = -1.7701307697799304f * xz * (xx - 3.f * yy);
    Y[24] = 0.6258357354491761f * (xx * (xx - 3.f * yy) - yy * (3.f * xx - yy));
    return 25;
}


}  // namespace gstex
