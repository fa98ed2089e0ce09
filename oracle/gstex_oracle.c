/*
 * CPU oracle for the textured 2D-Gaussian rasteriser hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference algorithm (victor-rong/GStex_cuda, paths relative to the
 * reference project; csrc = gstex_cuda/cuda/csrc).  It exists so that the
 * tests, the smoke check and the CPU baseline leg of the benchmark can check
 * the CUDA library against an independent implementation.  Nothing in the
 * product package imports, links or calls it.
 *
 * The file is compiled twice: with REAL = float (prefix or32_) to follow the
 * reference kernels' fp32 arithmetic in the same operation order, and with
 * REAL = double (prefix or64_) as the high-precision oracle.  Thresholds are
 * the reference's float constants in both builds, so the two builds differ
 * only by rounding.  Build with -ffp-contract=off so that x86 and Arm hosts
 * give identical results.
 *
 * Integer work (tile counts, intersection keys, sorting, tile ranges) always
 * runs on float32 inputs, because the reference's 64-bit sort keys embed the
 * float32 bit pattern of the depth.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef OR_F64
typedef double REAL;
#define FN(name) or64_##name
#define R_EXP exp
#define R_SQRT sqrt
#define R_FABS fabs
#define R_FMIN fmin
#define R_FMAX fmax
#else
typedef float REAL;
#define FN(name) or32_##name
#define R_EXP expf
#define R_SQRT sqrtf
#define R_FABS fabsf
#define R_FMIN fminf
#define R_FMAX fmaxf
#endif

/* Reference float constants (csrc/texture.cu:198, 213-217, 494-500;
 * csrc/texture_helpers.cuh:305; csrc/get_aabb_2d.cu:19). */
#define K_T_NEAR ((REAL)0.01f)
#define K_T_FAR ((REAL)1000.0f)
#define K_ALPHA_MAX ((REAL)0.99f)
#define K_ALPHA_MIN ((REAL)(1.f / 255.f))
#define K_T_DONE ((REAL)1e-4f)
#define K_DENOM_EPS ((REAL)1e-6f)
#define K_PROJ_EPS ((REAL)1e-6f)
#define K_BLUR_FSQ ((REAL)2.0f)

typedef struct { REAL x, y, z; } v3;

static inline REAL dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* CUDA's float->int conversion (cvt.rzi.s32): truncate, NaN -> 0, saturate. */
static inline int f2i_rz(double x) {
    if (x != x) return 0;
    if (x >= 2147483647.0) return 2147483647;
    if (x <= -2147483648.0) return (-2147483647 - 1);
    return (int)x;
}

/* helpers.cuh:124-131 (row-major 4x4, first 12 entries) */
static inline v3 transform_4x3(const REAL* m, v3 p) {
    v3 o = { m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
             m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
             m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11] };
    return o;
}

/* helpers.cuh:114-121 */
static inline v3 transform_4x3_rot_t(const REAL* m, v3 p) {
    v3 o = { m[0] * p.x + m[4] * p.y + m[8] * p.z,
             m[1] * p.x + m[5] * p.y + m[9] * p.z,
             m[2] * p.x + m[6] * p.y + m[10] * p.z };
    return o;
}

/* helpers.cuh:145-152 */
static inline void project_pix(REAL fx, REAL fy, v3 p, REAL cx, REAL cy, REAL* ox, REAL* oy) {
    REAL rw = (REAL)1 / (p.z + K_PROJ_EPS);
    REAL qx = p.x * rw, qy = p.y * rw;
    *ox = qx * fx + cx;
    *oy = qy * fy + cy;
}

/* helpers.cuh:155-164 */
static inline v3 project_pix_vjp(REAL fx, REAL fy, v3 p, REAL vx, REAL vy) {
    REAL rw = (REAL)1 / (p.z + K_PROJ_EPS);
    REAL px = fx * vx, py = fy * vy;
    v3 o = { px * rw, py * rw, -(px * p.x + py * p.y) * rw * rw };
    return o;
}

/* helpers.cuh:166-185: quaternion (w,x,y,z) -> rotation; the three columns
 * are the splat's tangent axes ax1, ax2 and its normal ax3. */
static inline void quat_axes(const REAL* q, v3* a1, v3* a2, v3* a3) {
    REAL w = q[0], x = q[1], y = q[2], z = q[3];
    a1->x = (REAL)1 - (REAL)2 * (y * y + z * z);
    a1->y = (REAL)2 * (x * y + w * z);
    a1->z = (REAL)2 * (x * z - w * y);
    a2->x = (REAL)2 * (x * y - w * z);
    a2->y = (REAL)1 - (REAL)2 * (x * x + z * z);
    a2->z = (REAL)2 * (y * z + w * x);
    a3->x = (REAL)2 * (x * z + w * y);
    a3->y = (REAL)2 * (y * z - w * x);
    a3->z = (REAL)1 - (REAL)2 * (x * x + y * y);
}

/* helpers.cuh:187-228. vR[c] is column c (the gradient w.r.t. axis c). */
static inline void quat_axes_vjp(const REAL* q, const v3 vR[3], REAL* out) {
    REAL w = q[0], x = q[1], y = q[2], z = q[3];
    /* vR[c].{x,y,z} = column c, rows 0..2, i.e. glm v_R[c][r]. */
    REAL r01 = vR[0].y, r02 = vR[0].z, r10 = vR[1].x, r12 = vR[1].z;
    REAL r20 = vR[2].x, r21 = vR[2].y, r00 = vR[0].x, r11 = vR[1].y, r22 = vR[2].z;
    out[0] = (REAL)2 * (x * (r12 - r21) + y * (r20 - r02) + z * (r01 - r10));
    out[1] = (REAL)2 * (-(REAL)2 * x * (r11 + r22) + y * (r01 + r10) + z * (r02 + r20) + w * (r12 - r21));
    out[2] = (REAL)2 * (x * (r01 + r10) - (REAL)2 * y * (r00 + r22) + z * (r12 + r21) + w * (r20 - r02));
    out[3] = (REAL)2 * (x * (r02 + r20) + y * (r12 + r21) - (REAL)2 * z * (r00 + r11) + w * (r01 - r10));
}

/* texture_helpers.cuh:336-352 */
static inline void get_ray(const REAL* c2w, REAL fx, REAL fy, REAL cx, REAL cy, REAL px, REAL py,
                           v3* origin, v3* ray) {
    origin->x = c2w[3]; origin->y = c2w[7]; origin->z = c2w[11];
    REAL u = (px - cx) / fx, v = (py - cy) / fy;
    v3 d = { u, v, (REAL)1 };
    v3 r = transform_4x3(c2w, d);
    r.x = r.x - origin->x; r.y = r.y - origin->y; r.z = r.z - origin->z;
    REAL n = R_SQRT(r.x * r.x + r.y * r.y + r.z * r.z);
    r.x = r.x / n; r.y = r.y / n; r.z = r.z / n;
    *ray = r;
}

/* texture_helpers.cuh:302-313, 322-327 (denominator clamp) */
static inline REAL clamp_denom(REAL d) {
    if ((REAL)0 <= d && d < K_DENOM_EPS) return K_DENOM_EPS;
    if (-K_DENOM_EPS < d && d <= (REAL)0) return -K_DENOM_EPS;
    return d;
}

/* texture_helpers.cuh:302-313 */
static inline REAL compute_tt(v3 o, v3 ray, v3 mean, v3 n) {
    v3 diff = { mean.x - o.x, mean.y - o.y, mean.z - o.z };
    REAL den = clamp_denom(dot3(n, ray));
    return dot3(n, diff) / den;
}

/* texture_helpers.cuh:315-334 */
static inline void compute_tt_vjp(v3 o, v3 ray, v3 mean, v3 n, REAL t, REAL v_t, v3* v_mean, v3* v_n) {
    v3 diff = { mean.x - o.x, mean.y - o.y, mean.z - o.z };
    REAL den = clamp_denom(dot3(n, ray));
    v_mean->x += n.x * v_t / den;
    v_mean->y += n.y * v_t / den;
    v_mean->z += n.z * v_t / den;
    v_n->x += (diff.x - ray.x * t) * v_t / den;
    v_n->y += (diff.y - ray.y * t) * v_t / den;
    v_n->z += (diff.z - ray.z * t) * v_t / den;
}

/* texture_helpers.cuh:37-51 (replicate padding clamps uv to [0,1]) */
static inline void clamp_coord(REAL* u, REAL* v) {
    if (*u <= (REAL)0) *u = (REAL)0;
    if (*u >= (REAL)1) *u = (REAL)1;
    if (*v <= (REAL)0) *v = (REAL)0;
    if (*v >= (REAL)1) *v = (REAL)1;
}

/* texture_helpers.cuh:162-215: bilinear (or nearest) weights and texel
 * indices inside chart (h, w, start) for channel ch of C channels. */
static inline void chart_weights(int h, int w, int si, int C, int ch, REAL u, REAL v, int bilinear,
                                 REAL wts[4], long idx[4], REAL* fx_out, REAL* fy_out) {
    REAL tcx = (REAL)h * u, tcy = (REAL)w * v;
    int iix = f2i_rz(tcx), iiy = f2i_rz(tcy);
    int jjx = iix + 1 < h - 1 ? iix + 1 : h - 1;
    int jjy = iiy + 1 < w - 1 ? iiy + 1 : w - 1;
    REAL wx = tcx - (REAL)iix, wy = tcy - (REAL)iiy;
    iix = iix < h - 1 ? iix : h - 1;
    iiy = iiy < w - 1 ? iiy : w - 1;
    REAL wii = ((REAL)1 - wx) * ((REAL)1 - wy);
    REAL wij = ((REAL)1 - wx) * (wy);
    REAL wji = (wx) * ((REAL)1 - wy);
    REAL wjj = (wx) * (wy);
    idx[0] = ((long)si + (long)iix * w + iiy) * C + ch;
    idx[1] = ((long)si + (long)iix * w + jjy) * C + ch;
    idx[2] = ((long)si + (long)jjx * w + iiy) * C + ch;
    idx[3] = ((long)si + (long)jjx * w + jjy) * C + ch;
    if (bilinear) {
        wts[0] = wii; wts[1] = wij; wts[2] = wji; wts[3] = wjj;
    } else {
        wts[0] = wts[1] = wts[2] = wts[3] = (REAL)0;
        if (wii >= wij && wii >= wji && wii >= wjj) wts[0] = (REAL)1;
        else if (wij >= wii && wij >= wji && wij >= wjj) wts[1] = (REAL)1;
        else if (wji >= wii && wji >= wij && wji >= wjj) wts[2] = (REAL)1;
        else wts[3] = (REAL)1;
    }
    *fx_out = wx; *fy_out = wy;
}

/* helpers.cuh:259-264 */
static inline void distortion(REAL val, REAL w, REAL s[3], REAL* err) {
    *err += w * (val * val * s[0] + s[2] - (REAL)2 * val * s[1]);
    s[0] += w;
    s[1] += w * val;
    s[2] += w * val * val;
}

/* helpers.cuh:266-269 */
static inline void distortion_vjp(REAL val, REAL w, const REAL s[3], REAL v_err, REAL* v_val, REAL* v_w) {
    *v_val += (REAL)2 * (w * val * s[0] - w * s[1]) * v_err;
    *v_w += (val * val * s[0] - (REAL)2 * val * s[1] + s[2]) * v_err;
}

/* texture_helpers.cuh:355-366 */
static inline void pixel_to_plane(const REAL* c2w, REAL fx, REAL fy, REAL cx, REAL cy, REAL px, REAL py,
                                  v3 mean, v3 a1, v3 a2, v3 a3, REAL* u, REAL* v) {
    v3 o, ray;
    get_ray(c2w, fx, fy, cx, cy, px, py, &o, &ray);
    REAL t = compute_tt(o, ray, mean, a3);
    v3 d = { o.x + t * ray.x - mean.x, o.y + t * ray.y - mean.y, o.z + t * ray.z - mean.z };
    *u = dot3(d, a1);
    *v = dot3(d, a2);
}

/* texture_helpers.cuh:390-417 */
static REAL local_outline(const REAL* c2w, REAL fx, REAL fy, REAL cx, REAL cy, REAL px, REAL py, v3 mean,
                          v3 a1, v3 a2, v3 a3, REAL s1, REAL s2, int width, REAL sigma_thresh) {
    REAL min_dis = (REAL)1000.0f;
    for (int dx = -width; dx <= width; dx++) {
        for (int dy = -width; dy <= width; dy++) {
            REAL u, v;
            pixel_to_plane(c2w, fx, fy, cx, cy, px + (REAL)dx, py + (REAL)dy, mean, a1, a2, a3, &u, &v);
            REAL as1 = u / s1, as2 = v / s2;
            REAL sg = (REAL)0.5f * (as1 * as1 + as2 * as2);
            if (sg > sigma_thresh) {
                REAL cd = R_SQRT((REAL)(dx * dx + dy * dy));
                if (min_dis > cd) min_dis = cd;
            }
        }
    }
    return min_dis;
}

static inline void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* ------------------------------------------------------------------------
 * get_aabb_2d: csrc/get_aabb_2d.cu:11-89
 * ---------------------------------------------------------------------- */
void FN(get_aabb_2d)(int n, const REAL* means, const REAL* scales, REAL glob_scale, const REAL* quats,
                     const REAL* viewmat, REAL fx, REAL fy, REAL cx, REAL cy, REAL* centers, REAL* extents) {
    for (int i = 0; i < n; i++) {
        v3 p = { means[3 * i], means[3 * i + 1], means[3 * i + 2] };
        v3 pv = transform_4x3(viewmat, p);
        int clipped = pv.z <= K_T_NEAR;
        REAL xyx, xyy;
        project_pix(fx, fy, pv, cx, cy, &xyx, &xyy);
        v3 a1, a2, a3;
        quat_axes(quats + 4 * i, &a1, &a2, &a3);
        REAL ell = (REAL)3.0f * glob_scale;
        REAL sx = scales[3 * i], sy = scales[3 * i + 1];
        v3 c[4];
        for (int k = 0; k < 4; k++) {
            REAL s1 = (k < 2) ? (REAL)1 : (REAL)-1;  /* corner00, 01: +ax1 */
            REAL s2 = (k % 2 == 0) ? (REAL)1 : (REAL)-1;
            /* point + ell*sx*ax1 (+/-) ell*sy*ax2, evaluated left to right */
            REAL e1 = ell * sx, e2 = ell * sy;
            c[k].x = (s1 > 0 ? p.x + e1 * a1.x : p.x - e1 * a1.x);
            c[k].x = (s2 > 0 ? c[k].x + e2 * a2.x : c[k].x - e2 * a2.x);
            c[k].y = (s1 > 0 ? p.y + e1 * a1.y : p.y - e1 * a1.y);
            c[k].y = (s2 > 0 ? c[k].y + e2 * a2.y : c[k].y - e2 * a2.y);
            c[k].z = (s1 > 0 ? p.z + e1 * a1.z : p.z - e1 * a1.z);
            c[k].z = (s2 > 0 ? c[k].z + e2 * a2.z : c[k].z - e2 * a2.z);
        }
        REAL px[4], py[4];
        for (int k = 0; k < 4; k++) {
            v3 cv = transform_4x3(viewmat, c[k]);
            cv.z = R_FMAX(cv.z, K_T_NEAR);  /* helpers.cuh:250-257 */
            project_pix(fx, fy, cv, cx, cy, &px[k], &py[k]);
        }
#define MAXR(a, b) R_FMAX(a, b)
#define MINR(a, b) R_FMIN(a, b)
        REAL mxx = MAXR(MAXR(px[0], px[1]), MAXR(px[2], px[3]));
        REAL mxy = MAXR(MAXR(py[0], py[1]), MAXR(py[2], py[3]));
        REAL mnx = MINR(MINR(px[0], px[1]), MINR(px[2], px[3]));
        REAL mny = MINR(MINR(py[0], py[1]), MINR(py[2], py[3]));
        if (clipped) {
            centers[2 * i] = xyx; centers[2 * i + 1] = xyy;
            extents[2 * i] = 0; extents[2 * i + 1] = 0;
        } else {
            centers[2 * i] = (REAL)0.5f * (mxx + mnx);
            centers[2 * i + 1] = (REAL)0.5f * (mxy + mny);
            extents[2 * i] = (REAL)0.5f * (mxx - mnx);
            extents[2 * i + 1] = (REAL)0.5f * (mxy - mny);
        }
    }
}

/* ------------------------------------------------------------------------
 * Spherical harmonics: csrc/sh.cuh:46-118 (forward), 120-210 (vjp);
 * the basis polynomials are the ones of gstex_cuda/_torch_impl.py:62-113.
 * ---------------------------------------------------------------------- */
static const double SHC0 = 0.28209479177387814;
static const double SHC1 = 0.4886025119029199;
static const double SHC2[5] = { 1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
                                -1.0925484305920792, 0.5462742152960396 };
static const double SHC3[7] = { -0.5900435899266435, 2.890611442640554, -0.4570457994644658,
                                0.3731763325901154, -0.4570457994644658, 1.445305721320277,
                                -0.5900435899266435 };
static const double SHC4[9] = { 2.5033429417967046, -1.7701307697799304, 0.9461746957575601,
                                -0.6690465435572892, 0.10578554691520431, -0.6690465435572892,
                                0.47308734787878004, -1.7701307697799304, 0.6258357354491761 };

static int sh_bases(int deg) { return deg == 0 ? 1 : deg == 1 ? 4 : deg == 2 ? 9 : deg == 3 ? 16 : 25; }

/* Basis values Y_b(dir) for b < sh_bases(deg); dir is normalised first
 * (sh.cuh:61-66). */
static int sh_basis(int deg, const REAL* dir, REAL* Y) {
    Y[0] = (REAL)SHC0;
    if (deg < 1) return 1;
    REAL nrm = R_SQRT(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    REAL x = dir[0] / nrm, y = dir[1] / nrm, z = dir[2] / nrm;
    REAL xx = x * x, xy = x * y, xz = x * z, yy = y * y, yz = y * z, zz = z * z;
    Y[1] = -(REAL)SHC1 * y;
    Y[2] = (REAL)SHC1 * z;
    Y[3] = -(REAL)SHC1 * x;
    if (deg < 2) return 4;
    Y[4] = (REAL)SHC2[0] * xy;
    Y[5] = (REAL)SHC2[1] * yz;
    Y[6] = (REAL)SHC2[2] * ((REAL)2 * zz - xx - yy);
    Y[7] = (REAL)SHC2[3] * xz;
    Y[8] = (REAL)SHC2[4] * (xx - yy);
    if (deg < 3) return 9;
    Y[9] = (REAL)SHC3[0] * y * ((REAL)3 * xx - yy);
    Y[10] = (REAL)SHC3[1] * xy * z;
    Y[11] = (REAL)SHC3[2] * y * ((REAL)4 * zz - xx - yy);
    Y[12] = (REAL)SHC3[3] * z * ((REAL)2 * zz - (REAL)3 * xx - (REAL)3 * yy);
    Y[13] = (REAL)SHC3[4] * x * ((REAL)4 * zz - xx - yy);
    Y[14] = (REAL)SHC3[5] * z * (xx - yy);
    Y[15] = (REAL)SHC3[6] * x * (xx - (REAL)3 * yy);
    if (deg < 4) return 16;
    Y[16] = (REAL)SHC4[0] * xy * (xx - yy);
    Y[17] = (REAL)SHC4[1] * yz * ((REAL)3 * xx - yy);
    Y[18] = (REAL)SHC4[2] * xy * ((REAL)7 * zz - (REAL)1);
    Y[19] = (REAL)SHC4[3] * yz * ((REAL)7 * zz - (REAL)3);
    Y[20] = (REAL)SHC4[4] * (zz * ((REAL)35 * zz - (REAL)30) + (REAL)3);
    Y[21] = (REAL)SHC4[5] * xz * ((REAL)7 * zz - (REAL)3);
    Y[22] = (REAL)SHC4[6] * (xx - yy) * ((REAL)7 * zz - (REAL)1);
    Y[23] = (REAL)SHC4[7] * xz * (xx - (REAL)3 * yy);
    Y[24] = (REAL)SHC4[8] * (xx * (xx - (REAL)3 * yy) - yy * ((REAL)3 * xx - yy));
    return 25;
}

/* compute_sh_forward: coeffs [n, sh_bases(degree), 3] -> colors [n, 3] using
 * the first sh_bases(degrees_to_use) bases, summed per degree band as in
 * sh.cuh:54-117 (kernel sh.cuh:212-232). */
void FN(sh_forward)(int n, int degree, int degrees_to_use, const REAL* dirs, const REAL* coeffs, REAL* colors) {
    static const int band_lo[5] = { 0, 1, 4, 9, 16 };
    static const int band_hi[5] = { 1, 4, 9, 16, 25 };
    int B = sh_bases(degree);
    for (int i = 0; i < n; i++) {
        REAL Y[25];
        int nb = sh_basis(degrees_to_use, dirs + 3 * i, Y);
        const REAL* k = coeffs + (long)i * B * 3;
        for (int c = 0; c < 3; c++) {
            REAL acc = Y[0] * k[c];
            for (int band = 1; band < 5 && band_hi[band] <= nb; band++) {
                REAL part;
                if (band == 1) {
                    /* SH_C1 * (-y*k1 + z*k2 - x*k3), sh.cuh:77-79 */
                    REAL s1 = (REAL)SHC1;
                    REAL x = -Y[3] / s1, y = -Y[1] / s1, z = Y[2] / s1;
                    part = s1 * (-y * k[3 + c] + z * k[6 + c] - x * k[9 + c]);
                } else {
                    part = 0;
                    for (int b = band_lo[band]; b < band_hi[band]; b++) part += Y[b] * k[3 * b + c];
                }
                acc += part;
            }
            colors[3 * i + c] = acc;
        }
    }
}

/* compute_sh_backward: v_coeffs[i,b,c] = Y_b * v_colors[i,c]; entries beyond
 * sh_bases(degrees_to_use) are zero (sh.cuh:234-253, bindings.cu:66-67). */
void FN(sh_backward)(int n, int degree, int degrees_to_use, const REAL* dirs, const REAL* v_colors, REAL* v_coeffs) {
    int B = sh_bases(degree);
    for (int i = 0; i < n; i++) {
        REAL Y[25];
        int nb = sh_basis(degrees_to_use, dirs + 3 * i, Y);
        for (int b = 0; b < B; b++)
            for (int c = 0; c < 3; c++)
                v_coeffs[((long)i * B + b) * 3 + c] = b < nb ? Y[b] * v_colors[3 * i + c] : (REAL)0;
    }
}

/* ------------------------------------------------------------------------
 * texture_sample: bilinear lookup in jagged charts with uv clamped to
 * [0,1] (gstex_cuda/_torch_impl.py:149-194; csrc/texture_sample.cu:11-36).
 * The backward returns the texel and uv gradients of that lookup; the
 * reference's own backward is unused (gstex_cuda/texture_sample.py:70-78).
 * ---------------------------------------------------------------------- */
void FN(texture_sample_forward)(int nq, int C, const int32_t* dims, const REAL* uvs, const REAL* texture, REAL* out) {
    for (int q = 0; q < nq; q++) {
        REAL u = uvs[2 * q], v = uvs[2 * q + 1];
        clamp_coord(&u, &v);
        for (int ch = 0; ch < C; ch++) {
            REAL w[4], fx, fy;
            long id[4];
            chart_weights(dims[3 * q], dims[3 * q + 1], dims[3 * q + 2], C, ch, u, v, 1, w, id, &fx, &fy);
            out[(long)q * C + ch] = w[0] * texture[id[0]] + w[1] * texture[id[1]] + w[2] * texture[id[2]] +
                                    w[3] * texture[id[3]];
        }
    }
}

void FN(texture_sample_backward)(int nq, int C, const int32_t* dims, const REAL* uvs, const REAL* texture,
                                 const REAL* v_out, REAL* v_texture, REAL* v_uvs) {
    for (int q = 0; q < nq; q++) {
        REAL u0 = uvs[2 * q], v0 = uvs[2 * q + 1];
        REAL u = u0, v = v0;
        clamp_coord(&u, &v);
        int h = dims[3 * q], w = dims[3 * q + 1];
        REAL gu = 0, gv = 0;
        for (int ch = 0; ch < C; ch++) {
            REAL wt[4], fx, fy;
            long id[4];
            chart_weights(h, w, dims[3 * q + 2], C, ch, u, v, 1, wt, id, &fx, &fy);
            REAL g = v_out[(long)q * C + ch];
            for (int k = 0; k < 4; k++) v_texture[id[k]] += wt[k] * g;
            REAL t00 = texture[id[0]], t01 = texture[id[1]], t10 = texture[id[2]], t11 = texture[id[3]];
            gu += g * (-((REAL)1 - fy) * t00 - fy * t01 + ((REAL)1 - fy) * t10 + fy * t11) * (REAL)h;
            gv += g * (-((REAL)1 - fx) * t00 + ((REAL)1 - fx) * t01 - fx * t10 + fx * t11) * (REAL)w;
        }
        /* clamp passes the gradient through only inside [0,1] */
        v_uvs[2 * q] = (u0 >= 0 && u0 <= 1) ? gu : (REAL)0;
        v_uvs[2 * q + 1] = (v0 >= 0 && v0 <= 1) ? gv : (REAL)0;
    }
}

/* ------------------------------------------------------------------------
 * Textured compositor forward: csrc/texture.cu:11-329, one pixel at a time.
 * The per-tile batching of the reference does not change per-pixel results,
 * so each pixel walks its tile's sorted range front to back.
 * ---------------------------------------------------------------------- */
typedef struct {
    int tiles_x, tiles_y, bw, img_w, img_h, C;
    const int32_t *texture_dims, *gids, *tile_bins;
    const REAL *colors, *opac, *means, *scales;
    REAL glob_scale;
    const REAL *quats, *uv0, *umap, *vmap, *texture, *viewmat, *c2w;
    REAL fx, fy, cx, cy;
    int settings;
    const REAL* bg;
} raster_args;

int FN(texture_forward)(int tiles_x, int tiles_y, int bw, int img_w, int img_h, int C,
                        const int32_t* texture_dims, const int32_t* gids, const int32_t* tile_bins,
                        const REAL* colors, const REAL* opac, const REAL* means, const REAL* scales,
                        REAL glob_scale, const REAL* quats, const REAL* uv0, const REAL* umap, const REAL* vmap,
                        const REAL* texture, const REAL* viewmat, const REAL* c2w, REAL fx, REAL fy, REAL cx,
                        REAL cy, int settings, const REAL* bg, REAL* final_T, int32_t* final_idx,
                        int32_t* depth_idx, REAL* reg_s, REAL* out_img, REAL* out_depth, REAL* out_reg,
                        REAL* out_tex, REAL* out_normal, int nthreads) {
    if (C > 64) return 1;
    const int use_blur = (settings & (1 << 9)) != 0;
    const int use_ndc = (settings & (1 << 10)) != 0;
    const int vis_mode = (settings & (1 << 15)) != 0;
    const int alpha_vis = (settings & (1 << 16)) != 0;
    const REAL alpha_bound = (REAL)((float)((settings & (0x1f << 17)) >> 17) / 8.0f);
    const REAL outline_bound = (REAL)((float)((settings & (0xf << 26)) >> 26) / 4.0f);
    const int accept_opac = (settings & (1 << 25)) != 0;
    const int white_outline = (settings & (1 << 24)) != 0;
    const int bilinear = !(settings & (1 << 2));
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int bi = 0; bi < img_h; bi++) {
        for (int bj = 0; bj < img_w; bj++) {
            const int tile = (bi / bw) * tiles_x + (bj / bw);
            const long pix = (long)bi * img_w + bj;
            REAL px = (REAL)bj + (REAL)0.5, py = (REAL)bi + (REAL)0.5;
            v3 o, ray;
            get_ray(c2w, fx, fy, cx, cy, px, py, &o, &ray);
            REAL view_depth = viewmat[8] * ray.x + viewmat[9] * ray.y + viewmat[10] * ray.z;
            int rs = tile_bins[2 * tile], re = tile_bins[2 * tile + 1];
            REAL T = 1, out[3] = { 0, 0, 0 }, nrm[3] = { 0, 0, 0 }, depth = 0, reg = 0;
            REAL ts[3] = { 0, 0, 0 }, otex[64];
            int didx = -1, cur = 0, done = 0;
            for (int k = 0; k < C; k++) otex[k] = 0;
            for (int idx = rs; idx < re && !done; idx++) {
                const int g = gids[idx];
                v3 mean = { means[3 * g], means[3 * g + 1], means[3 * g + 2] };
                REAL sx = scales[3 * g], sy = scales[3 * g + 1];
                REAL op = opac[g];
                v3 a1, a2, a3;
                quat_axes(quats + 4 * g, &a1, &a2, &a3);
                REAL t = compute_tt(o, ray, mean, a3);
                v3 pos = { o.x + t * ray.x, o.y + t * ray.y, o.z + t * ray.z };
                v3 d = { pos.x - mean.x, pos.y - mean.y, pos.z - mean.z };
                REAL l1 = dot3(d, a1), l2 = dot3(d, a2);
                REAL is1 = (REAL)1 / (sx * glob_scale), is2 = (REAL)1 / (sy * glob_scale);
                REAL sigma = (REAL)0.5f * (is1 * is1 * l1 * l1 + is2 * is2 * l2 * l2);
                v3 pv = transform_4x3(viewmat, mean);
                REAL xyx, xyy;
                project_pix(fx, fy, pv, cx, cy, &xyx, &xyy);
                REAL ddx = xyx - px, ddy = xyy - py;
                REAL sigma_blur = (REAL)0.5f * K_BLUR_FSQ * (ddx * ddx + ddy * ddy);
                REAL nbf = 1, bf = 0;
                if (use_blur && sigma_blur < sigma) { bf = 1; nbf = 0; }
                REAL alpha = R_FMIN(K_ALPHA_MAX, op * (nbf * R_EXP(-sigma) + bf * R_EXP(-sigma_blur)));
                REAL pixel_dis = (REAL)1000.0f;
                if (alpha_vis) {
                    alpha = K_ALPHA_MAX;
                    REAL sth = (REAL)0.5f * alpha_bound * alpha_bound;
                    if (sigma > sth) alpha = 0;
                    if (accept_opac && op < (REAL)0.5f) alpha = 0;
                    pixel_dis = local_outline(c2w, fx, fy, cx, cy, px, py, mean, a1, a2, a3, sx * glob_scale,
                                              sy * glob_scale, 3, sth);
                }
                int skip = (t < K_T_NEAR || t > K_T_FAR || alpha < K_ALPHA_MIN);
                REAL next_T = T * ((REAL)1 - alpha);
                if (next_T <= K_T_DONE) done = 1;  /* texture.cu:216-221, also for skipped */
                if (skip || done) continue;
                REAL vis = alpha * T;
                const REAL* c = colors + 3 * g;
                int plain = (!alpha_vis || pixel_dis > outline_bound);
                if (plain) {
                    out[0] = out[0] + c[0] * vis; out[1] = out[1] + c[1] * vis; out[2] = out[2] + c[2] * vis;
                } else if (white_outline) {
                    out[0] = out[0] + vis; out[1] = out[1] + vis; out[2] = out[2] + vis;
                }
                v3 hn = a3;
                if (vis_mode && ray.x * a3.x + ray.y * a3.y + ray.z * a3.z > 0) { hn.x = -a3.x; hn.y = -a3.y; hn.z = -a3.z; }
                nrm[0] += vis * hn.x; nrm[1] += vis * hn.y; nrm[2] += vis * hn.z;
                REAL t_view = t * view_depth;
                const int32_t* dm = texture_dims + 3 * g;
                v3 um = { umap[3 * g], umap[3 * g + 1], umap[3 * g + 2] };
                v3 vm = { vmap[3 * g], vmap[3 * g + 1], vmap[3 * g + 2] };
                REAL uu = uv0[2 * g] + dot3(um, d), vv = uv0[2 * g + 1] + dot3(vm, d);
                clamp_coord(&uu, &vv);
                for (int k = 0; k < C; k++) {
                    REAL w[4], wx, wy;
                    long id[4];
                    chart_weights(dm[0], dm[1], dm[2], C, k, uu, vv, bilinear, w, id, &wx, &wy);
                    REAL val = w[0] * texture[id[0]] + w[1] * texture[id[1]] + w[2] * texture[id[2]] + w[3] * texture[id[3]];
                    if (plain) otex[k] += vis * val;
                    else if (white_outline) otex[k] += vis;
                }
                if (T > (REAL)0.5f) { depth = t_view; didx = idx; }
                if (use_ndc) {
                    REAL t_ndc = (K_T_FAR * t_view - K_T_FAR * K_T_NEAR) / ((K_T_FAR - K_T_NEAR) * t_view);
                    distortion(t_ndc, vis, ts, &reg);
                } else {
                    distortion(t, vis, ts, &reg);
                }
                T = next_T;
                cur = idx;
            }
            final_T[pix] = T;
            final_idx[pix] = cur;
            depth_idx[pix] = didx;
            for (int k = 0; k < 3; k++) {
                out_img[3 * pix + k] = out[k] + T * bg[k];
                out_normal[3 * pix + k] = nrm[k];
                reg_s[3 * pix + k] = ts[k];
            }
            out_depth[pix] = depth;
            out_reg[pix] = reg;
            for (int k = 0; k < C; k++) out_tex[pix * C + k] = otex[k];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * Textured compositor backward: csrc/texture.cu:331-760, one pixel at a
 * time, back to front from the pixel's last contributor.  Gradients are
 * accumulated with atomics as in the reference.
 * ---------------------------------------------------------------------- */
#define ATOMIC_ADD(ptr, val)        \
    do {                            \
        REAL _v = (val);            \
        _Pragma("omp atomic")       \
        (ptr)[0] += _v;             \
    } while (0)

int FN(texture_backward)(int tiles_x, int tiles_y, int bw, int img_w, int img_h, int C,
                         const int32_t* texture_dims, const int32_t* gids, const int32_t* tile_bins,
                         const REAL* colors, const REAL* opac, const REAL* means, const REAL* scales,
                         REAL glob_scale, const REAL* quats, const REAL* uv0, const REAL* umap,
                         const REAL* vmap, const REAL* texture, const REAL* viewmat, const REAL* c2w, REAL fx,
                         REAL fy, REAL cx, REAL cy, int settings, const REAL* bg, const REAL* final_T,
                         const int32_t* final_idx, const int32_t* depth_idx, const REAL* final_s,
                         const REAL* v_img, const REAL* v_depth, const REAL* v_reg, const REAL* v_alpha_out,
                         const REAL* v_tex, const REAL* v_normal, REAL* v_colors, REAL* v_opac, REAL* v_means,
                         REAL* v_scales, REAL* v_quats, REAL* v_uv0, REAL* v_umap, REAL* v_vmap,
                         REAL* v_texture, int nthreads) {
    if (C > 64) return 1;
    const int propagate_uv = (settings & (1 << 8)) != 0;
    const int use_blur = (settings & (1 << 9)) != 0;
    const int use_ndc = (settings & (1 << 10)) != 0;
    const int bilinear = !(settings & (1 << 2));
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int bi = 0; bi < img_h; bi++) {
        for (int bj = 0; bj < img_w; bj++) {
            const int tile = (bi / bw) * tiles_x + (bj / bw);
            const long pix = (long)bi * img_w + bj;
            REAL px = (REAL)bj + (REAL)0.5, py = (REAL)bi + (REAL)0.5;
            v3 o, ray;
            get_ray(c2w, fx, fy, cx, cy, px, py, &o, &ray);
            REAL view_depth = viewmat[8] * ray.x + viewmat[9] * ray.y + viewmat[10] * ray.z;
            REAL T = final_T[pix];
            const REAL* sfin = final_s + 3 * pix;
            int dfin = depth_idx[pix];
            int bfin = final_idx[pix];
            int rs = tile_bins[2 * tile], re = tile_bins[2 * tile + 1];
            v3 vout = { v_img[3 * pix], v_img[3 * pix + 1], v_img[3 * pix + 2] };
            REAL vdepth = v_depth[pix], vreg = v_reg[pix], valpha = v_alpha_out[pix];
            v3 vnorm = { v_normal[3 * pix], v_normal[3 * pix + 1], v_normal[3 * pix + 2] };
            const REAL* vt = v_tex + pix * C;
            v3 bgv = { bg[0], bg[1], bg[2] };
            REAL vT_run = dot3(bgv, vout) - valpha;
            /* entries after the pixel's last contributor are skipped
               (texture.cu:483-487): start the walk at it */
            for (int idx = (bfin < re - 1 ? bfin : re - 1); idx >= rs; idx--) {
                const int g = gids[idx];
                v3 mean = { means[3 * g], means[3 * g + 1], means[3 * g + 2] };
                REAL sx = scales[3 * g], sy = scales[3 * g + 1];
                REAL op = opac[g];
                v3 a1, a2, a3;
                quat_axes(quats + 4 * g, &a1, &a2, &a3);
                REAL t = compute_tt(o, ray, mean, a3);
                v3 pos = { o.x + t * ray.x, o.y + t * ray.y, o.z + t * ray.z };
                v3 d = { pos.x - mean.x, pos.y - mean.y, pos.z - mean.z };
                REAL l1 = dot3(d, a1), l2 = dot3(d, a2);
                REAL sf = (REAL)0.5f / (glob_scale * glob_scale);
                REAL sg1 = l1 * l1 / (sx * sx), sg2 = l2 * l2 / (sy * sy);
                REAL sigma = sf * (sg1 + sg2);
                v3 pv = transform_4x3(viewmat, mean);
                REAL xyx, xyy;
                project_pix(fx, fy, pv, cx, cy, &xyx, &xyy);
                REAL ddx = xyx - px, ddy = xyy - py;
                REAL sigma_blur = (REAL)0.5f * K_BLUR_FSQ * (ddx * ddx + ddy * ddy);
                REAL nbf = 1, bf = 0;
                if (use_blur && sigma_blur < sigma) { bf = 1; nbf = 0; }
                REAL es = R_EXP(-sigma), esb = R_EXP(-sigma_blur);
                REAL alpha = R_FMIN(K_ALPHA_MAX, op * (nbf * es + bf * esb));
                if (t < K_T_NEAR || t > K_T_FAR || alpha < K_ALPHA_MIN) continue;

                REAL ra = (REAL)1 / ((REAL)1 - alpha);
                T *= ra;
                REAL vis = alpha * T;
                const REAL* rgb = colors + 3 * g;
                REAL v_vis = rgb[0] * vout.x + rgb[1] * vout.y + rgb[2] * vout.z;
                v_vis += dot3(a3, vnorm);
                v3 v_diff = { 0, 0, 0 };
                REAL vuv0x = 0, vuv0y = 0;
                v3 vum = { 0, 0, 0 }, vvm = { 0, 0, 0 };
                {
                    const int32_t* dm = texture_dims + 3 * g;
                    v3 um = { umap[3 * g], umap[3 * g + 1], umap[3 * g + 2] };
                    v3 vm = { vmap[3 * g], vmap[3 * g + 1], vmap[3 * g + 2] };
                    REAL uu = uv0[2 * g] + dot3(um, d), vv = uv0[2 * g + 1] + dot3(vm, d);
                    clamp_coord(&uu, &vv);
                    REAL vu = 0, vv_ = 0;
                    for (int k = 0; k < C; k++) {
                        REAL w[4], wx, wy;
                        long id[4];
                        chart_weights(dm[0], dm[1], dm[2], C, k, uu, vv, bilinear, w, id, &wx, &wy);
                        REAL c00 = texture[id[0]], c01 = texture[id[1]], c10 = texture[id[2]], c11 = texture[id[3]];
                        REAL val = w[0] * c00 + w[1] * c01 + w[2] * c10 + w[3] * c11;
                        REAL vval = vis * vt[k];
                        for (int q = 0; q < 4; q++) ATOMIC_ADD(v_texture + id[q], w[q] * vval);
                        if (bilinear) {
                            /* texture_helpers.cuh:283-298 */
                            REAL vwx = vval * (-((REAL)1 - wy) * c00 - (wy) * c01 + ((REAL)1 - wy) * c10 + (wy) * c11);
                            REAL vwy = vval * (-((REAL)1 - wx) * c00 + ((REAL)1 - wx) * c01 - (wx) * c10 + (wx) * c11);
                            if (propagate_uv) { vu += (REAL)dm[0] * vwx; vv_ += (REAL)dm[1] * vwy; }
                        }
                        v_vis += val * vt[k];
                    }
                    /* texture_helpers.cuh:62-80 */
                    vuv0x += vu; vuv0y += vv_;
                    vum.x += d.x * vu; vum.y += d.y * vu; vum.z += d.z * vu;
                    vvm.x += d.x * vv_; vvm.y += d.y * vv_; vvm.z += d.z * vv_;
                    if (propagate_uv) {
                        v_diff.x += um.x * vu + vm.x * vv_;
                        v_diff.y += um.y * vu + vm.y * vv_;
                        v_diff.z += um.z * vu + vm.z * vv_;
                    }
                }
                REAL v_alpha = T * v_vis - T * vT_run;
                REAL vT_cur = alpha * v_vis + ((REAL)1 - alpha) * vT_run;
                REAL t_view = t * view_depth;
                REAL t_ndc = (K_T_FAR * t_view - K_T_FAR * K_T_NEAR) / ((K_T_FAR - K_T_NEAR) * t_view);
                REAL v_t = 0, v_t_ndc = 0, v_t_view = 0, v_w = 0;
                if (use_ndc) distortion_vjp(t_ndc, vis, sfin, vreg, &v_t_ndc, &v_w);
                else distortion_vjp(t, vis, sfin, vreg, &v_t, &v_w);
                v_alpha += v_w * T;
                vT_cur += v_w * alpha;
                vT_run = vT_cur;

                REAL v_sigma = -nbf * op * es * v_alpha;
                REAL vsx = -(REAL)2 * sf * sg1 * v_sigma / sx;
                REAL vsy = -(REAL)2 * sf * sg2 * v_sigma / sy;
                REAL v_l1 = (REAL)2 * sf * l1 * v_sigma / (sx * sx);
                REAL v_l2 = (REAL)2 * sf * l2 * v_sigma / (sy * sy);
                v_t += (v_l1 * dot3(ray, a1) + v_l2 * dot3(ray, a2));
                v_t += dot3(ray, v_diff);
                if (idx == dfin && dfin != -1) v_t_view += vdepth;
                v_t_view += (K_T_FAR * K_T_NEAR) / ((K_T_FAR - K_T_NEAR) * t_view * t_view) * v_t_ndc;
                v_t += view_depth * v_t_view;
                REAL v_sb = -bf * op * esb * v_alpha;
                v3 vme = transform_4x3_rot_t(
                    viewmat, project_pix_vjp(fx, fy, pv, K_BLUR_FSQ * v_sb * (xyx - px), K_BLUR_FSQ * v_sb * (xyy - py)));
                v3 vmt = { 0, 0, 0 }, vnt = { 0, 0, 0 };
                compute_tt_vjp(o, ray, mean, a3, t, v_t, &vmt, &vnt);
                v3 vmean = { -(a1.x * v_l1 + a2.x * v_l2) + vmt.x + vme.x - v_diff.x,
                             -(a1.y * v_l1 + a2.y * v_l2) + vmt.y + vme.y - v_diff.y,
                             -(a1.z * v_l1 + a2.z * v_l2) + vmt.z + vme.z - v_diff.z };
                v3 vR[3] = { { d.x * v_l1, d.y * v_l1, d.z * v_l1 },
                             { d.x * v_l2, d.y * v_l2, d.z * v_l2 },
                             { vnt.x + vis * vnorm.x, vnt.y + vis * vnorm.y, vnt.z + vis * vnorm.z } };
                REAL vq[4];
                quat_axes_vjp(quats + 4 * g, vR, vq);
                REAL vop = (nbf * es + bf * esb) * v_alpha;

                ATOMIC_ADD(v_colors + 3 * g + 0, vis * vout.x);
                ATOMIC_ADD(v_colors + 3 * g + 1, vis * vout.y);
                ATOMIC_ADD(v_colors + 3 * g + 2, vis * vout.z);
                ATOMIC_ADD(v_scales + 3 * g + 0, vsx);
                ATOMIC_ADD(v_scales + 3 * g + 1, vsy);
                ATOMIC_ADD(v_means + 3 * g + 0, vmean.x);
                ATOMIC_ADD(v_means + 3 * g + 1, vmean.y);
                ATOMIC_ADD(v_means + 3 * g + 2, vmean.z);
                for (int q = 0; q < 4; q++) ATOMIC_ADD(v_quats + 4 * g + q, vq[q]);
                ATOMIC_ADD(v_opac + g, vop);
                ATOMIC_ADD(v_uv0 + 2 * g + 0, vuv0x);
                ATOMIC_ADD(v_uv0 + 2 * g + 1, vuv0y);
                ATOMIC_ADD(v_umap + 3 * g + 0, vum.x);
                ATOMIC_ADD(v_umap + 3 * g + 1, vum.y);
                ATOMIC_ADD(v_umap + 3 * g + 2, vum.z);
                ATOMIC_ADD(v_vmap + 3 * g + 0, vvm.x);
                ATOMIC_ADD(v_vmap + 3 * g + 1, vvm.y);
                ATOMIC_ADD(v_vmap + 3 * g + 2, vvm.z);
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------
 * Texture editing: csrc/texture_edit.cu:11-236.  Front to back like the
 * forward compositor (blur is settings bit 0 here), and for every pair that
 * contributes with its camera depth inside [depth_lower, depth_upper] of the
 * pixel, the values (r*a, g*a, b*a, a, 1) of the edited pixel are splatted
 * with the bilinear weights of the hit's texture coordinate into the five
 * channels of the chart's texels (out is [num_texels, 5], accumulated).
 * ---------------------------------------------------------------------- */
void FN(texture_edit)(int tiles_x, int tiles_y, int bw, int img_w, int img_h, const int32_t* texture_dims,
                      const REAL* upd_img, const REAL* upd_alpha, const REAL* depth_lower, const REAL* depth_upper,
                      const int32_t* gids, const int32_t* tile_bins, const REAL* opac, const REAL* means,
                      const REAL* scales, REAL glob_scale, const REAL* quats, const REAL* uv0, const REAL* umap,
                      const REAL* vmap, const REAL* viewmat, const REAL* c2w, REAL fx, REAL fy, REAL cx, REAL cy,
                      int settings, REAL* out, int nthreads) {
    const int use_blur = (settings & 1) != 0;
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
    for (int bi = 0; bi < img_h; bi++) {
        for (int bj = 0; bj < img_w; bj++) {
            const int tile = (bi / bw) * tiles_x + (bj / bw);
            const long pix = (long)bi * img_w + bj;
            REAL px = (REAL)bj + (REAL)0.5, py = (REAL)bi + (REAL)0.5;
            v3 o, ray;
            get_ray(c2w, fx, fy, cx, cy, px, py, &o, &ray);
            REAL view_depth = viewmat[8] * ray.x + viewmat[9] * ray.y + viewmat[10] * ray.z;
            const REAL a = upd_alpha[pix];
            const REAL vals[5] = { upd_img[3 * pix] * a, upd_img[3 * pix + 1] * a, upd_img[3 * pix + 2] * a, a, 1 };
            const REAL lo = depth_lower[pix], hi = depth_upper[pix];
            int rs = tile_bins[2 * tile], re = tile_bins[2 * tile + 1];
            REAL T = 1;
            int done = 0;
            for (int idx = rs; idx < re && !done; idx++) {
                const int g = gids[idx];
                v3 mean = { means[3 * g], means[3 * g + 1], means[3 * g + 2] };
                REAL sx = scales[3 * g], sy = scales[3 * g + 1];
                v3 a1, a2, a3;
                quat_axes(quats + 4 * g, &a1, &a2, &a3);
                REAL t = compute_tt(o, ray, mean, a3);
                v3 pos = { o.x + t * ray.x, o.y + t * ray.y, o.z + t * ray.z };
                v3 d = { pos.x - mean.x, pos.y - mean.y, pos.z - mean.z };
                REAL l1 = dot3(d, a1), l2 = dot3(d, a2);
                REAL is1 = (REAL)1 / (sx * glob_scale), is2 = (REAL)1 / (sy * glob_scale);
                REAL sigma = (REAL)0.5f * (is1 * is1 * l1 * l1 + is2 * is2 * l2 * l2);
                v3 pv = transform_4x3(viewmat, mean);
                REAL xyx, xyy;
                project_pix(fx, fy, pv, cx, cy, &xyx, &xyy);
                REAL ddx = xyx - px, ddy = xyy - py;
                REAL sigma_blur = (REAL)0.5f * K_BLUR_FSQ * (ddx * ddx + ddy * ddy);
                REAL nbf = 1, bf = 0;
                if (use_blur && sigma_blur < sigma) { bf = 1; nbf = 0; }
                REAL alpha = R_FMIN(K_ALPHA_MAX, opac[g] * (nbf * R_EXP(-sigma) + bf * R_EXP(-sigma_blur)));
                int skip = (t < K_T_NEAR || t > K_T_FAR || alpha < K_ALPHA_MIN);
                REAL next_T = T * ((REAL)1 - alpha);
                if (next_T <= K_T_DONE) done = 1;
                if (skip || done) continue;
                REAL t_view = t * view_depth;
                if (t_view >= lo && t_view <= hi) {
                    const int32_t* dm = texture_dims + 3 * g;
                    v3 um = { umap[3 * g], umap[3 * g + 1], umap[3 * g + 2] };
                    v3 vm = { vmap[3 * g], vmap[3 * g + 1], vmap[3 * g + 2] };
                    REAL uu = uv0[2 * g] + dot3(um, d), vv = uv0[2 * g + 1] + dot3(vm, d);
                    clamp_coord(&uu, &vv);
                    for (int k = 0; k < 5; k++) {
                        REAL w[4], wx, wy;
                        long id[4];
                        chart_weights(dm[0], dm[1], dm[2], 5, k, uu, vv, 1, w, id, &wx, &wy);
                        for (int q = 0; q < 4; q++) ATOMIC_ADD(out + id[q], w[q] * vals[k]);
                    }
                }
                T = next_T;
            }
        }
    }
}

/* ------------------------------------------------------------------------
 * Integer binning (float32 inputs in both builds; defined once, in the
 * float build).
 * ---------------------------------------------------------------------- */
#ifndef OR_F64

/* gstex_cuda/get_aabb_2d.py:70-91, in float32 like the torch code. */
void or_num_tiles_hit(int n, const float* centers, const float* extents, int img_h, int img_w, int bw, int32_t* out) {
    int tx = (img_w + bw - 1) / bw, ty = (img_h + bw - 1) / bw;
    float fbw = (float)bw;
    for (int i = 0; i < n; i++) {
        int tl[2], br[2], lim[2] = { tx, ty };
        for (int a = 0; a < 2; a++) {
            float c = centers[2 * i + a], e = extents[2 * i + a];
            float lo = floorf((c - e) / fbw);
            float hi = floorf((c + e) / fbw + 1.0f);
            tl[a] = f2i_rz(lo);
            br[a] = f2i_rz(hi);
            tl[a] = tl[a] < 0 ? 0 : (tl[a] > lim[a] ? lim[a] : tl[a]);
            br[a] = br[a] < 0 ? 0 : (br[a] > lim[a] ? lim[a] : br[a]);
        }
        out[i] = (br[0] - tl[0]) * (br[1] - tl[1]);
    }
}

/* helpers.cuh:37-51, 53-73, 75-111 */
static void tile_bbox(float cx, float cy, float ex, float ey, int tiles_x, int tiles_y, int bw, int wrapped,
                      int* x0, int* y0, int* x1, int* y1) {
    float tcx = cx / (float)bw, tcy = cy / (float)bw;
    float tex = ex / (float)bw, tey = ey / (float)bw;
    if (wrapped) {
        *x0 = f2i_rz(tcx - tex);
        if (*x0 <= 0) *x0 -= 1;
        *x1 = f2i_rz(tcx + tex + 1.0f);
        *y0 = f2i_rz(tcy - tey);
        if (*y0 <= 0) *y0 -= 1;
        *y1 = f2i_rz(tcy + tey + 1.0f);
        return;
    }
#define CLAMPI(v, hi) ((v) < 0 ? 0 : ((v) > (hi) ? (hi) : (v)))
    *x0 = CLAMPI(f2i_rz(tcx - tex), tiles_x);
    *x1 = CLAMPI(f2i_rz(tcx + tex + 1.0f), tiles_x);
    *y0 = CLAMPI(f2i_rz(tcy - tey), tiles_y);
    *y1 = CLAMPI(f2i_rz(tcy + tey + 1.0f), tiles_y);
}

/* csrc/forward.cu:13-71.  Slots come from the caller's inclusive cumsum; a
 * Gaussian that is skipped (both extents <= 1e-4) leaves its slots at the
 * zero-initialised value, as the reference's torch::zeros buffers do.  Each
 * Gaussian writes only inside its own slots [cum[i-1], cum[i]): with a
 * power-of-two tile width the emitted count always equals the slot count;
 * otherwise the reference would race into its neighbour's slots. */
void or_map_gaussian_to_intersects(int n, const float* centers, const float* extents, const float* depths,
                                   const int32_t* cum, int tiles_x, int tiles_y, int bw, int wrapped,
                                   long n_isect, int64_t* isect_ids, int32_t* gids) {
    memset(isect_ids, 0, sizeof(int64_t) * n_isect);
    memset(gids, 0, sizeof(int32_t) * n_isect);
    for (int i = 0; i < n; i++) {
        float ex = extents[2 * i], ey = extents[2 * i + 1];
        if ((double)ex <= 1e-4 && (double)ey <= 1e-4) continue;
        int x0, y0, x1, y1;
        tile_bbox(centers[2 * i], centers[2 * i + 1], ex, ey, tiles_x, tiles_y, bw, wrapped, &x0, &y0, &x1, &y1);
        long cur = i == 0 ? 0 : cum[i - 1];
        long hi = cum[i] < n_isect ? cum[i] : n_isect;
        int32_t dbits;
        memcpy(&dbits, depths + i, 4);
        int64_t depth_id = (int64_t)dbits;  /* sign-extends, forward.cu:47 */
        for (int ty = y0; ty < y1; ty++) {
            for (int tx = x0; tx < x1; tx++) {
                int ti = ty, tj = tx;
                if (wrapped) {
                    ti = ti % tiles_y; if (ti < 0) ti += tiles_y;
                    tj = tj % tiles_x; if (tj < 0) tj += tiles_x;
                }
                int64_t tile_id = (int64_t)(ti * tiles_x + tj);
                if (cur >= 0 && cur < hi) {
                    isect_ids[cur] = (int64_t)(((uint64_t)tile_id << 32) | (uint64_t)depth_id);
                    gids[cur] = i;
                }
                cur++;
            }
        }
    }
}

/* Stable ascending sort of signed 64-bit keys with int32 payload (the
 * reference uses torch.sort, gstex_cuda/utils.py:159-160; for equal keys the
 * original order is kept, which is what a radix sort gives). */
typedef struct { int64_t k; int32_t v; int32_t pos; } kv_t;
static int kv_cmp(const void* a, const void* b) {
    const kv_t* x = (const kv_t*)a;
    const kv_t* y = (const kv_t*)b;
    if (x->k < y->k) return -1;
    if (x->k > y->k) return 1;
    return x->pos < y->pos ? -1 : (x->pos > y->pos);
}
void or_sort_pairs(long n, const int64_t* keys, const int32_t* vals, int64_t* keys_out, int32_t* vals_out) {
    kv_t* a = (kv_t*)malloc(sizeof(kv_t) * (n > 0 ? n : 1));
    for (long i = 0; i < n; i++) { a[i].k = keys[i]; a[i].v = vals[i]; a[i].pos = (int32_t)i; }
    qsort(a, (size_t)n, sizeof(kv_t), kv_cmp);
    for (long i = 0; i < n; i++) { keys_out[i] = a[i].k; vals_out[i] = a[i].v; }
    free(a);
}

/* csrc/forward.cu:76-98 with the zero-initialised output of
 * bindings.cu:123-140.  Tile indices outside [0, num_tiles) are ignored. */
void or_get_tile_bin_edges(long n, const int64_t* sorted, int num_tiles, int32_t* bins) {
    memset(bins, 0, sizeof(int32_t) * 2 * (size_t)num_tiles);
    for (long i = 0; i < n; i++) {
        int32_t cur = (int32_t)(sorted[i] >> 32);
        int ok = cur >= 0 && cur < num_tiles;
        if (i == 0 && ok) bins[2 * cur] = 0;
        if (i == n - 1 && ok) bins[2 * cur + 1] = (int32_t)n;
        if (i == 0) continue;
        int32_t prev = (int32_t)(sorted[i - 1] >> 32);
        if (prev != cur) {
            if (prev >= 0 && prev < num_tiles) bins[2 * prev + 1] = (int32_t)i;
            if (ok) bins[2 * cur] = (int32_t)i;
        }
    }
}

#endif /* !OR_F64 */
