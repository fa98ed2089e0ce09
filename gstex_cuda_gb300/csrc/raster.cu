// Textured 2D-Gaussian compositor: forward, backward and gradient finalize.
//
// Reference: csrc/texture.cu:11-329 (forward), 331-760 (backward).  One CTA
// per screen tile and one thread per pixel as in the reference; each CTA
// stages batches of block_size Gaussians of its depth-sorted range into
// shared memory as camera-space records (common.cuh), so a pixel evaluates a
// splat with a handful of FMAs instead of the reference's per-pixel
// quaternion, ray-plane and projection work.
//
// Backward: per (pixel, Gaussian) the adjoint reduces to 26 scalar
// "moments" whose sums over pixels determine every parameter gradient
// (because delta = l1*ax1 + l2*ax2 on the splat plane and the quaternion
// adjoint is linear in dR).  Moments are reduced across a warp with a
// 31-shuffle transpose reduction, summed per CTA in shared memory, and
// flushed with one set of vector atomics per (tile, Gaussian).  A finalize
// kernel turns the per-Gaussian sums into v_means, v_quats, ...
#include "common.cuh"

namespace gstex {

constexpr int kMoments = 26;       // per-pair moments reduced in the CTA
constexpr int kMomStride = 28;     // per-Gaussian global stride (24 + 3 blur + pad)

struct RasterArgs {
    int N, W, H, bw, tiles_x, tiles_y, C, T;
    const int3* dims;
    const int32_t* gids;
    const int2* bins;
    const float3* colors;
    const float* opac;
    const float3* means;
    const float* scales;
    float glob;
    const float4* quats;
    const float2* uv0;
    const float3* umap;
    const float3* vmap;
    const void* tex;
    const float* viewmat;
    float fx, fy, cx, cy;
    int settings;
    const float* bg;
};

struct FwdOut {
    float3* img;
    float* depth;
    float* reg;
    float* tex;
    float3* normal;
    float* final_T;
    int32_t* final_idx;
    int32_t* depth_idx;
    float3* reg_s;
};

struct BwdArgs {
    const float* final_T;
    const int32_t* final_idx;
    const int32_t* depth_idx;
    const float3* reg_s;
    const float3* v_img;
    const float* v_depth;
    const float* v_reg;
    const float* v_alpha;
    const float* v_tex;
    const float3* v_normal;
    float* moments;   // [N, kMomStride]
    float* v_texgrad; // [T, C] (fp32 texture) or [T, 4] (bf16 texture)
};

__device__ __forceinline__ void stage(GaussRec& R, const RasterArgs& a, const View& V, int gid) {
    make_record(R, gid, V, a.means[gid], a.quats[gid], make_float2(a.scales[3 * gid], a.scales[3 * gid + 1]), a.glob,
                a.opac[gid], a.colors[gid], a.uv0[gid], a.umap[gid], a.vmap[gid], a.dims[gid]);
}

// All channels of the 4 bilinear corners (C == 3 fast path).
template <int TEXMODE>
__device__ __forceinline__ void fetch3(const void* tex, const Bilerp& B, float c[4][3]) {
    const int rows[4] = { B.i00, B.i01, B.i10, B.i11 };
    if (TEXMODE == 1) {
        const uint2* t = (const uint2*)tex;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint2 raw = __ldg(t + rows[q]);
            const __nv_bfloat162 lo = *reinterpret_cast<const __nv_bfloat162*>(&raw.x);
            const __nv_bfloat162 hi = *reinterpret_cast<const __nv_bfloat162*>(&raw.y);
            c[q][0] = __low2float(lo);
            c[q][1] = __high2float(lo);
            c[q][2] = __low2float(hi);
        }
    } else {
        const float* t = (const float*)tex;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            c[q][0] = __ldg(t + 3 * rows[q] + 0);
            c[q][1] = __ldg(t + 3 * rows[q] + 1);
            c[q][2] = __ldg(t + 3 * rows[q] + 2);
        }
    }
}

// ---------------------------------------------------------------------------
// Forward
// ---------------------------------------------------------------------------
template <int TEXMODE, int CT>
__global__ void __launch_bounds__(256) fwd_kernel(RasterArgs a, FwdOut o) {
    extern __shared__ __align__(16) unsigned char smem[];
    GaussRec* recs = reinterpret_cast<GaussRec*>(smem);
    const int bs = blockDim.x * blockDim.y;
    const int tr = threadIdx.y * blockDim.x + threadIdx.x;
    const int tile = blockIdx.y * a.tiles_x + blockIdx.x;
    const int pi = blockIdx.y * blockDim.y + threadIdx.y;
    const int pj = blockIdx.x * blockDim.x + threadIdx.x;
    const View V = load_view(a.viewmat, a.fx, a.fy, a.cx, a.cy);
    const PixelRay P = make_pixel(V, pi, pj);
    const bool inside = pi < a.H && pj < a.W;
    bool done = !inside;
    const int2 range = a.bins[tile];
    const int nb = ceil_div(range.y - range.x, bs);
    const bool use_blur = a.settings & (1 << 9);
    const bool use_ndc = a.settings & (1 << 10);
    const bool flip = a.settings & (1 << 15);
    const bool bilinear = !(a.settings & (1 << 2));
    const int C = CT >= 0 ? CT : a.C;
    constexpr int CA = CT > 0 ? CT : (CT == 0 ? 1 : kMaxChannels);
    float otex[CA];
#pragma unroll
    for (int k = 0; k < CA; k++) otex[k] = 0.f;
    float T = 1.f;
    int cur = 0, didx = -1;
    float3 out = make_float3(0.f, 0.f, 0.f), nrm = make_float3(0.f, 0.f, 0.f), ts = make_float3(0.f, 0.f, 0.f);
    float depth = 0.f, reg = 0.f;

    for (int b = 0; b < nb; ++b) {
        if (__syncthreads_count(done) >= bs) break;
        const int bstart = range.x + bs * b;
        const int idx = bstart + tr;
        if (idx < range.y) stage(recs[tr], a, V, a.gids[idx]);
        __syncthreads();
        const int bsize = min(bs, range.y - bstart);
        if (done) continue;
        for (int k = 0; k < bsize; ++k) {
            const GaussRec& R = recs[k];
            const Hit H = intersect(R, P);
            const float l1s = H.l1 * R.is1, l2s = H.l2 * R.is2;
            const float sigma = 0.5f * (l1s * l1s + l2s * l2s);
            float nbf = 1.f, bf = 0.f, sigma_blur = 0.f;
            if (use_blur) {
                const float dx = R.bx - P.px, dy = R.by - P.py;
                sigma_blur = 0.5f * kBlurFsq * (dx * dx + dy * dy);
                if (sigma_blur < sigma) { bf = 1.f; nbf = 0.f; }
            }
            const float alpha = fminf(kAlphaMax, R.opac * (nbf * __expf(-sigma) + bf * __expf(-sigma_blur)));
            const bool skip = H.t < kTNear || H.t > kTFar || alpha < kAlphaMin;
            const float next_T = T * (1.f - alpha);
            if (next_T <= kTDone) { done = true; break; }
            if (skip) continue;
            const float vis = alpha * T;
            out.x = out.x + R.color.x * vis;
            out.y = out.y + R.color.y * vis;
            out.z = out.z + R.color.z * vis;
            float3 hn = R.nw;
            if (flip && dot3(make_float3(P.u, P.v, 1.f), R.nc) > 0.f) hn = make_float3(-hn.x, -hn.y, -hn.z);
            nrm.x += vis * hn.x; nrm.y += vis * hn.y; nrm.z += vis * hn.z;
            if (C > 0) {
                const Bilerp B = bilerp(R.h, R.w, R.start, clamp01(H.tu), clamp01(H.tv), bilinear);
                if (CT == 3) {
                    float c[4][3];
                    fetch3<TEXMODE>(a.tex, B, c);
#pragma unroll
                    for (int ch = 0; ch < 3; ch++)
                        otex[ch] += vis * (B.w00 * c[0][ch] + B.w01 * c[1][ch] + B.w10 * c[2][ch] + B.w11 * c[3][ch]);
                } else if (CT != 0) {
                    const float* t = (const float*)a.tex;
                    for (int ch = 0; ch < C; ch++) {
                        const float v = B.w00 * __ldg(t + (size_t)B.i00 * C + ch) + B.w01 * __ldg(t + (size_t)B.i01 * C + ch) +
                                        B.w10 * __ldg(t + (size_t)B.i10 * C + ch) + B.w11 * __ldg(t + (size_t)B.i11 * C + ch);
                        otex[ch] += vis * v;
                    }
                }
            }
            const float t_view = H.tcam;
            if (T > 0.5f) { depth = t_view; didx = bstart + k; }
            const float dv = use_ndc ? (kTFar * t_view - kTFar * kTNear) / ((kTFar - kTNear) * t_view) : H.t;
            reg += vis * (dv * dv * ts.x + ts.z - 2.f * dv * ts.y);
            ts.x += vis;
            ts.y += vis * dv;
            ts.z += vis * dv * dv;
            T = next_T;
            cur = bstart + k;
        }
    }
    if (inside) {
        const int pix = pi * a.W + pj;
        o.final_T[pix] = T;
        o.final_idx[pix] = cur;
        o.depth_idx[pix] = didx;
        o.img[pix] = make_float3(out.x + T * a.bg[0], out.y + T * a.bg[1], out.z + T * a.bg[2]);
        o.normal[pix] = nrm;
        o.depth[pix] = depth;
        o.reg[pix] = reg;
        o.reg_s[pix] = ts;
        for (int ch = 0; ch < C; ch++) o.tex[(size_t)pix * C + ch] = otex[ch];
    }
}

// ---------------------------------------------------------------------------
// Backward
// ---------------------------------------------------------------------------
// Transpose reduction: lane l ends with the warp sum of m[l].
__device__ __forceinline__ float warp_transpose_reduce(float (&m)[32], unsigned lane) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const bool upper = lane & off;
#pragma unroll
        for (int j = 0; j < off; j++) {
            const float send = upper ? m[j] : m[j + off];
            const float keep = upper ? m[j + off] : m[j];
            m[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return m[0];
}

template <int TEXMODE, int CT>
__global__ void __launch_bounds__(256) bwd_kernel(RasterArgs a, BwdArgs g) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int bs = blockDim.x * blockDim.y;
    GaussRec* recs = reinterpret_cast<GaussRec*>(smem);
    float* smom = reinterpret_cast<float*>(smem + sizeof(GaussRec) * bs);
    const int tr = threadIdx.y * blockDim.x + threadIdx.x;
    const unsigned lane = tr & 31;
    const unsigned wmask = __activemask();
    const bool full_warp = wmask == 0xffffffffu;
    const int tile = blockIdx.y * a.tiles_x + blockIdx.x;
    const int pi = blockIdx.y * blockDim.y + threadIdx.y;
    const int pj = blockIdx.x * blockDim.x + threadIdx.x;
    const View V = load_view(a.viewmat, a.fx, a.fy, a.cx, a.cy);
    const PixelRay P = make_pixel(V, pi, pj);
    const bool inside = pi < a.H && pj < a.W;
    const int pix = inside ? pi * a.W + pj : 0;
    const bool use_blur = a.settings & (1 << 9);
    const bool use_ndc = a.settings & (1 << 10);
    const bool prop_uv = a.settings & (1 << 8);
    const bool bilinear = !(a.settings & (1 << 2));
    const int C = CT >= 0 ? CT : a.C;
    constexpr int CA = CT > 0 ? CT : (CT == 0 ? 1 : kMaxChannels);

    float T = inside ? g.final_T[pix] : 1.f;
    const float3 sfin = inside ? g.reg_s[pix] : make_float3(0.f, 0.f, 0.f);
    const int dfin = inside ? g.depth_idx[pix] : -1;
    const int bfin = inside ? g.final_idx[pix] : 0;
    const float3 vout = inside ? g.v_img[pix] : make_float3(0.f, 0.f, 0.f);
    const float vdepth = inside ? g.v_depth[pix] : 0.f;
    const float vreg = inside ? g.v_reg[pix] : 0.f;
    const float valph = inside ? g.v_alpha[pix] : 0.f;
    const float3 vnorm = inside ? g.v_normal[pix] : make_float3(0.f, 0.f, 0.f);
    float vtex[CA];
    for (int ch = 0; ch < CA; ch++) vtex[ch] = (inside && ch < C) ? g.v_tex[(size_t)pix * C + ch] : 0.f;
    float vT_run = a.bg[0] * vout.x + a.bg[1] * vout.y + a.bg[2] * vout.z - valph;
    const int warp_bfin = __reduce_max_sync(wmask, bfin);

    const int2 range = a.bins[tile];
    const int nb = ceil_div(range.y - range.x, bs);
    for (int b = 0; b < nb; ++b) {
        __syncthreads();
        const int bend = range.y - 1 - bs * b;
        const int bsize = min(bs, bend + 1 - range.x);
        const int idx = bend - tr;
        if (idx >= range.x) stage(recs[tr], a, V, a.gids[idx]);
        for (int q = tr; q < bs * kMoments; q += bs) smom[q] = 0.f;
        __syncthreads();
        for (int k = max(0, bend - warp_bfin); k < bsize; ++k) {
            const int gidx = bend - k;
            bool valid = inside && gidx <= bfin;
            const GaussRec& R = recs[k];
            Hit H;
            float l1s = 0.f, l2s = 0.f, e = 0.f, eb = 0.f, nbf = 1.f, bf = 0.f, alpha = 0.f;
            if (valid) {
                H = intersect(R, P);
                l1s = H.l1 * R.is1;
                l2s = H.l2 * R.is2;
                const float sigma = 0.5f * (l1s * l1s + l2s * l2s);
                float sigma_blur = 0.f;
                if (use_blur) {
                    const float dx = R.bx - P.px, dy = R.by - P.py;
                    sigma_blur = 0.5f * kBlurFsq * (dx * dx + dy * dy);
                    if (sigma_blur < sigma) { bf = 1.f; nbf = 0.f; }
                }
                e = __expf(-sigma);
                eb = use_blur ? __expf(-sigma_blur) : 0.f;
                alpha = fminf(kAlphaMax, R.opac * (nbf * e + bf * eb));
                if (H.t < kTNear || H.t > kTFar || alpha < kAlphaMin) valid = false;
            }
            if (!__any_sync(wmask, valid)) continue;
            float m[32];
#pragma unroll
            for (int q = 0; q < 32; q++) m[q] = 0.f;
            if (valid) {
                T = T * __frcp_rn(1.f - alpha);
                const float vis = alpha * T;
                float v_vis = R.color.x * vout.x + R.color.y * vout.y + R.color.z * vout.z + dot3(R.nw, vnorm);
                float v_u = 0.f, v_v = 0.f;
                if (C > 0) {
                    const Bilerp B = bilerp(R.h, R.w, R.start, clamp01(H.tu), clamp01(H.tv), bilinear);
                    if (CT == 3) {
                        float c[4][3];
                        fetch3<TEXMODE>(a.tex, B, c);
                        float gv[3];
#pragma unroll
                        for (int ch = 0; ch < 3; ch++) {
                            const float val = B.w00 * c[0][ch] + B.w01 * c[1][ch] + B.w10 * c[2][ch] + B.w11 * c[3][ch];
                            const float vv = vis * vtex[ch];
                            gv[ch] = vv;
                            if (bilinear && prop_uv) {
                                v_u += (float)R.h * (vv * (-(1.f - B.fy) * c[0][ch] - B.fy * c[1][ch] + (1.f - B.fy) * c[2][ch] + B.fy * c[3][ch]));
                                v_v += (float)R.w * (vv * (-(1.f - B.fx) * c[0][ch] + (1.f - B.fx) * c[1][ch] - B.fx * c[2][ch] + B.fx * c[3][ch]));
                            }
                            v_vis += val * vtex[ch];
                        }
                        const int rows[4] = { B.i00, B.i01, B.i10, B.i11 };
                        const float wts[4] = { B.w00, B.w01, B.w10, B.w11 };
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            if (wts[q] == 0.f) continue;
                            if (TEXMODE == 1) {
                                atomicAdd(reinterpret_cast<float4*>(g.v_texgrad) + rows[q],
                                          make_float4(wts[q] * gv[0], wts[q] * gv[1], wts[q] * gv[2], 0.f));
                            } else {
                                float* dst = g.v_texgrad + 3 * (size_t)rows[q];
                                atomicAdd(dst + 0, wts[q] * gv[0]);
                                atomicAdd(dst + 1, wts[q] * gv[1]);
                                atomicAdd(dst + 2, wts[q] * gv[2]);
                            }
                        }
                    } else if (CT != 0) {
                        const float* t = (const float*)a.tex;
                        for (int ch = 0; ch < C; ch++) {
                            const float c00 = __ldg(t + (size_t)B.i00 * C + ch), c01 = __ldg(t + (size_t)B.i01 * C + ch);
                            const float c10 = __ldg(t + (size_t)B.i10 * C + ch), c11 = __ldg(t + (size_t)B.i11 * C + ch);
                            const float val = B.w00 * c00 + B.w01 * c01 + B.w10 * c10 + B.w11 * c11;
                            const float vv = vis * vtex[ch];
                            if (B.w00 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i00 * C + ch, B.w00 * vv);
                            if (B.w01 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i01 * C + ch, B.w01 * vv);
                            if (B.w10 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i10 * C + ch, B.w10 * vv);
                            if (B.w11 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i11 * C + ch, B.w11 * vv);
                            if (bilinear && prop_uv) {
                                v_u += (float)R.h * (vv * (-(1.f - B.fy) * c00 - B.fy * c01 + (1.f - B.fy) * c10 + B.fy * c11));
                                v_v += (float)R.w * (vv * (-(1.f - B.fx) * c00 + (1.f - B.fx) * c01 - B.fx * c10 + B.fx * c11));
                            }
                            v_vis += val * vtex[ch];
                        }
                    }
                }
                float v_alpha = T * v_vis - T * vT_run;
                float vT_cur = alpha * v_vis + (1.f - alpha) * vT_run;
                const float t_view = H.tcam;
                float v_t = 0.f, v_t_ndc = 0.f, v_w = 0.f;
                if (use_ndc) {
                    const float t_ndc = (kTFar * t_view - kTFar * kTNear) / ((kTFar - kTNear) * t_view);
                    v_t_ndc = 2.f * (vis * t_ndc * sfin.x - vis * sfin.y) * vreg;
                    v_w = (t_ndc * t_ndc * sfin.x - 2.f * t_ndc * sfin.y + sfin.z) * vreg;
                } else {
                    v_t = 2.f * (vis * H.t * sfin.x - vis * sfin.y) * vreg;
                    v_w = (H.t * H.t * sfin.x - 2.f * H.t * sfin.y + sfin.z) * vreg;
                }
                v_alpha += v_w * T;
                vT_cur += v_w * alpha;
                vT_run = vT_cur;
                const float v_sigma = -nbf * R.opac * e * v_alpha;
                const float v_l1 = H.l1 * R.is1 * R.is1 * v_sigma;
                const float v_l2 = H.l2 * R.is2 * R.is2 * v_sigma;
                const float ra1 = (R.a1c.x * P.u + R.a1c.y * P.v + R.a1c.z) * P.idn;
                const float ra2 = (R.a2c.x * P.u + R.a2c.y * P.v + R.a2c.z) * P.idn;
                v_t += v_l1 * ra1 + v_l2 * ra2;
                if (prop_uv) {
                    const float rum = (R.umc.x * P.u + R.umc.y * P.v + R.umc.z) * P.idn;
                    const float rvm = (R.vmc.x * P.u + R.vmc.y * P.v + R.vmc.z) * P.idn;
                    v_t += v_u * rum + v_v * rvm;
                }
                float v_t_view = 0.f;
                if (gidx == dfin && dfin != -1) v_t_view += vdepth;
                if (use_ndc) v_t_view += (kTFar * kTNear) / ((kTFar - kTNear) * t_view * t_view) * v_t_ndc;
                v_t += P.idn * v_t_view;
                const float vtd = v_t * (P.dn * H.inv);  // v_t / (n . r)
                const float v_sb = -bf * R.opac * eb * v_alpha;
                m[0] = vis * vout.x;
                m[1] = vis * vout.y;
                m[2] = vis * vout.z;
                m[3] = (nbf * e + bf * eb) * v_alpha;
                m[4] = -(l1s * l1s) * v_sigma * R.is1 * a.glob;
                m[5] = -(l2s * l2s) * v_sigma * R.is2 * a.glob;
                m[6] = v_l1;
                m[7] = v_l2;
                m[8] = vtd;
                m[9] = H.l1 * v_l1;
                m[10] = H.l2 * v_l1;
                m[11] = H.l1 * v_l2;
                m[12] = H.l2 * v_l2;
                m[13] = H.l1 * vtd;
                m[14] = H.l2 * vtd;
                m[15] = vis * vnorm.x;
                m[16] = vis * vnorm.y;
                m[17] = vis * vnorm.z;
                m[18] = v_u;
                m[19] = v_v;
                m[20] = H.l1 * v_u;
                m[21] = H.l2 * v_u;
                m[22] = H.l1 * v_v;
                m[23] = H.l2 * v_v;
                m[24] = kBlurFsq * v_sb * (R.bx - P.px);
                m[25] = kBlurFsq * v_sb * (R.by - P.py);
            }
            float* dst = smom + k * kMoments;
            if (full_warp) {
                const float s = warp_transpose_reduce(m, lane);
                if (lane < (unsigned)kMoments) atomicAdd(dst + lane, s);
            } else if (valid) {
#pragma unroll
                for (int q = 0; q < kMoments; q++) atomicAdd(dst + q, m[q]);
            }
        }
        __syncthreads();
        if (idx >= range.x) {
            const float* sm = smom + tr * kMoments;
            bool any = false;
#pragma unroll
            for (int q = 0; q < kMoments; q++) any |= sm[q] != 0.f;
            if (any) {
                const GaussRec& R = recs[tr];
                float4* dst = reinterpret_cast<float4*>(g.moments + (size_t)R.gid * kMomStride);
                // blur moments -> world-space mean gradient (helpers.cuh:155-164, 114-121)
                const float3 p = R.mu_c;
                const float rw = 1.f / (p.z + 1e-6f);
                const float vx = a.fx * sm[24], vy = a.fy * sm[25];
                const float3 vview = make_float3(vx * rw, vy * rw, -(vx * p.x + vy * p.y) * rw * rw);
                const float3 vmb = V.rot_t(vview);
                float v[kMomStride];
#pragma unroll
                for (int q = 0; q < 24; q++) v[q] = sm[q];
                v[24] = vmb.x; v[25] = vmb.y; v[26] = vmb.z; v[27] = 0.f;
#pragma unroll
                for (int q = 0; q < kMomStride / 4; q++)
                    atomicAdd(dst + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
            }
        }
    }
}

// Moments -> parameter gradients (one thread per Gaussian).
__global__ void finalize_kernel(int N, const float* __restrict__ mom, const float4* __restrict__ quats,
                                const float3* __restrict__ umap, const float3* __restrict__ vmap, float3* v_colors,
                                float* v_opac, float3* v_means, float3* v_scales, float4* v_quats, float2* v_uv0,
                                float3* v_umap, float3* v_vmap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float M[kMomStride];
    const float4* src = reinterpret_cast<const float4*>(mom + (size_t)i * kMomStride);
#pragma unroll
    for (int q = 0; q < kMomStride / 4; q++) {
        const float4 v = src[q];
        M[4 * q] = v.x; M[4 * q + 1] = v.y; M[4 * q + 2] = v.z; M[4 * q + 3] = v.w;
    }
    const float4 q = quats[i];
    const Axes A = quat_axes(q);
    const float3 um = umap[i], vm = vmap[i];
    v_colors[i] = make_float3(M[0], M[1], M[2]);
    v_opac[i] = M[3];
    v_scales[i] = make_float3(M[4], M[5], 0.f);
    v_uv0[i] = make_float2(M[18], M[19]);
    v_umap[i] = M[20] * A.a1 + M[21] * A.a2;
    v_vmap[i] = M[22] * A.a1 + M[23] * A.a2;
    const float3 vdiff = M[18] * um + M[19] * vm;
    float3 vm_ = (M[8] * A.a3) - (M[6] * A.a1 + M[7] * A.a2) - vdiff;
    v_means[i] = vm_ + make_float3(M[24], M[25], M[26]);
    const float3 c0 = M[9] * A.a1 + M[10] * A.a2;
    const float3 c1 = M[11] * A.a1 + M[12] * A.a2;
    const float3 c2 = make_float3(M[15], M[16], M[17]) - (M[13] * A.a1 + M[14] * A.a2);
    v_quats[i] = quat_axes_vjp(q, c0, c1, c2);
}

template <typename K>
static int launch_raster(K kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t stream, const char* what) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) { set_cuda_error(e, what); return GSTEX_ERR_CUDA; }
    return GSTEX_OK;
}

static int fill_args(const gstex_raster_inputs* in, RasterArgs& a) {
    GSTEX_REQUIRE(in);
    GSTEX_REQUIRE(in->num_points >= 0 && in->img_width > 0 && in->img_height > 0);
    GSTEX_REQUIRE(in->block_width >= 2 && in->block_width <= kMaxBlockWidth);
    GSTEX_REQUIRE(in->channels >= 0);
    if (in->channels > kMaxChannels) return GSTEX_ERR_UNSUPPORTED;
    if (in->texture_dtype == 1 && in->channels != 3) return GSTEX_ERR_UNSUPPORTED;
    GSTEX_REQUIRE(in->texture_dtype == 0 || in->texture_dtype == 1);
    if (in->settings & (1 << 16)) return GSTEX_ERR_UNSUPPORTED;  // alpha-visualisation mode
    GSTEX_REQUIRE(in->tile_bins && in->viewmat && in->background);
    if (in->num_points > 0)
        GSTEX_REQUIRE(in->texture_dims && in->colors && in->opacities && in->means && in->scales && in->quats &&
                      in->uv0 && in->umap && in->vmap);
    if (in->channels > 0 && in->num_points > 0) GSTEX_REQUIRE(in->texture);
    a.N = in->num_points;
    a.W = in->img_width;
    a.H = in->img_height;
    a.bw = in->block_width;
    a.tiles_x = ceil_div(a.W, a.bw);
    a.tiles_y = ceil_div(a.H, a.bw);
    a.C = in->channels;
    a.T = in->num_texels;
    a.dims = (const int3*)in->texture_dims;
    a.gids = in->gaussian_ids_sorted;
    a.bins = (const int2*)in->tile_bins;
    a.colors = (const float3*)in->colors;
    a.opac = in->opacities;
    a.means = (const float3*)in->means;
    a.scales = in->scales;
    a.glob = in->glob_scale;
    a.quats = (const float4*)in->quats;
    a.uv0 = (const float2*)in->uv0;
    a.umap = (const float3*)in->umap;
    a.vmap = (const float3*)in->vmap;
    a.tex = in->texture;
    a.viewmat = in->viewmat;
    a.fx = in->fx; a.fy = in->fy; a.cx = in->cx; a.cy = in->cy;
    a.settings = in->settings;
    a.bg = in->background;
    return GSTEX_OK;
}

}  // namespace gstex

using namespace gstex;

extern "C" int gstex_texture_forward(const gstex_raster_inputs* in, const gstex_forward_outputs* out,
                                     gstex_stream_t s) {
    RasterArgs a;
    int rc = fill_args(in, a);
    if (rc) return rc;
    GSTEX_REQUIRE(out && out->img && out->depth && out->reg && out->normal && out->final_T && out->final_idx &&
                  out->depth_idx && out->reg_s);
    if (a.C > 0) GSTEX_REQUIRE(out->texture);
    FwdOut o{ (float3*)out->img, out->depth, out->reg, out->texture, (float3*)out->normal, out->final_T,
              out->final_idx, out->depth_idx, (float3*)out->reg_s };
    cudaStream_t stream = (cudaStream_t)s;
    const dim3 grid(a.tiles_x, a.tiles_y), block(a.bw, a.bw);
    const size_t smem = sizeof(GaussRec) * a.bw * a.bw;
    void (*k)(RasterArgs, FwdOut);
    if (a.C == 0) k = fwd_kernel<0, 0>;
    else if (a.C == 3) k = in->texture_dtype == 1 ? fwd_kernel<1, 3> : fwd_kernel<0, 3>;
    else k = fwd_kernel<0, -1>;
    if ((rc = launch_raster(k, grid, block, smem, stream, "texture_forward"))) return rc;
    k<<<grid, block, smem, stream>>>(a, o);
    return check_launch("texture_forward");
}

extern "C" size_t gstex_backward_workspace_bytes(int num_points) {
    return (size_t)(num_points > 0 ? num_points : 1) * kMomStride * sizeof(float);
}

extern "C" int gstex_texture_backward(const gstex_raster_inputs* in, const gstex_backward_io* io, gstex_stream_t s) {
    RasterArgs a;
    int rc = fill_args(in, a);
    if (rc) return rc;
    GSTEX_REQUIRE(io && io->final_T && io->final_idx && io->depth_idx && io->reg_s && io->v_img && io->v_depth &&
                  io->v_reg && io->v_alpha && io->v_normal);
    GSTEX_REQUIRE(io->v_colors && io->v_opacity && io->v_means && io->v_scales && io->v_quats && io->v_uv0 &&
                  io->v_umap && io->v_vmap && io->workspace);
    if (a.C > 0) GSTEX_REQUIRE(io->v_texture && io->v_tex_grad);
    if (io->workspace_bytes < gstex_backward_workspace_bytes(a.N)) return GSTEX_ERR_CAPACITY;
    if (a.N == 0) return GSTEX_OK;
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(io->workspace, 0, gstex_backward_workspace_bytes(a.N), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "texture_backward memset"); return GSTEX_ERR_CUDA; }
    BwdArgs g{ io->final_T, io->final_idx, io->depth_idx, (const float3*)io->reg_s, (const float3*)io->v_img,
               io->v_depth, io->v_reg, io->v_alpha, io->v_texture, (const float3*)io->v_normal,
               (float*)io->workspace, io->v_tex_grad };
    const dim3 grid(a.tiles_x, a.tiles_y), block(a.bw, a.bw);
    const size_t smem = (sizeof(GaussRec) + kMoments * sizeof(float)) * a.bw * a.bw;
    void (*k)(RasterArgs, BwdArgs);
    if (a.C == 0) k = bwd_kernel<0, 0>;
    else if (a.C == 3) k = in->texture_dtype == 1 ? bwd_kernel<1, 3> : bwd_kernel<0, 3>;
    else k = bwd_kernel<0, -1>;
    if ((rc = launch_raster(k, grid, block, smem, stream, "texture_backward"))) return rc;
    k<<<grid, block, smem, stream>>>(a, g);
    if ((rc = check_launch("texture_backward"))) return rc;
    finalize_kernel<<<ceil_div(a.N, 256), 256, 0, stream>>>(
        a.N, (const float*)io->workspace, a.quats, a.umap, a.vmap, (float3*)io->v_colors, io->v_opacity,
        (float3*)io->v_means, (float3*)io->v_scales, (float4*)io->v_quats, (float2*)io->v_uv0, (float3*)io->v_umap,
        (float3*)io->v_vmap);
    return check_launch("texture_backward finalize");
}
