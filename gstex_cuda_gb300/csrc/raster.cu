// Textured 2D-Gaussian compositor: forward, backward and gradient finalize.
//
// Reference: csrc/texture.cu:11-329 (forward), 331-760 (backward).  A CTA of
// bw x bw threads renders one screen tile, one thread per pixel; it stages
// batches of bw*bw Gaussians of the tile's depth-sorted range into shared
// memory as camera-space records (common.cuh), so a pixel evaluates a splat
// with a handful of FMAs instead of the reference's per-pixel quaternion,
// ray-plane and projection work.
//
// Backward: per (pixel, Gaussian) the adjoint reduces to 23 scalar moments
// whose sums over pixels determine every parameter gradient (on the splat
// plane delta = l1*ax1 + l2*ax2, and the quaternion adjoint is linear in dR).
// Moments are reduced across a warp with a 24-shuffle transpose reduction,
// summed per CTA in shared memory, and flushed with one set of vector atomics
// per (tile, Gaussian).  A finalize kernel turns the per-Gaussian sums into
// v_means, v_quats, ...
//
// Two launch forms share the per-tile bodies: one CTA per tile of a single
// view (the reference's texture_forward/backward), and a persistent kernel
// that pulls tiles of many views from one global queue (batched rendering).
#include "common.cuh"
#include "raster.cuh"

namespace gstex {

__device__ __forceinline__ void stage(const Recs& R, int slot, const SceneArgs& a, const View& V, const float3* colors,
                                      int gid, bool use_blur) {
    make_record(R.hot[slot], R.warm[slot], R.cold[slot], gid, V, a.means[gid], a.quats[gid],
                make_float2(a.scales[3 * gid], a.scales[3 * gid + 1]), a.glob, a.opac[gid],
                colors ? colors[gid] : make_float3(0.f, 0.f, 0.f), a.uv0[gid],
                a.umap[gid], a.vmap[gid], a.dims[gid], use_blur, true, R.edge ? R.edge + slot : nullptr,
                !(a.settings & (1 << 16)));
}

// Stages the record of Gaussian gid for one tile: a copy of the prebuilt
// (view, Gaussian) record when the batched path built them, else built here.
__device__ __forceinline__ void stage_job(const Recs& R, int slot, const SceneArgs& a, const TileJob& J, int gid,
                                          bool use_blur) {
    if (J.recs) {
        const uint4* src = reinterpret_cast<const uint4*>(J.recs + gid);
        uint4 v[kRecBytes / 16];
#pragma unroll
        for (int q = 0; q < kRecBytes / 16; q++) v[q] = __ldg(src + q);
        uint4* hot = reinterpret_cast<uint4*>(R.hot + slot);
        uint4* warm = reinterpret_cast<uint4*>(R.warm + slot);
        uint4* cold = reinterpret_cast<uint4*>(R.cold + slot);
        constexpr int nh = sizeof(RecHot) / 16, nw = sizeof(RecWarm) / 16, nc = sizeof(RecCold) / 16;
#pragma unroll
        for (int q = 0; q < nh; q++) hot[q] = v[q];
#pragma unroll
        for (int q = 0; q < nw; q++) warm[q] = v[nh + q];
#pragma unroll
        for (int q = 0; q < nc; q++) cold[q] = v[nh + nw + q];
        if (R.edge) {
            uint4* edge = reinterpret_cast<uint4*>(R.edge + slot);
#pragma unroll
            for (int q = 0; q < kEdgeBytes / 16; q++) edge[q] = __ldg(src + kRecBytes / 16 + q);
        }
    } else {
        stage(R, slot, a, J.V, J.colors, gid, use_blur);
    }
}

// Gaussians staged per round of a tile: a.batch when set (at most the
// threads of the CTA, which stage one each), else one per thread.
__device__ __forceinline__ int batch_of(const SceneArgs& a, int nthr) {
    return (a.batch > 0 && a.batch < nthr) ? a.batch : nthr;
}

// Completes a Hit in the direct form, rebuilding the Gaussian's camera-space
// frame from its parameters (rare: splats at the camera plane and pixels within
// the reference's denominator clamp).
__device__ __forceinline__ void direct_hit(Hit& H, const float4* __restrict__ quats, const float3* __restrict__ means,
                                           const float* __restrict__ scales, float glob, const float2* __restrict__ uv0s,
                                           const float3* __restrict__ umaps, const float3* __restrict__ vmaps,
                                           const View& V, int gid, const PixelRay& P, float tvn) {
    const Axes A = quat_axes(quats[gid]);
    const float3 mc = V.xform(means[gid]);
    const float is1 = 1.f / (scales[3 * gid] * glob), is2 = 1.f / (scales[3 * gid + 1] * glob);
    const float2 uv0 = uv0s[gid];
    intersect_direct(H, P, tvn, mc, V.rot(A.a1), V.rot(A.a2), V.rot(A.a3), V.rot(umaps[gid]), V.rot(vmaps[gid]), is1,
                     is2, uv0.x, uv0.y);
}

__device__ __forceinline__ Hit hit_pixel(const RecHot& Hr, const Recs& R, int k, const SceneArgs& a, const View& V,
                                         const PixelRay& P) {
    Hit H = intersect(Hr, P);
    if (H.direct)
        direct_hit(H, a.quats, a.means, a.scales, a.glob, a.uv0, a.umap, a.vmap, V, R.warm[k].tex.w, P, Hr.org.w);
    return H;
}

// Distance (in pixels) from the pixel to the nearest pixel of its 7x7
// neighbourhood whose ray meets the splat outside sigma <= sth
// (texture_helpers.cuh:390-417); 1000 when there is none.
__device__ __noinline__ float local_outline(const RecHot& Hr, const Recs& R, int k, const SceneArgs& a, const View& V,
                                            const TileJob& J, const PixelRay& P, float sth) {
    float best = 1000.f;
    const int pi = (int)(P.py - 0.5f), pj = (int)(P.px - 0.5f);
    for (int dx = -3; dx <= 3; dx++) {
        for (int dy = -3; dy <= 3; dy++) {
            const PixelRay Q = make_pixel(V, pi + dy, pj + dx);
            const Hit H = hit_pixel(Hr, R, k, a, V, Q);
            if (0.5f * (H.l1s * H.l1s + H.l2s * H.l2s) > sth) best = fminf(best, sqrtf((float)(dx * dx + dy * dy)));
        }
    }
    return best;
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

// Local (row, column) of a thread's first pixel.  When the tile width is a
// multiple of 8, each warp covers an 8-column block of 4 thread rows
// (8 x 4*PPT pixels): a warp's pixels stay close together, so a splat's screen
// box splits fewer warps than with 16 x 2 strips.  Otherwise thread (x, y)
// owns column x and rows PPT*y + p.
#ifndef GSTEX_WARP_BLOCK
#define GSTEX_WARP_BLOCK 1
#endif
//
// Inside a warp's 8 x 4 block, GS < 32 splits the lanes into groups of GS
// lanes, each covering a compact sub-block (16: two 4 x 4 halves; 8: four
// 4 x 2 quarters; 4: eight 2 x 2 blocks).
template <int PPT, int GS = 32>
__device__ __forceinline__ int2 thread_pixel(int bw) {
#if GSTEX_WARP_BLOCK
    if ((bw & 7) == 0) {
        const int tr = threadIdx.y * blockDim.x + threadIdx.x;
        const int lane = tr & 31, w = tr >> 5, wx = bw >> 3;
        int col = lane & 7, row = lane >> 3;
        if (GS == 4) {  // eight 2 x 2 blocks
            const int g = lane >> 2, lg = lane & 3;
            col = (g & 3) * 2 + (lg & 1);
            row = (g >> 2) * 2 + (lg >> 1);
        } else if (GS < 32) {
            const int g = lane / GS, lg = lane % GS;
            col = (g & 1) * 4 + (lg & 3);
            row = (g >> 1) * (GS / 4) + (lg >> 2);
        }
        return make_int2(((w / wx) * 4 + row) * PPT, (w % wx) * 8 + col);
    }
#endif
    return make_int2(threadIdx.y * PPT, threadIdx.x);
}

// Maximum / minimum over the GS-lane group of a full warp (GS a power of two).
template <int GS>
__device__ __forceinline__ int group_max(int v) {
#pragma unroll
    for (int o = GS / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int GS>
__device__ __forceinline__ int group_min(int v) {
#pragma unroll
    for (int o = GS / 2; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Candidate list of one warp: the staged slots k in [k0, bsize), in order,
// whose screen box overlaps the rectangle of the warp's pixel centres.  A
// splat left out is outside its alpha >= 1/255 box for every pixel of the
// warp.  Returns the count; the entries are in wl[0, count).  The lanes of a
// partial warp (tile widths that are not a multiple of 8) are its low lanes.
__device__ __forceinline__ bool splat_meets_rect(const Recs& R, int kk, float rx0, float rx1, float ry0, float ry1) {
    const float4 bx = R.hot[kk].box;
    bool hit = !(bx.y < rx0 || bx.x > rx1 || bx.w < ry0 || bx.z > ry1);
    if (hit && R.edge) {
        // separating axes of the splat's quad: the rectangle's corner
        // furthest inside each edge must be inside it
        const RecEdge e = R.edge[kk];
        const float ea[4] = { e.A.x, e.A.y, e.A.z, e.A.w }, eb[4] = { e.B.x, e.B.y, e.B.z, e.B.w };
        const float ec[4] = { e.C.x, e.C.y, e.C.z, e.C.w };
#pragma unroll
        for (int q = 0; q < 4; q++)
            hit = hit && ea[q] * (ea[q] > 0.f ? rx1 : rx0) + eb[q] * (eb[q] > 0.f ? ry1 : ry0) + ec[q] >= 0.f;
    }
    return hit;
}

__device__ __forceinline__ int build_list(uint8_t* wl, const Recs& R, int k0, int bsize, float rx0, float rx1,
                                          float ry0, float ry1, unsigned wmask, unsigned lane) {
    const int nl = __popc(wmask);
    int cnt = 0;
    for (int base = k0; base < bsize; base += nl) {
        const int kk = base + (int)lane;
        const bool hit = kk < bsize && splat_meets_rect(R, kk, rx0, rx1, ry0, ry1);
        const unsigned m = __ballot_sync(wmask, hit);
        if (hit) wl[cnt + __popc(m & ((1u << lane) - 1u))] = (uint8_t)kk;
        cnt += __popc(m);
    }
    __syncwarp(wmask);
    return cnt;
}

// The same for the GS-lane group of a full warp that holds this lane: the
// entries of the warp's list wl[0, cntw) (built with the warp's rectangle)
// that are at or after slot k0 (k0 per group) and whose box and quad meet the
// group's rectangle, in order.
template <int GS>
__device__ __forceinline__ int build_group_list(uint8_t* gl, const uint8_t* wl, int cntw, const Recs& R, int k0,
                                                float rx0, float rx1, float ry0, float ry1, unsigned lane) {
    const unsigned lg = lane & (GS - 1);
    const unsigned gm = ((1u << GS) - 1u) << (lane & ~(unsigned)(GS - 1));
    int cnt = 0;
    for (int base = 0; base < cntw; base += GS) {
        const int e = base + (int)lg;
        const int kk = e < cntw ? wl[e] : 0;
        const bool hit = e < cntw && kk >= k0 && splat_meets_rect(R, kk, rx0, rx1, ry0, ry1);
        const unsigned m = __ballot_sync(0xffffffffu, hit) & gm;
        if (hit) gl[cnt + __popc(m & ((1u << lane) - 1u))] = (uint8_t)kk;
        cnt += __popc(m);
    }
    __syncwarp();
    return cnt;
}

// ---------------------------------------------------------------------------
// Forward body: one tile.  A block of bw x (bw / PPT) threads covers the
// bw x bw tile; each thread owns PPT vertically adjacent pixels, so every
// staged record read from shared memory is used for PPT pixels.
// ---------------------------------------------------------------------------
template <int TEXMODE, int CT, int PPT, int FIX = 0>
__device__ __forceinline__ void fwd_tile(const SceneArgs& a, const TileJob& J, const FwdOut& o, const Recs& R) {
    const int nthr = blockDim.x * blockDim.y;
    const int tr = threadIdx.y * blockDim.x + threadIdx.x;
    const int bw = blockDim.x;
    const unsigned wmask = __activemask();
    const View& V = J.V;
    // FIX = 1: compiled for the default settings (kFixedFwdMask bits off)
    const bool use_blur = FIX ? false : (a.settings & (1 << 9)) != 0;
    const bool use_ndc = FIX ? false : (a.settings & (1 << 10)) != 0;
    const bool flip = FIX ? false : (a.settings & (1 << 15)) != 0;
    const bool bilinear = FIX ? true : !(a.settings & (1 << 2));
    // alpha-visualisation mode (texture.cu:58-63, 201-241; settings bit 16,
    // selected at launch as TEXMODE | 2): alpha 0.99 inside
    // sigma <= alpha_bound^2 / 2, outlines within outline_bound pixels of its edge
    constexpr bool alpha_vis = (TEXMODE & 2) != 0;
    constexpr int TM = TEXMODE & 1;
    const float alpha_bound = (float)((a.settings >> 17) & 31) / 8.f;
    const float vis_sth = 0.5f * alpha_bound * alpha_bound;
    const float outline_bound = (float)((a.settings >> 26) & 15) / 4.f;
    const bool accept_opac = a.settings & (1 << 25);
    const bool white_outline = a.settings & (1 << 24);
    const int C = CT >= 0 ? CT : a.C;
    constexpr int CA = CT > 0 ? CT : (CT == 0 ? 1 : kMaxChannels);
    const int2 lp = thread_pixel<PPT>(bw);
    const int pj = J.tx * bw + lp.y;
    PixelRay P[PPT];
    bool inside[PPT], done[PPT];
    float T[PPT], depth[PPT], reg[PPT];
    int cur[PPT], didx[PPT];
    float3 out[PPT], nrm[PPT], ts[PPT];
    float otex[PPT][CA];
    bool all_done = true;
#pragma unroll
    for (int p = 0; p < PPT; p++) {
        const int pi = J.ty * bw + lp.x + p;
        P[p] = make_pixel(V, pi, pj);
        inside[p] = pi < J.H && pj < J.W;
        done[p] = !inside[p];
        all_done = all_done && done[p];
        T[p] = 1.f;
        depth[p] = 0.f;
        reg[p] = 0.f;
        cur[p] = 0;
        didx[p] = -1;
        out[p] = nrm[p] = ts[p] = make_float3(0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < CA; k++) otex[p][k] = 0.f;
    }
    const int2 range = J.range;
    const int bsz = batch_of(a, nthr);  // Gaussians staged per round
    const int nb = ceil_div(range.y - range.x, bsz);

    for (int b = 0; b < nb; ++b) {
        if (__syncthreads_count(all_done) >= nthr) break;
        const int bstart = range.x + bsz * b;
        const int idx = bstart + tr;
        if (tr < bsz && idx < range.y) stage_job(R, tr, a, J, a.gids[idx], use_blur);
        __syncthreads();
        const int bsize = min(bsz, range.y - bstart);
        if (__all_sync(wmask, all_done)) continue;
        // Every staged slot in order; each pixel tests the splat's box first.
        for (int k = 0; k < bsize; ++k) {
            const float4 bx = R.hot[k].box;
            bool need = false;
#pragma unroll
            for (int p = 0; p < PPT; p++) {
                const bool out_box = P[p].px < bx.x || P[p].px > bx.y || P[p].py < bx.z || P[p].py > bx.w;
                need = need || (!done[p] && !(out_box && T[p] > 1.01e-4f));
            }
            if (need) {
            const RecHot Hr = R.hot[k];
#pragma unroll
            for (int p = 0; p < PPT; p++) {
                if (done[p]) continue;
                if (outside_box(Hr, P[p]) && T[p] > 1.01e-4f) continue;
                const Hit H = hit_pixel(Hr, R, k, a, V, P[p]);
                const float sigma = 0.5f * (H.l1s * H.l1s + H.l2s * H.l2s);
                float nbf = 1.f, bf = 0.f, sigma_blur = 0.f;
                if (use_blur) {
                    const float4 uvs = R.warm[k].uvs;
                    const float dx = uvs.z - P[p].px, dy = uvs.w - P[p].py;
                    sigma_blur = 0.5f * kBlurFsq * (dx * dx + dy * dy);
                    if (sigma_blur < sigma) { bf = 1.f; nbf = 0.f; }
                }
                float alpha = fminf(kAlphaMax, Hr.nop.z * (nbf * __expf(-sigma) + bf * __expf(-sigma_blur)));
                float pixel_dis = 1000.f;
                if (alpha_vis) {
                    alpha = sigma > vis_sth ? 0.f : kAlphaMax;
                    if (accept_opac && Hr.nop.z < 0.5f) alpha = 0.f;
                    pixel_dis = local_outline(Hr, R, k, a, V, J, P[p], vis_sth);
                }
                const bool skip = H.t < kTNear || H.t > kTFar || alpha < kAlphaMin;
                const float next_T = T[p] * (1.f - alpha);
                if (next_T <= kTDone) { done[p] = true; continue; }
                if (skip) continue;
                const RecWarm& Wm = R.warm[k];
                const float vis = alpha * T[p];
                const float4 col = Wm.col;
                // outside the outline: the colour; on it: white (bit 24) or nothing
                const bool plain = !alpha_vis || pixel_dis > outline_bound;
                const float wv = plain ? 0.f : (white_outline ? vis : 0.f);
                if (!alpha_vis) {
                    const float2 o2 = fma2(make_float2(col.x, col.y), dup2(vis), make_float2(out[p].x, out[p].y));
                    out[p].x = o2.x;
                    out[p].y = o2.y;
                    out[p].z = out[p].z + col.z * vis;
                } else {
                    out[p].x = out[p].x + (plain ? col.x * vis : wv);
                    out[p].y = out[p].y + (plain ? col.y * vis : wv);
                    out[p].z = out[p].z + (plain ? col.z * vis : wv);
                }
                float3 hn = f3(Wm.nrm);
                if (flip && H.nd > 0.f) hn = make_float3(-hn.x, -hn.y, -hn.z);
                const float2 n2 = fma2(dup2(vis), make_float2(hn.x, hn.y), make_float2(nrm[p].x, nrm[p].y));
                nrm[p].x = n2.x;
                nrm[p].y = n2.y;
                nrm[p].z += vis * hn.z;
                if (C > 0) {
                    const float2 uv = hit_uv(H, Wm);
                    const int4 tx = Wm.tex;
                    const Bilerp B = bilerp(tx.x, tx.y, tx.z, clamp01(uv.x), clamp01(uv.y), bilinear);
                    if (CT == 3) {
                        float c[4][3];
                        fetch3<TM>(a.tex, B, c);
                        if (!alpha_vis) {  // channels 0 and 1 as one pair
                            float2 v = mul2(dup2(B.w00), make_float2(c[0][0], c[0][1]));
                            v = fma2(dup2(B.w01), make_float2(c[1][0], c[1][1]), v);
                            v = fma2(dup2(B.w10), make_float2(c[2][0], c[2][1]), v);
                            v = fma2(dup2(B.w11), make_float2(c[3][0], c[3][1]), v);
                            const float2 o2 = fma2(dup2(vis), v, make_float2(otex[p][0], otex[p][1]));
                            otex[p][0] = o2.x;
                            otex[p][1] = o2.y;
                            otex[p][2] += vis * (B.w00 * c[0][2] + B.w01 * c[1][2] + B.w10 * c[2][2] + B.w11 * c[3][2]);
                        } else {
#pragma unroll
                            for (int ch = 0; ch < 3; ch++)
                                otex[p][ch] += plain ? vis * (B.w00 * c[0][ch] + B.w01 * c[1][ch] + B.w10 * c[2][ch] +
                                                              B.w11 * c[3][ch])
                                                     : wv;
                        }
                    } else if (CT != 0) {
                        const float* t = (const float*)a.tex;
                        for (int ch = 0; ch < C; ch++) {
                            const float v = B.w00 * __ldg(t + (size_t)B.i00 * C + ch) + B.w01 * __ldg(t + (size_t)B.i01 * C + ch) +
                                            B.w10 * __ldg(t + (size_t)B.i10 * C + ch) + B.w11 * __ldg(t + (size_t)B.i11 * C + ch);
                            otex[p][ch] += plain ? vis * v : wv;
                        }
                    }
                }
                const float t_view = H.tcam;
                if (T[p] > 0.5f) { depth[p] = t_view; didx[p] = bstart + k; }
                const float dv = use_ndc ? (kTFar * t_view - kTFar * kTNear) / ((kTFar - kTNear) * t_view) : H.t;
                reg[p] += vis * (dv * dv * ts[p].x + ts[p].z - 2.f * dv * ts[p].y);
                ts[p].x += vis;
                const float2 t2 = fma2(dup2(vis), make_float2(dv, dv * dv), make_float2(ts[p].y, ts[p].z));
                ts[p].y = t2.x;
                ts[p].z = t2.y;
                T[p] = next_T;
                cur[p] = bstart + k;
            }
            }
            bool ad = true;
#pragma unroll
            for (int p = 0; p < PPT; p++) ad = ad && done[p];
            all_done = ad;
            if (__all_sync(wmask, all_done)) break;
        }
    }
#pragma unroll
    for (int p = 0; p < PPT; p++) {
        if (!inside[p]) continue;
        const int pi = J.ty * bw + lp.x + p;
        const size_t pix = J.pix_base + (size_t)pi * J.W + pj;
        o.final_T[pix] = T[p];
        o.final_idx[pix] = cur[p];
        o.depth_idx[pix] = didx[p];
        o.img[pix] = make_float3(out[p].x + T[p] * a.bg[0], out[p].y + T[p] * a.bg[1], out[p].z + T[p] * a.bg[2]);
        o.normal[pix] = nrm[p];
        o.depth[pix] = depth[p];
        o.reg[pix] = reg[p];
        o.reg_s[pix] = ts[p];
        for (int ch = 0; ch < C; ch++) o.tex[pix * C + ch] = otex[p][ch];
    }
}

// ---------------------------------------------------------------------------
// Backward body: one tile
// ---------------------------------------------------------------------------
// Transpose reduction of N values per lane over the lanes that differ in bits
// OFF, OFF/2, ..., 1: at each level a lane keeps the lower or the upper half
// of its values (H = ceil(N/2) of them) and receives its partner's copy of
// that half, one shuffle per kept value (N - 1 + log2 32 shuffles in all for
// N <= 32).  Starting at OFF = 16 every lane ends with one sum; starting at
// OFF = GS / 2 the reduction stays inside aligned groups of GS lanes and each
// lane ends with OUT sums m[0, OUT).  slot(lane, j) names the value index
// that m[j] belongs to (N when it holds padding).
template <int N, int OFF>
struct Ragged {
    static constexpr int H = (N + 1) / 2;
    static constexpr int OUT = Ragged<H, OFF / 2>::OUT;
    static __device__ __forceinline__ void reduce(float* m, unsigned lane) {
        const bool upper = lane & OFF;
        // two values per step: their sums as one f32x2 add
#pragma unroll
        for (int j = 0; j < H; j += 2) {
            const int j1 = j + 1 < H ? j + 1 : j;
            const float lo0 = m[j], lo1 = m[j1];
            const float hi0 = j + H < N ? m[j + H] : 0.f, hi1 = j1 + H < N ? m[j1 + H] : 0.f;
            const float r0 = __shfl_xor_sync(0xffffffffu, upper ? lo0 : hi0, OFF);
            const float r1 = __shfl_xor_sync(0xffffffffu, upper ? lo1 : hi1, OFF);
            const float2 sum = add2(make_float2(upper ? hi0 : lo0, upper ? hi1 : lo1), make_float2(r0, r1));
            m[j] = sum.x;
            if (j + 1 < H) m[j1] = sum.y;
        }
        Ragged<H, OFF / 2>::reduce(m, lane);
    }
    static __device__ __forceinline__ int slot(unsigned lane, int j = 0) {
        const int inner = Ragged<H, OFF / 2>::slot(lane, j);
        if (inner >= H) return N;
        const int idx = ((lane & OFF) ? H : 0) + inner;
        return idx < N ? idx : N;
    }
};
template <int N>
struct Ragged<N, 0> {
    static constexpr int OUT = N;
    static __device__ __forceinline__ void reduce(float*, unsigned) {}
    static __device__ __forceinline__ int slot(unsigned, int j = 0) { return j; }
};
static_assert(Ragged<23, 16>::OUT == 1, "a full warp reduces 23 moments to one per lane");

template <typename T>
__device__ __forceinline__ T ld_or(const T* p, size_t i, T z) {
    return p ? p[i] : z;
}

// Per-pixel state of the backward walk.
template <int CA>
struct BwdPix {
    PixelRay P;
    bool inside;
    float T, vT_run;
    float3 sfin, vout, vnorm;
    int dfin, bfin;
    float vdepth, vreg;
    float vtex[CA];
};

// Adjoint of one (pixel, Gaussian) pair; adds its moments to m and returns
// false when the pair is skipped.  Follows csrc/texture.cu:577-708.
template <int TEXMODE, int CT, int CA, int NM>
__device__ __forceinline__ void bwd_pair(const SceneArgs& a, const BwdArgs& g, const Recs& R, int k, int gidx,
                                         const RecHot& Hr, const Hit& H, float alpha, float e, float eb, float nbf,
                                         float bf, BwdPix<CA>& S, int C, bool use_ndc, bool prop_uv, bool bilinear,
                                         float (&m)[NM]) {
    static_assert(NM == kMoments || NM == kMoments - 2, "all moments, or all but the two blur moments");
    const RecWarm& Wm = R.warm[k];
    const float4 col = Wm.col, nw = Wm.nrm;
    const float is1 = col.w, is2 = nw.w;
    const PixelRay& P = S.P;
    S.T = __fdividef(S.T, 1.f - alpha);
    const float T = S.T;
    const float vis = alpha * T;
    const float3 vout = S.vout, vnorm = S.vnorm;
    float v_vis = col.x * vout.x + col.y * vout.y + col.z * vout.z + nw.x * vnorm.x + nw.y * vnorm.y + nw.z * vnorm.z;
    float v_u = 0.f, v_v = 0.f;
    if (C > 0) {
        const float2 uv = hit_uv(H, Wm);
        const int4 tx = Wm.tex;
        const Bilerp B = bilerp(tx.x, tx.y, tx.z, clamp01(uv.x), clamp01(uv.y), bilinear);
        const float fh = (float)tx.x, fw = (float)tx.y;
        if (CT == 3) {
            float c[4][3];
            fetch3<TEXMODE>(a.tex, B, c);
            // channels 0 and 1 as f32x2 pairs, channel 2 alone
            const float2 c0 = make_float2(c[0][0], c[0][1]), c1 = make_float2(c[1][0], c[1][1]);
            const float2 c2 = make_float2(c[2][0], c[2][1]), c3 = make_float2(c[3][0], c[3][1]);
            const float2 vt = make_float2(S.vtex[0], S.vtex[1]);
            float2 val = mul2(dup2(B.w00), c0);
            val = fma2(dup2(B.w01), c1, val);
            val = fma2(dup2(B.w10), c2, val);
            val = fma2(dup2(B.w11), c3, val);
            const float val2 = B.w00 * c[0][2] + B.w01 * c[1][2] + B.w10 * c[2][2] + B.w11 * c[3][2];
            const float2 gv01 = mul2(dup2(vis), vt);
            const float gv2 = vis * S.vtex[2];
            if (bilinear && prop_uv) {
                // d(val)/d(tcx) = (1 - fy)(c10 - c00) + fy (c11 - c01),
                // d(val)/d(tcy) = (1 - fx)(c01 - c00) + fx (c11 - c10)
                const float2 du = fma2(dup2(B.fy), sub2(c3, c1), mul2(dup2(1.f - B.fy), sub2(c2, c0)));
                const float2 dv = fma2(dup2(B.fx), sub2(c3, c2), mul2(dup2(1.f - B.fx), sub2(c1, c0)));
                const float du2 = (1.f - B.fy) * (c[2][2] - c[0][2]) + B.fy * (c[3][2] - c[1][2]);
                const float dv2 = (1.f - B.fx) * (c[1][2] - c[0][2]) + B.fx * (c[3][2] - c[2][2]);
                const float2 pu = mul2(gv01, du), pv = mul2(gv01, dv);
                v_u += fh * (pu.x + pu.y + gv2 * du2);
                v_v += fw * (pv.x + pv.y + gv2 * dv2);
            }
            const float2 vs = mul2(val, vt);
            v_vis += vs.x + vs.y + val2 * S.vtex[2];
            if (gv01.x != 0.f || gv01.y != 0.f || gv2 != 0.f) {
                const int rows[4] = { B.i00, B.i01, B.i10, B.i11 };
                const float wts[4] = { B.w00, B.w01, B.w10, B.w11 };
                const float gv[3] = { gv01.x, gv01.y, gv2 };
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (wts[q] == 0.f) continue;
                    if (TEXMODE == 1) {
                        const float2 g01 = mul2(dup2(wts[q]), gv01);
                        atomicAdd(reinterpret_cast<float4*>(g.v_texgrad) + rows[q],
                                  make_float4(g01.x, g01.y, wts[q] * gv2, 0.f));
                    } else {
                        float* dst = g.v_texgrad + 3 * (size_t)rows[q];
                        atomicAdd(dst + 0, wts[q] * gv[0]);
                        atomicAdd(dst + 1, wts[q] * gv[1]);
                        atomicAdd(dst + 2, wts[q] * gv[2]);
                    }
                }
            }
        } else if (CT != 0) {
            const float* t = (const float*)a.tex;
            for (int ch = 0; ch < C; ch++) {
                const float c00 = __ldg(t + (size_t)B.i00 * C + ch), c01 = __ldg(t + (size_t)B.i01 * C + ch);
                const float c10 = __ldg(t + (size_t)B.i10 * C + ch), c11 = __ldg(t + (size_t)B.i11 * C + ch);
                const float val = B.w00 * c00 + B.w01 * c01 + B.w10 * c10 + B.w11 * c11;
                const float vv = vis * S.vtex[ch];
                if (vv != 0.f) {
                    if (B.w00 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i00 * C + ch, B.w00 * vv);
                    if (B.w01 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i01 * C + ch, B.w01 * vv);
                    if (B.w10 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i10 * C + ch, B.w10 * vv);
                    if (B.w11 != 0.f) atomicAdd(g.v_texgrad + (size_t)B.i11 * C + ch, B.w11 * vv);
                }
                if (bilinear && prop_uv) {
                    v_u += fh * (vv * (-(1.f - B.fy) * c00 - B.fy * c01 + (1.f - B.fy) * c10 + B.fy * c11));
                    v_v += fw * (vv * (-(1.f - B.fx) * c00 + (1.f - B.fx) * c01 - B.fx * c10 + B.fx * c11));
                }
                v_vis += val * S.vtex[ch];
            }
        }
    }
    const float vT_run = S.vT_run;
    float v_alpha = T * v_vis - T * vT_run;
    float vT_cur = alpha * v_vis + (1.f - alpha) * vT_run;
    const float t_view = H.tcam;
    const float3 sfin = S.sfin;
    float v_t = 0.f, v_t_ndc = 0.f, v_w = 0.f;
    if (use_ndc) {
        const float t_ndc = (kTFar * t_view - kTFar * kTNear) / ((kTFar - kTNear) * t_view);
        v_t_ndc = 2.f * (vis * t_ndc * sfin.x - vis * sfin.y) * S.vreg;
        v_w = (t_ndc * t_ndc * sfin.x - 2.f * t_ndc * sfin.y + sfin.z) * S.vreg;
    } else {
        v_t = 2.f * (vis * H.t * sfin.x - vis * sfin.y) * S.vreg;
        v_w = (H.t * H.t * sfin.x - 2.f * H.t * sfin.y + sfin.z) * S.vreg;
    }
    v_alpha += v_w * T;
    vT_cur += v_w * alpha;
    S.vT_run = vT_cur;
    const float v_sigma = -nbf * Hr.nop.z * e * v_alpha;
    // sigma = (l1s^2 + l2s^2) / 2 with l_ks = l_k * is_k, so v_lk = is_k l_ks v_sigma;
    // the per-Gaussian factors is_k, 1 / is_k and glob are applied at the flush
    const float p1 = H.l1s * v_sigma, p2 = H.l2s * v_sigma;
    const float l1 = __fdividef(H.l1s, is1), l2 = __fdividef(H.l2s, is2);
    // ray . axis from the hit: l = a . (t r - mu) gives a . r = (l + a . mu) / t
    const RecCold& Cd = R.cold[k];
    const float it = __fdividef(1.f, H.t);
    const float ra1 = (l1 + Cd.mu.w) * it;
    const float ra2 = (l2 + Cd.dt.x) * it;
    v_t += is1 * p1 * ra1 + is2 * p2 * ra2;
    if (prop_uv) {
        const float2 uvr = hit_uv(H, Wm);
        const float rum = (uvr.x - Wm.uvs.x + Cd.dt.y) * it;
        const float rvm = (uvr.y - Wm.uvs.y + Cd.dt.z) * it;
        v_t += v_u * rum + v_v * rvm;
    }
    float v_t_view = 0.f;
    if (gidx == S.dfin && S.dfin != -1) v_t_view += S.vdepth;
    if (use_ndc) v_t_view += (kTFar * kTNear) / ((kTFar - kTNear) * t_view * t_view) * v_t_ndc;
    v_t += P.idn * v_t_view;
    const float vtd = v_t * (P.dn * H.inv);  // v_t / (n . r)
    const float v_sb = -bf * Hr.nop.z * eb * v_alpha;
    // (pairs of moments as one f32x2 operation where they line up)
    const float2 ls = make_float2(H.l1s, H.l2s);
    float2 t2 = fma2(dup2(vis), make_float2(vout.x, vout.y), make_float2(m[0], m[1]));
    m[0] = t2.x; m[1] = t2.y;
    m[2] += vis * vout.z;
    m[3] += (nbf * e + bf * eb) * v_alpha;
    t2 = fma2(ls, make_float2(p1, p2), make_float2(m[4], m[5]));  // l1 v_l1, l2 v_l2; v_scale1 = -is1 glob m4
    m[4] = t2.x; m[5] = t2.y;
    m[6] += H.l1s * p2;  // l2 v_l1 = (is1 / is2) m6, l1 v_l2 = (is2 / is1) m6
    t2 = add2(make_float2(m[7], m[8]), make_float2(p1, p2));  // v_l1 / is1, v_l2 / is2
    m[7] = t2.x; m[8] = t2.y;
    m[9] += vtd;
    t2 = fma2(ls, dup2(vtd), make_float2(m[10], m[11]));  // l1 vtd is1, l2 vtd is2
    m[10] = t2.x; m[11] = t2.y;
    t2 = fma2(dup2(vis), make_float2(vnorm.x, vnorm.y), make_float2(m[12], m[13]));
    m[12] = t2.x; m[13] = t2.y;
    m[14] += vis * vnorm.z;
    t2 = add2(make_float2(m[15], m[16]), make_float2(v_u, v_v));
    m[15] = t2.x; m[16] = t2.y;
    t2 = fma2(ls, dup2(v_u), make_float2(m[17], m[18]));  // l1 v_u is1, l2 v_u is2
    m[17] = t2.x; m[18] = t2.y;
    t2 = fma2(ls, dup2(v_v), make_float2(m[19], m[20]));
    m[19] = t2.x; m[20] = t2.y;
    if constexpr (NM == kMoments) {
        m[21] += kBlurFsq * v_sb * (Wm.uvs.z - P.px);
        m[22] += kBlurFsq * v_sb * (Wm.uvs.w - P.py);
    }
}

// GS: lanes per splat walk.  32 = the warp walks one candidate list; 16, 8 or
// 4 (full warps only) = each group of GS lanes (a compact pixel block, see
// thread_pixel) walks its own list, so a warp works on 32 / GS splats at once
// and a small splat occupies the lanes of the pixels it can reach, not a whole
// warp.
template <int TEXMODE, int CT, int PPT, int GS = 32, int FIX = 0>
__device__ __forceinline__ void bwd_tile(const SceneArgs& a, const TileJob& J, const BwdArgs& g, const Recs& R,
                                         float* smom, uint8_t* lists, uint8_t* touched) {
    static_assert(GS == 32 || GS == 16 || GS == 8 || GS == 4, "group of 32, 16, 8 or 4 lanes");
    // FIX = 1: compiled for the default settings (kFixedBwdSettings): no
    // blur (its two moments are dropped), no NDC depth, uv gradients
    // propagated, bilinear texels
    constexpr int NM = FIX ? kMoments - 2 : kMoments;
    using Red = Ragged<NM, GS / 2>;
    const int nthr = blockDim.x * blockDim.y;
    const int tr = threadIdx.y * blockDim.x + threadIdx.x;
    const int bw = blockDim.x;
    const unsigned lane = tr & 31;
    const unsigned wmask = __activemask();
    // Gaussians staged per round (the shared-memory slots); candidate lists
    // of that length: one per warp, then (GS < 32) one per group
    const int bsz = batch_of(a, nthr);
    uint8_t* wl = lists + (tr >> 5) * bsz;
    uint8_t* gl = lists + ((size_t)ceil_div(nthr, 32) + tr / GS) * bsz;
    const bool full_warp = wmask == 0xffffffffu;
    int my_slot[Red::OUT];
#pragma unroll
    for (int q = 0; q < Red::OUT; q++) my_slot[q] = Red::slot(lane, q);
    const View& V = J.V;
    const bool use_blur = FIX ? false : (a.settings & (1 << 9)) != 0;
    const bool use_ndc = FIX ? false : (a.settings & (1 << 10)) != 0;
    const bool prop_uv = FIX ? true : (a.settings & (1 << 8)) != 0;
    const bool bilinear = FIX ? true : !(a.settings & (1 << 2));
    const int C = CT >= 0 ? CT : a.C;
    constexpr int CA = CT > 0 ? CT : (CT == 0 ? 1 : kMaxChannels);
    const float3 z3 = make_float3(0.f, 0.f, 0.f);
    const int2 lp = thread_pixel<PPT, GS>(bw);
    const int pj = J.tx * bw + lp.y;
    BwdPix<CA> S[PPT];
    int my_bfin = -1;
#pragma unroll
    for (int p = 0; p < PPT; p++) {
        const int pi = J.ty * bw + lp.x + p;
        BwdPix<CA>& s = S[p];
        s.P = make_pixel(V, pi, pj);
        s.inside = pi < J.H && pj < J.W;
        const size_t pix = s.inside ? J.pix_base + (size_t)pi * J.W + pj : 0;
        s.T = s.inside ? g.final_T[pix] : 1.f;
        s.sfin = s.inside ? g.reg_s[pix] : z3;
        s.dfin = s.inside ? g.depth_idx[pix] : -1;
        s.bfin = s.inside ? g.final_idx[pix] : 0;
        s.vout = s.inside ? ld_or(g.v_img, pix, z3) : z3;
        s.vdepth = s.inside ? ld_or(g.v_depth, pix, 0.f) : 0.f;
        s.vreg = s.inside ? ld_or(g.v_reg, pix, 0.f) : 0.f;
        const float valph = s.inside ? ld_or(g.v_alpha, pix, 0.f) : 0.f;
        s.vnorm = s.inside ? ld_or(g.v_normal, pix, z3) : z3;
        for (int ch = 0; ch < CA; ch++) s.vtex[ch] = (s.inside && ch < C && g.v_tex) ? g.v_tex[pix * C + ch] : 0.f;
        s.vT_run = a.bg[0] * s.vout.x + a.bg[1] * s.vout.y + a.bg[2] * s.vout.z - valph;
        if (s.inside) my_bfin = max(my_bfin, s.bfin);
    }
    // last contributor and rectangle of the pixel centres of the warp, and
    // (GS < 32) of the lane's group
    const int pi0 = J.ty * bw + lp.x;
    const int warp_bfin = __reduce_max_sync(wmask, my_bfin);
    const float rx0 = (float)__reduce_min_sync(wmask, pj) + 0.5f, rx1 = (float)__reduce_max_sync(wmask, pj) + 0.5f;
    const float ry0 = (float)__reduce_min_sync(wmask, pi0) + 0.5f;
    const float ry1 = (float)__reduce_max_sync(wmask, pi0 + PPT - 1) + 0.5f;
    int group_bfin = warp_bfin;
    float qx0 = rx0, qx1 = rx1, qy0 = ry0, qy1 = ry1;
    if (GS < 32) {
        group_bfin = group_max<GS>(my_bfin);
        qx0 = (float)group_min<GS>(pj) + 0.5f;
        qx1 = (float)group_max<GS>(pj) + 0.5f;
        qy0 = (float)group_min<GS>(pi0) + 0.5f;
        qy1 = (float)group_max<GS>(pi0 + PPT - 1) + 0.5f;
    }
    const unsigned gmask = (GS == 32) ? wmask : (((1u << GS) - 1u) << (lane & ~(unsigned)(GS - 1)));

    const int2 range = J.range;
    const int nb = ceil_div(range.y - range.x, bsz);
    for (int b = 0; b < nb; ++b) {
        __syncthreads();
        const int bend = range.y - 1 - bsz * b;
        const int bsize = min(bsz, bend + 1 - range.x);
        const int idx = bend - tr;
        const bool mine = tr < bsz && idx >= range.x;  // this thread stages and flushes slot tr
        if (mine) stage_job(R, tr, a, J, a.gids[idx], use_blur);
        for (int q = tr; q < bsz * (kMomSlot / 4); q += nthr)
            reinterpret_cast<float4*>(smom)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (tr < bsz) touched[tr] = 0;
        __syncthreads();
        // splats outside their alpha >= 1/255 box contribute nothing here:
        // walk the candidates of the warp or group, back to front
        const int cntw = build_list(wl, R, max(0, bend - warp_bfin), bsize, rx0, rx1, ry0, ry1, wmask, lane);
        int cnt = cntw, cmax = cntw;
        const uint8_t* list = wl;
        if (GS < 32) {
            cnt = build_group_list<GS>(gl, wl, cntw, R, max(0, bend - group_bfin), qx0, qx1, qy0, qy1, lane);
            cmax = __reduce_max_sync(0xffffffffu, cnt);
            list = gl;
        }
        for (int j = 0; j < cmax; ++j) {
            const bool act = j < cnt;
            const int k = act ? list[j] : 0;
            const int gidx = bend - k;
            {
                const float4 bx = R.hot[k].box;
                bool need = false;
#pragma unroll
                for (int p = 0; p < PPT; p++)
                    need = need || (S[p].inside && gidx <= S[p].bfin &&
                                    !(S[p].P.px < bx.x || S[p].P.px > bx.y || S[p].P.py < bx.z || S[p].P.py > bx.w));
                if (!__any_sync(wmask, act && need)) continue;
            }
            const RecHot Hr = R.hot[k];
            bool valid[PPT];
            Hit H[PPT];
            float e[PPT], eb[PPT], nbf[PPT], bf[PPT], alpha[PPT];
            bool any = false;
#pragma unroll
            for (int p = 0; p < PPT; p++) {
                valid[p] = act && S[p].inside && gidx <= S[p].bfin && !outside_box(Hr, S[p].P);
                e[p] = eb[p] = alpha[p] = bf[p] = 0.f;
                nbf[p] = 1.f;
                if (valid[p]) {
                    H[p] = hit_pixel(Hr, R, k, a, V, S[p].P);
                    const float sigma = 0.5f * (H[p].l1s * H[p].l1s + H[p].l2s * H[p].l2s);
                    float sigma_blur = 0.f;
                    if (use_blur) {
                        const float4 uvs = R.warm[k].uvs;
                        const float dx = uvs.z - S[p].P.px, dy = uvs.w - S[p].P.py;
                        sigma_blur = 0.5f * kBlurFsq * (dx * dx + dy * dy);
                        if (sigma_blur < sigma) { bf[p] = 1.f; nbf[p] = 0.f; }
                    }
                    e[p] = __expf(-sigma);
                    eb[p] = use_blur ? __expf(-sigma_blur) : 0.f;
                    alpha[p] = fminf(kAlphaMax, Hr.nop.z * (nbf[p] * e[p] + bf[p] * eb[p]));
                    if (H[p].t < kTNear || H[p].t > kTFar || alpha[p] < kAlphaMin) valid[p] = false;
                }
                any = any || valid[p];
            }
            const unsigned vmask = __ballot_sync(wmask, any);
            if (!vmask) continue;
            float m[NM];
#pragma unroll
            for (int q = 0; q < NM; q++) m[q] = 0.f;
#pragma unroll
            for (int p = 0; p < PPT; p++)
                if (valid[p])
                    bwd_pair<TEXMODE, CT, CA, NM>(a, g, R, k, gidx, Hr, H[p], alpha[p], e[p], eb[p], nbf[p], bf[p],
                                                  S[p], C, use_ndc, prop_uv, bilinear, m);
            float* dst = smom + k * kMomSlot;
            if (GS == 32 && !full_warp) {
                if (lane == 0) touched[k] = 1;
                if (any) {
#pragma unroll
                    for (int q = 0; q < NM; q++) atomicAdd(dst + q, m[q]);
                }
            } else {
                Red::reduce(m, lane);
                if (vmask & gmask) {
                    if ((lane & (GS - 1)) == 0) touched[k] = 1;
#pragma unroll
                    for (int q = 0; q < Red::OUT; q++)
                        if (my_slot[q] < NM) atomicAdd(dst + my_slot[q], m[q]);
                }
            }
        }
        __syncthreads();
        if (mine && touched[tr]) {
            float sm[kMomSlot];
#pragma unroll
            for (int q = 0; q < kMomSlot / 4; q++) {
                const float4 v4 = reinterpret_cast<const float4*>(smom + tr * kMomSlot)[q];
                sm[4 * q] = v4.x; sm[4 * q + 1] = v4.y; sm[4 * q + 2] = v4.z; sm[4 * q + 3] = v4.w;
            }
            {
                const int gid = R.warm[tr].tex.w;
                if (J.vc_stride == 4) {
                    atomicAdd(reinterpret_cast<float4*>(J.vcolors) + gid, make_float4(sm[0], sm[1], sm[2], 0.f));
                } else {
                    float* vc = J.vcolors + 3 * (size_t)gid;
                    atomicAdd(vc + 0, sm[0]);
                    atomicAdd(vc + 1, sm[1]);
                    atomicAdd(vc + 2, sm[2]);
                }
                float4* dst = reinterpret_cast<float4*>(g.moments + (size_t)gid * kMomStride);
                // blur moments -> world-space mean gradient (helpers.cuh:155-164, 114-121)
                const float3 p = f3(R.cold[tr].mu);
                const float rw = 1.f / (p.z + 1e-6f);
                const float vx = V.fx * sm[21], vy = V.fy * sm[22];
                const float3 vmb = V.rot_t(make_float3(vx * rw, vy * rw, -(vx * p.x + vy * p.y) * rw * rw));
                // the per-Gaussian factors left out of the pixel sums
                const float is1 = R.warm[tr].col.w, is2 = R.warm[tr].nrm.w;
                const float r1 = 1.f / is1, r2 = 1.f / is2;
                float v[kMomStride];
                v[0] = sm[3];
                v[1] = -is1 * a.glob * sm[4];
                v[2] = -is2 * a.glob * sm[5];
                v[3] = is1 * sm[7];
                v[4] = is2 * sm[8];
                v[5] = sm[9];
                v[6] = sm[4];
                v[7] = is1 * r2 * sm[6];
                v[8] = is2 * r1 * sm[6];
                v[9] = sm[5];
                v[10] = r1 * sm[10];
                v[11] = r2 * sm[11];
                v[12] = sm[12]; v[13] = sm[13]; v[14] = sm[14];
                v[15] = sm[15]; v[16] = sm[16];
                v[17] = r1 * sm[17];
                v[18] = r2 * sm[18];
                v[19] = r1 * sm[19];
                v[20] = r2 * sm[20];
                v[21] = vmb.x; v[22] = vmb.y; v[23] = vmb.z;
#pragma unroll
                for (int q = 0; q < kMomStride / 4; q++)
                    atomicAdd(dst + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Texture editing (csrc/texture_edit.cu:11-236): the forward walk, front to
// back (blur is settings bit 0 here), and for every contributing pair whose
// camera depth lies in the pixel's [lower, upper] range a bilinear splat of
// (r a, g a, b a, a, 1) of the edited pixel into the chart's [T, 5] texels.
// ---------------------------------------------------------------------------
struct EditIO {
    const float3* img;
    const float* alpha;
    const float* lower;
    const float* upper;
    float* out;  // [T, 5]
};

__device__ __forceinline__ void edit_tile(const SceneArgs& a, const TileJob& J, const EditIO& E, const Recs& R) {
    const int nthr = blockDim.x * blockDim.y;
    const int tr = threadIdx.y * blockDim.x + threadIdx.x;
    const int bw = blockDim.x;
    const View& V = J.V;
    const bool use_blur = a.settings & 1;
    const int2 lp = thread_pixel<1>(bw);
    const int pj = J.tx * bw + lp.y, pi = J.ty * bw + lp.x;
    const PixelRay P = make_pixel(V, pi, pj);
    const bool inside = pi < J.H && pj < J.W;
    bool done = !inside;
    float vals[5] = { 0.f, 0.f, 0.f, 0.f, 1.f };
    float lo = 0.f, hi = 0.f;
    if (inside) {
        const size_t pix = J.pix_base + (size_t)pi * J.W + pj;
        const float3 c = E.img[pix];
        const float m = E.alpha[pix];
        vals[0] = c.x * m; vals[1] = c.y * m; vals[2] = c.z * m; vals[3] = m;
        lo = E.lower[pix];
        hi = E.upper[pix];
    }
    float T = 1.f;
    const int2 range = J.range;
    const int nb = ceil_div(range.y - range.x, nthr);
    for (int b = 0; b < nb; ++b) {
        if (__syncthreads_count(done) >= nthr) break;
        const int bstart = range.x + nthr * b;
        const int idx = bstart + tr;
        if (idx < range.y) stage_job(R, tr, a, J, a.gids[idx], use_blur);
        __syncthreads();
        const int bsize = min(nthr, range.y - bstart);
        for (int k = 0; k < bsize && !done; ++k) {
            const RecHot Hr = R.hot[k];
            // outside the alpha >= 1/255 box a splat is skipped; it can end the
            // pixel there only when T <= 1e-4 * 255/254
            if (outside_box(Hr, P) && T > 1.01e-4f) continue;
            const Hit H = hit_pixel(Hr, R, k, a, V, P);
            const float sigma = 0.5f * (H.l1s * H.l1s + H.l2s * H.l2s);
            float nbf = 1.f, bf = 0.f, sigma_blur = 0.f;
            if (use_blur) {
                const float4 uvs = R.warm[k].uvs;
                const float dx = uvs.z - P.px, dy = uvs.w - P.py;
                sigma_blur = 0.5f * kBlurFsq * (dx * dx + dy * dy);
                if (sigma_blur < sigma) { bf = 1.f; nbf = 0.f; }
            }
            const float alpha = fminf(kAlphaMax, Hr.nop.z * (nbf * __expf(-sigma) + bf * __expf(-sigma_blur)));
            const bool skip = H.t < kTNear || H.t > kTFar || alpha < kAlphaMin;
            const float next_T = T * (1.f - alpha);
            if (next_T <= kTDone) { done = true; continue; }
            if (skip) continue;
            if (H.tcam >= lo && H.tcam <= hi) {
                const RecWarm& Wm = R.warm[k];
                const float2 uv = hit_uv(H, Wm);
                const int4 tx = Wm.tex;
                const Bilerp B = bilerp(tx.x, tx.y, tx.z, clamp01(uv.x), clamp01(uv.y), true);
                const int rows[4] = { B.i00, B.i01, B.i10, B.i11 };
                const float wts[4] = { B.w00, B.w01, B.w10, B.w11 };
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    float* dst = E.out + 5 * (size_t)rows[q];
#pragma unroll
                    for (int c = 0; c < 5; c++) atomicAdd(dst + c, wts[q] * vals[c]);
                }
            }
            T = next_T;
        }
    }
}

template <int PPT>
__global__ void __launch_bounds__(256, 4) edit_view_kernel(SceneArgs a, ViewArgs va, EditIO E) {
    extern __shared__ __align__(16) unsigned char smem[];
    TileJob J;
    J.V = load_view(va.viewmat, va.fx, va.fy, va.cx, va.cy);
    J.W = va.W; J.H = va.H;
    J.tx = blockIdx.x; J.ty = blockIdx.y;
    J.range = va.bins[blockIdx.y * va.tiles_x + blockIdx.x];
    J.pix_base = 0;
    J.colors = nullptr;
    J.vcolors = nullptr;
    J.vc_stride = 3;
    J.recs = nullptr;
    edit_tile(a, J, E, Recs::carve(smem, blockDim.x * blockDim.y, false));
}

// ---------------------------------------------------------------------------
// Launch forms
// ---------------------------------------------------------------------------
// Minimum resident CTAs per SM asked of the register allocator.
#ifndef GSTEX_FWD_MINB
#define GSTEX_FWD_MINB 5
#endif
#ifndef GSTEX_BWD_MINB
#define GSTEX_BWD_MINB 4
#endif
#ifndef GSTEX_FWD_MINB1
#define GSTEX_FWD_MINB1 4
#endif
#ifndef GSTEX_BWD_MINB1
#define GSTEX_BWD_MINB1 2
#endif
#define FWD_BOUNDS(PPT) __launch_bounds__((PPT) == 2 ? 128 : 256, (PPT) == 2 ? GSTEX_FWD_MINB : GSTEX_FWD_MINB1)
#define BWD_BOUNDS(PPT) __launch_bounds__((PPT) == 2 ? 128 : 256, (PPT) == 2 ? GSTEX_BWD_MINB : GSTEX_BWD_MINB1)

template <int TEXMODE, int CT, int PPT>
__global__ void FWD_BOUNDS(PPT) fwd_view_kernel(SceneArgs a, ViewArgs va, FwdOut o) {
    extern __shared__ __align__(16) unsigned char smem[];
    TileJob J;
    J.V = load_view(va.viewmat, va.fx, va.fy, va.cx, va.cy);
    J.W = va.W; J.H = va.H;
    J.tx = blockIdx.x; J.ty = blockIdx.y;
    J.range = va.bins[blockIdx.y * va.tiles_x + blockIdx.x];
    J.pix_base = 0;
    J.colors = va.colors;
    J.vcolors = nullptr;
    J.vc_stride = 3;
    J.recs = va.recs;
    const int nthr = blockDim.x * blockDim.y;
    fwd_tile<TEXMODE, CT, PPT>(a, J, o, Recs::carve(smem, nthr, false));
}

template <int TEXMODE, int CT, int PPT, int GS>
__global__ void BWD_BOUNDS(PPT) bwd_view_kernel(SceneArgs a, ViewArgs va, BwdArgs g) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nthr = blockDim.x * blockDim.y;
    TileJob J;
    J.V = load_view(va.viewmat, va.fx, va.fy, va.cx, va.cy);
    J.W = va.W; J.H = va.H;
    J.tx = blockIdx.x; J.ty = blockIdx.y;
    J.range = va.bins[blockIdx.y * va.tiles_x + blockIdx.x];
    J.pix_base = 0;
    J.colors = va.colors;
    J.vcolors = va.vcolors;
    J.vc_stride = 3;
    J.recs = va.recs;
    uint8_t* lists = smem + (size_t)(kRecBytes + kEdgeBytes + kMomSlot * sizeof(float)) * nthr;
    bwd_tile<TEXMODE, CT, PPT, GS>(a, J, g, Recs::carve(smem, nthr, true),
                                   reinterpret_cast<float*>(smem + (size_t)(kRecBytes + kEdgeBytes) * nthr), lists,
                                   lists + ((size_t)ceil_div(nthr, 32) + (GS < 32 ? ceil_div(nthr, GS) : 0)) * nthr);
}

__device__ __forceinline__ bool next_job(const BatchArgs& ba, int* s_tile, TileJob& J) {
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) *s_tile = atomicAdd(ba.queue, 1);
    __syncthreads();
    int t = *s_tile;
    if (t >= ba.total_tiles) return false;
    if (ba.order) t = ba.order[t];
    const int v = ba.tile_view[t];
    const BatchView& bv = ba.views[v];
    J.V = bv.V;
    J.W = bv.W; J.H = bv.H;
    const int local = t - bv.tile_offset;
    J.ty = local / bv.tiles_x;
    J.tx = local - J.ty * bv.tiles_x;
    J.range = ba.bins[t];
    J.pix_base = bv.pix_offset;
    J.colors = ba.colors + (size_t)v * ba.num_points;
    J.vcolors = ba.vcolors ? ba.vcolors + (size_t)v * ba.num_points * 4 : nullptr;
    J.vc_stride = 4;
    J.recs = ba.recs ? ba.recs + (size_t)v * ba.num_points : nullptr;
    return true;
}

template <int TEXMODE, int CT, int PPT, int FIX = 0>
__global__ void FWD_BOUNDS(PPT) fwd_batch_kernel(SceneArgs a, BatchArgs ba, FwdOut o) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_tile;
    TileJob J;
    const int slots = batch_of(a, blockDim.x * blockDim.y);
    const Recs R = Recs::carve(smem, slots, false);
    while (next_job(ba, &s_tile, J)) fwd_tile<TEXMODE, CT, PPT, FIX>(a, J, o, R);
}

template <int TEXMODE, int CT, int PPT, int GS, int FIX = 0>
__device__ __forceinline__ void bwd_batch_body(const SceneArgs& a, const BatchArgs& ba, const BwdArgs& g) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_tile;
    const int nthr = blockDim.x * blockDim.y;
    const int slots = batch_of(a, nthr);
    TileJob J;
    const Recs R = Recs::carve(smem, slots, true);
    float* smom = reinterpret_cast<float*>(smem + (size_t)(kRecBytes + kEdgeBytes) * slots);
    uint8_t* lists = smem + (size_t)(kRecBytes + kEdgeBytes + kMomSlot * sizeof(float)) * slots;
    uint8_t* touched = lists + ((size_t)ceil_div(nthr, 32) + (GS < 32 ? ceil_div(nthr, GS) : 0)) * slots;
    while (next_job(ba, &s_tile, J)) bwd_tile<TEXMODE, CT, PPT, GS, FIX>(a, J, g, R, smom, lists, touched);
}

template <int TEXMODE, int CT, int PPT, int GS>
__global__ void BWD_BOUNDS(PPT) bwd_batch_kernel(SceneArgs a, BatchArgs ba, BwdArgs g) {
    bwd_batch_body<TEXMODE, CT, PPT, GS>(a, ba, g);
}

// Registers per thread that let NB CTAs of 64 threads reside on one SM.
constexpr int regs_for_ctas(int nb) { return (65536 / (64 * nb)) / 8 * 8; }

// 8x8 tiles (64 threads, one pixel each) with GS-lane groups, compiled for
// NB resident CTAs per SM: at most 65536 / (64 NB) registers per thread
// rounded down to a multiple of 8 (96 for 10 CTAs; the general kernel uses
// 124, which allows 8), in exchange for more warps per SM.  (9 CTAs at 112
// registers measured between the two; 11 and 12 CTAs, at 88 and 80 registers
// and with fewer Gaussians per batch so that the shared memory fits, spill
// 130-190 bytes and lose.)  FIX = 1: compiled for the default settings (see
// bwd_tile).
template <int TEXMODE, int CT, int NB, int FIX, int GS>
__global__ void __launch_bounds__(64) __maxnreg__(regs_for_ctas(NB))
    bwd_batch64_kernel(SceneArgs a, BatchArgs ba, BwdArgs g) {
    bwd_batch_body<TEXMODE, CT, 1, GS, FIX>(a, ba, g);
}

// Writes the 32 records of a warp, assembled in shared memory (src), to
// dst[0, 32) as contiguous 16-byte chunks, skipping the records of lanes not
// in `live`.
__device__ __forceinline__ void copy_out_records(const RecAll* __restrict__ src, RecAll* __restrict__ dst,
                                                 unsigned live, unsigned lane) {
    constexpr int kChunks = (int)(sizeof(RecAll) / 16);
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    __syncwarp();
#pragma unroll 2
    for (int c = (int)lane; c < 32 * kChunks; c += 32)
        if ((live >> (c / kChunks)) & 1u) d4[c] = s4[c];
}

// Records of every (view, Gaussian) pair with tiles in the view, and of
// Gaussian 0 in every view (the reference's zero-slot entries name it).
// Block b covers Gaussians [128 (b / V), +128) of view b % V, so the blocks of
// one Gaussian range run back to back and reread its parameters from cache.
// Near-edge-on pairs get fp32 coefficients here and are appended to `fix`
// for records_fixup_kernel: on this GPU one lane in the double branch would
// hold its whole warp at the fp64 rate.
__global__ void __launch_bounds__(128) records_kernel(SceneArgs a, BatchArgs ba, int num_views,
                                                      const int32_t* __restrict__ counts, RecAll* __restrict__ recs,
                                                      int* __restrict__ fix_count, uint32_t* __restrict__ fix) {
    __shared__ RecAll srec[128];
    const int v = blockIdx.x % num_views;
    const int i0 = (blockIdx.x / num_views) * 128;
    const int i = i0 + threadIdx.x;
    const size_t j = (size_t)v * ba.num_points + i;
    const bool live = i < ba.num_points && (i == 0 || counts[j] > 0);
    if (live) {
        const View V = ba.views[v].V;
        RecAll& r = srec[threadIdx.x];
        const bool defer = make_record(r.h, r.w, r.c, i, V, a.means[i], a.quats[i],
                                       make_float2(a.scales[3 * i], a.scales[3 * i + 1]), a.glob, a.opac[i],
                                       ba.colors[j], a.uv0[i], a.umap[i], a.vmap[i], a.dims[i],
                                       a.settings & (1 << 9), false, &r.e, !(a.settings & (1 << 16)));
        if (defer) fix[atomicAdd(fix_count, 1)] = (uint32_t)j;
    }
    const unsigned lane = threadIdx.x & 31;
    const int w0 = threadIdx.x & ~31;
    copy_out_records(srec + w0, recs + (size_t)v * ba.num_points + i0 + w0, __ballot_sync(0xffffffffu, live), lane);
}

// The double solve of one deferred near-edge-on record of Gaussian i.
__device__ __forceinline__ void fix_record(const SceneArgs& a, const View& V, int i, RecAll* __restrict__ rec) {
    const Axes A = quat_axes(a.quats[i]);
    const float3 mc = V.xform(a.means[i]);
    const float3 a1c = V.rot(A.a1), a2c = V.rot(A.a2), nc = V.rot(A.a3);
    const float3 umc = V.rot(a.umap[i]), vmc = V.rot(a.vmap[i]);
    const float is1 = 1.f / (a.scales[3 * i] * a.glob), is2 = 1.f / (a.scales[3 * i + 1] * a.glob);
    RecHot h = rec->h;
    RecWarm w = rec->w;
    edge_on_solve(h, w, V, mc, a1c, a2c, nc, umc, vmc, is1, is2, dot3(nc, mc));
    rec->h = h;
    rec->w.uvm = w.uvm;
}

// The double solve of the deferred near-edge-on records, densely.
__global__ void records_fixup_kernel(SceneArgs a, BatchArgs ba, const int* __restrict__ fix_count,
                                     const uint32_t* __restrict__ fix, RecAll* __restrict__ recs) {
    const int n = *fix_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t j = fix[t];
        const int v = (int)(j / (uint32_t)ba.num_points);
        const int i = (int)(j - (uint32_t)v * (uint32_t)ba.num_points);
        fix_record(a, ba.views[v].V, i, recs + j);
    }
}

// Per-view form (texture_forward / texture_backward): the record of every
// Gaussian of one view, so that any Gaussian a tile names has one.
__global__ void __launch_bounds__(128) view_records_kernel(SceneArgs a, ViewArgs va, RecAll* __restrict__ recs,
                                                           int* __restrict__ fix_count, uint32_t* __restrict__ fix) {
    __shared__ RecAll srec[128];
    const int i0 = blockIdx.x * 128;
    const int i = i0 + threadIdx.x;
    const bool live = i < a.N;
    if (live) {
        const View V = load_view(va.viewmat, va.fx, va.fy, va.cx, va.cy);
        RecAll& r = srec[threadIdx.x];
        const bool defer = make_record(r.h, r.w, r.c, i, V, a.means[i], a.quats[i],
                                       make_float2(a.scales[3 * i], a.scales[3 * i + 1]), a.glob, a.opac[i],
                                       va.colors[i], a.uv0[i], a.umap[i], a.vmap[i], a.dims[i], a.settings & (1 << 9),
                                       false, &r.e, !(a.settings & (1 << 16)));
        if (defer) fix[atomicAdd(fix_count, 1)] = (uint32_t)i;
    }
    const unsigned lane = threadIdx.x & 31;
    const int w0 = threadIdx.x & ~31;
    copy_out_records(srec + w0, recs + i0 + w0, __ballot_sync(0xffffffffu, live), lane);
}

__global__ void view_records_fixup_kernel(SceneArgs a, ViewArgs va, const int* __restrict__ fix_count,
                                          const uint32_t* __restrict__ fix, RecAll* __restrict__ recs) {
    const int n = *fix_count;
    if (blockIdx.x * blockDim.x >= n) return;
    const View V = load_view(va.viewmat, va.fx, va.fy, va.cx, va.cy);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int i = (int)fix[t];
        fix_record(a, V, i, recs + i);
    }
}

int launch_records(const SceneArgs& a, const BatchArgs& ba, int num_views, const int32_t* counts, RecAll* recs,
                   int* fix_count, uint32_t* fix, cudaStream_t stream) {
    if (a.N == 0) return GSTEX_OK;
    cudaError_t e = cudaMemsetAsync(fix_count, 0, sizeof(int), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "batch_records"); return GSTEX_ERR_CUDA; }
    const long long blocks = (long long)ceil_div(a.N, 128) * num_views;
    if (blocks > 0x7fffffffLL) return GSTEX_ERR_UNSUPPORTED;
    records_kernel<<<(unsigned)blocks, 128, 0, stream>>>(a, ba, num_views, counts, recs, fix_count, fix);
    records_fixup_kernel<<<152 * 4, 128, 0, stream>>>(a, ba, fix_count, fix, recs);
    return check_launch("batch_records", 2);
}

// Moments -> parameter gradients (one thread per Gaussian).  Colour gradients
// are written by the tile flushes directly.  With rg.raw_quats set the
// gradients are carried on through the parameter activation (preprocess.cuh)
// to the trainer's raw parameters, from the activated values the projection
// wrote: exp' = scale, sigmoid' = o (1 - o); the chart maps umap = us (cs a1 +
// sn a2), vmap = us (cs a2 - sn a1) give d/d log-scale = vu.u + vv.v,
// d/d theta = vu.v - vv.u and, with us cs = u.a1 and us sn = u.a2, the
// gradients into the axes a1, a2 that join the quaternion's; the
// normalisation adds (I - q q^T) / |raw q|.
__global__ void finalize_kernel(int N, const float* __restrict__ mom, const float4* __restrict__ quats,
                                const float3* __restrict__ umap, const float3* __restrict__ vmap, float* v_opac,
                                float3* v_means, float3* v_scales, float4* v_quats, float2* v_uv0, float3* v_umap,
                                float3* v_vmap, RawGradArgs rg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float M[kMomStride];
    const float4* src = reinterpret_cast<const float4*>(mom + (size_t)i * kMomStride);
#pragma unroll
    for (int q = 0; q < kMomStride / 4; q++) {
        const float4 v = src[q];
        M[4 * q] = v.x; M[4 * q + 1] = v.y; M[4 * q + 2] = v.z; M[4 * q + 3] = v.w;
    }
    // M: 0 v_opac, 1-2 v_scale, 3-4 sum v_l, 5 sum v_t/(n.r), 6-9 S_lk v_lj, 10-11 S_l v_t/(n.r),
    //    12-14 sum vis*v_normal, 15-16 sum v_uv, 17-20 S_l v_uv, 21-23 blur mean gradient
    const float4 q = quats[i];
    const Axes A = quat_axes(q);
    const float3 um = umap[i], vm = vmap[i];
    const float3 vu = M[17] * A.a1 + M[18] * A.a2;  // v_umap
    const float3 vv = M[19] * A.a1 + M[20] * A.a2;  // v_vmap
    const float3 vdiff = M[15] * um + M[16] * vm;
    const float3 vmean = (M[5] * A.a3) - (M[3] * A.a1 + M[4] * A.a2) - vdiff;
    v_means[i] = vmean + make_float3(M[21], M[22], M[23]);
    float3 c0 = M[6] * A.a1 + M[7] * A.a2;
    float3 c1 = M[8] * A.a1 + M[9] * A.a2;
    const float3 c2 = make_float3(M[12], M[13], M[14]) - (M[10] * A.a1 + M[11] * A.a2);
    if (!rg.raw_quats) {
        v_opac[i] = M[0];
        v_scales[i] = make_float3(M[1], M[2], 0.f);
        v_uv0[i] = make_float2(M[15], M[16]);
        v_umap[i] = vu;
        v_vmap[i] = vv;
        v_quats[i] = quat_axes_vjp(q, c0, c1, c2);
        return;
    }
    if (rg.v_raw_opacity) {
        const float o = rg.opacity[i];
        rg.v_raw_opacity[i] = M[0] * o * (1.f - o);
    }
    rg.v_raw_scales[3 * i] = M[1] * rg.scales[3 * i];
    rg.v_raw_scales[3 * i + 1] = M[2] * rg.scales[3 * i + 1];
    rg.v_raw_scales[3 * i + 2] = 0.f;
    const float usc = dot3(um, A.a1), uss = dot3(um, A.a2);
    rg.v_mapping[i] = make_float4(M[15], M[16], dot3(vu, um) + dot3(vv, vm), dot3(vu, vm) - dot3(vv, um));
    c0 = c0 + (usc * vu - uss * vv);
    c1 = c1 + (uss * vu + usc * vv);
    const float4 vq = quat_axes_vjp(q, c0, c1, c2);
    const float4 r = rg.raw_quats[i];
    const float in = 1.f / sqrtf(r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w);
    const float qv = q.x * vq.x + q.y * vq.y + q.z * vq.z + q.w * vq.w;
    rg.v_raw_quats[i] = make_float4((vq.x - q.x * qv) * in, (vq.y - q.y * qv) * in, (vq.z - q.z * qv) * in,
                                    (vq.w - q.w * qv) * in);
}

template <typename K>
static int set_smem(K kernel, size_t smem, const char* what) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) { set_cuda_error(e, what); return GSTEX_ERR_CUDA; }
    return GSTEX_OK;
}

int fill_scene(const gstex_raster_inputs* in, SceneArgs& a, bool need_bins) {
    GSTEX_REQUIRE(in);
    GSTEX_REQUIRE(in->num_points >= 0 && in->img_width > 0 && in->img_height > 0);
    GSTEX_REQUIRE(in->block_width >= 2 && in->block_width <= kMaxBlockWidth);
    GSTEX_REQUIRE(in->channels >= 0);
    if (in->channels > kMaxChannels) return GSTEX_ERR_UNSUPPORTED;
    if (in->texture_dtype == 1 && in->channels != 3) return GSTEX_ERR_UNSUPPORTED;
    GSTEX_REQUIRE(in->texture_dtype == 0 || in->texture_dtype == 1);
    GSTEX_REQUIRE(in->viewmat && in->background);
    if (need_bins) GSTEX_REQUIRE(in->tile_bins);
    // prebuilt records are copied as 16-byte vectors
    GSTEX_REQUIRE(((uintptr_t)in->records & 15) == 0);
    if (in->num_points > 0)
        GSTEX_REQUIRE(in->texture_dims && in->colors && in->opacities && in->means && in->scales && in->quats &&
                      in->uv0 && in->umap && in->vmap);
    if (in->channels > 0 && in->num_points > 0) GSTEX_REQUIRE(in->texture);
    a.N = in->num_points;
    a.C = in->channels;
    a.T = in->num_texels;
    a.dims = (const int3*)in->texture_dims;
    a.gids = in->gaussian_ids_sorted;
    a.means = (const float3*)in->means;
    a.scales = in->scales;
    a.glob = in->glob_scale;
    a.quats = (const float4*)in->quats;
    a.opac = in->opacities;
    a.uv0 = (const float2*)in->uv0;
    a.umap = (const float3*)in->umap;
    a.vmap = (const float3*)in->vmap;
    a.tex = in->texture;
    a.settings = in->settings;
    a.bg = in->background;
    a.batch = 0;
    return GSTEX_OK;
}

// Kernel tables ------------------------------------------------------------
// Pixels per thread: 1 (block bw x bw) or 2 (block bw x bw/2, even bw only).
int ppt_of(int bw, int requested) { return (requested == 2 && bw % 2 == 0) ? 2 : 1; }

// Lanes per splat walk actually used: groups below 32 need block widths that
// are multiples of 8 (full warps), one pixel per thread and 0 or 3 channels.
int gs_of(int bw, int ppt, int C, int requested) {
    if ((bw & 7) != 0 || ppt != 1 || (C != 0 && C != 3)) return 32;
    return (requested == 16 || requested == 8 || requested == 4) ? requested : 32;
}
// Backward kernel variant of (channels, texel type, pixels per thread, lanes
// per splat walk gs from gs_of): 1 or 2 pixels per thread with gs = 32;
// gs < 32 with one pixel per thread and 0 or 3 channels.
template <template <int, int, int, int> class Sel>
static typename Sel<0, 0, 1, 32>::type pick(int C, int texmode, int ppt, int gs) {
    if (gs == 16) {
        if (C == 0) return Sel<0, 0, 1, 16>::get();
        return texmode == 1 ? Sel<1, 3, 1, 16>::get() : Sel<0, 3, 1, 16>::get();
    }
    if (gs == 8) {
        if (C == 0) return Sel<0, 0, 1, 8>::get();
        return texmode == 1 ? Sel<1, 3, 1, 8>::get() : Sel<0, 3, 1, 8>::get();
    }
    if (gs == 4) {
        if (C == 0) return Sel<0, 0, 1, 4>::get();
        return texmode == 1 ? Sel<1, 3, 1, 4>::get() : Sel<0, 3, 1, 4>::get();
    }
    if (ppt == 2) {
        if (C == 0) return Sel<0, 0, 2, 32>::get();
        if (C == 3) return texmode == 1 ? Sel<1, 3, 2, 32>::get() : Sel<0, 3, 2, 32>::get();
        return Sel<0, -1, 2, 32>::get();
    }
    if (C == 0) return Sel<0, 0, 1, 32>::get();
    if (C == 3) return texmode == 1 ? Sel<1, 3, 1, 32>::get() : Sel<0, 3, 1, 32>::get();
    return Sel<0, -1, 1, 32>::get();
}
// Forward kernel (pixels per thread only): the alpha-visualisation variants
// (settings bit 16) come with 1 pixel per thread and the generic fp32 or the
// bf16 texel path.
template <template <int, int, int> class Sel>
static typename Sel<0, 0, 1>::type pick_fwd(int C, int texmode, int& ppt, int settings) {
    if (settings & (1 << 16)) {
        ppt = 1;
        return texmode == 1 ? Sel<3, 3, 1>::get() : Sel<2, -1, 1>::get();
    }
    if (ppt == 2) {
        if (C == 0) return Sel<0, 0, 2>::get();
        if (C == 3) return texmode == 1 ? Sel<1, 3, 2>::get() : Sel<0, 3, 2>::get();
        return Sel<0, -1, 2>::get();
    }
    if (C == 0) return Sel<0, 0, 1>::get();
    if (C == 3) return texmode == 1 ? Sel<1, 3, 1>::get() : Sel<0, 3, 1>::get();
    return Sel<0, -1, 1>::get();
}
template <int M, int C, int P> struct FwdView { typedef void (*type)(SceneArgs, ViewArgs, FwdOut); static type get() { return fwd_view_kernel<M, C, P>; } };
template <int M, int C, int P, int G> struct BwdView { typedef void (*type)(SceneArgs, ViewArgs, BwdArgs); static type get() { return bwd_view_kernel<M, C, P, G>; } };
template <int M, int C, int P> struct FwdBatch { typedef void (*type)(SceneArgs, BatchArgs, FwdOut); static type get() { return fwd_batch_kernel<M, C, P>; } };
template <int M, int C, int P, int G> struct BwdBatch { typedef void (*type)(SceneArgs, BatchArgs, BwdArgs); static type get() { return bwd_batch_kernel<M, C, P, G>; } };

static dim3 block_of(int bw, int ppt) { return dim3(bw, bw / ppt); }
static int threads_of(int bw, int ppt) { return bw * (bw / ppt); }
// records, then (backward) the moment slots, then one candidate list per warp
// Shared-memory slots of a launch: `batch` Gaussians per round when set
// below the threads of the CTA, else one per thread.
static int slots_of(int bw, int ppt, int batch) {
    const int n = threads_of(bw, ppt);
    return (batch > 0 && batch < n) ? batch : n;
}
static size_t list_bytes(int bw, int ppt, int gs, int batch) {
    const int n = threads_of(bw, ppt);
    return ((size_t)ceil_div(n, 32) + (gs < 32 ? (size_t)ceil_div(n, gs) : 0)) * slots_of(bw, ppt, batch);
}
size_t fwd_smem(int bw, int ppt, int batch) { return (size_t)kRecBytes * slots_of(bw, ppt, batch); }
size_t bwd_smem(int bw, int ppt, int gs, int batch) {
    // ... then one "touched" flag per slot
    return ((size_t)kRecBytes + kEdgeBytes + kMomSlot * sizeof(float) + 1) * slots_of(bw, ppt, batch) +
           list_bytes(bw, ppt, gs, batch);
}

int launch_finalize(const SceneArgs& a, const float* moments, float* v_opac, float* v_means, float* v_scales,
                    float* v_quats, float* v_uv0, float* v_umap, float* v_vmap, cudaStream_t stream,
                    const RawGradArgs& rg) {
    if (a.N == 0) return GSTEX_OK;
    finalize_kernel<<<ceil_div(a.N, 256), 256, 0, stream>>>(a.N, moments, a.quats, a.umap, a.vmap, v_opac,
                                                           (float3*)v_means, (float3*)v_scales, (float4*)v_quats,
                                                           (float2*)v_uv0, (float3*)v_umap, (float3*)v_vmap, rg);
    return check_launch("finalize");
}

// The batched forward kernel: compiled for the default settings where they
// apply (one pixel per thread, bf16 RGB texels), else pick_fwd's.
// (Kernels of 8x8 tiles compiled for 12, 14, 18 or 20 CTAs per SM, i.e. 80,
// 72, 56 or 48 registers instead of 64 at 16, all measured slower.)
static FwdBatch<0, 0, 1>::type pick_fwd_batch(int C, int texmode, int& ppt, int settings) {
    if (ppt == 1 && C == 3 && texmode == 1 && (settings & kFixedFwdMask) == 0) return fwd_batch_kernel<1, 3, 1, 1>;
    return pick_fwd<FwdBatch>(C, texmode, ppt, settings);
}

int launch_fwd_batch(const SceneArgs& a, const BatchArgs& ba, const FwdOut& o, int bw, int texmode, int ppt, int grid,
                     cudaStream_t stream) {
    ppt = ppt_of(bw, ppt);
    auto k = pick_fwd_batch(a.C, texmode, ppt, a.settings);
    const size_t smem = fwd_smem(bw, ppt, a.batch);
    int rc = set_smem(k, smem, "batch forward");
    if (rc) return rc;
    k<<<grid, block_of(bw, ppt), smem, stream>>>(a, ba, o);
    return check_launch("batch forward");
}

// The backward kernel of a launch: the 64-thread variant compiled for
// `ctas` resident CTAs per SM where one exists (8x8 tiles, one pixel per
// thread, bf16 texels with 3 channels, ctas 10; 8-lane groups, or 32 with the
// default settings), else the general kernel.
static BwdBatch<0, 0, 1, 32>::type pick_bwd_batch(int bw, int C, int texmode, int ppt, int gs, int ctas,
                                                   int settings) {
    if (threads_of(bw, ppt) == 64 && ppt == 1 && C == 3 && texmode == 1 && ctas == 10) {
        const bool fixed = (settings & kFixedBwdMask) == kFixedBwdSettings;
        if (gs == 8) return fixed ? bwd_batch64_kernel<1, 3, 10, 1, 8> : bwd_batch64_kernel<1, 3, 10, 0, 8>;
        if (gs == 32 && fixed) return bwd_batch64_kernel<1, 3, 10, 1, 32>;
    }
    return pick<BwdBatch>(C, texmode, ppt, gs);
}

// Dynamic shared memory of a backward kernel; the 64-thread variants also ask
// for the largest shared-memory carveout, which 10 CTAs of 22 KB need.
template <typename K>
static int set_bwd_smem(K k, size_t smem, const char* what) {
    int rc = set_smem(k, smem, what);
    if (rc) return rc;
    if (k == (K)bwd_batch64_kernel<1, 3, 10, 0, 8> || k == (K)bwd_batch64_kernel<1, 3, 10, 1, 8> ||
        k == (K)bwd_batch64_kernel<1, 3, 10, 1, 32>) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) { set_cuda_error(e, what); return GSTEX_ERR_CUDA; }
    }
    return GSTEX_OK;
}

int launch_bwd_batch(const SceneArgs& a, const BatchArgs& ba, const BwdArgs& g, int bw, int texmode, int ppt, int gs,
                     int ctas, int grid, cudaStream_t stream) {
    ppt = ppt_of(bw, ppt);
    gs = gs_of(bw, ppt, a.C, gs);
    auto k = pick_bwd_batch(bw, a.C, texmode, ppt, gs, ctas, a.settings);
    const size_t smem = bwd_smem(bw, ppt, gs, a.batch);
    int rc = set_bwd_smem(k, smem, "batch backward");
    if (rc) return rc;
    k<<<grid, block_of(bw, ppt), smem, stream>>>(a, ba, g);
    return check_launch("batch backward");
}

int resident_ctas(int bw, bool backward, int texmode, int C, int ppt, int gs, int ctas, int batch, int settings) {
    int n = 0;
    cudaError_t e;
    ppt = ppt_of(bw, ppt);
    gs = gs_of(bw, ppt, C, gs);
    if (backward) {
        auto k = pick_bwd_batch(bw, C, texmode, ppt, gs, ctas, settings);
        const size_t smem = bwd_smem(bw, ppt, gs, batch);
        if (set_bwd_smem(k, smem, "occupancy")) return 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, threads_of(bw, ppt), smem);
    } else {
        auto k = pick_fwd_batch(C, texmode, ppt, settings);
        const size_t smem = fwd_smem(bw, ppt, batch);
        if (set_smem(k, smem, "occupancy")) return 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, threads_of(bw, ppt), smem);
    }
    if (e != cudaSuccess) return 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return n * sms;
}

}  // namespace gstex

using namespace gstex;

static ViewArgs view_args(const gstex_raster_inputs* in) {
    ViewArgs va;
    va.viewmat = in->viewmat;
    va.fx = in->fx; va.fy = in->fy; va.cx = in->cx; va.cy = in->cy;
    va.W = in->img_width; va.H = in->img_height;
    va.tiles_x = ceil_div(va.W, in->block_width);
    va.bins = (const int2*)in->tile_bins;
    va.colors = (const float3*)in->colors;
    va.vcolors = nullptr;
    va.recs = (const RecAll*)in->records;
    return va;
}

// records [N], then the count and list of deferred near-edge-on records
static size_t view_records_fix_offset(int n) { return (size_t)n * sizeof(RecAll); }

extern "C" size_t gstex_view_records_bytes(int num_points) {
    const int n = num_points > 0 ? num_points : 0;
    return view_records_fix_offset(n) + 16 + (size_t)n * sizeof(uint32_t);
}

extern "C" int gstex_view_records(const gstex_raster_inputs* in, void* records, size_t records_bytes,
                                  gstex_stream_t s) {
    SceneArgs a;
    int rc = fill_scene(in, a, false);
    if (rc) return rc;
    GSTEX_REQUIRE(records && ((uintptr_t)records & 15) == 0);
    if (records_bytes < gstex_view_records_bytes(a.N)) return GSTEX_ERR_CAPACITY;
    if (a.N == 0) return GSTEX_OK;
    ViewArgs va = view_args(in);
    RecAll* recs = (RecAll*)records;
    int* fix_count = (int*)((char*)records + view_records_fix_offset(a.N));
    uint32_t* fix = (uint32_t*)((char*)records + view_records_fix_offset(a.N) + 16);
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(fix_count, 0, sizeof(int), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "view_records"); return GSTEX_ERR_CUDA; }
    view_records_kernel<<<ceil_div(a.N, 128), 128, 0, stream>>>(a, va, recs, fix_count, fix);
    view_records_fixup_kernel<<<152 * 2, 128, 0, stream>>>(a, va, fix_count, fix, recs);
    return check_launch("view_records", 2);
}

extern "C" int gstex_texture_forward(const gstex_raster_inputs* in, const gstex_forward_outputs* out,
                                     gstex_stream_t s) {
    SceneArgs a;
    int rc = fill_scene(in, a, true);
    if (rc) return rc;
    GSTEX_REQUIRE(out && out->img && out->depth && out->reg && out->normal && out->final_T && out->final_idx &&
                  out->depth_idx && out->reg_s);
    if (a.C > 0) GSTEX_REQUIRE(out->texture);
    FwdOut o{ (float3*)out->img, out->depth, out->reg, out->texture, (float3*)out->normal, out->final_T,
              out->final_idx, out->depth_idx, (float3*)out->reg_s };
    const int bw = in->block_width;
    ViewArgs va = view_args(in);
    cudaStream_t stream = (cudaStream_t)s;
    const dim3 grid(va.tiles_x, ceil_div(va.H, bw));
    int ppt = ppt_of(bw, in->pixels_per_thread);
    auto k = pick_fwd<FwdView>(a.C, in->texture_dtype, ppt, a.settings);
    const size_t smem = fwd_smem(bw, ppt, 0);
    if ((rc = set_smem(k, smem, "texture_forward"))) return rc;
    k<<<grid, block_of(bw, ppt), smem, stream>>>(a, va, o);
    return check_launch("texture_forward");
}

extern "C" int gstex_texture_edit(const gstex_raster_inputs* in, const gstex_edit_io* io, gstex_stream_t s) {
    GSTEX_REQUIRE(in && io);
    GSTEX_REQUIRE(in->num_points >= 0 && in->img_width > 0 && in->img_height > 0);
    GSTEX_REQUIRE(in->block_width >= 2 && in->block_width <= kMaxBlockWidth);
    // the reference writes five channels at a stride of texture_info[2]
    if (in->channels != 5) return GSTEX_ERR_UNSUPPORTED;
    GSTEX_REQUIRE(in->tile_bins && in->viewmat && io->num_texels >= 0);
    GSTEX_REQUIRE(io->updated_img && io->updated_alpha && io->depth_lower && io->depth_upper);
    if (io->num_texels > 0) GSTEX_REQUIRE(io->updated_texture);
    if (in->num_points > 0)
        GSTEX_REQUIRE(in->texture_dims && in->gaussian_ids_sorted && in->opacities && in->means && in->scales &&
                      in->quats && in->uv0 && in->umap && in->vmap);
    cudaStream_t stream = (cudaStream_t)s;
    if (io->num_texels > 0) {
        cudaError_t e = cudaMemsetAsync(io->updated_texture, 0, (size_t)io->num_texels * 5 * sizeof(float), stream);
        if (e != cudaSuccess) { set_cuda_error(e, "texture_edit"); return GSTEX_ERR_CUDA; }
    }
    if (in->num_points == 0) return GSTEX_OK;
    SceneArgs a{};
    a.N = in->num_points;
    a.C = 5;
    a.T = (int)io->num_texels;
    a.dims = (const int3*)in->texture_dims;
    a.gids = in->gaussian_ids_sorted;
    a.means = (const float3*)in->means;
    a.scales = in->scales;
    a.glob = in->glob_scale;
    a.quats = (const float4*)in->quats;
    a.opac = in->opacities;
    a.uv0 = (const float2*)in->uv0;
    a.umap = (const float3*)in->umap;
    a.vmap = (const float3*)in->vmap;
    a.settings = in->settings;
    const int bw = in->block_width;
    ViewArgs va{};
    va.viewmat = in->viewmat;
    va.fx = in->fx; va.fy = in->fy; va.cx = in->cx; va.cy = in->cy;
    va.W = in->img_width; va.H = in->img_height;
    va.tiles_x = ceil_div(va.W, bw);
    va.bins = (const int2*)in->tile_bins;
    EditIO E{ (const float3*)io->updated_img, io->updated_alpha, io->depth_lower, io->depth_upper,
              io->updated_texture };
    const size_t smem = (size_t)kRecBytes * bw * bw;
    int rc = set_smem(edit_view_kernel<1>, smem, "texture_edit");
    if (rc) return rc;
    edit_view_kernel<1><<<dim3(va.tiles_x, ceil_div(va.H, bw)), dim3(bw, bw), smem, stream>>>(a, va, E);
    return check_launch("texture_edit");
}

extern "C" size_t gstex_backward_workspace_bytes(int num_points) {
    return (size_t)(num_points > 0 ? num_points : 1) * kMomStride * sizeof(float);
}

extern "C" int gstex_texture_backward(const gstex_raster_inputs* in, const gstex_backward_io* io, gstex_stream_t s) {
    SceneArgs a;
    int rc = fill_scene(in, a, true);
    if (rc) return rc;
    // alpha-visualisation mode is a forward-only view: its alpha has no adjoint
    if (in->settings & (1 << 16)) return GSTEX_ERR_UNSUPPORTED;
    GSTEX_REQUIRE(io && io->final_T && io->final_idx && io->depth_idx && io->reg_s && io->v_img && io->v_depth &&
                  io->v_reg && io->v_alpha && io->v_normal);
    GSTEX_REQUIRE(io->v_colors && io->v_opacity && io->v_means && io->v_scales && io->v_quats && io->v_uv0 &&
                  io->v_umap && io->v_vmap && io->workspace);
    if (a.C > 0) GSTEX_REQUIRE(io->v_texture && io->v_tex_grad);
    if (io->workspace_bytes < gstex_backward_workspace_bytes(a.N)) return GSTEX_ERR_CAPACITY;
    if (a.N == 0) return GSTEX_OK;
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(io->workspace, 0, gstex_backward_workspace_bytes(a.N), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(io->v_colors, 0, (size_t)a.N * 3 * sizeof(float), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "texture_backward memset"); return GSTEX_ERR_CUDA; }
    BwdArgs g{ io->final_T, io->final_idx, io->depth_idx, (const float3*)io->reg_s, (const float3*)io->v_img,
               io->v_depth, io->v_reg, io->v_alpha, io->v_texture, (const float3*)io->v_normal,
               (float*)io->workspace, io->v_tex_grad };
    const int bw = in->block_width;
    ViewArgs va = view_args(in);
    va.vcolors = io->v_colors;
    const dim3 grid(va.tiles_x, ceil_div(va.H, bw));
    const int ppt = ppt_of(bw, in->pixels_per_thread);
    const int gs = gs_of(bw, ppt, a.C, in->group_lanes);
    auto k = pick<BwdView>(a.C, in->texture_dtype, ppt, gs);
    const size_t smem = bwd_smem(bw, ppt, gs, 0);
    if ((rc = set_smem(k, smem, "texture_backward"))) return rc;
    k<<<grid, block_of(bw, ppt), smem, stream>>>(a, va, g);
    if ((rc = check_launch("texture_backward"))) return rc;
    return launch_finalize(a, (const float*)io->workspace, io->v_opacity, io->v_means, io->v_scales, io->v_quats,
                           io->v_uv0, io->v_umap, io->v_vmap, stream);
}
