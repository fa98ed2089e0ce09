// Batched multi-view rendering: projection of every (view, Gaussian) pair,
// capacity-bounded intersection emission, device-count sort and tile ranges,
// the demo's image losses, and the SH adjoint over all views.
//
// Nothing here reads a size back to the host, so one forward + backward step
// over all views can be captured in a CUDA graph.  Global tiles of all views
// are numbered view by view (tile_offset); sort keys are
// (global tile << 32 | float bits of the camera depth), so one sort orders
// every view's tiles front to back.
#include <vector>

#include "common.cuh"
#include "preprocess.cuh"
#include "project.cuh"
#include "raster.cuh"

namespace gstex {

// ---------------------------------------------------------------------------
// Projection: AABB, tile count, depth and SH colour of each (view, Gaussian).
// One thread per Gaussian loops over the views so parameters and SH
// coefficients are read once.
// ---------------------------------------------------------------------------
// SH degree DEG is a template parameter so that the coefficient and basis
// arrays stay in registers.  With raw.raw_scales set, each Gaussian is first
// activated from the trainer's raw parameters (preprocess.cuh) and its
// activated parameters are written for the later stages.
template <typename SHT, int DEG>
__global__ void batch_project_kernel(int N, int V, const BatchView* __restrict__ views, const float3* __restrict__ means,
                                     const float* __restrict__ scales, float glob, const float4* __restrict__ quats,
                                     const SHT* __restrict__ sh, int bw, float3* __restrict__ colors,
                                     int32_t* __restrict__ counts, uint32_t* __restrict__ depth_keys,
                                     int32_t* __restrict__ pair_ids, uint2* __restrict__ rects, RawParams raw) {
    constexpr int B = (DEG + 1) * (DEG + 1);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float3 p = means[i];
    float4 q;
    float sx, sy;
    if (raw.raw_scales) {
        activate(raw, i, sx, sy, q);
    } else {
        q = quats[i];
        sx = scales[3 * i];
        sy = scales[3 * i + 1];
    }
    float k[B][3];
#pragma unroll
    for (int b = 0; b < B; b++)
#pragma unroll
        for (int c = 0; c < 3; c++) k[b][c] = (float)sh[((size_t)i * B + b) * 3 + c];
    for (int v = 0; v < V; v++) {
        const BatchView& bv = views[v];
        float m[12];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            m[4 * r + 0] = bv.V.r[3 * r + 0];
            m[4 * r + 1] = bv.V.r[3 * r + 1];
            m[4 * r + 2] = bv.V.r[3 * r + 2];
            m[4 * r + 3] = bv.V.t[r];
        }
        float2 c, e;
        float z;
        aabb_2d(m, bv.V.fx, bv.V.fy, bv.V.cx, bv.V.cy, p, q, sx, sy, glob, c, e, z);
        const size_t j = (size_t)v * N + i;
        const int cnt = tiles_hit(c, e, bv.tiles_x, bv.tiles_y, (float)bw);
        counts[j] = cnt;
        if (depth_keys) {
            // depth-first binning: the pair's sort key (pairs without tiles last)
            // and the tile rectangle its emission walks (empty: fillers only)
            depth_keys[j] = cnt > 0 ? __float_as_uint(z) : 0xffffffffu;
            pair_ids[j] = (int32_t)j;
            uint2 rc = make_uint2(0u, 0u);
            if (cnt > 0 && !((double)e.x <= 1e-4 && (double)e.y <= 1e-4)) {
                int x0, y0, x1, y1;
                tile_rect(c, e, bv.tiles_x, bv.tiles_y, bw, x0, y0, x1, y1);
                rc = make_uint2((uint32_t)x0 | ((uint32_t)x1 << 16), (uint32_t)y0 | ((uint32_t)y1 << 16));
            }
            rects[j] = rc;
        }
        float Y[25];
        sh_basis(DEG, make_float3(p.x - bv.campos[0], p.y - bv.campos[1], p.z - bv.campos[2]), Y);
        float3 col = make_float3(0.f, 0.f, 0.f);
#pragma unroll
        for (int b = 0; b < B; b++) {
            col.x += Y[b] * k[b][0];
            col.y += Y[b] * k[b][1];
            col.z += Y[b] * k[b][2];
        }
        colors[(size_t)v * N + i] = col;
    }
}

// Emission into [cum[j-1], cum[j]) for j = v*N + i, clipped to the capacity.
// Slots a Gaussian does not write (tiny or culled extents) hold the view's
// tile 0 with depth bits 0 and Gaussian 0, the reference's zero-slot value.
__global__ void batch_emit_kernel(int N, int V, const BatchView* __restrict__ views, const float3* __restrict__ means,
                                  const float* __restrict__ scales, float glob, const float4* __restrict__ quats,
                                  int bw, const int32_t* __restrict__ cum, long long capacity,
                                  int64_t* __restrict__ keys, int32_t* __restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float3 p = means[i];
    const float4 q = quats[i];
    const float sx = scales[3 * i], sy = scales[3 * i + 1];
    for (int v = 0; v < V; v++) {
        const BatchView& bv = views[v];
        const size_t j = (size_t)v * N + i;
        long long lo = j == 0 ? 0 : (long long)(uint32_t)cum[j - 1];
        long long hi = (long long)(uint32_t)cum[j];
        if (hi > capacity) hi = capacity;
        if (lo >= hi) continue;
        float m[12];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            m[4 * r + 0] = bv.V.r[3 * r + 0];
            m[4 * r + 1] = bv.V.r[3 * r + 1];
            m[4 * r + 2] = bv.V.r[3 * r + 2];
            m[4 * r + 3] = bv.V.t[r];
        }
        float2 c, e;
        float z;
        aabb_2d(m, bv.V.fx, bv.V.fy, bv.V.cx, bv.V.cy, p, q, sx, sy, glob, c, e, z);
        long long cur = lo;
        if (!((double)e.x <= 1e-4 && (double)e.y <= 1e-4)) {
            int x0, y0, x1, y1;
            tile_rect(c, e, bv.tiles_x, bv.tiles_y, bw, x0, y0, x1, y1);
            const uint64_t dbits = (uint64_t)(int64_t)__float_as_int(z);
            for (int ty = y0; ty < y1 && cur < hi; ++ty)
                for (int tx = x0; tx < x1 && cur < hi; ++tx) {
                    const uint64_t tile = (uint64_t)(bv.tile_offset + ty * bv.tiles_x + tx);
                    keys[cur] = (int64_t)((tile << 32) | dbits);
                    vals[cur] = i;
                    ++cur;
                }
        }
        for (; cur < hi; ++cur) {
            keys[cur] = (int64_t)((uint64_t)bv.tile_offset << 32);
            vals[cur] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// Depth-first binning.  The (view, Gaussian) pairs are sorted by the bits of
// their camera depth (stable: ties keep (view, Gaussian) order), each pair
// emits its tiles in that order, and one stable sort by
// (global tile << 1 | real) orders every tile front to back.  This is the
// order of the reference's sort by (tile << 32 | depth bits) with ties in
// emission order, built from 32-bit keys: 4 passes over the pairs and 3 over
// the intersections instead of 7 over 64-bit intersection keys.  Slots a
// Gaussian does not write (filler bit 0) take the place the reference's zero
// entries take: first in the view's tile 0, with Gaussian 0.
// ---------------------------------------------------------------------------
__global__ void gather_counts_kernel(int n, const int32_t* __restrict__ order, const int32_t* __restrict__ counts,
                                     int32_t* __restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) out[p] = counts[order[p]];
}

// Pair p of the depth order writes [cum[p-1], cum[p]) (clipped to the capacity).
__global__ void batch_emit_sorted_kernel(int VN, int N, const BatchView* __restrict__ views,
                                         const int32_t* __restrict__ order, const int32_t* __restrict__ cum,
                                         const uint2* __restrict__ rects, long long capacity,
                                         uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
    // A warp emits the slots of its 32 pairs, which are contiguous: each lane
    // takes every 32nd slot of the range, finds its pair by a binary search
    // over the pairs' first slots and writes one key, so the stores are
    // coalesced whatever the pairs' tile counts.
    const unsigned lane = threadIdx.x & 31;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const long long last = VN > 0 ? min((long long)(uint32_t)cum[VN - 1], capacity) : 0;
    long long lo = last, hi = last;
    if (p < VN) {
        lo = min(p == 0 ? 0 : (long long)(uint32_t)cum[p - 1], capacity);
        hi = min((long long)(uint32_t)cum[p], capacity);
    }
    uint32_t rx = 0, ry = 0;
    int toff = 0, tiles_x = 1, gi = 0;
    if (lo < hi) {
        const int j = order[p];
        const int v = j / N;
        gi = j - v * N;
        const uint2 rc = rects[j];
        rx = rc.x;
        ry = rc.y;
        toff = views[v].tile_offset;
        tiles_x = views[v].tiles_x;
    }
    const long long wlo = __shfl_sync(0xffffffffu, lo, 0);
    const long long whi = __shfl_sync(0xffffffffu, hi, 31);
    for (long long base = wlo; base < whi; base += 32) {  // warp-uniform trip count
        const long long t = base + lane;
        int q = 0;  // the last lane whose first slot is <= t (its pair owns t)
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const long long l = __shfl_sync(0xffffffffu, lo, q + step);
            if (l <= t) q += step;
        }
        const long long qlo = __shfl_sync(0xffffffffu, lo, q);
        const uint32_t qx = __shfl_sync(0xffffffffu, rx, q), qy = __shfl_sync(0xffffffffu, ry, q);
        const int qoff = __shfl_sync(0xffffffffu, toff, q), qtx = __shfl_sync(0xffffffffu, tiles_x, q);
        const int qgi = __shfl_sync(0xffffffffu, gi, q);
        if (t < whi) {
            const int x0 = (int)(qx & 0xffffu), x1 = (int)(qx >> 16), y0 = (int)(qy & 0xffffu), y1 = (int)(qy >> 16);
            const int w = x1 - x0;
            const long long u = t - qlo;
            if (w > 0 && y1 > y0 && u < (long long)w * (y1 - y0)) {
                const int ty = y0 + (int)(u / w), tx = x0 + (int)(u % w);
                keys[t] = ((uint32_t)(qoff + ty * qtx + tx) << 1) | 1u;
                vals[t] = qgi;
            } else {  // slots beyond the tiles emitted: the reference's zero entries
                keys[t] = (uint32_t)qoff << 1;
                vals[t] = 0;
            }
        }
    }
}

// Queue order of the forward: groups of G x G neighbouring tiles of a view by
// decreasing intersection count of the group (ties in tile order), the tiles
// of a group back to back in tile order.  The heaviest work does not start
// last and leave the end of the persistent launch to a few CTAs, and the
// tiles of a group, which share most of their splats, run close together in
// time (their records are still in L2).  First pass: the key of a tile is its
// group (the global index of the group's first tile) and the group's cost is
// kept; a stable sort by group, then one by decreasing cost, gives the order.
__global__ void tile_group_keys_kernel(int T, const int2* __restrict__ bins, const int32_t* __restrict__ tile_view,
                                       const BatchView* __restrict__ views, int G, uint32_t* __restrict__ group_key,
                                       int32_t* __restrict__ ids, uint32_t* __restrict__ cost_key) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    ids[t] = t;
    if (G <= 1) {
        const int2 b = bins[t];
        group_key[t] = (uint32_t)t;
        cost_key[t] = ~(uint32_t)max(b.y - b.x, 0);
        return;
    }
    const BatchView& bv = views[tile_view[t]];
    const int local = t - bv.tile_offset;
    const int gx = local % bv.tiles_x / G * G, gy = local / bv.tiles_x / G * G;
    group_key[t] = (uint32_t)(bv.tile_offset + gy * bv.tiles_x + gx);
    uint32_t c = 0;
    for (int dy = 0; dy < G && gy + dy < bv.tiles_y; dy++)
        for (int dx = 0; dx < G && gx + dx < bv.tiles_x; dx++) {
            const int2 b = bins[bv.tile_offset + (gy + dy) * bv.tiles_x + gx + dx];
            c += (uint32_t)max(b.y - b.x, 0);
        }
    cost_key[t] = ~c;
}

__global__ void gather_keys_kernel(int T, const int32_t* __restrict__ ids, const uint32_t* __restrict__ key,
                                   uint32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < T) out[i] = key[ids[i]];
}

// ---------------------------------------------------------------------------
// Image losses of the reference demo (example.py:189-209) with their
// gradients, over the concatenated pixels of all views:
//   per view: w_img * MSE(img, tgt) + w_tex * MSE(tex, tgt_tex)
//           + w_reg * mean(reg) + w_normal * mean(nx^2 + ny^2 + (1 - nz)^2)
// ---------------------------------------------------------------------------
__global__ void batch_loss_kernel(long long total, int V, const long long* __restrict__ pix_off, int C,
                                  const float3* __restrict__ img, const float* __restrict__ tex,
                                  const float3* __restrict__ normal, const float* __restrict__ reg,
                                  const float3* __restrict__ tgt_img, const float* __restrict__ tgt_tex, float w_img,
                                  float w_tex, float w_reg, float w_normal, float3* __restrict__ v_img,
                                  float* __restrict__ v_tex, float3* __restrict__ v_normal, float* __restrict__ v_reg,
                                  float* __restrict__ loss) {
    __shared__ float part[32];
    float acc = 0.f;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = V;  // view of pixel p: pix_off[v] <= p < pix_off[v+1]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (pix_off[mid] <= p) lo = mid; else hi = mid;
        }
        const float inv = 1.f / (float)(pix_off[lo + 1] - pix_off[lo]);
        const float3 a = img[p], t = tgt_img[p];
        const float3 d = make_float3(a.x - t.x, a.y - t.y, a.z - t.z);
        acc += w_img * inv / 3.f * (d.x * d.x + d.y * d.y + d.z * d.z);
        const float gi = 2.f * w_img * inv / 3.f;
        v_img[p] = make_float3(gi * d.x, gi * d.y, gi * d.z);
        if (C > 0) {
            const float gt = 2.f * w_tex * inv / (float)C;
            for (int c = 0; c < C; c++) {
                const float dt = tex[p * C + c] - tgt_tex[p * C + c];
                acc += w_tex * inv / (float)C * dt * dt;
                v_tex[p * C + c] = gt * dt;
            }
        }
        acc += w_reg * inv * reg[p];
        v_reg[p] = w_reg * inv;
        const float3 n = normal[p];
        acc += w_normal * inv * (n.x * n.x + n.y * n.y + (1.f - n.z) * (1.f - n.z));
        const float gn = 2.f * w_normal * inv;
        v_normal[p] = make_float3(gn * n.x, gn * n.y, gn * (n.z - 1.f));
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(loss, s);
    }
}

// SH adjoint summed over views: v_coeffs[i,b,c] = sum_v Y_b(dir_v) v_color[v,i,c].
template <int DEG>
__global__ void batch_sh_backward_kernel(int N, int V, const BatchView* __restrict__ views,
                                         const float3* __restrict__ means, const float4* __restrict__ vcol,
                                         float* __restrict__ v_coeffs) {
    constexpr int B = (DEG + 1) * (DEG + 1);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float acc[B][3];
#pragma unroll
    for (int b = 0; b < B; b++) acc[b][0] = acc[b][1] = acc[b][2] = 0.f;
    const float3 p = means[i];
    for (int v = 0; v < V; v++) {
        const float4 g = vcol[(size_t)v * N + i];
        if (g.x == 0.f && g.y == 0.f && g.z == 0.f) continue;
        const BatchView& bv = views[v];
        float Y[25];
        sh_basis(DEG, make_float3(p.x - bv.campos[0], p.y - bv.campos[1], p.z - bv.campos[2]), Y);
#pragma unroll
        for (int b = 0; b < B; b++) {
            acc[b][0] += Y[b] * g.x;
            acc[b][1] += Y[b] * g.y;
            acc[b][2] += Y[b] * g.z;
        }
    }
    float* o = v_coeffs + (size_t)i * B * 3;
#pragma unroll
    for (int b = 0; b < B; b++) {
        o[3 * b + 0] = acc[b][0];
        o[3 * b + 1] = acc[b][1];
        o[3 * b + 2] = acc[b][2];
    }
}

__global__ void clamp_count_kernel(const int64_t* __restrict__ total, long long capacity, int64_t* __restrict__ n,
                                   int* __restrict__ overflow) {
    const long long t = *total;
    *n = t < capacity ? t : capacity;
    if (t > capacity) atomicOr(overflow, 1);
}

}  // namespace gstex

using namespace gstex;

extern "C" size_t gstex_batch_views_bytes(int num_views) { return sizeof(BatchView) * (size_t)(num_views > 0 ? num_views : 1); }

extern "C" int gstex_batch_layout(int num_views, const gstex_view_desc* views, int block_width, int* total_tiles,
                                  long long* total_pixels) {
    GSTEX_REQUIRE(num_views > 0 && views && block_width >= 2 && block_width <= kMaxBlockWidth && total_tiles &&
                  total_pixels);
    long long tiles = 0, pix = 0;
    for (int v = 0; v < num_views; v++) {
        GSTEX_REQUIRE(views[v].width > 0 && views[v].height > 0);
        tiles += (long long)ceil_div(views[v].width, block_width) * ceil_div(views[v].height, block_width);
        pix += (long long)views[v].width * views[v].height;
    }
    if (tiles >= (1ll << 31) - 1) return GSTEX_ERR_UNSUPPORTED;
    *total_tiles = (int)tiles;
    *total_pixels = pix;
    return GSTEX_OK;
}

extern "C" int gstex_batch_prepare(int num_views, const gstex_view_desc* views, int block_width, void* views_dev,
                                   int32_t* tile_view_dev, long long* pix_offsets_dev, gstex_stream_t s) {
    int total_tiles = 0;
    long long total_pix = 0;
    int rc = gstex_batch_layout(num_views, views, block_width, &total_tiles, &total_pix);
    if (rc) return rc;
    GSTEX_REQUIRE(views_dev && tile_view_dev && pix_offsets_dev);
    std::vector<BatchView> bv(num_views);
    std::vector<int32_t> tv(total_tiles);
    std::vector<long long> po(num_views + 1);
    int toff = 0;
    long long poff = 0;
    for (int v = 0; v < num_views; v++) {
        const gstex_view_desc& d = views[v];
        BatchView& b = bv[v];
        for (int r = 0; r < 3; r++) {
            for (int c = 0; c < 3; c++) b.V.r[3 * r + c] = d.viewmat[4 * r + c];
            b.V.t[r] = d.viewmat[4 * r + 3];
        }
        b.V.fx = d.fx; b.V.fy = d.fy; b.V.cx = d.cx; b.V.cy = d.cy;
        b.W = d.width; b.H = d.height;
        b.tiles_x = ceil_div(d.width, block_width);
        b.tiles_y = ceil_div(d.height, block_width);
        b.tile_offset = toff;
        b.pix_offset = (int)poff;
        // camera centre = -R^T t
        for (int c = 0; c < 3; c++)
            b.campos[c] = -(b.V.r[c] * b.V.t[0] + b.V.r[3 + c] * b.V.t[1] + b.V.r[6 + c] * b.V.t[2]);
        b.pad = 0;
        for (int k = 0; k < b.tiles_x * b.tiles_y; k++) tv[toff + k] = v;
        po[v] = poff;
        toff += b.tiles_x * b.tiles_y;
        poff += (long long)d.width * d.height;
    }
    po[num_views] = poff;
    if (poff >= (1ll << 31)) return GSTEX_ERR_UNSUPPORTED;
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemcpyAsync(views_dev, bv.data(), sizeof(BatchView) * num_views, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(tile_view_dev, tv.data(), sizeof(int32_t) * total_tiles, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(pix_offsets_dev, po.data(), sizeof(long long) * (num_views + 1), cudaMemcpyHostToDevice,
                            stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);  // host vectors go out of scope
    if (e != cudaSuccess) { set_cuda_error(e, "batch_prepare"); return GSTEX_ERR_CUDA; }
    return GSTEX_OK;
}

template <typename SHT>
static void project_launch(int deg, int N, int V, const BatchView* bv, const float* means, const float* scales,
                           float glob, const float* quats, const SHT* sh, int bw, float* colors, int32_t* counts,
                           uint32_t* dk, int32_t* ids, uint2* rects, const RawParams& raw, cudaStream_t stream) {
    const dim3 grid(ceil_div(N, 128)), block(128);
    const float3* m = (const float3*)means;
    const float4* q = (const float4*)quats;
    float3* c = (float3*)colors;
    switch (deg) {
        case 0: batch_project_kernel<SHT, 0><<<grid, block, 0, stream>>>(N, V, bv, m, scales, glob, q, sh, bw, c, counts, dk, ids, rects, raw); break;
        case 1: batch_project_kernel<SHT, 1><<<grid, block, 0, stream>>>(N, V, bv, m, scales, glob, q, sh, bw, c, counts, dk, ids, rects, raw); break;
        case 2: batch_project_kernel<SHT, 2><<<grid, block, 0, stream>>>(N, V, bv, m, scales, glob, q, sh, bw, c, counts, dk, ids, rects, raw); break;
        case 3: batch_project_kernel<SHT, 3><<<grid, block, 0, stream>>>(N, V, bv, m, scales, glob, q, sh, bw, c, counts, dk, ids, rects, raw); break;
        default: batch_project_kernel<SHT, 4><<<grid, block, 0, stream>>>(N, V, bv, m, scales, glob, q, sh, bw, c, counts, dk, ids, rects, raw); break;
    }
}

static int project_impl(int N, int V, const void* views_dev, const float* means, const float* scales,
                        float glob_scale, const float* quats, const void* sh_coeffs, int sh_dtype, int sh_degree,
                        int block_width, float* colors, int32_t* counts, uint32_t* depth_keys, int32_t* pair_ids,
                        uint2* rects, cudaStream_t stream, const RawParams& raw = RawParams{}) {
    GSTEX_REQUIRE(N >= 0 && V > 0 && views_dev && block_width >= 2 && block_width <= kMaxBlockWidth);
    GSTEX_REQUIRE(sh_degree >= 0 && sh_degree <= 4 && (sh_dtype == 0 || sh_dtype == 1));
    if (N == 0) return GSTEX_OK;
    GSTEX_REQUIRE(means && scales && quats && sh_coeffs && colors && counts);
    const BatchView* bv = (const BatchView*)views_dev;
    if (sh_dtype == 1)
        project_launch<__nv_bfloat16>(sh_degree, N, V, bv, means, scales, glob_scale, quats,
                                      (const __nv_bfloat16*)sh_coeffs, block_width, colors, counts, depth_keys,
                                      pair_ids, rects, raw, stream);
    else
        project_launch<float>(sh_degree, N, V, bv, means, scales, glob_scale, quats, (const float*)sh_coeffs,
                              block_width, colors, counts, depth_keys, pair_ids, rects, raw, stream);
    return check_launch("batch_project");
}

extern "C" int gstex_batch_project(int N, int V, const void* views_dev, const float* means, const float* scales,
                                   float glob_scale, const float* quats, const void* sh_coeffs, int sh_dtype,
                                   int sh_degree, int block_width, float* colors, int32_t* counts, gstex_stream_t s) {
    return project_impl(N, V, views_dev, means, scales, glob_scale, quats, sh_coeffs, sh_dtype, sh_degree,
                        block_width, colors, counts, nullptr, nullptr, nullptr, (cudaStream_t)s);
}

extern "C" int gstex_batch_project_keys(int N, int V, const void* views_dev, const float* means, const float* scales,
                                        float glob_scale, const float* quats, const void* sh_coeffs, int sh_dtype,
                                        int sh_degree, int block_width, float* colors, int32_t* counts,
                                        uint32_t* depth_keys, int32_t* pair_ids, uint32_t* rects, gstex_stream_t s) {
    if ((unsigned long long)N * (unsigned long long)V > 0x7fffffffull) return GSTEX_ERR_UNSUPPORTED;
    if (N > 0) GSTEX_REQUIRE(depth_keys && pair_ids && rects && ((uintptr_t)rects & 7) == 0);
    return project_impl(N, V, views_dev, means, scales, glob_scale, quats, sh_coeffs, sh_dtype, sh_degree,
                        block_width, colors, counts, depth_keys, pair_ids, (uint2*)rects, (cudaStream_t)s);
}

extern "C" int gstex_batch_project_keys_raw(int N, int V, const void* views_dev, const float* means,
                                            const float* raw_scales, const float* raw_quats, const float* mapping,
                                            const float* raw_opacity, float glob_scale, const void* sh_coeffs,
                                            int sh_dtype, int sh_degree, int block_width, float* scales, float* quats,
                                            float* uv0, float* umap, float* vmap, float* opacity, float* colors,
                                            int32_t* counts, uint32_t* depth_keys, int32_t* pair_ids, uint32_t* rects,
                                            gstex_stream_t s) {
    if ((unsigned long long)N * (unsigned long long)V > 0x7fffffffull) return GSTEX_ERR_UNSUPPORTED;
    if (N > 0) {
        GSTEX_REQUIRE(depth_keys && pair_ids && rects && ((uintptr_t)rects & 7) == 0);
        GSTEX_REQUIRE(raw_scales && raw_quats && mapping && scales && quats && uv0 && umap && vmap);
        GSTEX_REQUIRE(((uintptr_t)raw_quats & 15) == 0 && ((uintptr_t)mapping & 15) == 0 &&
                      ((uintptr_t)quats & 15) == 0 && ((uintptr_t)uv0 & 7) == 0);
        if (raw_opacity) GSTEX_REQUIRE(opacity);
    }
    const RawParams raw{ raw_scales, (const float4*)raw_quats, (const float4*)mapping, raw_opacity, 1, scales,
                         (float4*)quats, (float2*)uv0, umap, vmap, opacity };
    // the kernel reads means and writes the activated scales and quats itself
    return project_impl(N, V, views_dev, means, scales, glob_scale, quats, sh_coeffs, sh_dtype, sh_degree,
                        block_width, colors, counts, depth_keys, pair_ids, (uint2*)rects, (cudaStream_t)s, raw);
}

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

extern "C" size_t gstex_batch_tile_order_workspace_bytes(int total_tiles) {
    const int n = total_tiles > 0 ? total_tiles : 1;
    return 6 * align256((size_t)n * 4) + gstex_sort32_workspace_bytes(n);
}

extern "C" int gstex_batch_tile_order(int total_tiles, const int32_t* tile_bins, const int32_t* tile_view,
                                      const void* views_dev, int group, int32_t* order, void* workspace,
                                      size_t workspace_bytes, gstex_stream_t s) {
    GSTEX_REQUIRE(total_tiles >= 0 && group >= 1 && group <= 64);
    if (total_tiles == 0) return GSTEX_OK;
    GSTEX_REQUIRE(tile_bins && order && workspace && ((uintptr_t)workspace & 15) == 0);
    if (group > 1) GSTEX_REQUIRE(tile_view && views_dev);
    if (workspace_bytes < gstex_batch_tile_order_workspace_bytes(total_tiles)) return GSTEX_ERR_CAPACITY;
    const size_t a = align256((size_t)total_tiles * 4);
    unsigned char* w = (unsigned char*)workspace;
    uint32_t* group_key = (uint32_t*)w;
    int32_t* ids = (int32_t*)(w + a);
    uint32_t* cost_key = (uint32_t*)(w + 2 * a);
    uint32_t* keys_sorted = (uint32_t*)(w + 3 * a);
    int32_t* by_group = (int32_t*)(w + 4 * a);
    uint32_t* cost_in = (uint32_t*)(w + 5 * a);
    unsigned char* sort_ws = w + 6 * a;
    const size_t sort_bytes = workspace_bytes - 6 * a;
    cudaStream_t st = (cudaStream_t)s;
    const int blocks = ceil_div(total_tiles, 256);
    tile_group_keys_kernel<<<blocks, 256, 0, st>>>(total_tiles, (const int2*)tile_bins, tile_view,
                                                   (const BatchView*)views_dev, group, group_key, ids, cost_key);
    int rc = check_launch("batch_tile_order");
    if (rc) return rc;
    if (group == 1)  // tiles are already in tile order
        return gstex_sort_pairs32(total_tiles, nullptr, 32, cost_key, ids, keys_sorted, order, sort_ws, sort_bytes, s);
    int bits = 1;
    while (bits < 31 && (1u << bits) < (uint32_t)total_tiles) bits++;
    rc = gstex_sort_pairs32(total_tiles, nullptr, bits, group_key, ids, keys_sorted, by_group, sort_ws, sort_bytes, s);
    if (rc) return rc;
    gather_keys_kernel<<<blocks, 256, 0, st>>>(total_tiles, by_group, cost_key, cost_in);
    rc = check_launch("batch_tile_order");
    if (rc) return rc;
    return gstex_sort_pairs32(total_tiles, nullptr, 32, cost_in, by_group, keys_sorted, order, sort_ws, sort_bytes, s);
}

extern "C" int gstex_batch_gather_counts(int n, const int32_t* order, const int32_t* counts, int32_t* out,
                                         gstex_stream_t s) {
    GSTEX_REQUIRE(n >= 0);
    if (n == 0) return GSTEX_OK;
    GSTEX_REQUIRE(order && counts && out);
    gather_counts_kernel<<<ceil_div(n, 256), 256, 0, (cudaStream_t)s>>>(n, order, counts, out);
    return check_launch("batch_gather_counts");
}

extern "C" int gstex_batch_emit_sorted(int N, int V, const void* views_dev, const int32_t* order, const int32_t* cum,
                                       const uint32_t* rects, const int64_t* total, long long capacity,
                                       uint32_t* keys, int32_t* vals, int64_t* count, int* overflow,
                                       gstex_stream_t s) {
    GSTEX_REQUIRE(N >= 0 && V > 0 && views_dev && capacity >= 0 && total && count && overflow);
    if ((unsigned long long)N * (unsigned long long)V > 0x7fffffffull) return GSTEX_ERR_UNSUPPORTED;
    cudaStream_t stream = (cudaStream_t)s;
    clamp_count_kernel<<<1, 1, 0, stream>>>(total, capacity, count, overflow);
    if (N == 0 || capacity == 0) return check_launch("batch_emit_sorted");
    GSTEX_REQUIRE(order && cum && rects && keys && vals && ((uintptr_t)rects & 7) == 0);
    const int VN = N * V;
    batch_emit_sorted_kernel<<<ceil_div(VN, 256), 256, 0, stream>>>(VN, N, (const BatchView*)views_dev, order, cum,
                                                                     (const uint2*)rects, capacity, keys, vals);
    return check_launch("batch_emit_sorted", 2);
}

extern "C" int gstex_batch_emit(int N, int V, const void* views_dev, const float* means, const float* scales,
                                float glob_scale, const float* quats, int block_width, const int32_t* cum,
                                const int64_t* total, long long capacity, int64_t* keys, int32_t* vals,
                                int64_t* count, int* overflow, gstex_stream_t s) {
    GSTEX_REQUIRE(N >= 0 && V > 0 && views_dev && capacity >= 0 && total && count && overflow);
    cudaStream_t stream = (cudaStream_t)s;
    clamp_count_kernel<<<1, 1, 0, stream>>>(total, capacity, count, overflow);
    if (N == 0 || capacity == 0) return check_launch("batch_emit");
    GSTEX_REQUIRE(means && scales && quats && cum && keys && vals);
    batch_emit_kernel<<<ceil_div(N, 128), 128, 0, stream>>>(N, V, (const BatchView*)views_dev, (const float3*)means,
                                                            scales, glob_scale, (const float4*)quats, block_width, cum,
                                                            capacity, keys, vals);
    return check_launch("batch_emit", 2);
}

static int batch_scene(const gstex_batch_inputs* in, SceneArgs& a, BatchArgs& ba) {
    GSTEX_REQUIRE(in && in->num_points >= 0 && in->num_views > 0 && in->total_tiles > 0);
    GSTEX_REQUIRE(in->block_width >= 2 && in->block_width <= kMaxBlockWidth);
    GSTEX_REQUIRE(in->channels >= 0);
    GSTEX_REQUIRE(in->batch_size >= 0 && in->resident_ctas >= 0);
    if (in->channels > kMaxChannels) return GSTEX_ERR_UNSUPPORTED;
    if (in->texture_dtype == 1 && in->channels != 3) return GSTEX_ERR_UNSUPPORTED;
    GSTEX_REQUIRE(in->views && in->tile_view && in->tile_bins && in->background && in->queue);
    if (in->num_points > 0)
        GSTEX_REQUIRE(in->gaussian_ids_sorted && in->colors && in->texture_dims && in->opacities && in->means &&
                      in->scales && in->quats && in->uv0 && in->umap && in->vmap);
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
    a.batch = in->batch_size;
    a.bg = in->background;
    ba.num_points = in->num_points;
    ba.total_tiles = in->total_tiles;
    ba.views = (const BatchView*)in->views;
    ba.tile_view = in->tile_view;
    ba.order = in->tile_order;
    ba.bins = (const int2*)in->tile_bins;
    ba.colors = (const float3*)in->colors;
    ba.vcolors = nullptr;
    ba.queue = in->queue;
    ba.recs = (const RecAll*)in->records;
    return GSTEX_OK;
}

extern "C" size_t gstex_batch_records_bytes(int num_points, int num_views) {
    return (size_t)(num_points > 0 ? num_points : 0) * (num_views > 0 ? num_views : 0) * sizeof(RecAll);
}

extern "C" size_t gstex_batch_records_workspace_bytes(int num_points, int num_views) {
    return 16 + (size_t)(num_points > 0 ? num_points : 0) * (num_views > 0 ? num_views : 0) * sizeof(uint32_t);
}

extern "C" int gstex_batch_records(const gstex_batch_inputs* in, const int32_t* counts, void* records,
                                   void* workspace, size_t workspace_bytes, gstex_stream_t s) {
    SceneArgs a;
    BatchArgs ba;
    int rc = batch_scene(in, a, ba);
    if (rc) return rc;
    if (a.N == 0) return GSTEX_OK;
    GSTEX_REQUIRE(records && ((uintptr_t)records & 15) == 0 && workspace && ((uintptr_t)workspace & 15) == 0);
    if ((unsigned long long)a.N * (unsigned long long)in->num_views > 0xffffffffull) return GSTEX_ERR_UNSUPPORTED;
    if (workspace_bytes < gstex_batch_records_workspace_bytes(a.N, in->num_views)) return GSTEX_ERR_CAPACITY;
    if (a.N > 0) GSTEX_REQUIRE(counts);
    unsigned char* ws = (unsigned char*)workspace;
    return launch_records(a, ba, in->num_views, counts, (RecAll*)records, (int*)ws, (uint32_t*)(ws + 16),
                          (cudaStream_t)s);
}

static int grid_of(const gstex_batch_inputs* in, bool backward) {
    if (in->grid > 0) return in->grid;
    int g = resident_ctas(in->block_width, backward, in->texture_dtype, in->channels, in->pixels_per_thread,
                          in->group_lanes, backward ? in->resident_ctas : 0, in->batch_size, in->settings);
    return g > 0 ? g : 152;
}

extern "C" int gstex_batch_forward(const gstex_batch_inputs* in, const gstex_forward_outputs* out, gstex_stream_t s) {
    SceneArgs a;
    BatchArgs ba;
    int rc = batch_scene(in, a, ba);
    if (rc) return rc;
    GSTEX_REQUIRE(out && out->img && out->depth && out->reg && out->normal && out->final_T && out->final_idx &&
                  out->depth_idx && out->reg_s);
    if (a.C > 0) GSTEX_REQUIRE(out->texture);
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(in->queue, 0, sizeof(int), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "batch_forward"); return GSTEX_ERR_CUDA; }
    FwdOut o{ (float3*)out->img, out->depth, out->reg, out->texture, (float3*)out->normal, out->final_T,
              out->final_idx, out->depth_idx, (float3*)out->reg_s };
    return launch_fwd_batch(a, ba, o, in->block_width, in->texture_dtype, in->pixels_per_thread, grid_of(in, false),
                            stream);
}

extern "C" size_t gstex_batch_backward_workspace_bytes(int num_points) {
    return (size_t)(num_points > 0 ? num_points : 1) * kMomStride * sizeof(float);
}

static int batch_backward_impl(const gstex_batch_inputs* in, const gstex_backward_io* io, const gstex_raw_grads* raw,
                               gstex_stream_t s) {
    SceneArgs a;
    BatchArgs ba;
    int rc = batch_scene(in, a, ba);
    if (rc) return rc;
    if (in->settings & (1 << 16)) return GSTEX_ERR_UNSUPPORTED;  // alpha-visualisation mode: forward only
    GSTEX_REQUIRE(io);
    if (a.N == 0) return GSTEX_OK;  // no Gaussian, no gradient
    GSTEX_REQUIRE(io->final_T && io->final_idx && io->depth_idx && io->reg_s && io->workspace);
    GSTEX_REQUIRE(io->v_colors && io->v_means);
    RawGradArgs rg{};
    if (raw) {
        GSTEX_REQUIRE(raw->raw_quats && raw->v_raw_scales && raw->v_raw_quats && raw->v_mapping);
        GSTEX_REQUIRE(((uintptr_t)raw->raw_quats & 15) == 0 && ((uintptr_t)raw->v_raw_quats & 15) == 0 &&
                      ((uintptr_t)raw->v_mapping & 15) == 0);
        rg = RawGradArgs{ (const float4*)raw->raw_quats, in->scales, in->opacities, raw->v_raw_scales,
                          (float4*)raw->v_raw_quats, (float4*)raw->v_mapping, raw->v_raw_opacity };
    } else {
        GSTEX_REQUIRE(io->v_opacity && io->v_scales && io->v_quats && io->v_uv0 && io->v_umap && io->v_vmap);
    }
    if (a.C > 0) GSTEX_REQUIRE(io->v_tex_grad);
    if (io->workspace_bytes < gstex_batch_backward_workspace_bytes(a.N)) return GSTEX_ERR_CAPACITY;
    if (a.N == 0) return GSTEX_OK;
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(in->queue, 0, sizeof(int), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(io->workspace, 0, gstex_batch_backward_workspace_bytes(a.N), stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(io->v_colors, 0, (size_t)in->num_views * a.N * 4 * sizeof(float), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "batch_backward"); return GSTEX_ERR_CUDA; }
    ba.vcolors = io->v_colors;
    BwdArgs g{ io->final_T, io->final_idx, io->depth_idx, (const float3*)io->reg_s, (const float3*)io->v_img,
               io->v_depth, io->v_reg, io->v_alpha, io->v_texture, (const float3*)io->v_normal,
               (float*)io->workspace, io->v_tex_grad };
    if ((rc = launch_bwd_batch(a, ba, g, in->block_width, in->texture_dtype, in->pixels_per_thread,
                               in->group_lanes, in->resident_ctas, grid_of(in, true), stream)))
        return rc;
    return launch_finalize(a, (const float*)io->workspace, io->v_opacity, io->v_means, io->v_scales, io->v_quats,
                           io->v_uv0, io->v_umap, io->v_vmap, stream, rg);
}

extern "C" int gstex_batch_backward(const gstex_batch_inputs* in, const gstex_backward_io* io, gstex_stream_t s) {
    return batch_backward_impl(in, io, nullptr, s);
}

extern "C" int gstex_batch_backward_raw(const gstex_batch_inputs* in, const gstex_backward_io* io,
                                        const gstex_raw_grads* raw, gstex_stream_t s) {
    GSTEX_REQUIRE(raw);
    return batch_backward_impl(in, io, raw, s);
}

extern "C" int gstex_batch_sh_backward(int N, int V, const void* views_dev, const float* means, int sh_degree,
                                       const float* v_colors, float* v_coeffs, gstex_stream_t s) {
    GSTEX_REQUIRE(N >= 0 && V > 0 && views_dev && sh_degree >= 0 && sh_degree <= 4);
    if (N == 0) return GSTEX_OK;
    GSTEX_REQUIRE(means && v_colors && v_coeffs);
    const dim3 grid(ceil_div(N, 128)), block(128);
    const BatchView* bv = (const BatchView*)views_dev;
    const float3* m = (const float3*)means;
    const float4* vc = (const float4*)v_colors;
    cudaStream_t stream = (cudaStream_t)s;
    switch (sh_degree) {
        case 0: batch_sh_backward_kernel<0><<<grid, block, 0, stream>>>(N, V, bv, m, vc, v_coeffs); break;
        case 1: batch_sh_backward_kernel<1><<<grid, block, 0, stream>>>(N, V, bv, m, vc, v_coeffs); break;
        case 2: batch_sh_backward_kernel<2><<<grid, block, 0, stream>>>(N, V, bv, m, vc, v_coeffs); break;
        case 3: batch_sh_backward_kernel<3><<<grid, block, 0, stream>>>(N, V, bv, m, vc, v_coeffs); break;
        default: batch_sh_backward_kernel<4><<<grid, block, 0, stream>>>(N, V, bv, m, vc, v_coeffs); break;
    }
    return check_launch("batch_sh_backward");
}

extern "C" int gstex_batch_image_loss(long long total_pixels, int V, const long long* pix_offsets, int channels,
                                      const float* img, const float* tex, const float* normal, const float* reg,
                                      const float* tgt_img, const float* tgt_tex, float w_img, float w_tex,
                                      float w_reg, float w_normal, float* v_img, float* v_tex, float* v_normal,
                                      float* v_reg, float* loss, gstex_stream_t s) {
    GSTEX_REQUIRE(total_pixels >= 0 && V > 0 && pix_offsets && channels >= 0 && loss);
    GSTEX_REQUIRE(img && normal && reg && tgt_img && v_img && v_normal && v_reg);
    if (channels > 0) GSTEX_REQUIRE(tex && tgt_tex && v_tex);
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(float), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "batch_image_loss"); return GSTEX_ERR_CUDA; }
    if (total_pixels == 0) return GSTEX_OK;
    const int blocks = (int)std::min<long long>(ceil_div((int)std::min<long long>(total_pixels, 1ll << 30), 256), 152 * 16);
    batch_loss_kernel<<<blocks, 256, 0, stream>>>(total_pixels, V, pix_offsets, channels, (const float3*)img, tex,
                                                  (const float3*)normal, reg, (const float3*)tgt_img, tgt_tex, w_img,
                                                  w_tex, w_reg, w_normal, (float3*)v_img, v_tex, (float3*)v_normal,
                                                  v_reg, loss);
    return check_launch("batch_image_loss");
}
