// Tile binning: intersection emission, stable LSD radix sort, tile ranges.
#include "common.cuh"

namespace gstex {

// ---------------------------------------------------------------------------
// Emission (reference csrc/forward.cu:13-71, helpers.cuh:37-111)
// ---------------------------------------------------------------------------
__global__ void emit_kernel(int n, int num_isect, const float2* __restrict__ centers,
                            const float2* __restrict__ extents, const float* __restrict__ depths,
                            const int32_t* __restrict__ cum, int tiles_x, int tiles_y, int bw, int wrapped,
                            int64_t* __restrict__ keys, int32_t* __restrict__ gids) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int lo = i == 0 ? 0 : cum[i - 1];
    const int hi = min(cum[i], num_isect);
    int cur = lo;
    const float2 e = extents[i];
    if (!((double)e.x <= 1e-4 && (double)e.y <= 1e-4)) {
        const float2 c = centers[i];
        const float fbw = (float)bw;
        const float tcx = __fdiv_rn(c.x, fbw), tcy = __fdiv_rn(c.y, fbw);
        const float tex = __fdiv_rn(e.x, fbw), tey = __fdiv_rn(e.y, fbw);
        int x0 = __float2int_rz(__fsub_rn(tcx, tex));
        int x1 = __float2int_rz(__fadd_rn(__fadd_rn(tcx, tex), 1.0f));
        int y0 = __float2int_rz(__fsub_rn(tcy, tey));
        int y1 = __float2int_rz(__fadd_rn(__fadd_rn(tcy, tey), 1.0f));
        if (wrapped) {
            if (x0 <= 0) x0 -= 1;
            if (y0 <= 0) y0 -= 1;
        } else {
            x0 = min(max(0, x0), tiles_x);
            x1 = min(max(0, x1), tiles_x);
            y0 = min(max(0, y0), tiles_y);
            y1 = min(max(0, y1), tiles_y);
        }
        const int64_t depth_id = (int64_t)__float_as_int(depths[i]);  // sign-extended (forward.cu:47)
        for (int ty = y0; ty < y1 && cur < hi; ++ty) {
            for (int tx = x0; tx < x1 && cur < hi; ++tx) {
                int ti = ty, tj = tx;
                if (wrapped) {
                    ti %= tiles_y; if (ti < 0) ti += tiles_y;
                    tj %= tiles_x; if (tj < 0) tj += tiles_x;
                }
                const int64_t tile = (int64_t)(ti * tiles_x + tj);
                keys[cur] = (int64_t)(((uint64_t)tile << 32) | (uint64_t)depth_id);
                gids[cur] = i;
                ++cur;
            }
        }
    }
    // slots this Gaussian did not write keep the zero value of the reference's
    // torch::zeros buffers (bindings.cu:99-102)
    for (; cur < hi; ++cur) {
        keys[cur] = 0;
        gids[cur] = 0;
    }
}

// ---------------------------------------------------------------------------
// Tile ranges (reference csrc/forward.cu:76-98); tiles outside [0, num_tiles)
// are ignored.
// ---------------------------------------------------------------------------
constexpr int kEdgeItems = 4;

// Tile of a sorted key: bits [shift, ...) of a 64-bit (tile | depth) key or of
// a 32-bit (tile | filler bit) key.
template <typename K>
__global__ void bin_edges_kernel(int n, const int64_t* __restrict__ n_dev, const K* __restrict__ sorted, int shift,
                                 int num_tiles, int2* __restrict__ bins) {
    if (n_dev) {
        const int64_t m = *n_dev;
        n = (int)(m < (int64_t)n ? (m > 0 ? m : 0) : n);
    }
    // kEdgeItems consecutive items per thread, their keys loaded up front
    const long long i0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kEdgeItems;
    if (i0 >= n) return;
    int tile[kEdgeItems + 1];
    tile[0] = i0 > 0 ? (int)(sorted[i0 - 1] >> shift) : -1;
#pragma unroll
    for (int q = 0; q < kEdgeItems; q++) tile[q + 1] = i0 + q < n ? (int)(sorted[i0 + q] >> shift) : -1;
#pragma unroll
    for (int q = 0; q < kEdgeItems; q++) {
        const int i = (int)i0 + q;
        if (i >= n) break;
        const int prev = tile[q], cur = tile[q + 1];
        const bool ok = cur >= 0 && cur < num_tiles;
        if (i == 0 && ok) bins[cur].x = 0;
        if (i == n - 1 && ok) bins[cur].y = n;
        if (i > 0 && prev != cur) {
            if (prev >= 0 && prev < num_tiles) bins[prev].y = i;
            if (ok) bins[cur].x = i;
        }
    }
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (u64 key, u32 value), 8-bit digits.
//
// Each pass: per-block digit histograms -> one exclusive scan in
// (digit, block) order -> stable scatter.  Blocks own contiguous chunks; a
// block ranks each 2048-item tile with warp match + per-warp counters, so the
// order of equal digits is the input order.
// ---------------------------------------------------------------------------
constexpr int kRadix = 256;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortMaxBlocks = 1216;

struct SortPlan {
    int blocks, chunk;
};

static SortPlan sort_plan(int n) {
    SortPlan p;
    int tiles = ceil_div(n, kSortTile);
    int tiles_per_block = ceil_div(tiles, kSortMaxBlocks);
    p.chunk = tiles_per_block * kSortTile;
    p.blocks = ceil_div(n, p.chunk);
    if (p.blocks < 1) p.blocks = 1;
    return p;
}

// With n_dev set, the item count is read on the device (clamped to n) and the
// chunk of each block is derived from it, so the launch shape does not depend
// on the count.
__device__ __forceinline__ void resolve_count(const int64_t* n_dev, int& n, int& chunk) {
    if (n_dev) {
        const int64_t m = *n_dev;
        n = (int)(m < (int64_t)n ? (m > 0 ? m : 0) : n);
        chunk = ceil_div(ceil_div(n, kSortTile), (int)gridDim.x) * kSortTile;
        if (chunk < kSortTile) chunk = kSortTile;
    }
}

// Per-block digit counts: each warp loads its kSortItems keys per thread of a
// 2048-item tile up front (so the loads overlap) and counts them in its own
// shared-memory histogram with plain atomics; the warps' histograms are summed
// at the end.
template <typename K>
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const K* __restrict__ keys, int n, int chunk,
                                                                  const int64_t* __restrict__ n_dev, int shift,
                                                                  uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[kSortWarps][kRadix];
    for (int i = threadIdx.x; i < kSortWarps * kRadix; i += blockDim.x) (&h[0][0])[i] = 0;
    resolve_count(n_dev, n, chunk);
    __syncthreads();
    const int start = blockIdx.x * chunk;
    const int end = min(start + chunk, n);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    uint32_t* hw = h[warp];
    for (int tbase = start; tbase < end; tbase += kSortTile) {
        K key[kSortItems];
#pragma unroll
        for (int k = 0; k < kSortItems; k++) {
            const int i = tbase + warp * (32 * kSortItems) + k * 32 + lane;
            key[k] = i < end ? keys[i] : K(0);
        }
#pragma unroll
        for (int k = 0; k < kSortItems; k++) {
            const int i = tbase + warp * (32 * kSortItems) + k * 32 + lane;
            if (i < end) atomicAdd(&hw[(unsigned)(key[k] >> shift) & (kRadix - 1)], 1u);
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x) {
        uint32_t c = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; w++) c += h[w][d];
        hist[(size_t)d * gridDim.x + blockIdx.x] = c;
    }
}

// Block-wide exclusive scan of one value per thread (blockDim.x == kSortThreads);
// *total receives the sum.  Ends with a barrier.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* wsum, uint32_t* total) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (unsigned)o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < (unsigned)kSortWarps ? wsum[lane] : 0u;
#pragma unroll
        for (int o = 1; o < kSortWarps; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (unsigned)o) t += y;
        }
        if (lane < (unsigned)kSortWarps) wsum[lane] = t;
    }
    __syncthreads();
    const uint32_t before = (warp ? wsum[warp - 1] : 0u) + x - v;
    if (total) *total = wsum[kSortWarps - 1];
    __syncthreads();
    return before;
}

// Exclusive scan of each digit's row of per-block counts, one block per
// digit; the row total goes to totals[digit].
__global__ void __launch_bounds__(kSortThreads) radix_scan_rows_kernel(uint32_t* __restrict__ hist, int blocks,
                                                                       uint32_t* __restrict__ totals) {
    __shared__ uint32_t wsum[kSortWarps];
    uint32_t* row = hist + (size_t)blockIdx.x * blocks;
    uint32_t carry = 0;
    for (int base = 0; base < blocks; base += kSortThreads) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < blocks ? row[i] : 0u;
        uint32_t sum;
        const uint32_t before = block_exclusive_scan(v, wsum, &sum);
        if (i < blocks) row[i] = carry + before;
        carry += sum;
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

// Stable scatter of one block's chunk, 2048 items at a time: items are ranked
// by digit (warp match + per-warp counters, so equal digits keep their input
// order), regrouped by digit in shared memory, and written out as runs of
// consecutive positions.  K: 64- or 32-bit keys.
template <typename K>
__global__ void __launch_bounds__(kSortThreads) radix_scatter_kernel(
    const K* __restrict__ kin, const uint32_t* __restrict__ vin, K* __restrict__ kout,
    uint32_t* __restrict__ vout, int n, int chunk, const int64_t* __restrict__ n_dev, int shift,
    const uint32_t* __restrict__ offsets, const uint32_t* __restrict__ totals) {
    __shared__ uint32_t run_off[kRadix];
    __shared__ uint32_t tile_base[kRadix];
    __shared__ uint32_t wsum[kSortWarps];
    __shared__ uint32_t wcnt[kSortWarps][kRadix];
    __shared__ K skey[kSortTile];
    __shared__ uint32_t sval[kSortTile];
    resolve_count(n_dev, n, chunk);
    const int tid = threadIdx.x, warp = tid >> 5;
    const unsigned lane = tid & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    // digit d starts at (sum of the totals of smaller digits) + (this block's row prefix)
    {
        const uint32_t base = block_exclusive_scan(totals[tid], wsum, nullptr);
        run_off[tid] = base + offsets[(size_t)tid * gridDim.x + blockIdx.x];
    }
    const int start = blockIdx.x * chunk;
    const int end = min(start + chunk, n);
    for (int tbase = start; tbase < end; tbase += kSortTile) {
        for (int k = tid; k < kSortWarps * kRadix; k += blockDim.x) (&wcnt[0][0])[k] = 0;
        __syncthreads();
        K key[kSortItems];
        uint32_t val[kSortItems];
        uint32_t rank[kSortItems];
        // all loads first, so that they overlap
#pragma unroll
        for (int k = 0; k < kSortItems; k++) {
            const int i = tbase + warp * (32 * kSortItems) + k * 32 + (int)lane;
            key[k] = i < end ? kin[i] : K(0);
            val[k] = i < end ? vin[i] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kSortItems; k++) {
            const int i = tbase + warp * (32 * kSortItems) + k * 32 + (int)lane;
            const bool valid = i < end;
            const unsigned mask = __ballot_sync(0xffffffffu, valid);
            uint32_t d = 0, before = 0, peers = 0;
            if (valid) {
                d = (uint32_t)(key[k] >> shift) & (kRadix - 1);
                peers = __match_any_sync(mask, d);
                before = wcnt[warp][d];
                rank[k] = before + __popc(peers & lt_mask);
            }
            __syncwarp();
            if (valid && lane == (unsigned)(31 - __clz(peers))) wcnt[warp][d] = before + __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        // per-warp offsets within each digit, then the digit's start in the tile
        uint32_t tot = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; w++) {
            const uint32_t c = wcnt[w][tid];
            wcnt[w][tid] = tot;
            tot += c;
        }
        const uint32_t tb = block_exclusive_scan(tot, wsum, nullptr);
        tile_base[tid] = tb;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSortItems; k++) {
            const int i = tbase + warp * (32 * kSortItems) + k * 32 + (int)lane;
            if (i < end) {
                const uint32_t d = (uint32_t)(key[k] >> shift) & (kRadix - 1);
                const uint32_t local = tile_base[d] + wcnt[warp][d] + rank[k];
                skey[local] = key[k];
                sval[local] = val[k];
            }
        }
        __syncthreads();
        const int tile_n = min(kSortTile, end - tbase);
        for (int l = tid; l < tile_n; l += kSortThreads) {
            const K kk = skey[l];
            const uint32_t d = (uint32_t)(kk >> shift) & (kRadix - 1);
            const uint32_t pos = run_off[d] + (uint32_t)l - tile_base[d];
            kout[pos] = kk;
            vout[pos] = sval[l];
        }
        __syncthreads();
        // advance each digit's cursor by the tile's count of that digit
        {
            const uint32_t next = (tid + 1 < kRadix) ? tile_base[tid + 1] : (uint32_t)tile_n;
            run_off[tid] += next - tile_base[tid];
        }
        __syncthreads();
    }
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace gstex

using namespace gstex;

extern "C" int gstex_map_gaussian_to_intersects(int n, int num_isect, const float* centers, const float* extents,
                                                const float* depths, const int32_t* cum, int tiles_x, int tiles_y,
                                                int bw, int wrapped, int64_t* keys, int32_t* gids,
                                                gstex_stream_t stream) {
    GSTEX_REQUIRE(n >= 0 && num_isect >= 0 && tiles_x > 0 && tiles_y > 0 && bw > 0);
    if (n == 0 || num_isect == 0) return GSTEX_OK;
    GSTEX_REQUIRE(centers && extents && depths && cum && keys && gids);
    emit_kernel<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(n, num_isect, (const float2*)centers,
                                                                     (const float2*)extents, depths, cum, tiles_x,
                                                                     tiles_y, bw, wrapped, keys, gids);
    return check_launch("map_gaussian_to_intersects");
}

static size_t sort_workspace_bytes(int n, size_t key_bytes) {
    if (n < 1) n = 1;
    const SortPlan p = sort_plan(n);
    return align_up((size_t)n * key_bytes, 256) + align_up((size_t)n * 4, 256) + (size_t)kRadix * p.blocks * 4 +
           (size_t)kRadix * 4;
}

extern "C" size_t gstex_sort_workspace_bytes(int n) { return sort_workspace_bytes(n, 8); }
extern "C" size_t gstex_sort32_workspace_bytes(int n) { return sort_workspace_bytes(n, 4); }

template <typename K>
static int sort_impl(int n, const int64_t* n_dev, int end_bit, const K* keys_in, const int32_t* vals_in,
                     K* keys_out, int32_t* vals_out, void* ws, size_t ws_bytes, cudaStream_t stream) {
    GSTEX_REQUIRE(n >= 0 && end_bit >= 0 && end_bit <= (int)(8 * sizeof(K)));
    if (n == 0) return GSTEX_OK;
    GSTEX_REQUIRE(keys_in && vals_in && keys_out && vals_out);
    const int passes = ceil_div(end_bit, 8);
    if (passes == 0 || (n == 1 && !n_dev)) {
        cudaError_t e = cudaMemcpyAsync(keys_out, keys_in, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(vals_out, vals_in, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
        if (e != cudaSuccess) { set_cuda_error(e, "sort_pairs copy"); return GSTEX_ERR_CUDA; }
        return GSTEX_OK;
    }
    GSTEX_REQUIRE(ws);
    if (ws_bytes < sort_workspace_bytes(n, sizeof(K))) return GSTEX_ERR_CAPACITY;
    const SortPlan p = sort_plan(n);
    char* w = (char*)ws;
    K* kalt = (K*)w;
    w += align_up((size_t)n * sizeof(K), 256);
    uint32_t* valt = (uint32_t*)w;
    w += align_up((size_t)n * 4, 256);
    uint32_t* hist = (uint32_t*)w;
    uint32_t* totals = hist + (size_t)kRadix * p.blocks;
    // Ping-pong so that the last pass lands in the output buffers.
    const K* ksrc = keys_in;
    const uint32_t* vsrc = (const uint32_t*)vals_in;
    for (int pass = 0; pass < passes; pass++) {
        const bool to_out = ((passes - 1 - pass) % 2) == 0;
        K* kdst = to_out ? keys_out : kalt;
        uint32_t* vdst = to_out ? (uint32_t*)vals_out : valt;
        const int shift = pass * 8;
        radix_hist_kernel<K><<<p.blocks, kSortThreads, 0, stream>>>(ksrc, n, p.chunk, n_dev, shift, hist);
        radix_scan_rows_kernel<<<kRadix, kSortThreads, 0, stream>>>(hist, p.blocks, totals);
        radix_scatter_kernel<K><<<p.blocks, kSortThreads, 0, stream>>>(ksrc, vsrc, kdst, vdst, n, p.chunk, n_dev,
                                                                       shift, hist, totals);
        ksrc = kdst;
        vsrc = vdst;
    }
    return check_launch("sort_pairs", 3 * passes);
}

extern "C" int gstex_sort_pairs(int n, int end_bit, const int64_t* keys_in, const int32_t* vals_in,
                                int64_t* keys_out, int32_t* vals_out, void* ws, size_t ws_bytes, gstex_stream_t s) {
    return sort_impl<uint64_t>(n, nullptr, end_bit, (const uint64_t*)keys_in, vals_in, (uint64_t*)keys_out, vals_out,
                               ws, ws_bytes, (cudaStream_t)s);
}

extern "C" int gstex_sort_pairs_dyn(int capacity, const int64_t* count, int end_bit, const int64_t* keys_in,
                                    const int32_t* vals_in, int64_t* keys_out, int32_t* vals_out, void* ws,
                                    size_t ws_bytes, gstex_stream_t s) {
    GSTEX_REQUIRE(count);
    return sort_impl<uint64_t>(capacity, count, end_bit, (const uint64_t*)keys_in, vals_in, (uint64_t*)keys_out,
                               vals_out, ws, ws_bytes, (cudaStream_t)s);
}

extern "C" int gstex_sort_pairs32(int n, const int64_t* count, int end_bit, const uint32_t* keys_in,
                                  const int32_t* vals_in, uint32_t* keys_out, int32_t* vals_out, void* ws,
                                  size_t ws_bytes, gstex_stream_t s) {
    return sort_impl<uint32_t>(n, count, end_bit, keys_in, vals_in, keys_out, vals_out, ws, ws_bytes,
                               (cudaStream_t)s);
}

extern "C" int gstex_get_tile_bin_edges(int num_isect, const int64_t* sorted, int num_tiles, int32_t* bins,
                                        gstex_stream_t s) {
    GSTEX_REQUIRE(num_isect >= 0 && num_tiles > 0 && bins);
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)num_tiles * 2 * sizeof(int32_t), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "tile_bin_edges memset"); return GSTEX_ERR_CUDA; }
    if (num_isect == 0) return GSTEX_OK;
    GSTEX_REQUIRE(sorted);
    bin_edges_kernel<int64_t><<<ceil_div(num_isect, 256 * kEdgeItems), 256, 0, stream>>>(num_isect, nullptr, sorted, 32,
                                                                             num_tiles, (int2*)bins);
    return check_launch("get_tile_bin_edges");
}

extern "C" int gstex_get_tile_bin_edges_dyn(int capacity, const int64_t* count, const int64_t* sorted, int num_tiles,
                                            int32_t* bins, gstex_stream_t s) {
    GSTEX_REQUIRE(capacity >= 0 && num_tiles > 0 && bins && count);
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)num_tiles * 2 * sizeof(int32_t), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "tile_bin_edges memset"); return GSTEX_ERR_CUDA; }
    if (capacity == 0) return GSTEX_OK;
    GSTEX_REQUIRE(sorted);
    bin_edges_kernel<int64_t><<<ceil_div(capacity, 256 * kEdgeItems), 256, 0, stream>>>(capacity, count, sorted, 32, num_tiles,
                                                                            (int2*)bins);
    return check_launch("get_tile_bin_edges_dyn");
}

extern "C" int gstex_get_tile_bin_edges32_dyn(int capacity, const int64_t* count, const uint32_t* sorted, int shift,
                                              int num_tiles, int32_t* bins, gstex_stream_t s) {
    GSTEX_REQUIRE(capacity >= 0 && num_tiles > 0 && bins && count && shift >= 0 && shift < 32);
    cudaStream_t stream = (cudaStream_t)s;
    cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)num_tiles * 2 * sizeof(int32_t), stream);
    if (e != cudaSuccess) { set_cuda_error(e, "tile_bin_edges32 memset"); return GSTEX_ERR_CUDA; }
    if (capacity == 0) return GSTEX_OK;
    GSTEX_REQUIRE(sorted);
    bin_edges_kernel<uint32_t><<<ceil_div(capacity, 256 * kEdgeItems), 256, 0, stream>>>(capacity, count, sorted, shift, num_tiles,
                                                                             (int2*)bins);
    return check_launch("get_tile_bin_edges32_dyn");
}
