// Per-Gaussian projection work: screen AABB, tile counts, prefix sum, SH.
//
// Built with -fmad=false and IEEE division so that the AABB and tile counts
// are reproducible bit for bit by a CPU restatement of the same operations.
#include "common.cuh"
#include "project.cuh"

namespace gstex {

// Reference: csrc/get_aabb_2d.cu:11-89
__global__ void aabb_kernel(int n, const float3* __restrict__ means, const float* __restrict__ scales,
                            float glob_scale, const float4* __restrict__ quats, const float* __restrict__ viewmat,
                            float fx, float fy, float cx, float cy, float2* __restrict__ centers,
                            float2* __restrict__ extents) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float m[12];
#pragma unroll
    for (int k = 0; k < 12; k++) m[k] = viewmat[k];
    float2 c, e;
    float z;
    aabb_2d(m, fx, fy, cx, cy, means[i], quats[i], scales[3 * i], scales[3 * i + 1], glob_scale, c, e, z);
    centers[i] = c;
    extents[i] = e;
}

// gstex_cuda/get_aabb_2d.py:70-91 in float32: floor((c-e)/bw), floor((c+e)/bw + 1),
// clamped to the tile grid.
__global__ void tiles_hit_kernel(int n, const float2* __restrict__ centers, const float2* __restrict__ extents,
                                 int tiles_x, int tiles_y, float fbw, int32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = tiles_hit(centers[i], extents[i], tiles_x, tiles_y, fbw);
}

// ---------------------------------------------------------------------------
// Inclusive int32 scan (decomposed: block sums, scan of sums, block scan)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    total = warp_sums[(blockDim.x >> 5) - 1];
    const int before = warp > 0 ? warp_sums[warp - 1] : 0;
    __syncthreads();
    return before + x - v;
}

__global__ void scan_block_sums(int n, const int32_t* __restrict__ in, int64_t* __restrict__ sums) {
    __shared__ int ws[32];
    const int base = blockIdx.x * kScanTile;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int idx = base + k * kScanThreads + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    int total;
    block_exclusive_scan(s, ws, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// single block: exclusive scan of the block sums (64-bit to detect overflow)
__global__ void scan_sums(int nb, int64_t* __restrict__ sums, int64_t* __restrict__ total) {
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += blockDim.x) {
        const int i = base + threadIdx.x;
        long long v = i < nb ? sums[i] : 0;
        // warp-serial inclusive scan over the block (small nb)
        __shared__ long long buf[1024];
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < (int)blockDim.x; o <<= 1) {
            long long y = threadIdx.x >= (unsigned)o ? buf[threadIdx.x - o] : 0;
            __syncthreads();
            buf[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + buf[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += buf[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_apply(int n, const int32_t* __restrict__ in, const int64_t* __restrict__ offsets,
                           int32_t* __restrict__ out) {
    __shared__ int ws[32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        const int idx = base + k;
        v[k] = idx < n ? in[idx] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive_scan(s, ws, total) + (int)offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        run += v[k];
        const int idx = base + k;
        if (idx < n) out[idx] = run;
    }
}

// ---------------------------------------------------------------------------
// Spherical harmonics (csrc/sh.cuh:46-253; basis of gstex_cuda/_torch_impl.py:62-113)
// ---------------------------------------------------------------------------
// Templated on the degree in use (DTU), so the basis stays in registers; the
// coefficient stride follows the stored degree.
template <int DTU>
__global__ void sh_forward_kernel(int n, int degree, const float3* __restrict__ dirs,
                                  const float* __restrict__ coeffs, float* __restrict__ colors) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    constexpr int NB = (DTU + 1) * (DTU + 1);
    float Y[25];
    sh_basis(DTU, dirs[i], Y);
    const float* k = coeffs + (size_t)i * sh_bases(degree) * 3;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
    for (int b = 0; b < NB; b++) {
        c0 += Y[b] * k[3 * b + 0];
        c1 += Y[b] * k[3 * b + 1];
        c2 += Y[b] * k[3 * b + 2];
    }
    colors[3 * i + 0] = c0;
    colors[3 * i + 1] = c1;
    colors[3 * i + 2] = c2;
}

template <int DTU>
__global__ void sh_backward_kernel(int n, int degree, const float3* __restrict__ dirs,
                                   const float* __restrict__ v_colors, float* __restrict__ v_coeffs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    constexpr int NB = (DTU + 1) * (DTU + 1);
    float Y[25];
    sh_basis(DTU, dirs[i], Y);
    const int B = sh_bases(degree);
    const float v0 = v_colors[3 * i], v1 = v_colors[3 * i + 1], v2 = v_colors[3 * i + 2];
    float* o = v_coeffs + (size_t)i * B * 3;
#pragma unroll
    for (int b = 0; b < NB; b++) {
        o[3 * b + 0] = Y[b] * v0;
        o[3 * b + 1] = Y[b] * v1;
        o[3 * b + 2] = Y[b] * v2;
    }
    for (int b = NB; b < B; b++) {
        o[3 * b + 0] = 0.f;
        o[3 * b + 1] = 0.f;
        o[3 * b + 2] = 0.f;
    }
}

}  // namespace gstex

using namespace gstex;

extern "C" int gstex_get_aabb_2d(int n, const float* means, const float* scales, float glob_scale,
                                 const float* quats, const float* viewmat, float fx, float fy, float cx, float cy,
                                 float* centers, float* extents, gstex_stream_t stream) {
    GSTEX_REQUIRE(n >= 0);
    if (n == 0) return GSTEX_OK;
    GSTEX_REQUIRE(means && scales && quats && viewmat && centers && extents);
    aabb_kernel<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, (const float3*)means, scales, glob_scale, (const float4*)quats, viewmat, fx, fy, cx, cy,
        (float2*)centers, (float2*)extents);
    return check_launch("get_aabb_2d");
}

extern "C" int gstex_num_tiles_hit(int n, const float* centers, const float* extents, int img_height,
                                   int img_width, int block_width, int32_t* out, gstex_stream_t stream) {
    GSTEX_REQUIRE(n >= 0 && img_height > 0 && img_width > 0 && block_width > 0);
    if (n == 0) return GSTEX_OK;
    GSTEX_REQUIRE(centers && extents && out);
    const int tx = ceil_div(img_width, block_width), ty = ceil_div(img_height, block_width);
    tiles_hit_kernel<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(
        n, (const float2*)centers, (const float2*)extents, tx, ty, (float)block_width, out);
    return check_launch("num_tiles_hit");
}

extern "C" size_t gstex_scan_workspace_bytes(int n) {
    return (size_t)(ceil_div(n > 0 ? n : 1, kScanTile) + 1) * sizeof(int64_t);
}

extern "C" int gstex_inclusive_scan_i32(int n, const int32_t* counts, int32_t* cum, int64_t* total, void* ws,
                                        size_t ws_bytes, gstex_stream_t s) {
    GSTEX_REQUIRE(n >= 0 && total);
    cudaStream_t stream = (cudaStream_t)s;
    if (n == 0) {
        cudaError_t e = cudaMemsetAsync(total, 0, sizeof(int64_t), stream);
        if (e != cudaSuccess) { set_cuda_error(e, "scan"); return GSTEX_ERR_CUDA; }
        return GSTEX_OK;
    }
    GSTEX_REQUIRE(counts && cum && ws);
    if (ws_bytes < gstex_scan_workspace_bytes(n)) return GSTEX_ERR_CAPACITY;
    const int nb = ceil_div(n, kScanTile);
    int64_t* sums = (int64_t*)ws;
    scan_block_sums<<<nb, kScanThreads, 0, stream>>>(n, counts, sums);
    scan_sums<<<1, 1024, 0, stream>>>(nb, sums, total);
    scan_apply<<<nb, kScanThreads, 0, stream>>>(n, counts, sums, cum);
    return check_launch("inclusive_scan", 3);
}

// Degrees above 4 are not supported (sh.cuh:46-253 stops at 4); the degree in
// use must not exceed the stored one (the reference's wrapper asserts it,
// sh.py:54, and its kernel would read the next Gaussian's coefficients).
static int sh_degrees_ok(int degree, int degrees_to_use) {
    if (degree < 0 || degrees_to_use < 0 || degrees_to_use > degree) return GSTEX_ERR_INVALID_ARGUMENT;
    if (degree > 4) return GSTEX_ERR_UNSUPPORTED;
    return GSTEX_OK;
}

extern "C" int gstex_compute_sh_forward(int n, int degree, int degrees_to_use, const float* viewdirs,
                                        const float* coeffs, float* colors, gstex_stream_t stream) {
    GSTEX_REQUIRE(n >= 0);
    int rc = sh_degrees_ok(degree, degrees_to_use);
    if (rc) return rc;
    if (n == 0) return GSTEX_OK;
    GSTEX_REQUIRE(viewdirs && coeffs && colors);
    const dim3 grid(ceil_div(n, 256)), block(256);
    cudaStream_t st = (cudaStream_t)stream;
    const float3* d = (const float3*)viewdirs;
    switch (degrees_to_use) {
        case 0: sh_forward_kernel<0><<<grid, block, 0, st>>>(n, degree, d, coeffs, colors); break;
        case 1: sh_forward_kernel<1><<<grid, block, 0, st>>>(n, degree, d, coeffs, colors); break;
        case 2: sh_forward_kernel<2><<<grid, block, 0, st>>>(n, degree, d, coeffs, colors); break;
        case 3: sh_forward_kernel<3><<<grid, block, 0, st>>>(n, degree, d, coeffs, colors); break;
        default: sh_forward_kernel<4><<<grid, block, 0, st>>>(n, degree, d, coeffs, colors); break;
    }
    return check_launch("compute_sh_forward");
}

extern "C" int gstex_compute_sh_backward(int n, int degree, int degrees_to_use, const float* viewdirs,
                                         const float* v_colors, float* v_coeffs, gstex_stream_t stream) {
    GSTEX_REQUIRE(n >= 0);
    int rc = sh_degrees_ok(degree, degrees_to_use);
    if (rc) return rc;
    if (n == 0) return GSTEX_OK;
    GSTEX_REQUIRE(viewdirs && v_colors && v_coeffs);
    const dim3 grid(ceil_div(n, 256)), block(256);
    cudaStream_t st = (cudaStream_t)stream;
    const float3* d = (const float3*)viewdirs;
    switch (degrees_to_use) {
        case 0: sh_backward_kernel<0><<<grid, block, 0, st>>>(n, degree, d, v_colors, v_coeffs); break;
        case 1: sh_backward_kernel<1><<<grid, block, 0, st>>>(n, degree, d, v_colors, v_coeffs); break;
        case 2: sh_backward_kernel<2><<<grid, block, 0, st>>>(n, degree, d, v_colors, v_coeffs); break;
        case 3: sh_backward_kernel<3><<<grid, block, 0, st>>>(n, degree, d, v_colors, v_coeffs); break;
        default: sh_backward_kernel<4><<<grid, block, 0, st>>>(n, degree, d, v_colors, v_coeffs); break;
    }
    return check_launch("compute_sh_backward");
}
