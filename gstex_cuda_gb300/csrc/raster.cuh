// Argument structs and launch helpers of the compositor kernels.
#pragma once

#include "common.cuh"

namespace gstex {

constexpr int kMoments = 23;    // per-pair moments reduced inside a CTA
constexpr int kMomSlot = 24;    // shared-memory slot stride: 6 float4
constexpr int kMomStride = 24;  // per-Gaussian global moments (colour gradients live elsewhere)

// View-independent scene inputs.
struct SceneArgs {
    int N, C, T;
    const int3* dims;
    const int32_t* gids;  // depth-sorted Gaussian ids of all tiles
    const float3* means;
    const float* scales;
    float glob;
    const float4* quats;
    const float* opac;
    const float2* uv0;
    const float3* umap;
    const float3* vmap;
    const void* tex;
    int settings;
    const float* bg;      // [3] device
    int batch;            // Gaussians staged per round (0: one per thread)
};

// One view rendered by a tile grid (the reference's launch form).
struct ViewArgs {
    const float* viewmat;
    float fx, fy, cx, cy;
    int W, H, tiles_x;
    const int2* bins;
    const float3* colors;
    float* vcolors;       // [N,3] colour gradients (backward)
    const RecAll* recs;   // optional [N] prebuilt records of the view; null: built per tile
};

// Per-view constants of a batched launch (device array).
struct BatchView {
    View V;
    int W, H, tiles_x, tiles_y;
    int tile_offset;      // global index of the view's first tile
    int pix_offset;       // global index of the view's first pixel
    float campos[3];      // camera centre in world space (SH view directions)
    int pad;
};

struct BatchArgs {
    int num_points, total_tiles;
    const BatchView* views;
    const int32_t* tile_view;  // [total_tiles] view of each global tile
    const int32_t* order;      // optional queue order of global tiles
    const int2* bins;          // [total_tiles]
    const float3* colors;      // [V, N, 3]
    float* vcolors;            // [V, N, 4] (rgb + pad: one vector atomic per flush)
    int* queue;                // tile counter, zero before each launch
    const RecAll* recs;        // optional [V, N] prebuilt records; null: built per tile
};

// What one CTA needs to render one tile.
struct TileJob {
    View V;
    int W, H, tx, ty;
    int2 range;
    size_t pix_base;
    const float3* colors;
    float* vcolors;       // colour gradients: [N, 3] (per-view launch) or [N, 4] rows (batched)
    int vc_stride;        // 3 or 4 floats per Gaussian in vcolors
    const RecAll* recs;   // the view's prebuilt records, or null
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
    const float3* v_img;    // upstream gradients; null means zero
    const float* v_depth;
    const float* v_reg;
    const float* v_alpha;
    const float* v_tex;
    const float3* v_normal;
    float* moments;         // [N, kMomStride]
    float* v_texgrad;       // [T, C] (fp32 texture) or [T, 4] (bf16 texture)
};

int fill_scene(const gstex_raster_inputs* in, SceneArgs& a, bool need_bins);
int ppt_of(int bw, int requested);
int gs_of(int bw, int ppt, int C, int requested);
// shared memory of a compositor CTA staging `batch` Gaussians per round (0: one per thread)
size_t fwd_smem(int bw, int ppt, int batch);
size_t bwd_smem(int bw, int ppt, int gs, int batch);
int launch_fwd_batch(const SceneArgs& a, const BatchArgs& ba, const FwdOut& o, int bw, int texmode, int ppt, int grid,
                     cudaStream_t stream);
int launch_bwd_batch(const SceneArgs& a, const BatchArgs& ba, const BwdArgs& g, int bw, int texmode, int ppt, int gs,
                     int ctas, int grid, cudaStream_t stream);
// Gradients w.r.t. the trainer's raw parameters (raw_quats == nullptr: the
// activated parameters' gradients are written instead).
struct RawGradArgs {
    const float4* raw_quats;   // [N, 4]
    const float* scales;       // [N, 3] activated
    const float* opacity;      // [N] activated
    float* v_raw_scales;       // [N, 3]
    float4* v_raw_quats;       // [N, 4]
    float4* v_mapping;         // [N, 4] (one chart)
    float* v_raw_opacity;      // [N] or null
};

int launch_finalize(const SceneArgs& a, const float* moments, float* v_opac, float* v_means, float* v_scales,
                    float* v_quats, float* v_uv0, float* v_umap, float* v_vmap, cudaStream_t stream,
                    const RawGradArgs& rg = RawGradArgs{});
int resident_ctas(int bw, bool backward, int texmode, int C, int ppt, int gs, int ctas = 0, int batch = 0,
                  int settings = 0);
// Settings bits the backward reads (bilinear off, uv-gradient propagation,
// blur, NDC depth) and the value for which kernels compiled for fixed
// settings exist: uv gradients propagated, everything else off.
constexpr int kFixedBwdMask = (1 << 2) | (1 << 8) | (1 << 9) | (1 << 10);
constexpr int kFixedBwdSettings = 1 << 8;
// Settings bits the forward reads besides the alpha-visualisation mode
// (bilinear off, blur, NDC depth, flipped normals, alpha visualisation): the
// kernel compiled for fixed settings applies when all are off.
constexpr int kFixedFwdMask = (1 << 2) | (1 << 9) | (1 << 10) | (1 << 15) | (1 << 16);
int launch_records(const SceneArgs& a, const BatchArgs& ba, int num_views, const int32_t* counts, RecAll* recs,
                   int* fix_count, uint32_t* fix, cudaStream_t stream);

}  // namespace gstex
