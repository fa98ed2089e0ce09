/*
 * gstex_gb300 - C ABI of the GB300-native textured 2D-Gaussian rasteriser.
 *
 * Each entry point replaces one native op of the reference's Python
 * extension (gstex_cuda.csrc, bound in gstex_cuda/cuda/csrc/ext.cpp:8-25 and
 * looked up lazily in gstex_cuda/cuda/__init__.py:4-27; paths relative to
 * the reference project).  The conventions differ from the reference in the
 * ways a C ABI needs:
 *   - every array is a raw device pointer to contiguous memory, allocated by
 *     the caller (outputs included); the library allocates nothing;
 *   - every call takes the CUDA stream to launch on and is asynchronous;
 *   - every call returns a status code (GSTEX_OK = 0) after validating its
 *     arguments on the host and checking the launch with cudaGetLastError.
 * Matrices are row-major float[16]; quaternions are (w, x, y, z).
 */
#ifndef GSTEX_GB300_H
#define GSTEX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gstex_stream_t; /* same type as cudaStream_t */

enum gstex_status {
    GSTEX_OK = 0,
    GSTEX_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size or shape */
    GSTEX_ERR_CAPACITY = 2,         /* a caller-provided buffer is too small */
    GSTEX_ERR_UNSUPPORTED = 3,      /* e.g. more than 64 texture channels */
    GSTEX_ERR_CUDA = 4              /* a CUDA launch or runtime call failed */
};

/* Text for a status code (static storage). */
const char* gstex_status_string(int status);
/* Text of the last CUDA error seen by this library on this thread. */
const char* gstex_last_cuda_error(void);
/* Library version, e.g. "0.1.0". */
const char* gstex_version(void);
/* Number of kernels this library has launched since it was loaded. */
unsigned long long gstex_launch_count(void);

/* ---------------------------------------------------------------------
 * Projection
 * ------------------------------------------------------------------- */

/* Screen-space AABB of each 2D Gaussian's +-3 sigma rectangle.
 * Replaces _C.get_aabb_2d (csrc/get_aabb_2d.cu:91-126).
 * means/scales [n,3], quats [n,4] -> centers/extents [n,2]. */
int gstex_get_aabb_2d(int n, const float* means, const float* scales, float glob_scale, const float* quats,
                      const float* viewmat, float fx, float fy, float cx, float cy, float* centers,
                      float* extents, gstex_stream_t stream);

/* Per-Gaussian number of tiles hit, bit-exact with the reference's torch
 * tile counter.  Replaces get_num_tiles_hit_2d (gstex_cuda/get_aabb_2d.py:70-91). */
int gstex_num_tiles_hit(int n, const float* centers, const float* extents, int img_height, int img_width,
                        int block_width, int32_t* num_tiles_hit, gstex_stream_t stream);

/* Inclusive int32 prefix sum of n counts (the reference's torch.cumsum in
 * compute_cumulative_intersects, gstex_cuda/utils.py:40-59).  total (device,
 * int64) receives the last value.  workspace: gstex_scan_workspace_bytes(n). */
size_t gstex_scan_workspace_bytes(int n);
int gstex_inclusive_scan_i32(int n, const int32_t* counts, int32_t* cum, int64_t* total, void* workspace,
                             size_t workspace_bytes, gstex_stream_t stream);

/* Spherical harmonics colours from coefficients [n, bases(degree), 3] using
 * the first bases(degrees_to_use) bases.  Replaces _C.compute_sh_forward
 * (csrc/bindings.cu:18-43). */
int gstex_compute_sh_forward(int n, int degree, int degrees_to_use, const float* viewdirs, const float* coeffs,
                             float* colors, gstex_stream_t stream);
/* v_coeffs [n, bases(degree), 3] (fully written). Replaces
 * _C.compute_sh_backward (csrc/bindings.cu:45-75). */
int gstex_compute_sh_backward(int n, int degree, int degrees_to_use, const float* viewdirs,
                              const float* v_colors, float* v_coeffs, gstex_stream_t stream);

/* ---------------------------------------------------------------------
 * Tile binning
 * ------------------------------------------------------------------- */

/* Emits one (tile << 32 | depth-bits) key and Gaussian id per tile hit into
 * the slots [cum[i-1], cum[i]) of each Gaussian.  Slots a Gaussian does not
 * write (tiny extents) are set to zero, as in the reference.  Replaces
 * _C.map_gaussian_to_intersects (csrc/bindings.cu:77-121, forward.cu:13-71). */
int gstex_map_gaussian_to_intersects(int n, int num_intersects, const float* centers, const float* extents,
                                     const float* depths, const int32_t* cum_tiles_hit, int tiles_x, int tiles_y,
                                     int block_width, int wrapped, int64_t* isect_ids, int32_t* gaussian_ids,
                                     gstex_stream_t stream);

/* Stable ascending LSD radix sort of (int64 key, int32 value) pairs on key
 * bits [0, end_bit).  Replaces torch.sort + torch.gather in
 * bin_and_sort_gaussians (gstex_cuda/utils.py:159-160).  The caller passes
 * end_bit = 32 + bit_length(num_tiles), which orders every key with a
 * non-negative depth exactly as a signed 64-bit sort does. */
size_t gstex_sort_workspace_bytes(int n);
int gstex_sort_pairs(int n, int end_bit, const int64_t* keys_in, const int32_t* vals_in, int64_t* keys_out,
                     int32_t* vals_out, void* workspace, size_t workspace_bytes, gstex_stream_t stream);

/* Largest n accepted by gstex_sort_pairs_static. */
#define GSTEX_SORT_STATIC_MAX_ITEMS 1048576

/* The same stable pair sort for callers that cannot allocate device memory
 * (a host framework that owns all device allocations, a plugin handed only a
 * stream and raw pointers, real-time code where an allocation could stall or
 * fail mid-frame).  No counterpart in the reference, which allocates with
 * torch inside each op.  Scratch is one file-scope device array of 13.1 MB
 * sized for GSTEX_SORT_STATIC_MAX_ITEMS pairs, held by every GPU that loads
 * the library until exit; larger n returns GSTEX_ERR_CAPACITY.  The first
 * call in each CUDA context (per device, and again after a device reset)
 * looks up the array's device address (do it before any stream capture).  All calls on a device share the array: calls that
 * overlap on the GPU race and must be serialised by the caller; nothing in it
 * needs clearing between calls.  Allocates nothing and calls no allocating
 * routine. */
int gstex_sort_pairs_static(int n, int end_bit, const int64_t* keys_in, const int32_t* vals_in,
                            int64_t* keys_out, int32_t* vals_out, gstex_stream_t stream);

/* Same sort with the number of items read from device memory (*count,
 * clamped to capacity): the launch shape depends only on capacity, so the
 * call can be captured in a CUDA graph.  Workspace:
 * gstex_sort_workspace_bytes(capacity).  Batched form of utils.py:159-160. */
int gstex_sort_pairs_dyn(int capacity, const int64_t* count, int end_bit, const int64_t* keys_in,
                         const int32_t* vals_in, int64_t* keys_out, int32_t* vals_out, void* workspace,
                         size_t workspace_bytes, gstex_stream_t stream);

/* Per-tile [start, end) ranges of a sorted key list (zero for empty tiles).
 * Replaces _C.get_tile_bin_edges (csrc/bindings.cu:123-140, forward.cu:76-98). */
int gstex_get_tile_bin_edges(int num_intersects, const int64_t* isect_ids_sorted, int num_tiles,
                             int32_t* tile_bins, gstex_stream_t stream);
/* Same with the key count read from device memory (clamped to capacity). */
int gstex_get_tile_bin_edges_dyn(int capacity, const int64_t* count, const int64_t* isect_ids_sorted,
                                 int num_tiles, int32_t* tile_bins, gstex_stream_t stream);

/* Stable LSD radix sort of (uint32 key, int32 value) pairs on key bits
 * [0, end_bit); with count non-NULL the number of items is read from device
 * memory (clamped to n) and the call can be captured in a CUDA graph.
 * Workspace: gstex_sort32_workspace_bytes(n).  The two sorts of the
 * depth-first batched binning, which together replace the 64-bit sort of
 * bin_and_sort_gaussians (gstex_cuda/utils.py:159-160). */
size_t gstex_sort32_workspace_bytes(int n);
int gstex_sort_pairs32(int n, const int64_t* count, int end_bit, const uint32_t* keys_in, const int32_t* vals_in,
                       uint32_t* keys_out, int32_t* vals_out, void* workspace, size_t workspace_bytes,
                       gstex_stream_t stream);
/* Tile ranges of 32-bit sorted keys whose tile is key >> shift; batched form
 * of _C.get_tile_bin_edges (csrc/forward.cu:76-98). */
int gstex_get_tile_bin_edges32_dyn(int capacity, const int64_t* count, const uint32_t* keys_sorted, int shift,
                                   int num_tiles, int32_t* tile_bins, gstex_stream_t stream);

/* ---------------------------------------------------------------------
 * Textured compositor (texture_forward / texture_backward)
 * ------------------------------------------------------------------- */

/* Inputs shared by forward and backward (csrc/texture.cuh:92-167). */
typedef struct gstex_raster_inputs {
    int num_points;       /* N */
    int img_width, img_height, block_width;
    int channels;         /* texture channels C (texture_info[2]), 0..64 */
    int num_texels;       /* T = rows of texture */
    int texture_dtype;    /* 0: float32 [T,C]; 1: bfloat16 [T,4] (C == 3 only) */
    const int32_t* texture_dims;        /* [N,3] (h, w, start) */
    const int32_t* gaussian_ids_sorted; /* [num_intersects] */
    const int32_t* tile_bins;           /* [tiles, 2] */
    const float* colors;                /* [N,3] */
    const float* opacities;             /* [N] */
    const float* means;                 /* [N,3] */
    const float* scales;                /* [N,3] */
    float glob_scale;
    const float* quats;                 /* [N,4] */
    const float* uv0;                   /* [N,2] */
    const float* umap;                  /* [N,3] */
    const float* vmap;                  /* [N,3] */
    const void* texture;                /* see texture_dtype */
    const float* viewmat;               /* [16] device */
    float fx, fy, cx, cy;
    int settings;                       /* reference settings bitfield */
    const float* background;            /* [3] device */
    int pixels_per_thread;              /* 0 = default (1); 2 needs an even block width */
    /* Optional splat records of this view built by gstex_view_records from
     * the same inputs (16-byte aligned); NULL: every tile derives the records
     * of its Gaussians itself.  Read by texture_forward / texture_backward,
     * not by texture_edit. */
    const void* records;
    /* texture_backward: lanes that walk one list of staged splats, 32 (a
     * warp's 8x4 pixel block), 16 (4x4), 8 (4x2) or 4 (2x2); 0 = 32.  Values
     * below 32 apply to block widths that are multiples of 8, one pixel per
     * thread and 0 or 3 channels; elsewhere 32 is used.  Gradients do not
     * depend on it beyond float summation order.  texture_forward ignores it. */
    int group_lanes;
} gstex_raster_inputs;

/* Bytes of the records buffer of one view: 224 per Gaussian plus the list
 * of near-edge-on records solved in double precision. */
size_t gstex_view_records_bytes(int num_points);
/* One camera-space splat record per Gaussian of the view (all N, whatever
 * the binning), from the scene, camera, colours and settings of `in`
 * (tile_bins and gaussian_ids_sorted are not read).  Two launches; the
 * texture_forward / texture_backward calls that pass them copy a record per
 * (tile, Gaussian) instead of recomputing it.  No counterpart in the
 * reference, whose kernels derive the same per pixel (csrc/texture.cu:160-181). */
int gstex_view_records(const gstex_raster_inputs* in, void* records, size_t records_bytes, gstex_stream_t stream);

typedef struct gstex_forward_outputs {
    float* img;        /* [H,W,3] */
    float* depth;      /* [H,W] */
    float* reg;        /* [H,W] */
    float* texture;    /* [H,W,C] */
    float* normal;     /* [H,W,3] */
    float* final_T;    /* [H,W] */
    int32_t* final_idx; /* [H,W] */
    int32_t* depth_idx; /* [H,W] */
    float* reg_s;      /* [H,W,3] */
} gstex_forward_outputs;

/* Replaces _C.texture_forward (csrc/texture.cu:766-901). */
int gstex_texture_forward(const gstex_raster_inputs* in, const gstex_forward_outputs* out, gstex_stream_t stream);

typedef struct gstex_edit_io {
    const float* updated_img;    /* [H,W,3] edited colours */
    const float* updated_alpha;  /* [H,W] edit mask (0 where nothing is edited) */
    const float* depth_lower;    /* [H,W] camera depths outside [lower, upper] are not edited */
    const float* depth_upper;    /* [H,W] */
    long long num_texels;        /* rows of updated_texture (sum of h*w over the charts) */
    float* updated_texture;      /* [num_texels, 5]: r*a, g*a, b*a, a, total weight; zeroed, then accumulated */
} gstex_edit_io;

/* Replaces _C.texture_edit (csrc/texture_edit.cu:238-346): in->channels must
 * be 5 (texture_info[2]; the reference writes five channels at that stride),
 * in->colors / in->texture / in->background are not read, blur is settings
 * bit 0. */
int gstex_texture_edit(const gstex_raster_inputs* in, const gstex_edit_io* io, gstex_stream_t stream);

typedef struct gstex_backward_io {
    /* saved forward state */
    const float* final_T;
    const int32_t* final_idx;
    const int32_t* depth_idx;
    const float* reg_s;
    /* upstream gradients */
    const float* v_img;     /* [H,W,3] */
    const float* v_depth;   /* [H,W] */
    const float* v_reg;     /* [H,W] */
    const float* v_alpha;   /* [H,W] */
    const float* v_texture; /* [H,W,C] */
    const float* v_normal;  /* [H,W,3] */
    /* outputs (fully written; v_tex_grad is accumulated into and must be
     * zeroed by the caller) */
    float* v_colors;  /* [N,3] */
    float* v_opacity; /* [N] */
    float* v_means;   /* [N,3] */
    float* v_scales;  /* [N,3] */
    float* v_quats;   /* [N,4] */
    float* v_uv0;     /* [N,2] */
    float* v_umap;    /* [N,3] */
    float* v_vmap;    /* [N,3] */
    float* v_tex_grad; /* [T,C] float32 (or [T,4] when texture_dtype == 1) */
    /* caller-provided scratch of gstex_backward_workspace_bytes(N) bytes */
    void* workspace;
    size_t workspace_bytes;
} gstex_backward_io;

size_t gstex_backward_workspace_bytes(int num_points);

/* Replaces _C.texture_backward (csrc/texture.cu:915-1053). */
int gstex_texture_backward(const gstex_raster_inputs* in, const gstex_backward_io* io, gstex_stream_t stream);

/* ---------------------------------------------------------------------
 * texture_sample
 * ------------------------------------------------------------------- */

/* Bilinear lookup of nq queries in jagged charts, uv clamped to [0,1].
 * Replaces _C.texture_sample_forward (csrc/texture_sample.cu:72-105). */
int gstex_texture_sample_forward(int nq, int channels, const int32_t* texture_dims, const float* uvs,
                                 const float* texture, float* out, gstex_stream_t stream);
/* Texel gradients (accumulated into v_texture, zeroed by the caller) and uv
 * gradients (written).  Replaces _C.texture_sample_backward
 * (csrc/texture_sample.cu:107-141), which read its upstream gradient from the
 * wrong buffer and was never called. v_uvs may be null. */
int gstex_texture_sample_backward(int nq, int channels, const int32_t* texture_dims, const float* uvs,
                                  const float* texture, const float* v_out, float* v_texture, float* v_uvs,
                                  gstex_stream_t stream);

/* ---------------------------------------------------------------------
 * Batched multi-view rendering.  The reference renders one view per call
 * (gstex_cuda/texture.py:14-150, called once per camera by its trainer);
 * these entry points render many views of one scene with one launch per
 * stage and no size read back to the host, so a whole forward + backward
 * step can be captured in a CUDA graph.  Global tiles and pixels of all
 * views are numbered view by view.
 * ------------------------------------------------------------------- */
typedef struct gstex_view_desc {
    float viewmat[16]; /* world->camera, row-major */
    float fx, fy, cx, cy;
    int width, height;
} gstex_view_desc;

/* Total tiles and pixels of a set of views (host only). */
int gstex_batch_layout(int num_views, const gstex_view_desc* views, int block_width, int* total_tiles,
                       long long* total_pixels);
/* Bytes of the device view table written by gstex_batch_prepare. */
size_t gstex_batch_views_bytes(int num_views);
/* Writes the device view table, the view of every global tile
 * (tile_view [total_tiles]) and the pixel offsets of the views
 * (pix_offsets [num_views + 1]); synchronises the stream. */
int gstex_batch_prepare(int num_views, const gstex_view_desc* views, int block_width, void* views_dev,
                        int32_t* tile_view, long long* pix_offsets, gstex_stream_t stream);

/* AABB, tile count (counts [V*N], view-major) and SH colour
 * (colors [V,N,3]) of every (view, Gaussian); sh_dtype 0 float32, 1 bfloat16.
 * Batched form of get_aabb_2d + get_num_tiles_hit_2d + spherical_harmonics. */
int gstex_batch_project(int num_points, int num_views, const void* views_dev, const float* means,
                        const float* scales, float glob_scale, const float* quats, const void* sh_coeffs,
                        int sh_dtype, int sh_degree, int block_width, float* colors, int32_t* counts,
                        gstex_stream_t stream);

/* Emission of (global tile << 32 | depth bits) keys into the slots of the
 * inclusive scan cum [V*N] of the counts (total = its last value, device).
 * Writes stop at capacity; count receives min(total, capacity) and
 * *overflow is set when total exceeds capacity.  Batched form of
 * map_gaussian_to_intersects. */
int gstex_batch_emit(int num_points, int num_views, const void* views_dev, const float* means, const float* scales,
                     float glob_scale, const float* quats, int block_width, const int32_t* cum,
                     const int64_t* total, long long capacity, int64_t* keys, int32_t* gaussian_ids,
                     int64_t* count, int* overflow, gstex_stream_t stream);

/* Depth-first binning, the order of gstex_batch_emit + a 64-bit sort from
 * 32-bit sorts (batched form of get_aabb_2d + get_num_tiles_hit_2d +
 * compute_cumulative_intersects + map_gaussian_to_intersects + the sort,
 * gstex_cuda/utils.py:40-161, csrc/forward.cu:13-71):
 *   1. gstex_batch_project_keys: as gstex_batch_project, plus per pair j the
 *      depth key (float bits of the camera depth; 0xffffffff without tiles),
 *      pair_ids[j] = j and the tile rectangle rects [V*N, 2] (uint32 x0 | x1 << 16,
 *      y0 | y1 << 16; 8-byte aligned);
 *   2. gstex_sort_pairs32 of (depth_keys, pair_ids), end_bit 32 -> order;
 *   3. gstex_batch_gather_counts(order) and gstex_inclusive_scan_i32 -> cum;
 *   4. gstex_batch_emit_sorted: pair order[p] writes [cum[p-1], cum[p]) with
 *      keys (global tile << 1 | 1) and its Gaussian id; slots it does not write
 *      get (view's first tile << 1 | 0) and Gaussian 0, which sort first in that
 *      tile like the reference's zero entries;
 *   5. gstex_sort_pairs32 of (keys, gaussian_ids) with the emitted count,
 *      end_bit 1 + bit_length(total_tiles), and gstex_get_tile_bin_edges32_dyn
 *      with shift 1.
 * The resulting gaussian_ids_sorted and tile_bins equal those of
 * gstex_batch_emit + gstex_sort_pairs_dyn bit for bit; needs V * N < 2^31. */
int gstex_batch_project_keys(int num_points, int num_views, const void* views_dev, const float* means,
                             const float* scales, float glob_scale, const float* quats, const void* sh_coeffs,
                             int sh_dtype, int sh_degree, int block_width, float* colors, int32_t* counts,
                             uint32_t* depth_keys, int32_t* pair_ids, uint32_t* rects, gstex_stream_t stream);
int gstex_batch_gather_counts(int n, const int32_t* order, const int32_t* counts, int32_t* out,
                              gstex_stream_t stream);
int gstex_batch_emit_sorted(int num_points, int num_views, const void* views_dev, const int32_t* order,
                            const int32_t* cum, const uint32_t* rects, const int64_t* total, long long capacity,
                            uint32_t* keys, int32_t* gaussian_ids, int64_t* count, int* overflow,
                            gstex_stream_t stream);

/* Queue order of the global tiles for gstex_batch_forward (in->tile_order)
 * from tile_bins [total_tiles, 2]: groups of group x group neighbouring
 * tiles of a view (tile_view / views_dev from gstex_batch_prepare; unused for
 * group 1) by decreasing intersection count of the group, ties in tile order,
 * the tiles of a group back to back in tile order.  The heaviest work starts
 * first, and the tiles of a group, which share most of their splats, run
 * close together.  (The backward is faster in plain tile order.)  Workspace:
 * gstex_batch_tile_order_workspace_bytes(total_tiles), 16-byte aligned. */
size_t gstex_batch_tile_order_workspace_bytes(int total_tiles);
int gstex_batch_tile_order(int total_tiles, const int32_t* tile_bins, const int32_t* tile_view,
                           const void* views_dev, int group, int32_t* order, void* workspace,
                           size_t workspace_bytes, gstex_stream_t stream);

typedef struct gstex_batch_inputs {
    int num_points, num_views, block_width;
    int channels, num_texels, texture_dtype, settings;
    int total_tiles;
    const void* views;                  /* gstex_batch_prepare */
    const int32_t* tile_view;           /* [total_tiles] */
    const int32_t* tile_order;          /* optional queue order of global tiles */
    const int32_t* gaussian_ids_sorted;
    const int32_t* tile_bins;           /* [total_tiles, 2] */
    const float* colors;                /* [V, N, 3] */
    const float* opacities;
    const float* means;
    const float* scales;
    float glob_scale;
    const float* quats;
    const float* uv0;
    const float* umap;
    const float* vmap;
    const int32_t* texture_dims;
    const void* texture;
    const float* background;            /* [3] device */
    int* queue;                         /* device int (tile queue counter) */
    int grid;                           /* persistent CTAs; 0 = all resident */
    int pixels_per_thread;              /* 0 = default (1); 2 needs an even block width */
    const void* records;                /* optional: gstex_batch_records output (16-byte aligned);
                                           null = each tile derives the records it stages */
    int group_lanes;                    /* backward: lanes per splat walk (see gstex_raster_inputs) */
    int batch_size;                     /* Gaussians a tile stages per round; 0, or at least the
                                           threads of a CTA: one per thread (the reference's bw^2) */
    int resident_ctas;                  /* backward, 8x8 tiles with bf16 RGB texels and 8-lane groups (or
                                           32 at the default settings): 10 selects a kernel compiled for
                                           10 CTAs per SM (96 registers per thread instead of 124); other
                                           values: the general kernel */
} gstex_batch_inputs;

/* Bytes of the per-(view, Gaussian) splat records of gstex_batch_records
 * (224 bytes per pair). */
size_t gstex_batch_records_bytes(int num_points, int num_views);

/* Workspace of gstex_batch_records: a counter and one index per pair. */
size_t gstex_batch_records_workspace_bytes(int num_points, int num_views);

/* Builds the splat record (camera-space plane coefficients, alpha >= 1/255
 * screen box and quad, colour, chart) of every (view, Gaussian) pair whose tile count
 * in `counts` ([V, N], from gstex_batch_project) is positive, and of
 * Gaussian 0 in every view, once per step; near-edge-on splats are solved in
 * double here (gathered first, then solved by a second kernel).  Pass the
 * buffer as in->records to the forward and backward, which then copy records
 * instead of deriving them per tile.  Reads in->colors, the Gaussian
 * parameters and in->views; needs N * V < 2^32.  No reference counterpart
 * (the reference derives the same quantities per pixel,
 * csrc/texture.cu:160-181). */
int gstex_batch_records(const gstex_batch_inputs* in, const int32_t* counts, void* records, void* workspace,
                        size_t workspace_bytes, gstex_stream_t stream);

/* Forward of all views: outputs are the concatenated per-view buffers
 * (pixel p of view v at pix_offsets[v] + p).  Batched texture_forward. */
int gstex_batch_forward(const gstex_batch_inputs* in, const gstex_forward_outputs* out, gstex_stream_t stream);

/* Backward of all views.  io->v_colors is [V, N, 4] (per-view colour
 * gradients rgb + one unused float per row, for the SH adjoint; 16-byte
 * aligned); the other Gaussian gradients are summed
 * over views; null upstream-gradient pointers mean zero.  Workspace:
 * gstex_batch_backward_workspace_bytes(N).  Batched texture_backward. */
size_t gstex_batch_backward_workspace_bytes(int num_points);
int gstex_batch_backward(const gstex_batch_inputs* in, const gstex_backward_io* io, gstex_stream_t stream);

/* A training step from the trainer's raw parameters (the demo trainer's
 * per-step activation, example.py:126-143 and 155-171, fused into the
 * batched step instead of a dozen PyTorch ops; no native counterpart in the
 * reference).  gstex_batch_project_keys_raw is gstex_batch_project_keys that
 * first activates each Gaussian from raw_scales [N,3] (log, first two
 * used), raw_quats [N,4] (wxyz, any norm, 16-byte aligned), mapping [N,1,4]
 * (uv0 x, uv0 y, log uv-scale, theta; 16-byte aligned) and raw_opacity [N]
 * (logits, or null to keep opacity) and writes the activated scales [N,3],
 * quats [N,4], uv0 [N,1,2], umap / vmap [N,1,3] and opacity [N], which the
 * later stages of the step read (pass them in gstex_batch_inputs). */
int gstex_batch_project_keys_raw(int num_points, int num_views, const void* views_dev, const float* means,
                                 const float* raw_scales, const float* raw_quats, const float* mapping,
                                 const float* raw_opacity, float glob_scale, const void* sh_coeffs, int sh_dtype,
                                 int sh_degree, int block_width, float* scales, float* quats, float* uv0,
                                 float* umap, float* vmap, float* opacity, float* colors, int32_t* counts,
                                 uint32_t* depth_keys, int32_t* pair_ids, uint32_t* rects, gstex_stream_t stream);

/* Gradients w.r.t. the raw parameters of gstex_batch_project_keys_raw. */
typedef struct gstex_raw_grads {
    const float* raw_quats;  /* [N,4] the step's raw quaternions (16-byte aligned) */
    float* v_raw_scales;     /* [N,3] (third entry 0: the third scale is tied) */
    float* v_raw_quats;      /* [N,4] (16-byte aligned) */
    float* v_mapping;        /* [N,1,4] (16-byte aligned) */
    float* v_raw_opacity;    /* [N], or null when opacity was not activated */
} gstex_raw_grads;

/* gstex_batch_backward carried on through the activation: writes io->v_means,
 * io->v_colors and the raw gradients (io->v_opacity, v_scales, v_quats,
 * v_uv0, v_umap, v_vmap are not written and may be null).  The activated
 * scales and opacities in `in` are the ones the projection wrote. */
int gstex_batch_backward_raw(const gstex_batch_inputs* in, const gstex_backward_io* io, const gstex_raw_grads* raw,
                             gstex_stream_t stream);

/* SH coefficient gradients [N, bases(degree), 3] summed over views, from
 * the [V, N, 4] colour gradients of gstex_batch_backward.  Batched
 * compute_sh_backward. */
int gstex_batch_sh_backward(int num_points, int num_views, const void* views_dev, const float* means,
                            int sh_degree, const float* v_colors, float* v_coeffs, gstex_stream_t stream);

/* The reference demo's image losses (example.py:189-209) over all views,
 * with their gradients; *loss (device) receives the sum over views. */
int gstex_batch_image_loss(long long total_pixels, int num_views, const long long* pix_offsets, int channels,
                           const float* img, const float* tex, const float* normal, const float* reg,
                           const float* tgt_img, const float* tgt_tex, float w_img, float w_tex, float w_reg,
                           float w_normal, float* v_img, float* v_tex, float* v_normal, float* v_reg, float* loss,
                           gstex_stream_t stream);

/* ------------------------------------------------------------------------
 * Parameter activation of a GStex training step on the device: the demo
 * trainer's per-step preprocessing (example.py:126-143 and the opacity
 * sigmoid of example.py:155-171) as one kernel each way.  No native
 * counterpart in the reference (there it is a dozen PyTorch ops).
 *   scales[:, :2] = exp(raw_scales[:, :2]); scales[:, 2] = 1e-5 * mean(scales[:, :2])
 *   quats = raw_quats / |raw_quats|
 *   uv0 = mapping[..., 0:2]
 *   umap = exp(mapping[..., 2]) * ( ax1 cos(theta) + ax2 sin(theta))
 *   vmap = exp(mapping[..., 2]) * (-ax1 sin(theta) + ax2 cos(theta)), theta = mapping[..., 3]
 *   opacity = sigmoid(raw_opacity)            (when raw_opacity is not null)
 * Shapes: raw_scales/scales [N,3], raw_quats/quats [N,4], mapping [N,P,4],
 * uv0 [N,P,2], umap/vmap [N,P,3], raw_opacity/opacity [N]. */
int gstex_preprocess_forward(int N, int P, const float* raw_scales, const float* raw_quats, const float* mapping,
                             const float* raw_opacity, float* scales, float* quats, float* uv0, float* umap,
                             float* vmap, float* opacity, gstex_stream_t stream);

/* The adjoint of gstex_preprocess_forward (null upstream gradients are zero;
 * the third scale is detached, as in the trainer): gradients with respect to
 * raw_scales, raw_quats, mapping and raw_opacity. */
int gstex_preprocess_backward(int N, int P, const float* raw_scales, const float* raw_quats, const float* mapping,
                              const float* raw_opacity, const float* v_scales, const float* v_quats,
                              const float* v_uv0, const float* v_umap, const float* v_vmap, const float* v_opacity,
                              float* v_raw_scales, float* v_raw_quats, float* v_mapping, float* v_raw_opacity,
                              gstex_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* GSTEX_GB300_H */
