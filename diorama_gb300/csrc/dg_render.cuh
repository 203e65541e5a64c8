// Internal view of the renderer's objects, shared with the trainer.
#pragma once
#include "dg_common.cuh"
#include "dg_scan.cuh"

// TileRasterizer (src/tileRasterizer.ts:29-317).
struct dg_tile_rasterizer {
  dg_context* ctx;
  dg_buffer* camera;  // borrowed: the 144-byte Camera uniform
  dg_buffer* splats;  // borrowed
  uint32_t count;
  dg_buffer* tile_offsets;   // per splat: tiles touched, then its first pair slot
  dg_buffer* scan_total;     // PrefixSum.total: pairs this frame needs
  dg_buffer* scan_scratch;
  dg_buffer* raster_params;  // background (rgb, 1)
  // Pairs (createPairs, src/tileRasterizer.ts:276-293)
  uint32_t pair_capacity;
  dg::SortPlan plan;
  dg_buffer* keys;
  dg_buffer* values;
  dg_buffer* keys_alt;
  dg_buffer* values_alt;
  dg_buffer* sort_scratch;
  dg_buffer* ranges;
  uint32_t ranges_tiles;
  dg_buffer* pixel_color;
  dg_buffer* pixel_last;
  uint32_t pixel_count;
  // Pair-count readbacks (src/tileRasterizer.ts:187-191, 229-244): a ring of
  // READBACKS pinned words, each with the event its copy completes, queued one
  // per frame and consumed in order, [readback_tail, readback_head).
  static constexpr uint32_t READBACKS = 4;
  uint32_t* pinned_totals;
  cudaEvent_t readback_events[READBACKS];
  uint32_t readback_head, readback_tail;
  uint32_t last_pair_count;
  uint32_t tiles_x, tiles_y;
  float viewport[2];
  // The depth-first tile sort (the renderer's path, dg_render.cu): splats sorted
  // by depth, their pairs emitted in that order and sorted by tile index alone.
  bool depth_first;
  bool keys_are_tiles;  // the last frame left u32 tile indices in `keys`
  dg::SortPlan depth_plan, tile_plan;
  dg_buffer* depth_keys;
  dg_buffer* depth_values;  // splat indices, sorted by depth
  dg_buffer* depth_keys_alt;
  dg_buffer* depth_values_alt;
  dg_buffer* depth_scratch;
  dg_buffer* counts_sorted;  // tile counts in depth order, then their scan
  dg_buffer* keys64;         // the reference's 64-bit sorted keys, rebuilt on request
  dg_buffer* work;           // item counters of the blend kernels
  // The blend kernels' work plan (plan_kernel, dg_render.cu): tile order, the
  // backward's (tile, chunk) pairs and the forward's per-chunk pixel states.
  dg_buffer* work_plan;
  dg_buffer* chunks;
  dg_buffer* checkpoints;
  dg_buffer* blend_mask;  // which entries each 8x4 block blended (dg_render.cu, publish_blended)
  uint32_t coop_min;      // tiles with more entries are blended by a whole CTA
  bool splat_cutoffs;     // the splats come from this build's preprocess, cutoffs in slot 7
};

namespace dg {
// Host-side preparation of a frame: buffer sizes and the background uniform.
dg_status rasterizer_prepare(dg_tile_rasterizer* tr, const float viewport[2], const float background[3]);
// The frame's kernels. counts_ready: tile_offsets already hold the per-splat
// tile counts (the renderer's preprocess writes them), so count_tiles is skipped.
dg_status rasterizer_launch(dg_tile_rasterizer* tr, dg_buffer* target, bool counts_ready);
// Queues this frame's pair-count readback (waiting for the oldest queued one first
// if the ring is full). Not while a graph is being captured.
dg_status rasterizer_queue_readback(dg_tile_rasterizer* tr);
// Grows the pair buffers to 2^ceil(log2(1.25 * pairs)) if pairs exceed them.
dg_status rasterizer_reserve_pairs(dg_tile_rasterizer* tr, uint64_t pairs);
dg_status rasterizer_launch_backward(dg_tile_rasterizer* tr, dg_buffer* pixel_grads, dg_buffer* splat_grads);
// own_splats: `splats` is written by this build's preprocess (blend cutoffs in slot 7).
dg_status rasterizer_create(dg_context* ctx, dg_buffer* camera, dg_buffer* splats, uint32_t count,
                            uint32_t initial_pair_capacity, bool depth_first, bool own_splats,
                            dg_tile_rasterizer** out);
dg_status launch_rasterize(dg_tile_rasterizer* tr, dg_buffer* target);
// Grid of a persistent blend kernel of `threads` threads per CTA over `items`
// warp items.
uint32_t blend_grid(dg_context* ctx, const void* kernel, uint32_t threads, uint32_t items);

// Blend tiles of 2^twl x 2^thl 16x16 tiles (dg_render_kernels.cuh, blend_rect):
// {0, 0} everywhere but batches of views.
struct BlendShape {
  uint32_t twl, thl;
  bool operator==(const BlendShape& o) const { return twl == o.twl && thl == o.thl; }
};
constexpr uint32_t MAX_BLEND_TILE_LOG2 = 1;  // blend tiles of up to 2 x 2 16x16 tiles

// The forward blend (plan + rasterize kernels) over `tiles` tiles of
// tiles_per_view each; checkpoints, blend_mask and chunks may be NULL when no
// backward pass follows, and must be with blend tiles larger than 16x16.
struct BlendForward {
  const Camera* camera;
  const float4* raster_params;
  const float* splats;
  const uint32_t* pair_splats;
  const uint2* ranges;
  uint32_t tiles, tiles_per_view, coop_min;
  uint32_t* plan;
  uint2* chunks;
  uchar4* target;
  float4* pixel_color;
  uint32_t* pixel_last;
  float4* checkpoints;
  uint32_t* blend_mask;
  uint32_t* counters;  // 4 words, cleared here
  BlendShape shape;
  bool splat_cutoffs;  // the splats carry their blend cutoff (this build's preprocess wrote them)
};
dg_status blend_forward(dg_context* ctx, const BlendForward& f);
// The batched views' stages (dg_render.cu; used by dg_views.cu).
dg_status views_preprocess_launch(dg_context* ctx, const Camera* cameras, uint32_t views, const float* gaussians,
                                  const float* sh, uint32_t count, const uint32_t* scene_params, float* splats,
                                  uint32_t* tile_counts, uint2* depth_keys, uint32_t* order, BlendShape shape);
dg_status duplicate_sorted_launch(dg_context* ctx, const Camera* camera, const float* splats, const uint32_t* order,
                                  const uint32_t* offsets, uint32_t count, uint32_t per_view, uint32_t view_shift,
                                  uint32_t capacity, uint32_t* keys, uint32_t* values, BlendShape shape);
// Per-tile ranges of the sorted pairs of a batch of views (dg_views.cu), whose
// keys are view << view_shift | the view's tile index.
dg_status find_view_ranges_launch(dg_context* ctx, const uint32_t* tile_keys, const uint32_t* pair_total,
                                  uint32_t capacity, uint32_t view_shift, uint32_t tiles_per_view, uint32_t tiles,
                                  uint2* ranges);
dg_buffer* rasterizer_sorted_keys(dg_tile_rasterizer* tr);
}  // namespace dg

struct dg_view_batch;

// GaussianRenderer (src/gaussianRenderer.ts:55-311).
struct dg_renderer {
  dg_context* ctx;
  uint32_t initial_pair_capacity;
  dg_buffer* camera;
  float last_viewport[2];
  // The scene (src/gaussianRenderer.ts:38-48)
  bool has_scene;
  uint32_t count;
  dg_buffer* gaussians;
  dg_buffer* splats;
  dg_buffer* sh;
  dg_buffer* scene_params;  // element 0: SH degree
  dg_buffer* radii;         // each splat's radius of the last preprocess, densely
  dg_tile_rasterizer* rasterizer;
  dg_buffer* grad_splats;
  dg_buffer* grad_gaussians;
  dg_buffer* grad_sh;
  dg_tile_rasterizer* draw_rasterizer;
  // Batched views (dg_views.cu): buffers, views per batch (0: all), the blend's
  // cooperative threshold, the blend tiles, and whether a batch is replayed as a
  // CUDA graph.
  dg_view_batch* views;
  uint32_t view_batch;
  uint32_t view_coop_min;
  dg::BlendShape view_shape;
  bool view_graph;
};

namespace dg {
dg_status renderer_write_camera(dg_renderer* r, const dg_camera* camera);
dg_status renderer_prepare(dg_renderer* r, const dg_camera* camera, const float background[3]);
dg_status renderer_launch_forward(dg_renderer* r, dg_buffer* target);
dg_status renderer_ensure_gradients(dg_renderer* r);
dg_status renderer_launch_backward(dg_renderer* r, dg_buffer* pixel_grads, bool write_gaussian_grads);
const Camera* renderer_camera(dg_renderer* r);
// The backward kernels (dg_render_bwd.cu).
dg_status launch_rasterize_backward(dg_tile_rasterizer* tr, dg_buffer* pixel_grads, dg_buffer* splat_grads);
dg_status launch_preprocess_backward(dg_renderer* r);
struct AdamParams;
// The training step's preprocess backward with Adam applied at once to each
// Gaussian's raw parameters and SH (src/shaders/adam.wgsl:52-106) and the
// densification statistics added up (src/shaders/adam.wgsl:126-134); with
// keep_gradients the gradients are stored as well.
dg_status launch_preprocess_backward_adam(dg_renderer* r, const AdamParams* adam, float* params, float2* moments,
                                         float4* stats, float2* aux, bool keep_gradients);
// Batched views (dg_views.cu): renders count views in batches of `batch` into
// targets (count rgba8 images, may be NULL) and pixel_colors (count vec4 images,
// may be NULL), blending in tiles of `shape`.
dg_status views_render(dg_renderer* r, const dg_camera* cams, uint32_t count, const float bg[3], uchar4* targets,
                       float4* pixel_colors, uint32_t batch, uint32_t coop_min, BlendShape shape);
void view_batch_destroy(dg_view_batch* b);
}  // namespace dg
