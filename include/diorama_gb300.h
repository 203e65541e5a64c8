/*
 * diorama_gb300: the C ABI of a GB300-native 3D Gaussian Splatting renderer and
 * trainer that stands in for seanfourman/diorama's WebGPU path.
 *
 * Every entry point returns a dg_status (0 = DG_OK). On failure,
 * dg_last_error() returns a message for the calling thread. Objects are opaque
 * handles; sizes are plain integers; no entry point takes a framework type.
 *
 * The model the reference's TypeScript classes assume is kept:
 *   - A dg_context is the GPUDevice plus its queue: one CUDA device and one
 *     in-order stream. "encode" entry points enqueue work on that stream right
 *     away; the work runs in call order, as a WebGPU queue runs submissions.
 *   - dg_buffer stands in for GPUBuffer (rgba8unorm textures become byte
 *     buffers of width*height*4). Objects own the buffers they create and free
 *     them in their destroy entry point; "adopt" entry points take ownership.
 *   - Readbacks (dg_buffer_read, *_read, *_after_submit with wait) block until
 *     the work before them is done, like awaiting mapAsync.
 * Each declaration names the reference interface it replaces (path:line in the
 * reference project).
 */
#ifndef DIORAMA_GB300_H
#define DIORAMA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t dg_status;
#define DG_OK 0
#define DG_ERROR_INVALID_ARGUMENT 1 /* a throw new Error(...) in the reference */
#define DG_ERROR_CUDA 2             /* the CUDA runtime failed */
#define DG_ERROR_OUT_OF_MEMORY 3
#define DG_ERROR_DEVICE_WAIT 4 /* a bounded wait on the GPU gave up (see dg_context_check) */
#define DG_ERROR_STATE 5       /* e.g. a backward pass before any forward pass */

typedef struct dg_context dg_context;
typedef struct dg_buffer dg_buffer;
typedef struct dg_prefix_sum dg_prefix_sum;
typedef struct dg_radix_sort dg_radix_sort;
typedef struct dg_tile_rasterizer dg_tile_rasterizer;
typedef struct dg_renderer dg_renderer;
typedef struct dg_training_loss dg_training_loss;
typedef struct dg_trainer dg_trainer;
typedef struct dg_densify_mlp dg_densify_mlp;

/* CameraData (src/gaussianRenderer.ts:11-15): column-major view and proj, viewport in pixels. */
typedef struct dg_camera {
  float view[16];
  float proj[16];
  float viewport[2];
} dg_camera;

/* ---- errors and version */
const char* dg_last_error(void);
int32_t dg_abi_version(void);

/* ---- context: GPUDevice + queue (src/gpu.ts:8-46) */
dg_status dg_context_create(int32_t device, dg_context** out);
dg_status dg_context_destroy(dg_context* ctx);
/* queue.onSubmittedWorkDone(): waits for everything enqueued so far. */
dg_status dg_context_synchronize(dg_context* ctx);
/* Reads and clears the device error word that bounded GPU waits set instead of
 * hanging; returns DG_ERROR_DEVICE_WAIT if any bit was set (bits in *bits). */
dg_status dg_context_check(dg_context* ctx, uint32_t* bits);
/* Number of kernels this library has launched through ctx (for launch accounting). */
dg_status dg_context_launch_count(dg_context* ctx, uint64_t* out);
/* Per-kernel timing: while enabled, every kernel launched outside graph capture is
 * bracketed by CUDA events on the context's stream. The report (synchronizes, then
 * clears) is one line per kernel name: "name launches total_ms". No reference
 * counterpart (the reference only times whole frames, src/checks/tiles.ts:188-218). */
dg_status dg_context_set_kernel_timing(dg_context* ctx, int32_t enabled);
/* Marks the work a profiler started with its collection off records: waits for
 * the context's stream, then starts (enabled = 1) or stops (0) the collection
 * (cudaProfilerStart / cudaProfilerStop). No reference counterpart. */
dg_status dg_context_profile(dg_context* ctx, int32_t enabled);
dg_status dg_context_kernel_timing_report(dg_context* ctx, char* text, uint64_t capacity);

/* ---- events on the context's stream, for timing work enqueued through it
 * (the reference's performance.now() around onSubmittedWorkDone, src/checks/depthSort.ts:148-168). */
typedef struct dg_event dg_event;
dg_status dg_event_create(dg_context* ctx, dg_event** out);
dg_status dg_event_record(dg_event* event);
/* Waits for `end`, then the milliseconds between the two records. */
dg_status dg_event_elapsed(dg_event* start, dg_event* end, float* ms);
dg_status dg_event_destroy(dg_event* event);

/* ---- pinned host memory, for uploads that overlap GPU work. */
dg_status dg_host_alloc(uint64_t bytes, void** out);
dg_status dg_host_free(void* ptr);

/* ---- buffers: device.createBuffer, queue.writeBuffer, readBuffer (src/readback.ts),
 *      encoder.clearBuffer, encoder.copyBufferToBuffer. New buffers are zero-filled. */
dg_status dg_buffer_create(dg_context* ctx, uint64_t bytes, dg_buffer** out);
/* Wraps device memory the caller owns; dg_buffer_destroy then only drops the handle. */
dg_status dg_buffer_wrap(dg_context* ctx, void* device_ptr, uint64_t bytes, dg_buffer** out);
dg_status dg_buffer_destroy(dg_buffer* buffer);
uint64_t dg_buffer_size(const dg_buffer* buffer);
void* dg_buffer_device_pointer(const dg_buffer* buffer);
dg_status dg_buffer_write(dg_buffer* buffer, uint64_t offset, const void* src, uint64_t bytes);
/* Like dg_buffer_write, but src is pinned memory from dg_host_alloc that the caller
 * keeps unchanged until the queue has run the copy (no snapshot is taken). */
dg_status dg_buffer_write_pinned(dg_buffer* buffer, uint64_t offset, const void* src, uint64_t bytes);
dg_status dg_buffer_read(dg_buffer* buffer, uint64_t offset, void* dst, uint64_t bytes);
dg_status dg_buffer_clear(dg_buffer* buffer, uint64_t offset, uint64_t bytes);
dg_status dg_buffer_copy(dg_buffer* src, uint64_t src_offset, dg_buffer* dst, uint64_t dst_offset, uint64_t bytes);

/* ---- PrefixSum (src/prefixSum.ts:10-103): exclusive u32 scan of data, in place.
 * count (nullable) holds in element 0 how many values to scan, at most capacity. */
dg_status dg_prefix_sum_create(dg_context* ctx, dg_buffer* data, uint32_t capacity, dg_buffer* count,
                               dg_prefix_sum** out);
dg_status dg_prefix_sum_encode(dg_prefix_sum* scan);
/* .total: element 0 holds the sum once the scan has run. */
dg_buffer* dg_prefix_sum_total(dg_prefix_sum* scan);
dg_status dg_prefix_sum_destroy(dg_prefix_sum* scan);
/* The same exclusive scan for callers that cannot allocate device memory (a fixed
 * memory budget, no implicit synchronization allowed, or a host that owns every
 * allocation). It has no counterpart in the reference. It allocates nothing: the
 * scan's look-back state lives in a ~32 KB array inside the library that every
 * GPU loading the library holds until exit. data (count u32 values, scanned in
 * place) and total (one u32) are device pointers the caller owns; stream is a
 * cudaStream_t (NULL for the legacy default stream) that must belong to the
 * current device (DG_ERROR_INVALID_ARGUMENT otherwise).
 * At most 16,777,216 values; larger counts return DG_ERROR_INVALID_ARGUMENT.
 * Each call looks up the array's device address on the current device; the
 * first call on a device also loads the library's GPU code there, so make that
 * first call before any stream capture. All calls share the one array, so calls
 * whose work overlaps on the GPU (other streams, other threads) race.
 * A look-back that waits too long gives up instead of hanging; the scan's
 * output is then wrong and a give-up word in the array is set, which
 * dg_prefix_sum_no_alloc_check reports. */
dg_status dg_prefix_sum_no_alloc(void* stream, uint32_t* data, uint32_t count, uint32_t* total);
/* Waits for stream, then reads and clears the give-up word of dg_prefix_sum_no_alloc
 * on the current device: DG_ERROR_DEVICE_WAIT (bits in *bits, which may be NULL)
 * if a scan since the last check gave up, so its results are wrong; DG_OK
 * otherwise. Allocates nothing. No counterpart in the reference. */
dg_status dg_prefix_sum_no_alloc_check(void* stream, uint32_t* bits);
/* Test hook: sets bits in that give-up word, as a look-back that gave up would,
 * so the reporting path can be tested without making a GPU wait run out. */
dg_status dg_prefix_sum_no_alloc_inject_error(void* stream, uint32_t bits);

/* ---- RadixSort (src/radixSort.ts:27-142): stable LSD sort of u32 keys (high_bits = 0)
 * or u64 keys stored as (low word, high word) sorting high_bits bits of the high word,
 * each key carrying a u32 value. Sorted in place in .keys / .values. */
dg_status dg_radix_sort_create(dg_context* ctx, uint32_t capacity, uint32_t high_bits, dg_buffer* count,
                               dg_radix_sort** out);
dg_buffer* dg_radix_sort_keys(dg_radix_sort* sort);
dg_buffer* dg_radix_sort_values(dg_radix_sort* sort);
uint32_t dg_radix_sort_capacity(const dg_radix_sort* sort);
dg_status dg_radix_sort_encode(dg_radix_sort* sort);
dg_status dg_radix_sort_destroy(dg_radix_sort* sort);

/* ---- TileRasterizer (src/tileRasterizer.ts:29-317). camera is a buffer holding the
 * 144-byte Camera uniform; splats FLOATS_PER_SPLAT floats each (Splat2D,
 * src/shaders/common.wgsl:20-26; its padding float, element 7, is not read).
 * initial_pair_capacity 0 picks max(2^16, 8*count) as the reference does. */
dg_status dg_tile_rasterizer_create(dg_context* ctx, dg_buffer* camera, dg_buffer* splats, uint32_t count,
                                    uint32_t initial_pair_capacity, dg_tile_rasterizer** out);
/* target: rgba8 bytes (width*height*4), may be NULL. */
dg_status dg_tile_rasterizer_encode(dg_tile_rasterizer* tr, dg_buffer* target, const float viewport[2],
                                    const float background[3]);
dg_status dg_tile_rasterizer_encode_backward(dg_tile_rasterizer* tr, const float viewport[2],
                                             dg_buffer* pixel_grads, dg_buffer* splat_grads);
/* afterSubmit(): reads back the last frame's pair count and grows the pair buffers
 * to 2^ceil(log2(1.25 * pairs)) if it did not fit. wait = 0 returns at once if the
 * frame has not finished. */
dg_status dg_tile_rasterizer_after_submit(dg_tile_rasterizer* tr, int32_t wait);
uint32_t dg_tile_rasterizer_last_pair_count(const dg_tile_rasterizer* tr);
uint32_t dg_tile_rasterizer_pair_capacity(const dg_tile_rasterizer* tr);
dg_buffer* dg_tile_rasterizer_pair_splats(dg_tile_rasterizer* tr); /* debugBuffers.pairSplats */
dg_buffer* dg_tile_rasterizer_ranges(dg_tile_rasterizer* tr);      /* debugBuffers.ranges */
dg_buffer* dg_tile_rasterizer_pair_keys(dg_tile_rasterizer* tr);   /* sorted (depth, tile) keys */
dg_buffer* dg_tile_rasterizer_pixel_color(dg_tile_rasterizer* tr); /* .pixelColor, vec4 per pixel */
dg_buffer* dg_tile_rasterizer_pixel_last(dg_tile_rasterizer* tr);  /* .pixelLast, u32 per pixel */
dg_buffer* dg_tile_rasterizer_tile_offsets(dg_tile_rasterizer* tr);/* scanned per-splat first pair slots */
dg_buffer* dg_tile_rasterizer_pair_total(dg_tile_rasterizer* tr);  /* element 0: pairs the last frame needed */
dg_status dg_tile_rasterizer_destroy(dg_tile_rasterizer* tr);

/* ---- GaussianRenderer (src/gaussianRenderer.ts:55-311) */
dg_status dg_renderer_create(dg_context* ctx, uint32_t initial_pair_capacity, dg_renderer** out);
/* setGaussians(data, {rest, degree}): count Gaussians of 16 floats; sh_rest may be NULL
 * (then sh_floats must be 0); otherwise sh_floats must equal 45 * count. count 0 clears. */
dg_status dg_renderer_set_gaussians(dg_renderer* r, const float* data, uint32_t count, const float* sh_rest,
                                    uint64_t sh_floats, uint32_t degree);
/* adoptGaussians(count, gaussians, sh, degree): takes ownership of both buffers. */
dg_status dg_renderer_adopt_gaussians(dg_renderer* r, uint32_t count, dg_buffer* gaussians, dg_buffer* sh,
                                      uint32_t degree);
dg_status dg_renderer_set_sh_degree(dg_renderer* r, uint32_t degree);
/* encode(encoder, target, camera, background): target may be NULL. */
dg_status dg_renderer_encode(dg_renderer* r, dg_buffer* target, const dg_camera* camera, const float background[3]);
/* encodeDraw(encoder, target, splats, count, viewport, background) */
dg_status dg_renderer_encode_draw(dg_renderer* r, dg_buffer* target, dg_buffer* splats, uint32_t count,
                                  const float viewport[2], const float background[3]);
/* encodeBackward(encoder, pixelGrads) */
dg_status dg_renderer_encode_backward(dg_renderer* r, dg_buffer* pixel_grads);
dg_status dg_renderer_after_submit(dg_renderer* r, int32_t wait);
uint32_t dg_renderer_count(const dg_renderer* r);
/* The renderer's Splat2D records. Element 7, the padding the reference leaves
 * unwritten, holds the splat's blend cutoff ln(1 / (255 opacity)) - 1e-3 (0 when
 * culled), which the blend kernels read instead of computing it per tile. */
dg_buffer* dg_renderer_splat_buffer(dg_renderer* r);
dg_buffer* dg_renderer_gaussian_buffer(dg_renderer* r);
dg_buffer* dg_renderer_sh_buffer(dg_renderer* r);
dg_buffer* dg_renderer_pixel_buffer(dg_renderer* r);
dg_buffer* dg_renderer_pixel_last_buffer(dg_renderer* r);
dg_buffer* dg_renderer_gradient_gaussians(dg_renderer* r);
dg_buffer* dg_renderer_gradient_sh(dg_renderer* r);
dg_buffer* dg_renderer_gradient_splats(dg_renderer* r);
dg_tile_rasterizer* dg_renderer_tiles(dg_renderer* r);
dg_tile_rasterizer* dg_renderer_draw_tiles(dg_renderer* r);
dg_status dg_renderer_destroy(dg_renderer* r);

/* ---- Batched views. No reference counterpart: the reference renders held-out
 * views one at a time (src/trainer.ts:371-386); these render many views of the
 * scene together, each stage once per batch, with images bit-identical to
 * dg_renderer_encode's. All views must share one viewport. */
/* Renders count views: targets (NULL or count rgba8 images of the viewport,
 * back to back) and pixel_colors (NULL or count vec4 images: rgb, final T). */
dg_status dg_renderer_render_views(dg_renderer* r, const dg_camera* cameras, uint32_t count, const float background[3],
                                   dg_buffer* targets, dg_buffer* pixel_colors);
/* Views per batch (0: all at once), the blend's cooperative threshold (0: the
 * default) and whether a batch replays as one CUDA graph. */
dg_status dg_renderer_set_view_batching(dg_renderer* r, uint32_t batch, uint32_t coop_min, int32_t graph);
dg_status dg_renderer_view_batching(const dg_renderer* r, uint32_t* batch, uint32_t* coop_min);
/* The blend tiles of batched views, in pixels: 16 or 32 wide, 16 or 32 high
 * (default 16x16, the reference's tile). A splat is listed once per blend tile its
 * 16x16-tile rectangle touches, and each pixel blends only its own 16x16 tile's
 * entries, so images are identical for every blend tile; larger ones make fewer
 * pairs to sort and longer lists to walk. No reference counterpart: the
 * reference renders one view at a time in 16x16 tiles
 * (src/shaders/common.wgsl:29). */
dg_status dg_renderer_set_view_tile(dg_renderer* r, uint32_t width, uint32_t height);
dg_status dg_renderer_view_tile(const dg_renderer* r, uint32_t* width, uint32_t* height);
/* The autotuner: times each (views per batch, cooperative threshold) candidate
 * with 16x16 blend tiles on these views, then 32x16, 16x32 and 32x32 blend tiles
 * at the fastest of those, and keeps the fastest (read the blend tile back with
 * dg_renderer_view_tile). seconds (NULL or room for 32) receives each
 * candidate's time in the order tried; tried, how many were tried. */
dg_status dg_renderer_tune_views(dg_renderer* r, const dg_camera* cameras, uint32_t count, const float background[3],
                                 dg_buffer* targets, uint32_t* best_batch, uint32_t* best_coop_min, double* seconds,
                                 uint32_t* tried);
/* The last batch's pixel_last (views x pixels u32), for inspection: positions in
 * the blend tile's list (the 16x16 tile's with 16x16 blend tiles). */
dg_buffer* dg_renderer_views_pixel_last(dg_renderer* r);

/* ---- TrainingLoss (src/trainingLoss.ts:16-130): 0.8 L1 + 0.2 (1 - SSIM). */
dg_status dg_training_loss_create(dg_context* ctx, uint32_t width, uint32_t height, dg_training_loss** out);
/* encode(encoder, rendered, target): rendered vec4 per pixel, target rgba8 bytes. */
dg_status dg_training_loss_encode(dg_training_loss* loss, dg_buffer* rendered, dg_buffer* target);
dg_buffer* dg_training_loss_pixel_grads(dg_training_loss* loss);
dg_buffer* dg_training_loss_pixel_loss(dg_training_loss* loss);
/* read(): Σ pixel_loss + λ of the last encode. */
dg_status dg_training_loss_read(dg_training_loss* loss, double* out);
dg_status dg_training_loss_destroy(dg_training_loss* loss);

/* ---- Trainer (src/trainer.ts:103-446) */

/* TrainingSettings (src/trainer.ts:37-63). DEFAULT_SETTINGS (src/trainer.ts:65-82) via
 * dg_training_settings_default. */
typedef struct dg_training_settings {
  double extent;
  double position_lr_steps;
  double position_lr[2];
  double opacity_lr;
  double scale_lr;
  double rotation_lr;
  double color_lr;
  double sh_lr;
  uint32_t sh_degree_interval;
  uint32_t densify_from;
  uint32_t densify_until;
  uint32_t densify_interval;
  double densify_grad_threshold;
  double percent_dense;
  double min_opacity;
  uint32_t opacity_reset_interval;
  float background[3];
} dg_training_settings;
void dg_training_settings_default(dg_training_settings* out, double extent);

/* TrainingView (src/trainer.ts:20-24): a camera and a photo (rgba8 bytes of the
 * viewport's size). The trainer keeps the pointer; the caller keeps the buffer alive. */
typedef struct dg_training_view {
  dg_camera camera;
  dg_buffer* image;
} dg_training_view;

/* Densification (src/trainer.ts:87-95) */
typedef struct dg_densification {
  uint32_t step, before, after, kept, cloned, split, removed;
} dg_densification;

/* new Trainer(device, {params, sh}, views, settings): params 16 raw floats per
 * Gaussian, sh 45 per Gaussian. Throws (DG_ERROR_INVALID_ARGUMENT) on views of mixed sizes. */
dg_status dg_trainer_create(dg_context* ctx, const float* params, const float* sh, uint32_t count,
                            const dg_training_view* views, uint32_t view_count, const dg_training_settings* settings,
                            dg_trainer** out);
dg_status dg_trainer_step(dg_trainer* t);     /* optimize() then maintain() */
dg_status dg_trainer_optimize(dg_trainer* t); /* render, loss, backward, stats, Adam */
dg_status dg_trainer_maintain(dg_trainer* t); /* densify / reset opacity when due */
dg_status dg_trainer_densify(dg_trainer* t, int32_t prune_large);
dg_status dg_trainer_reset_opacity(dg_trainer* t);
/* exportRaw(): params (16 * count floats) and sh (45 * count floats). */
dg_status dg_trainer_export_raw(dg_trainer* t, float* params, float* sh);
dg_status dg_trainer_last_loss(dg_trainer* t, double* out);
/* The same loss summed on the GPU in a fixed order (8 bytes come back instead of
 * one float per pixel). */
dg_status dg_trainer_loss_value(dg_trainer* t, double* out);
/* The same without waiting (no reference counterpart): request_loss enqueues the
 * last step's sum and its 8-byte copy into pinned memory; take_loss returns the
 * oldest requested value (*ready = 1), blocking until it has arrived when wait is
 * nonzero, else setting *ready = 0 if it has not. At most 16 may be outstanding.
 * A training loop that takes step k's loss after launching step k + 1 keeps the
 * GPU busy while the host reads it. */
dg_status dg_trainer_request_loss(dg_trainer* t);
/* Photos from pinned host memory (no reference counterpart): photos[k] holds view
 * k's rgba8 photo (viewport size, from dg_host_alloc; the caller keeps it alive
 * and unchanged). Each step then copies its photo to the GPU itself, the next
 * step's while the current one runs (two device slots, an upload stream), and the
 * views' image buffers are not read. NULL goes back to the image buffers. */
dg_status dg_trainer_set_host_photos(dg_trainer* t, const void* const* photos, uint32_t count);
dg_status dg_trainer_take_loss(dg_trainer* t, int32_t wait, double* out, int32_t* ready);
/* The index of the view the next optimize() renders (shuffling a new round first
 * if needed, exactly as optimize() would): lets a caller upload that view's photo
 * just in time. */
dg_status dg_trainer_next_view(dg_trainer* t, uint32_t* index);
/* evaluate(views, withSsim): mean PSNR and SSIM of 8-bit-quantized renders, computed on the GPU. */
dg_status dg_trainer_evaluate(dg_trainer* t, const dg_training_view* views, uint32_t view_count, int32_t with_ssim,
                              double* psnr, double* ssim);
uint32_t dg_trainer_iteration(const dg_trainer* t);
dg_status dg_trainer_set_iteration(dg_trainer* t, uint32_t iteration);
uint32_t dg_trainer_sh_degree(const dg_trainer* t);
/* The steps that ran Adam so far, which its bias correction counts (densification
 * steps do not; src/trainer.ts:209,217-218, private there; exposed for checks). */
uint32_t dg_trainer_adam_steps(const dg_trainer* t);
uint32_t dg_trainer_count(const dg_trainer* t);
dg_renderer* dg_trainer_renderer(dg_trainer* t);
dg_buffer* dg_trainer_params(dg_trainer* t);
/* buffers.moments: Adam's (m, v) per slot, the reference's 61 slots per Gaussian
 * (src/trainer.ts:17; MOMENT_SLOTS * 8 bytes per Gaussian) held in two planes:
 * the 16 parameter slots of every Gaussian (count x 16 (m, v), 128-byte records),
 * then the 45 SH slots of every Gaussian (count x 45 (m, v)). The reference
 * interleaves the 61 slots per Gaussian; the planes let Adam move 16-byte groups
 * (a run of Gaussians has its SH moments contiguous, indexed like its SH
 * coefficients). Checkpoint files keep the reference's per-Gaussian order. */
dg_buffer* dg_trainer_moments(dg_trainer* t);
dg_buffer* dg_trainer_stats(dg_trainer* t);
uint32_t dg_trainer_densification_count(const dg_trainer* t);
dg_status dg_trainer_densification(const dg_trainer* t, uint32_t index, dg_densification* out);
/* Runs each optimize() step as one replay of a captured CUDA graph (re-captured
 * when the Gaussian count or the pair capacity changes). enabled = 0 launches each
 * kernel directly. Results are identical either way. */
dg_status dg_trainer_set_graph(dg_trainer* t, int32_t enabled);
/* An optimize() step applies Adam to each Gaussian's gradients as the backward
 * pass produces them, without storing them; enabled = 1 stores them too, in the
 * renderer's gradient buffers (gradients{gaussians, sh}), as the reference's
 * separate passes leave them. The parameters are the same either way. */
dg_status dg_trainer_set_keep_gradients(dg_trainer* t, int32_t enabled);
/* Checkpoints. No reference counterpart: the reference writes trained Gaussians
 * (src/plyWriter.ts) but cannot resume. The file is a .ply whose vertex element
 * starts with writeGaussianPly's 62 properties (so the reference's reader and 3DGS
 * viewers open it as a scene) and goes on with each Gaussian's training state
 * (pad floats, Adam moments, densification statistics); further elements hold the
 * identities, the trainer's counters, the rest of the current round of views and
 * the densification history. A learned densification model and its sample log
 * are not part of it. */
dg_status dg_trainer_save_checkpoint(dg_trainer* t, const char* path);
/* A trainer in the state a checkpoint recorded, over the same views (the same
 * number, in the same order) and settings. */
dg_status dg_trainer_resume(dg_context* ctx, const char* path, const dg_training_view* views, uint32_t view_count,
                            const dg_training_settings* settings, dg_trainer** out);
dg_status dg_trainer_destroy(dg_trainer* t);

/* ---- Learned densification proposal. No reference counterpart: the reference
 * densifies by its gradient threshold alone (src/shaders/densify.wgsl:72-85),
 * which stays the fallback. A candidate's 12 features (DG_MLP_FEATURES):
 *   0 mean view-space gradient norm / threshold   1 gradient samples / interval
 *   2 log(1 + max screen radius)                  3-5 log-scales (raw)
 *   6 opacity                                     7 distance to the training cameras' centroid / extent
 *   8 luminance of the DC colour                  9 age in steps / 1000
 *  10 steps seen over its life / 1000            11 std of the gradient norm samples / threshold */
#define DG_MLP_FEATURES 12
#define DG_MLP_PARAMS 5122
/* The model: MLP 12 -> 64 -> 64 -> 2, GELU, BF16 weights, FP32 accumulation,
 * He-initialized from seed. */
dg_status dg_densify_mlp_create(dg_context* ctx, uint32_t seed, dg_densify_mlp** out);
/* Trains on count labelled samples (host arrays: features [count][12], labels
 * 0/1): sets the input normalization from their mean and deviation, then runs
 * `epochs` shuffled passes of minibatches of `batch` with AdamW (lr,
 * weight_decay). balance_classes weighs each class by count / (2 * its size).
 * mean_loss (NULL or room for `epochs`) receives each epoch's mean cross-entropy. */
dg_status dg_densify_mlp_train(dg_densify_mlp* m, const float* features, const uint8_t* labels, uint32_t count,
                               uint32_t epochs, uint32_t batch, float lr, float weight_decay, int32_t balance_classes,
                               uint32_t seed, double* mean_loss);
/* The gradient of the mean cross-entropy over count labelled samples (host
 * arrays, as for training) at the current weights and normalization, in the
 * DG_MLP_PARAMS layout of dg_densify_mlp_get_weights; the model is not changed. */
dg_status dg_densify_mlp_gradient(dg_densify_mlp* m, const float* features, const uint8_t* labels, uint32_t count,
                                  float* gradient);
/* survive[i] = P(the children of candidate i survive); device buffers holding
 * features [count][12] and survive [count]. */
dg_status dg_densify_mlp_predict(dg_densify_mlp* m, dg_buffer* features, uint32_t count, dg_buffer* survive);
/* The model as DG_MLP_PARAMS FP32 weights (W1 [12][64], b1, W2 [64][64], b2,
 * W3 [64][2], b3) followed by 24 normalization values (mean, 1/deviation). */
dg_status dg_densify_mlp_get_weights(dg_densify_mlp* m, float* out);
dg_status dg_densify_mlp_set_weights(dg_densify_mlp* m, const float* in);
dg_status dg_densify_mlp_destroy(dg_densify_mlp* m);
/* Logs, at each densification, every clone/split candidate's features with the
 * identities of its children; a sample is labelled once `horizon` steps have
 * passed: 1 if any of its children is still alive then. */
dg_status dg_trainer_set_densify_log(dg_trainer* t, int32_t enabled, uint32_t horizon);
/* Moves up to `capacity` labelled samples out of the log (features [n][12],
 * labels [n]; features may be NULL to only count) and sets *count = n and
 * *pending = the samples still waiting for their horizon. */
dg_status dg_trainer_take_densify_samples(dg_trainer* t, float* features, uint8_t* labels, uint32_t capacity,
                                          uint32_t* count, uint32_t* pending);
/* Learned densification: the model scores the plain rule's clone/split
 * candidates; one it is confident about (max(p, 1 - p) >= min_confidence) is
 * densified if p >= 0.5 and kept as it is otherwise; the rest follow the plain
 * rule. NULL restores the plain rule. The trainer does not own the model. */
dg_status dg_trainer_set_densify_mlp(dg_trainer* t, dg_densify_mlp* mlp, float min_confidence);
/* Totals over the learned densifications: candidates scored, confident ones,
 * and of those the ones not densified. */
dg_status dg_trainer_densify_mlp_stats(const dg_trainer* t, uint64_t* scored, uint64_t* confident, uint64_t* vetoed);

/* ---- .ply files (host only; no GPU needed) */
/* parseGaussianPly (src/plyLoader.ts:21-104): the activated Gaussians of a binary
 * little-endian 3DGS .ply (gaussians count × 16 f32, packed like packGaussians;
 * sh_rest count × 45 f32, zero past the file's degree) and its SH degree. With
 * gaussians = sh_rest = NULL only *count and *sh_degree are set. Fails
 * (DG_ERROR_INVALID_ARGUMENT, with the reference's message) where it throws. */
dg_status dg_parse_gaussian_ply(const void* bytes, uint64_t size, uint32_t* count, uint32_t* sh_degree,
                                float* gaussians, float* sh_rest);
/* writeGaussianPly (src/plyWriter.ts:14-43): raw params (count × 16) and sh
 * (count × 45) as .ply bytes. *size gets the file's length; out (capacity bytes)
 * may be NULL to ask for it. */
dg_status dg_write_gaussian_ply(const float* params, const float* sh, uint32_t count, void* out, uint64_t capacity,
                                uint64_t* size);

/* ---- COLMAP sparse reconstructions (host only; no GPU needed) */
typedef struct dg_colmap dg_colmap;
/* TrainingCamera (src/sceneCameras.ts:6-19): a photo's name, size, centre, axes in
 * world space (x right, y down, z forward) and focal lengths in pixels. */
typedef struct dg_training_camera {
  const char* name; /* owned by the reconstruction it came from */
  double width, height;
  double position[3], right[3], down[3], forward[3];
  double fx, fy;
} dg_training_camera;
/* parseColmap (src/colmap.ts:18-31): the contents of cameras.bin, images.bin and
 * points3D.bin. Cameras come sorted by photo name; only SIMPLE_PINHOLE and
 * PINHOLE camera models are accepted, as in the reference. */
dg_status dg_parse_colmap(const void* cameras_bin, uint64_t cameras_size, const void* images_bin,
                          uint64_t images_size, const void* points_bin, uint64_t points_size, dg_colmap** out);
uint32_t dg_colmap_camera_count(const dg_colmap* r);
dg_status dg_colmap_camera(const dg_colmap* r, uint32_t index, dg_training_camera* out);
uint64_t dg_colmap_point_count(const dg_colmap* r);
/* positions: count × 3 f32; colors: count × 3 u8. */
dg_status dg_colmap_points(const dg_colmap* r, float* positions, uint8_t* colors);
dg_status dg_colmap_destroy(dg_colmap* r);

/* ---- Starting Gaussians from a point cloud (src/loadDataset.ts:93-149). */
/* meanNeighborDistance2 (src/loadDataset.ts:124-149, src/shaders/nearestNeighbors.wgsl:13-44):
 * distance2[i] = the mean of the squared distances from point i to its 3 nearest
 * other points (duplicates count; with fewer than 4 points each missing neighbour
 * counts as 3.4e38, so 1 or 2 points give infinity). The same values as the
 * reference's brute force, found through a grid. positions: count × 3 f32 (host);
 * distance2: count f32 (host). Blocks until done. */
dg_status dg_mean_neighbor_distance2(dg_context* ctx, const float* positions, uint32_t count, float* distance2);
/* The same on device buffers: points holds count × 4 f32 (xyz and padding, the
 * reference's points buffer), distance2 count f32. Blocks on one 64-byte readback
 * of the points' bounds; the rest is enqueued on the context's stream. */
dg_status dg_mean_neighbor_distance2_buffers(dg_context* ctx, dg_buffer* points, uint32_t count,
                                             dg_buffer* distance2);
/* initialGaussians (src/loadDataset.ts:99-121): one raw Gaussian per point (params
 * count × 16 f32, host) with the point's position, colour (colors count × 3 u8,
 * host), opacity 0.1, rotation (1, 0, 0, 0) and log-scale 0.5 ln max(distance2,
 * 1e-7) on all three axes; sh (count × 45 f32, host) is zeroed. Blocks. */
dg_status dg_initial_gaussians(dg_context* ctx, const float* positions, const uint8_t* colors, uint32_t count,
                               float* params, float* sh);

#ifdef __cplusplus
}
#endif

#endif /* DIORAMA_GB300_H */
