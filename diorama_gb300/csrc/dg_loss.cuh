// Internal view of TrainingLoss, shared with the trainer.
#pragma once
#include "dg_common.cuh"

struct dg_training_loss {
  dg_context* ctx;
  uint32_t width, height;
  dg_buffer* pixel_grads;  // vec4 per pixel
  dg_buffer* pixel_loss;   // f32 per pixel
  dg_buffer* partials;     // 12 floats per pixel: three SSIM partials and S, rgb each
  dg_buffer* target_slot;  // device pointer to the photo (rgba8), read by the kernels
  dg_buffer* sum_scratch;  // per-block partial sums, then the total
  uint32_t sum_blocks;
};

namespace dg {
// Both loss kernels; the photo is whatever target_slot points at when they run.
dg_status loss_launch(dg_training_loss* l, dg_buffer* rendered);
// Σ pixel_loss + λ into sum_scratch[sum_blocks] (a double), in a fixed order.
dg_status loss_sum_launch(dg_training_loss* l);
// Adds Σ SSIM and Σ squared error of the 8-bit-quantized render against the photo
// to sums_device[0] and [1].
dg_status metrics_launch(dg_context* ctx, dg_buffer* rendered, dg_buffer* target_slot, uint32_t width, uint32_t height,
                         double* sums_device);
}  // namespace dg
