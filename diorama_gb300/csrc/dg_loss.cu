// TrainingLoss (src/trainingLoss.ts:16-130, src/shaders/loss.wgsl:53-121):
// 0.8 L1 + 0.2 (1 - SSIM) between a render and a photo, with an 11x11 Gaussian
// window (sigma 1.5, zero padding), and its gradient with respect to every
// rendered pixel.
//
// The reference makes 7 dispatches over 5-map and 3-map vec4 buffers (moments,
// blur h, blur v, ssim, blur h, blur v, gradient: ~900 B/pixel of traffic). Here
// it is 2 kernels. Each CTA owns a 16x16 block of pixels, loads its 26x26 halo
// once, and does the separable blurs in shared memory:
//   ssim_kernel:     moments -> blur h -> blur v -> SSIM and its three partials
//   gradient_kernel: partials -> blur h -> blur v -> dL/dpixel and the pixel loss
// Sums run over the taps -5..5 in order, one fused multiply-add per tap (two
// sums per packed FP32 instruction where they pair up); taps past the image add
// exactly 0 (the halo holds zeros there), the same as the WGSL's skipping them.
//
// The same ssim_kernel also measures held-out renders (PSNR and SSIM of the
// 8-bit-quantized image, src/trainer.ts:371-386 and src/metrics.ts) on the GPU.
#include "dg_common.cuh"
#include "dg_loss.cuh"

namespace dg {
namespace {

constexpr int LT = 16;             // pixels per side of a CTA's block
constexpr int HALO = 5;
constexpr int LS = LT + 2 * HALO;  // 26
constexpr float LAMBDA = 0.2f;
constexpr float C1 = 0.0001f;
constexpr float C2 = 0.0009f;

struct Window {
  float w[6];
};

__device__ __forceinline__ float3 load_x(const float4* rendered, int w, int h, int x, int y, bool quantize) {
  if (x < 0 || y < 0 || x >= w || y >= h) return make_float3(0.f, 0.f, 0.f);
  float4 v = rendered[(size_t)y * w + x];
  if (quantize) {
    // src/trainer.ts:381: round(min(1, max(0, v)) * 255) / 255, in double as the
    // TypeScript does, then stored as float32.
    auto q = [](float c) {
      double d = rint((double)fminf(1.0f, fmaxf(0.0f, c)) * 255.0);
      return __double2float_rn(d / 255.0);
    };
    return make_float3(q(v.x), q(v.y), q(v.z));
  }
  return make_float3(v.x, v.y, v.z);
}

// A byte's value as float, v / 255: the loss's float quotient, or for metrics
// (exact_quotient) Float32Array.from(bytes, v => v / 255), the double quotient
// rounded to float.
__device__ __forceinline__ float unorm8(uint32_t v, bool exact_quotient) {
  return exact_quotient ? __double2float_rn(v / 255.0) : (float)v / 255.0f;
}

// The 256 values of unorm8 in shared memory (thread t writes entry t of each
// 256-thread CTA), so a pixel's three channels take three loads, not divisions.
__device__ __forceinline__ void fill_unorm8(float* table, bool exact_quotient) {
  table[threadIdx.x] = unorm8(threadIdx.x, exact_quotient);
}

__device__ __forceinline__ float3 load_y(const uchar4* target, int w, int h, int x, int y, const float* unorm) {
  if (x < 0 || y < 0 || x >= w || y >= h) return make_float3(0.f, 0.f, 0.f);
  uchar4 t = target[(size_t)y * w + x];
  return make_float3(unorm[t.x], unorm[t.y], unorm[t.z]);
}

// Moments, both blurs and the SSIM partials for one 16x16 block. mode 0 (loss):
// writes the three partials and S per channel to `partials` (12 floats per pixel,
// laid out for the gradient pass's paired loads: (dS/dmu_x, dS/dE[x^2]) for r, g, b,
// then dS/dE[xy] rgb, then S rgb). mode 1 (metrics): the render is quantized
// first, and each CTA adds its Σ S and Σ squared error to `sums`.
//
// The x and y sums of each blur, and the x^2 and y^2 ones, run as pairs through
// packed FP32 fused multiply-adds (F2): each lane is the scalar fmaf sum.
__global__ void __launch_bounds__(256) ssim_kernel(const float4* __restrict__ rendered,
                                                   const uchar4* const* __restrict__ target_slot, int w, int h,
                                                   Window win, float* __restrict__ partials, int mode,
                                                   double* __restrict__ sums) {
  __shared__ float2 s_xy[LS][LS][3];   // (x, y) per halo pixel and channel
  __shared__ float2 s_h01[LS][LT][3];  // horizontal blurs of x and y
  __shared__ float2 s_h23[LS][LT][3];  // of x^2 and y^2
  __shared__ float s_h4[LS][LT][3];    // of xy
  __shared__ double s_red[2][8];
  __shared__ float s_unorm[256];
  const uchar4* target = *target_slot;
  const int x0 = blockIdx.x * LT - HALO, y0 = blockIdx.y * LT - HALO;
  const bool metrics = mode == 1;
  fill_unorm8(s_unorm, metrics);
  __syncthreads();
  for (int k = threadIdx.x; k < LS * LS; k += 256) {
    const int ly = k / LS, lx = k % LS;
    float3 xv = load_x(rendered, w, h, x0 + lx, y0 + ly, metrics);
    float3 yv = load_y(target, w, h, x0 + lx, y0 + ly, s_unorm);
    s_xy[ly][lx][0] = make_float2(xv.x, yv.x);
    s_xy[ly][lx][1] = make_float2(xv.y, yv.y);
    s_xy[ly][lx][2] = make_float2(xv.z, yv.z);
  }
  F2 wp[6];
#pragma unroll
  for (int k = 0; k < 6; k++) wp[k] = f2(win.w[k], win.w[k]);
  __syncthreads();
  // Horizontal pass over every halo row, for the 16 output columns, two adjacent
  // columns per item: their 11-tap windows share 10 halo values, read (and
  // squared) once. Each column's sums still run over its taps -5..5 in order.
  for (int k = threadIdx.x; k < LS * (LT / 2) * 3; k += 256) {
    const int ch = k % 3, col = 2 * ((k / 3) % (LT / 2)), row = k / (3 * (LT / 2));
    F2 a01 = f2(0.f, 0.f), a23 = f2(0.f, 0.f), b01 = a01, b23 = a01;
    float a4 = 0.f, b4 = 0.f;
    // Taps past the image read the halo's zeros and add exactly 0: the same sums
    // as skipping them, without a branch per tap.
#pragma unroll
    for (int t = -HALO; t <= HALO + 1; t++) {  // halo column col + HALO + t
      const F2 xy = f2_load(&s_xy[row][col + HALO + t][ch]);
      const F2 sq = f2_mul(xy, xy);
      const float pr = f2_lo(xy) * f2_hi(xy);
      if (t <= HALO) {  // column col, tap t
        const int at = t < 0 ? -t : t;
        a01 = f2_fma(wp[at], xy, a01);  // x, y
        a23 = f2_fma(wp[at], sq, a23);  // x^2, y^2
        a4 = fmaf(win.w[at], pr, a4);   // xy
      }
      if (t > -HALO) {  // column col + 1, tap t - 1
        const int at = t - 1 < 0 ? 1 - t : t - 1;
        b01 = f2_fma(wp[at], xy, b01);
        b23 = f2_fma(wp[at], sq, b23);
        b4 = fmaf(win.w[at], pr, b4);
      }
    }
    f2_store(&s_h01[row][col][ch], a01);
    f2_store(&s_h23[row][col][ch], a23);
    s_h4[row][col][ch] = a4;
    f2_store(&s_h01[row][col + 1][ch], b01);
    f2_store(&s_h23[row][col + 1][ch], b23);
    s_h4[row][col + 1][ch] = b4;
  }
  __syncthreads();
  const int lx = threadIdx.x % LT, ly = threadIdx.x / LT;
  const int gx = blockIdx.x * LT + lx, gy = blockIdx.y * LT + ly;
  const bool inside = gx < w && gy < h;
  double s_sum = 0.0, se_sum = 0.0;
  if (inside) {
    float out[12];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      F2 m01 = f2(0.f, 0.f), m23 = f2(0.f, 0.f);
      float m4 = 0.f;
#pragma unroll
      for (int t = -HALO; t <= HALO; t++) {  // rows past the image were blurred to 0
        const int at = t < 0 ? -t : t;
        m01 = f2_fma(wp[at], f2_load(&s_h01[ly + HALO + t][lx][ch]), m01);
        m23 = f2_fma(wp[at], f2_load(&s_h23[ly + HALO + t][lx][ch]), m23);
        m4 = fmaf(win.w[at], s_h4[ly + HALO + t][lx][ch], m4);
      }
      const float mx = f2_lo(m01), my = f2_hi(m01);
      const float vx = f2_lo(m23) - mx * mx, vy = f2_hi(m23) - my * my, cxy = m4 - mx * my;
      const float a1 = 2.0f * mx * my + C1, a2 = 2.0f * cxy + C2;
      const float b1 = mx * mx + my * my + C1, b2 = vx + vy + C2;
      const float s = a1 * a2 / (b1 * b2);
      out[2 * ch] = s * (2.0f * my / a1 - 2.0f * my / a2 - 2.0f * mx / b1 + 2.0f * mx / b2);
      out[2 * ch + 1] = -s / b2;
      out[6 + ch] = 2.0f * s / a2;
      out[9 + ch] = s;
      if (metrics) {
        s_sum += (double)s;
        const float2 xy = s_xy[ly + HALO][lx + HALO][ch];
        const double d = (double)xy.x - (double)xy.y;
        se_sum += d * d;
      }
    }
    if (!metrics) {
      float4* dst = reinterpret_cast<float4*>(partials + ((size_t)gy * w + gx) * 12);
      dst[0] = make_float4(out[0], out[1], out[2], out[3]);
      dst[1] = make_float4(out[4], out[5], out[6], out[7]);
      dst[2] = make_float4(out[8], out[9], out[10], out[11]);
    }
  }
  if (metrics) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      s_sum += __shfl_xor_sync(0xffffffffu, s_sum, d);
      se_sum += __shfl_xor_sync(0xffffffffu, se_sum, d);
    }
    if ((threadIdx.x & 31) == 0) {
      s_red[0][threadIdx.x >> 5] = s_sum;
      s_red[1][threadIdx.x >> 5] = se_sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0, b = 0;
      for (int k = 0; k < 8; k++) {
        a += s_red[0][k];
        b += s_red[1][k];
      }
      atomicAdd(&sums[0], a);
      atomicAdd(&sums[1], b);
    }
  }
}

// Blurs the three partials and forms dL/dpixel and the pixel loss
// (src/shaders/loss.wgsl:108-121). The first two partials' blurs run as a pair
// of packed FP32 sums.
__global__ void __launch_bounds__(256) gradient_kernel(const float4* __restrict__ rendered,
                                                       const uchar4* const* __restrict__ target_slot, int w, int h,
                                                       Window win, const float* __restrict__ partials,
                                                       float4* __restrict__ pixel_grads, float* __restrict__ pixel_loss) {
  __shared__ float2 s_p01[LS][LS][3];
  __shared__ float s_p2[LS][LS][3];
  __shared__ float2 s_h01[LS][LT][3];
  __shared__ float s_h2[LS][LT][3];
  __shared__ float s_unorm[256];  // read after the barriers below
  const uchar4* target = *target_slot;
  const int x0 = blockIdx.x * LT - HALO, y0 = blockIdx.y * LT - HALO;
  fill_unorm8(s_unorm, false);
  for (int k = threadIdx.x; k < LS * LS; k += 256) {
    const int ly = k / LS, lx = k % LS;
    const int gx = x0 + lx, gy = y0 + ly;
    const bool in = gx >= 0 && gy >= 0 && gx < w && gy < h;
    float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0, q2 = q0;
    if (in) {
      const float4* src = reinterpret_cast<const float4*>(partials + ((size_t)gy * w + gx) * 12);
      q0 = src[0];
      q1 = src[1];
      q2 = src[2];
    }
    s_p01[ly][lx][0] = make_float2(q0.x, q0.y);
    s_p01[ly][lx][1] = make_float2(q0.z, q0.w);
    s_p01[ly][lx][2] = make_float2(q1.x, q1.y);
    s_p2[ly][lx][0] = q1.z;
    s_p2[ly][lx][1] = q1.w;
    s_p2[ly][lx][2] = q2.x;
  }
  F2 wp[6];
#pragma unroll
  for (int k = 0; k < 6; k++) wp[k] = f2(win.w[k], win.w[k]);
  __syncthreads();
  // Two adjacent output columns per item, as in ssim_kernel.
  for (int k = threadIdx.x; k < LS * (LT / 2) * 3; k += 256) {
    const int ch = k % 3, col = 2 * ((k / 3) % (LT / 2)), row = k / (3 * (LT / 2));
    F2 a01 = f2(0.f, 0.f), b01 = a01;
    float a2 = 0.f, b2 = 0.f;
#pragma unroll
    for (int t = -HALO; t <= HALO + 1; t++) {  // the halo holds zeros past the image
      const F2 p01 = f2_load(&s_p01[row][col + HALO + t][ch]);
      const float p2 = s_p2[row][col + HALO + t][ch];
      if (t <= HALO) {  // column col, tap t
        const int at = t < 0 ? -t : t;
        a01 = f2_fma(wp[at], p01, a01);
        a2 = fmaf(win.w[at], p2, a2);
      }
      if (t > -HALO) {  // column col + 1, tap t - 1
        const int at = t - 1 < 0 ? 1 - t : t - 1;
        b01 = f2_fma(wp[at], p01, b01);
        b2 = fmaf(win.w[at], p2, b2);
      }
    }
    f2_store(&s_h01[row][col][ch], a01);
    s_h2[row][col][ch] = a2;
    f2_store(&s_h01[row][col + 1][ch], b01);
    s_h2[row][col + 1][ch] = b2;
  }
  __syncthreads();
  const int lx = threadIdx.x % LT, ly = threadIdx.x / LT;
  const int gx = blockIdx.x * LT + lx, gy = blockIdx.y * LT + ly;
  if (gx >= w || gy >= h) return;
  const size_t p = (size_t)gy * w + gx;
  const float scale = 1.0f / (float)(3u * (uint32_t)(w * h));
  const float4 xv4 = rendered[p];
  const uchar4 t4 = target[p];
  const float xs[3] = {xv4.x, xv4.y, xv4.z};
  const float ys[3] = {s_unorm[t4.x], s_unorm[t4.y], s_unorm[t4.z]};
  const float* own = partials + p * 12;
  float grad[3];
  float lsum = 0.0f;
#pragma unroll
  for (int ch = 0; ch < 3; ch++) {
    F2 m01 = f2(0.f, 0.f);
    float m2 = 0.f;
#pragma unroll
    for (int t = -HALO; t <= HALO; t++) {  // rows past the image were blurred to 0
      const int at = t < 0 ? -t : t;
      m01 = f2_fma(wp[at], f2_load(&s_h01[ly + HALO + t][lx][ch]), m01);
      m2 = fmaf(win.w[at], s_h2[ly + HALO + t][lx][ch], m2);
    }
    const float x = xs[ch], y = ys[ch];
    const float sg = f2_lo(m01) + 2.0f * x * f2_hi(m01) + y * m2;
    const float diff = x - y;
    const float sign = diff > 0.0f ? 1.0f : (diff < 0.0f ? -1.0f : 0.0f);
    grad[ch] = ((1.0f - LAMBDA) * sign - LAMBDA * sg) * scale;
    lsum = lsum + ((1.0f - LAMBDA) * fabsf(diff) - LAMBDA * own[9 + ch]);
  }
  pixel_grads[p] = make_float4(grad[0], grad[1], grad[2], 0.0f);
  pixel_loss[p] = lsum * scale;
}

// Σ pixel_loss in double, in a fixed order (per-CTA partial sums, then one CTA).
__global__ void __launch_bounds__(256) loss_sum_kernel(const float* __restrict__ pixel_loss, uint32_t n,
                                                       double* __restrict__ partial, uint32_t per_block) {
  __shared__ double s[8];
  const uint32_t begin = blockIdx.x * per_block, end = min(n, begin + per_block);
  double acc = 0.0;
  for (uint32_t i = begin + threadIdx.x; i < end; i += 256) acc += (double)pixel_loss[i];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < 8; k++) t += s[k];
    partial[blockIdx.x] = t;
  }
}

__global__ void loss_total_kernel(const double* __restrict__ partial, uint32_t blocks, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0;
    for (uint32_t k = 0; k < blocks; k++) t += partial[k];
    out[0] = t + (double)LAMBDA;
  }
}

Window window_weights() {
  double raw[6], total;
  for (int k = 0; k < 6; k++) raw[k] = std::exp(-(double)(k * k) / (2 * 1.5 * 1.5));
  total = raw[0] + 2 * (raw[1] + raw[2] + raw[3] + raw[4] + raw[5]);
  Window win;
  for (int k = 0; k < 6; k++) win.w[k] = (float)(raw[k] / total);
  return win;
}

}  // namespace

dg_status loss_launch(dg_training_loss* l, dg_buffer* rendered) {
  dg_context* ctx = l->ctx;
  const Window win = window_weights();
  dim3 grid(ceil_div(l->width, LT), ceil_div(l->height, LT));
  DG_LAUNCH(ctx, "loss_ssim",
            ssim_kernel<<<grid, 256, 0, ctx->stream>>>(
                typed<float4>(rendered), typed<const uchar4* const>(l->target_slot), (int)l->width, (int)l->height,
                win, typed<float>(l->partials), 0, nullptr));
  DG_LAUNCH(ctx, "loss_gradient",
            gradient_kernel<<<grid, 256, 0, ctx->stream>>>(
                typed<float4>(rendered), typed<const uchar4* const>(l->target_slot), (int)l->width, (int)l->height,
                win, typed<float>(l->partials), typed<float4>(l->pixel_grads), typed<float>(l->pixel_loss)));
  return DG_OK;
}

dg_status loss_sum_launch(dg_training_loss* l) {
  dg_context* ctx = l->ctx;
  const uint32_t n = l->width * l->height;
  const uint32_t per_block = 4096;
  const uint32_t blocks = std::max(1u, ceil_div(n, per_block));
  DG_LAUNCH(ctx, "loss_sum",
            loss_sum_kernel<<<blocks, 256, 0, ctx->stream>>>(typed<float>(l->pixel_loss), n,
                                                             typed<double>(l->sum_scratch), per_block));
  DG_LAUNCH(ctx, "loss_total",
            loss_total_kernel<<<1, 32, 0, ctx->stream>>>(typed<double>(l->sum_scratch), blocks,
                                                          typed<double>(l->sum_scratch) + l->sum_blocks));
  return DG_OK;
}

dg_status metrics_launch(dg_context* ctx, dg_buffer* rendered, dg_buffer* target_slot, uint32_t width, uint32_t height,
                         double* sums_device) {
  const Window win = window_weights();
  dim3 grid(ceil_div(width, LT), ceil_div(height, LT));
  DG_LAUNCH(ctx, "metrics_ssim",
            ssim_kernel<<<grid, 256, 0, ctx->stream>>>(typed<float4>(rendered),
                                                       typed<const uchar4* const>(target_slot), (int)width,
                                                       (int)height, win, nullptr, 1, sums_device));
  return DG_OK;
}

}  // namespace dg

using namespace dg;

extern "C" {

dg_status dg_training_loss_create(dg_context* ctx, uint32_t width, uint32_t height, dg_training_loss** out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  DG_REQUIRE(width > 0 && height > 0, "empty image");
  auto* l = new dg_training_loss();
  l->ctx = ctx;
  l->width = width;
  l->height = height;
  const size_t pixels = (size_t)width * height;
  l->sum_blocks = std::max(1u, ceil_div(pixels, 4096));
  dg_status st = alloc_buffer(ctx, pixels * 16, &l->pixel_grads);
  if (st == DG_OK) st = alloc_buffer(ctx, pixels * 4, &l->pixel_loss);
  if (st == DG_OK) st = alloc_buffer(ctx, pixels * 12 * 4, &l->partials);
  if (st == DG_OK) st = alloc_buffer(ctx, 8, &l->target_slot);
  if (st == DG_OK) st = alloc_buffer(ctx, (l->sum_blocks + 1) * 8, &l->sum_scratch);
  if (st != DG_OK) {
    dg_training_loss_destroy(l);
    return st;
  }
  *out = l;
  return DG_OK;
}

dg_status dg_training_loss_encode(dg_training_loss* l, dg_buffer* rendered, dg_buffer* target) {
  DG_REQUIRE(l && rendered && target, "NULL argument");
  const uint64_t pixels = (uint64_t)l->width * l->height;
  DG_REQUIRE(rendered->bytes >= pixels * 16, "rendered buffer smaller than the image");
  DG_REQUIRE(target->bytes >= pixels * 4, "target smaller than the image");
  const void* ptr = target->ptr;
  DG_TRY(write_async(l->ctx, l->target_slot->ptr, &ptr, sizeof(ptr)));
  return loss_launch(l, rendered);
}

dg_buffer* dg_training_loss_pixel_grads(dg_training_loss* l) { return l ? l->pixel_grads : nullptr; }
dg_buffer* dg_training_loss_pixel_loss(dg_training_loss* l) { return l ? l->pixel_loss : nullptr; }

dg_status dg_training_loss_read(dg_training_loss* l, double* out) {
  DG_REQUIRE(l && out, "NULL argument");
  const size_t pixels = (size_t)l->width * l->height;
  std::vector<float> shares(pixels);
  DG_CUDA(cudaMemcpyAsync(shares.data(), l->pixel_loss->ptr, pixels * 4, cudaMemcpyDeviceToHost, l->ctx->stream));
  DG_CUDA(cudaStreamSynchronize(l->ctx->stream));
  double sum = 0;
  for (float s : shares) sum += s;
  *out = sum + (double)LAMBDA;
  return DG_OK;
}

dg_status dg_training_loss_destroy(dg_training_loss* l) {
  if (!l) return DG_OK;
  for (dg_buffer* b : {l->pixel_grads, l->pixel_loss, l->partials, l->target_slot, l->sum_scratch}) free_buffer(b);
  delete l;
  return DG_OK;
}

}  // extern "C"
