// The Node-API addon that lets the reference's TypeScript classes run on this
// library: every function here is a thin wrapper over one entry point of
// include/diorama_gb300.h. Handles travel to JavaScript as napi externals;
// numbers, Float32Arrays and Uint8Arrays are copied in and out; a failing status
// becomes a thrown Error with dg_last_error()'s message, which repeats the
// reference's own messages where it throws (src/gaussianRenderer.ts:99-101,
// src/tileRasterizer.ts:135-138, :202, src/trainer.ts:133-135, :295).
//
// Readbacks and training steps are the reference's async methods (mapAsync,
// afterSubmit, Trainer.step): they run on the libuv thread pool as napi async
// work and resolve a Promise, so the JavaScript thread never blocks on the GPU.
//
// Untested: node is not installed on the machines this library was built and
// tested on, so this file has not been compiled. The C ABI it calls is exercised
// by every test through the Python binding (diorama_gb300/_lib.py).
#include <node_api.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/diorama_gb300.h"

namespace {

napi_value Throw(napi_env env) {
  napi_throw_error(env, nullptr, dg_last_error());
  return nullptr;
}

#define DG_CHECK(call)                       \
  do {                                       \
    if ((call) != DG_OK) return Throw(env);  \
  } while (0)

struct Args {
  size_t argc = 8;
  napi_value argv[8];
  Args(napi_env env, napi_callback_info info) { napi_get_cb_info(env, info, &argc, argv, nullptr, nullptr); }
};

template <typename T>
T* External(napi_env env, napi_value v) {
  napi_valuetype type;
  napi_typeof(env, v, &type);
  if (type != napi_external) return nullptr;  // undefined / null: an optional handle left out
  void* p = nullptr;
  napi_get_value_external(env, v, &p);
  return static_cast<T*>(p);
}

napi_value Wrap(napi_env env, void* p) {
  napi_value out;
  napi_create_external(env, p, nullptr, nullptr, &out);
  return out;
}

uint32_t U32(napi_env env, napi_value v) {
  uint32_t x = 0;
  napi_get_value_uint32(env, v, &x);
  return x;
}

double F64(napi_env env, napi_value v) {
  double x = 0;
  napi_get_value_double(env, v, &x);
  return x;
}

napi_value Number(napi_env env, double x) {
  napi_value out;
  napi_create_double(env, x, &out);
  return out;
}

napi_value Undefined(napi_env env) {
  napi_value out;
  napi_get_undefined(env, &out);
  return out;
}

// The bytes of a TypedArray argument (pointer and length in bytes).
void* Bytes(napi_env env, napi_value v, size_t* bytes) {
  napi_typedarray_type type;
  size_t length = 0, offset = 0;
  void* data = nullptr;
  napi_value buffer;
  napi_get_typedarray_info(env, v, &type, &length, &data, &buffer, &offset);
  size_t element = 1;
  if (type == napi_float32_array || type == napi_uint32_array || type == napi_int32_array) element = 4;
  *bytes = length * element;
  return data;
}

void Floats(napi_env env, napi_value v, float* out, uint32_t n) {
  bool is_array = false;
  napi_is_array(env, v, &is_array);
  if (is_array) {
    for (uint32_t k = 0; k < n; k++) {
      napi_value e;
      napi_get_element(env, v, k, &e);
      out[k] = (float)F64(env, e);
    }
    return;
  }
  size_t bytes = 0;
  const void* p = Bytes(env, v, &bytes);
  std::memcpy(out, p, std::min<size_t>(bytes, n * sizeof(float)));
}

napi_value Property(napi_env env, napi_value object, const char* name) {
  napi_value v;
  napi_get_named_property(env, object, name, &v);
  return v;
}

// CameraData (src/gaussianRenderer.ts:11-15): {view, proj, viewport}.
dg_camera Camera(napi_env env, napi_value v) {
  dg_camera c{};
  Floats(env, Property(env, v, "view"), c.view, 16);
  Floats(env, Property(env, v, "proj"), c.proj, 16);
  Floats(env, Property(env, v, "viewport"), c.viewport, 2);
  return c;
}

// ---- device, queue and buffers (src/gpu.ts, src/readback.ts)

napi_value ContextCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  dg_context* ctx = nullptr;
  DG_CHECK(dg_context_create(a.argc > 0 ? (int32_t)U32(env, a.argv[0]) : 0, &ctx));
  return Wrap(env, ctx);
}

napi_value ContextDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_context_destroy(External<dg_context>(env, a.argv[0])));
  return Undefined(env);
}

napi_value BufferCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  dg_buffer* b = nullptr;
  DG_CHECK(dg_buffer_create(External<dg_context>(env, a.argv[0]), (uint64_t)F64(env, a.argv[1]), &b));
  return Wrap(env, b);
}

napi_value BufferDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_buffer_destroy(External<dg_buffer>(env, a.argv[0])));
  return Undefined(env);
}

// queue.writeBuffer(buffer, offset, data)
napi_value BufferWrite(napi_env env, napi_callback_info info) {
  Args a(env, info);
  size_t bytes = 0;
  const void* src = Bytes(env, a.argv[2], &bytes);
  DG_CHECK(dg_buffer_write(External<dg_buffer>(env, a.argv[0]), (uint64_t)F64(env, a.argv[1]), src, bytes));
  return Undefined(env);
}

// readBuffer(device, buffer): Promise<ArrayBuffer>, read on the thread pool.
struct ReadWork {
  napi_async_work work;
  napi_deferred deferred;
  dg_buffer* buffer;
  std::vector<uint8_t> bytes;
  dg_status status;
  std::string error;
};

void ReadExecute(napi_env, void* data) {
  auto* w = static_cast<ReadWork*>(data);
  w->bytes.resize(dg_buffer_size(w->buffer));
  w->status = dg_buffer_read(w->buffer, 0, w->bytes.data(), w->bytes.size());
  if (w->status != DG_OK) w->error = dg_last_error();
}

void Settle(napi_env env, napi_deferred deferred, dg_status status, const std::string& error, napi_value value) {
  if (status == DG_OK) {
    napi_resolve_deferred(env, deferred, value);
  } else {
    napi_value msg, err;
    napi_create_string_utf8(env, error.c_str(), NAPI_AUTO_LENGTH, &msg);
    napi_create_error(env, nullptr, msg, &err);
    napi_reject_deferred(env, deferred, err);
  }
}

void ReadComplete(napi_env env, napi_status, void* data) {
  auto* w = static_cast<ReadWork*>(data);
  napi_value out = Undefined(env);
  if (w->status == DG_OK) {
    void* dst = nullptr;
    napi_create_arraybuffer(env, w->bytes.size(), &dst, &out);
    std::memcpy(dst, w->bytes.data(), w->bytes.size());
  }
  Settle(env, w->deferred, w->status, w->error, out);
  napi_delete_async_work(env, w->work);
  delete w;
}

napi_value BufferRead(napi_env env, napi_callback_info info) {
  Args a(env, info);
  auto* w = new ReadWork{};
  w->buffer = External<dg_buffer>(env, a.argv[0]);
  napi_value promise, name;
  napi_create_promise(env, &w->deferred, &promise);
  napi_create_string_utf8(env, "dg_buffer_read", NAPI_AUTO_LENGTH, &name);
  napi_create_async_work(env, nullptr, name, ReadExecute, ReadComplete, w, &w->work);
  napi_queue_async_work(env, w->work);
  return promise;
}

// ---- PrefixSum (src/prefixSum.ts:10-103)

napi_value PrefixSumCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  dg_prefix_sum* s = nullptr;
  DG_CHECK(dg_prefix_sum_create(External<dg_context>(env, a.argv[0]), External<dg_buffer>(env, a.argv[1]),
                                U32(env, a.argv[2]), a.argc > 3 ? External<dg_buffer>(env, a.argv[3]) : nullptr,
                                &s));
  return Wrap(env, s);
}

napi_value PrefixSumEncode(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_prefix_sum_encode(External<dg_prefix_sum>(env, a.argv[0])));
  return Undefined(env);
}

napi_value PrefixSumTotal(napi_env env, napi_callback_info info) {
  Args a(env, info);
  return Wrap(env, dg_prefix_sum_total(External<dg_prefix_sum>(env, a.argv[0])));
}

napi_value PrefixSumDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_prefix_sum_destroy(External<dg_prefix_sum>(env, a.argv[0])));
  return Undefined(env);
}

// ---- RadixSort (src/radixSort.ts:27-142)

napi_value RadixSortCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  dg_radix_sort* s = nullptr;
  DG_CHECK(dg_radix_sort_create(External<dg_context>(env, a.argv[0]), U32(env, a.argv[1]),
                                a.argc > 2 ? U32(env, a.argv[2]) : 0,
                                a.argc > 3 ? External<dg_buffer>(env, a.argv[3]) : nullptr, &s));
  return Wrap(env, s);
}

napi_value RadixSortKeys(napi_env env, napi_callback_info info) {
  Args a(env, info);
  return Wrap(env, dg_radix_sort_keys(External<dg_radix_sort>(env, a.argv[0])));
}

napi_value RadixSortValues(napi_env env, napi_callback_info info) {
  Args a(env, info);
  return Wrap(env, dg_radix_sort_values(External<dg_radix_sort>(env, a.argv[0])));
}

napi_value RadixSortEncode(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_radix_sort_encode(External<dg_radix_sort>(env, a.argv[0])));
  return Undefined(env);
}

napi_value RadixSortDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_radix_sort_destroy(External<dg_radix_sort>(env, a.argv[0])));
  return Undefined(env);
}

// ---- GaussianRenderer (src/gaussianRenderer.ts:55-311)

napi_value RendererCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  dg_renderer* r = nullptr;
  DG_CHECK(dg_renderer_create(External<dg_context>(env, a.argv[0]), a.argc > 1 ? U32(env, a.argv[1]) : 0, &r));
  return Wrap(env, r);
}

// setGaussians(data, {rest, degree}?)
napi_value RendererSetGaussians(napi_env env, napi_callback_info info) {
  Args a(env, info);
  size_t bytes = 0, sh_bytes = 0;
  const float* data = static_cast<const float*>(Bytes(env, a.argv[1], &bytes));
  const float* rest = nullptr;
  uint32_t degree = 0;
  if (a.argc > 2) {
    napi_valuetype type;
    napi_typeof(env, a.argv[2], &type);
    if (type == napi_object) {
      rest = static_cast<const float*>(Bytes(env, Property(env, a.argv[2], "rest"), &sh_bytes));
      degree = U32(env, Property(env, a.argv[2], "degree"));
    }
  }
  DG_CHECK(dg_renderer_set_gaussians(External<dg_renderer>(env, a.argv[0]), data, (uint32_t)(bytes / 64), rest,
                                     sh_bytes / 4, degree));
  return Undefined(env);
}

napi_value RendererSetShDegree(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_renderer_set_sh_degree(External<dg_renderer>(env, a.argv[0]), U32(env, a.argv[1])));
  return Undefined(env);
}

// encode(encoder, target, camera, background): the encoder argument is dropped
// (work is enqueued at once on the context's in-order stream).
napi_value RendererEncode(napi_env env, napi_callback_info info) {
  Args a(env, info);
  const dg_camera cam = Camera(env, a.argv[2]);
  float bg[3] = {0, 0, 0};
  Floats(env, a.argv[3], bg, 3);
  DG_CHECK(dg_renderer_encode(External<dg_renderer>(env, a.argv[0]), External<dg_buffer>(env, a.argv[1]), &cam, bg));
  return Undefined(env);
}

napi_value RendererEncodeBackward(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_renderer_encode_backward(External<dg_renderer>(env, a.argv[0]), External<dg_buffer>(env, a.argv[1])));
  return Undefined(env);
}

napi_value RendererAfterSubmit(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_renderer_after_submit(External<dg_renderer>(env, a.argv[0]), 1));
  return Undefined(env);
}

// The renderer's buffer getters, by name: splatBuffer, gaussianBuffer, shBuffer,
// pixelBuffer, pixelLastBuffer, gradients.{gaussians, sh, splats}.
napi_value RendererBuffer(napi_env env, napi_callback_info info) {
  Args a(env, info);
  auto* r = External<dg_renderer>(env, a.argv[0]);
  char name[32] = {0};
  size_t len = 0;
  napi_get_value_string_utf8(env, a.argv[1], name, sizeof name, &len);
  const std::string n(name);
  dg_buffer* b = n == "splat"       ? dg_renderer_splat_buffer(r)
                 : n == "gaussian"  ? dg_renderer_gaussian_buffer(r)
                 : n == "sh"        ? dg_renderer_sh_buffer(r)
                 : n == "pixel"     ? dg_renderer_pixel_buffer(r)
                 : n == "pixelLast" ? dg_renderer_pixel_last_buffer(r)
                 : n == "gradGaussians" ? dg_renderer_gradient_gaussians(r)
                 : n == "gradSh"        ? dg_renderer_gradient_sh(r)
                 : n == "gradSplats"    ? dg_renderer_gradient_splats(r)
                                        : nullptr;
  return b ? Wrap(env, b) : Undefined(env);
}

napi_value RendererDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_renderer_destroy(External<dg_renderer>(env, a.argv[0])));
  return Undefined(env);
}

// ---- TrainingLoss (src/trainingLoss.ts:16-130)

napi_value LossCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  dg_training_loss* l = nullptr;
  DG_CHECK(dg_training_loss_create(External<dg_context>(env, a.argv[0]), U32(env, a.argv[1]), U32(env, a.argv[2]),
                                   &l));
  return Wrap(env, l);
}

napi_value LossEncode(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_training_loss_encode(External<dg_training_loss>(env, a.argv[0]), External<dg_buffer>(env, a.argv[1]),
                                   External<dg_buffer>(env, a.argv[2])));
  return Undefined(env);
}

napi_value LossPixelGrads(napi_env env, napi_callback_info info) {
  Args a(env, info);
  return Wrap(env, dg_training_loss_pixel_grads(External<dg_training_loss>(env, a.argv[0])));
}

napi_value LossRead(napi_env env, napi_callback_info info) {
  Args a(env, info);
  double v = 0;
  DG_CHECK(dg_training_loss_read(External<dg_training_loss>(env, a.argv[0]), &v));
  return Number(env, v);
}

napi_value LossDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_training_loss_destroy(External<dg_training_loss>(env, a.argv[0])));
  return Undefined(env);
}

// ---- Trainer (src/trainer.ts:103-446)

// TrainingSettings from a JavaScript object with the reference's field names.
dg_training_settings Settings(napi_env env, napi_value v) {
  dg_training_settings s;
  dg_training_settings_default(&s, F64(env, Property(env, v, "extent")));
  s.position_lr_steps = F64(env, Property(env, v, "positionLrSteps"));
  napi_value lr = Property(env, v, "positionLr"), e0, e1;
  napi_get_element(env, lr, 0, &e0);
  napi_get_element(env, lr, 1, &e1);
  s.position_lr[0] = F64(env, e0);
  s.position_lr[1] = F64(env, e1);
  s.opacity_lr = F64(env, Property(env, v, "opacityLr"));
  s.scale_lr = F64(env, Property(env, v, "scaleLr"));
  s.rotation_lr = F64(env, Property(env, v, "rotationLr"));
  s.color_lr = F64(env, Property(env, v, "colorLr"));
  s.sh_lr = F64(env, Property(env, v, "shLr"));
  s.sh_degree_interval = U32(env, Property(env, v, "shDegreeInterval"));
  s.densify_from = U32(env, Property(env, v, "densifyFrom"));
  s.densify_until = U32(env, Property(env, v, "densifyUntil"));
  s.densify_interval = U32(env, Property(env, v, "densifyInterval"));
  s.densify_grad_threshold = F64(env, Property(env, v, "densifyGradThreshold"));
  s.percent_dense = F64(env, Property(env, v, "percentDense"));
  s.min_opacity = F64(env, Property(env, v, "minOpacity"));
  s.opacity_reset_interval = U32(env, Property(env, v, "opacityResetInterval"));
  Floats(env, Property(env, v, "background"), s.background, 3);
  return s;
}

// TrainingView[] ({camera, image: buffer handle}).
std::vector<dg_training_view> Views(napi_env env, napi_value v) {
  uint32_t n = 0;
  napi_get_array_length(env, v, &n);
  std::vector<dg_training_view> out(n);
  for (uint32_t k = 0; k < n; k++) {
    napi_value e;
    napi_get_element(env, v, k, &e);
    out[k].camera = Camera(env, Property(env, e, "camera"));
    out[k].image = External<dg_buffer>(env, Property(env, e, "image"));
  }
  return out;
}

// new Trainer(device, {params, sh}, views, settings)
napi_value TrainerCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  size_t pb = 0, sb = 0;
  const float* params = static_cast<const float*>(Bytes(env, Property(env, a.argv[1], "params"), &pb));
  const float* sh = static_cast<const float*>(Bytes(env, Property(env, a.argv[1], "sh"), &sb));
  const auto views = Views(env, a.argv[2]);
  const dg_training_settings s = Settings(env, a.argv[3]);
  dg_trainer* t = nullptr;
  DG_CHECK(dg_trainer_create(External<dg_context>(env, a.argv[0]), params, sh, (uint32_t)(pb / 64), views.data(),
                             (uint32_t)views.size(), &s, &t));
  return Wrap(env, t);
}

// step(): Promise<void>, on the thread pool (the step enqueues its kernels and,
// on densification steps, reads back the new count, as the reference awaits it).
struct StepWork {
  napi_async_work work;
  napi_deferred deferred;
  dg_trainer* t;
  dg_status status;
  std::string error;
};

void StepExecute(napi_env, void* data) {
  auto* w = static_cast<StepWork*>(data);
  w->status = dg_trainer_step(w->t);
  if (w->status != DG_OK) w->error = dg_last_error();
}

void StepComplete(napi_env env, napi_status, void* data) {
  auto* w = static_cast<StepWork*>(data);
  Settle(env, w->deferred, w->status, w->error, Undefined(env));
  napi_delete_async_work(env, w->work);
  delete w;
}

napi_value TrainerStep(napi_env env, napi_callback_info info) {
  Args a(env, info);
  auto* w = new StepWork{};
  w->t = External<dg_trainer>(env, a.argv[0]);
  napi_value promise, name;
  napi_create_promise(env, &w->deferred, &promise);
  napi_create_string_utf8(env, "dg_trainer_step", NAPI_AUTO_LENGTH, &name);
  napi_create_async_work(env, nullptr, name, StepExecute, StepComplete, w, &w->work);
  napi_queue_async_work(env, w->work);
  return promise;
}

napi_value TrainerLastLoss(napi_env env, napi_callback_info info) {
  Args a(env, info);
  double v = 0;
  DG_CHECK(dg_trainer_last_loss(External<dg_trainer>(env, a.argv[0]), &v));
  return Number(env, v);
}

// evaluate(views, withSsim): {psnr, ssim}
napi_value TrainerEvaluate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  const auto views = Views(env, a.argv[1]);
  bool with_ssim = true;
  if (a.argc > 2) napi_get_value_bool(env, a.argv[2], &with_ssim);
  double psnr = 0, ssim = 0;
  DG_CHECK(dg_trainer_evaluate(External<dg_trainer>(env, a.argv[0]), views.data(), (uint32_t)views.size(),
                               with_ssim ? 1 : 0, &psnr, &ssim));
  napi_value out;
  napi_create_object(env, &out);
  napi_set_named_property(env, out, "psnr", Number(env, psnr));
  napi_set_named_property(env, out, "ssim", Number(env, with_ssim ? ssim : NAN));
  return out;
}

// exportRaw(): {params: Float32Array, sh: Float32Array}
napi_value TrainerExportRaw(napi_env env, napi_callback_info info) {
  Args a(env, info);
  auto* t = External<dg_trainer>(env, a.argv[0]);
  const uint32_t n = dg_trainer_count(t);
  napi_value pbuf, sbuf, params, sh, out;
  void *pd = nullptr, *sd = nullptr;
  napi_create_arraybuffer(env, (size_t)n * 64, &pd, &pbuf);
  napi_create_arraybuffer(env, (size_t)n * 180, &sd, &sbuf);
  DG_CHECK(dg_trainer_export_raw(t, static_cast<float*>(pd), static_cast<float*>(sd)));
  napi_create_typedarray(env, napi_float32_array, (size_t)n * 16, pbuf, 0, &params);
  napi_create_typedarray(env, napi_float32_array, (size_t)n * 45, sbuf, 0, &sh);
  napi_create_object(env, &out);
  napi_set_named_property(env, out, "params", params);
  napi_set_named_property(env, out, "sh", sh);
  return out;
}

napi_value TrainerCount(napi_env env, napi_callback_info info) {
  Args a(env, info);
  return Number(env, dg_trainer_count(External<dg_trainer>(env, a.argv[0])));
}

napi_value TrainerIteration(napi_env env, napi_callback_info info) {
  Args a(env, info);
  return Number(env, dg_trainer_iteration(External<dg_trainer>(env, a.argv[0])));
}

napi_value TrainerRenderer(napi_env env, napi_callback_info info) {
  Args a(env, info);
  return Wrap(env, dg_trainer_renderer(External<dg_trainer>(env, a.argv[0])));
}

napi_value TrainerDestroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  DG_CHECK(dg_trainer_destroy(External<dg_trainer>(env, a.argv[0])));
  return Undefined(env);
}

napi_value Init(napi_env env, napi_value exports) {
  const napi_property_descriptor fns[] = {
      {"contextCreate", nullptr, ContextCreate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"contextDestroy", nullptr, ContextDestroy, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"bufferCreate", nullptr, BufferCreate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"bufferDestroy", nullptr, BufferDestroy, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"bufferWrite", nullptr, BufferWrite, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"bufferRead", nullptr, BufferRead, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"prefixSumCreate", nullptr, PrefixSumCreate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"prefixSumEncode", nullptr, PrefixSumEncode, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"prefixSumTotal", nullptr, PrefixSumTotal, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"prefixSumDestroy", nullptr, PrefixSumDestroy, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"radixSortCreate", nullptr, RadixSortCreate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"radixSortKeys", nullptr, RadixSortKeys, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"radixSortValues", nullptr, RadixSortValues, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"radixSortEncode", nullptr, RadixSortEncode, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"radixSortDestroy", nullptr, RadixSortDestroy, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererCreate", nullptr, RendererCreate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererSetGaussians", nullptr, RendererSetGaussians, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererSetShDegree", nullptr, RendererSetShDegree, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererEncode", nullptr, RendererEncode, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererEncodeBackward", nullptr, RendererEncodeBackward, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererAfterSubmit", nullptr, RendererAfterSubmit, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererBuffer", nullptr, RendererBuffer, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"rendererDestroy", nullptr, RendererDestroy, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"lossCreate", nullptr, LossCreate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"lossEncode", nullptr, LossEncode, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"lossPixelGrads", nullptr, LossPixelGrads, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"lossRead", nullptr, LossRead, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"lossDestroy", nullptr, LossDestroy, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerCreate", nullptr, TrainerCreate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerStep", nullptr, TrainerStep, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerLastLoss", nullptr, TrainerLastLoss, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerEvaluate", nullptr, TrainerEvaluate, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerExportRaw", nullptr, TrainerExportRaw, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerCount", nullptr, TrainerCount, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerIteration", nullptr, TrainerIteration, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerRenderer", nullptr, TrainerRenderer, nullptr, nullptr, nullptr, napi_default, nullptr},
      {"trainerDestroy", nullptr, TrainerDestroy, nullptr, nullptr, nullptr, napi_default, nullptr},
  };
  napi_define_properties(env, exports, sizeof fns / sizeof fns[0], fns);
  return exports;
}

}  // namespace

NAPI_MODULE(NODE_GYP_MODULE_NAME, Init)
