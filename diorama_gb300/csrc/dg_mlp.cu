// The learned densification proposal's model: an MLP 12 -> 64 -> 64 -> 2 with
// GELU activations, BF16 weights and activations, FP32 accumulation, scoring
// whether a clone/split candidate's children survive pruning. No reference
// counterpart: the reference densifies by its gradient threshold alone
// (src/shaders/densify.wgsl:72-85), which stays the fallback.
//
// Every product runs on the tensor cores with BF16 operands and FP32 accumulation:
// - inference (mlp_predict_kernel, once per densification over every candidate):
//   tcgen05.mma, 128 candidates a CTA, each layer one 128 x N product issued by
//   one thread from shared-memory descriptors into tensor memory, read back with
//   tcgen05.ld for the bias and GELU;
// - training (mlp_train_kernel), as mma.sync m16n8k16, one warp per 16 samples
//   (its backward needs the activations in registers per warp):
// - forward: X W1, A1 W2, A2 W3, the outputs of one layer feeding the next as
//   register fragments (the C fragments of two adjacent 8-column tiles are the A
//   fragment of one 16-deep step);
// - backward: dZ3 W3^T and dZ2 W2^T the same way, then the weight gradients
//   X^T dZ1, A1^T dZ2, A2^T dZ3 over a CTA's 64 samples from transposed copies in
//   shared memory, added to FP32 accumulators;
// - AdamW on FP32 master weights, which are then repacked to BF16 in the layouts
//   the fragments read.
#include "dg_common.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

namespace dg {
namespace {

constexpr uint32_t IN = 12, IN_PAD = 16, HID = 64, OUT = 2, OUT_PAD = 8, OUT_K = 16;
constexpr uint32_t MLP_THREADS = 128;  // 4 warps x 16 samples
constexpr uint32_t ROWS = 64;          // samples per CTA
// Master parameter layout (FP32): W1 [IN][HID], b1 [HID], W2 [HID][HID], b2 [HID], W3 [HID][OUT], b3 [OUT].
constexpr uint32_t OFF_W1 = 0, OFF_B1 = OFF_W1 + IN * HID, OFF_W2 = OFF_B1 + HID, OFF_B2 = OFF_W2 + HID * HID,
                   OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + HID * OUT, PARAMS = OFF_B3 + OUT;
// Packed BF16 layouts, each [n][k] (k contiguous) as the B fragments read them.
constexpr uint32_t P_W1T = 0;                    // [HID out][IN_PAD in]
constexpr uint32_t P_W2T = P_W1T + HID * IN_PAD;  // [HID out][HID in]
constexpr uint32_t P_W3T = P_W2T + HID * HID;     // [OUT_PAD out][HID in]
constexpr uint32_t P_W2B = P_W3T + OUT_PAD * HID;  // [HID in][HID out]: W2^T as B
constexpr uint32_t P_W3B = P_W2B + HID * HID;      // [HID in][OUT_K out]: W3^T as B
constexpr uint32_t PACKED = P_W3B + HID * OUT_K;

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// The B fragment of the 16x8 block (k0.., n0..) of a [n][k] BF16 matrix with row length K.
__device__ __forceinline__ void load_b(const __nv_bfloat16* __restrict__ m, uint32_t K, uint32_t n0, uint32_t k0,
                                       uint32_t lane, uint32_t& b0, uint32_t& b1) {
  const uint32_t g = lane >> 2, t = lane & 3u;
  const __nv_bfloat16* row = m + (size_t)(n0 + g) * K + k0 + 2 * t;
  b0 = *reinterpret_cast<const uint32_t*>(row);
  b1 = *reinterpret_cast<const uint32_t*>(row + 8);
}

// GELU, 0.5 x (1 + erf(x / sqrt 2)), and its derivative.
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// The A fragment of one 16-deep step from two adjacent 8-column C tiles.
__device__ __forceinline__ void to_a(const float (&lo)[4], const float (&hi)[4], uint32_t (&a)[4]) {
  a[0] = pack2(lo[0], lo[1]);
  a[1] = pack2(lo[2], lo[3]);
  a[2] = pack2(hi[0], hi[1]);
  a[3] = pack2(hi[2], hi[3]);
}

// One warp's 16 samples starting at `first` (rows past n are zeros): the
// normalized input as an A fragment, and its FP32 values for the weight gradient.
__device__ __forceinline__ void load_input(const float* __restrict__ features, const uint32_t* __restrict__ order,
                                           uint32_t first, uint32_t n, const float* __restrict__ norm, uint32_t lane,
                                           uint32_t (&a)[4], float (&x)[8]) {
  const uint32_t g = lane >> 2, t = lane & 3u;
#pragma unroll
  for (int h = 0; h < 2; h++) {  // rows g, g + 8
    const uint32_t r = first + g + 8 * h;
    const bool valid = r < n;
    const uint32_t src = valid ? (order ? order[r] : r) : 0u;
#pragma unroll
    for (int q = 0; q < 2; q++) {  // columns 2t, 2t+1 and 8+2t, 9+2t
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const uint32_t c = 8 * q + 2 * t + e;
        float v = 0.0f;
        if (valid && c < IN) v = (features[(size_t)src * IN + c] - norm[c]) * norm[IN + c];
        x[4 * q + 2 * h + e] = v;
      }
    }
  }
  a[0] = pack2(x[0], x[1]);
  a[1] = pack2(x[2], x[3]);
  a[2] = pack2(x[4], x[5]);
  a[3] = pack2(x[6], x[7]);
}

// The forward pass of one warp's 16 samples: pre-activations z1, z2 (FP32 C
// fragments, 8 tiles of 8 columns each) and logits z3 (columns 0-1 real).
__device__ __forceinline__ void forward16(const uint32_t (&ax)[4], const __nv_bfloat16* __restrict__ packed,
                                          const float* __restrict__ master, uint32_t lane, float (&z1)[8][4],
                                          float (&z2)[8][4], float (&z3)[4]) {
  const uint32_t t = lane & 3u;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const float b0 = master[OFF_B1 + 8 * j + 2 * t], b1 = master[OFF_B1 + 8 * j + 2 * t + 1];
    z1[j][0] = b0;
    z1[j][1] = b1;
    z1[j][2] = b0;
    z1[j][3] = b1;
    uint32_t w0, w1;
    load_b(packed + P_W1T, IN_PAD, 8 * j, 0, lane, w0, w1);
    mma16816(z1[j], ax, w0, w1);
  }
  uint32_t a1[4][4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    float lo[4], hi[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      lo[e] = gelu(z1[2 * q][e]);
      hi[e] = gelu(z1[2 * q + 1][e]);
    }
    to_a(lo, hi, a1[q]);
  }
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const float b0 = master[OFF_B2 + 8 * j + 2 * t], b1 = master[OFF_B2 + 8 * j + 2 * t + 1];
    z2[j][0] = b0;
    z2[j][1] = b1;
    z2[j][2] = b0;
    z2[j][3] = b1;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      uint32_t w0, w1;
      load_b(packed + P_W2T, HID, 8 * j, 16 * q, lane, w0, w1);
      mma16816(z2[j], a1[q], w0, w1);
    }
  }
  uint32_t a2[4][4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    float lo[4], hi[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      lo[e] = gelu(z2[2 * q][e]);
      hi[e] = gelu(z2[2 * q + 1][e]);
    }
    to_a(lo, hi, a2[q]);
  }
  const float c0 = 2 * t < OUT ? master[OFF_B3 + 2 * t] : 0.0f, c1 = 2 * t + 1 < OUT ? master[OFF_B3 + 2 * t + 1] : 0.0f;
  z3[0] = c0;
  z3[1] = c1;
  z3[2] = c0;
  z3[3] = c1;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    uint32_t w0, w1;
    load_b(packed + P_W3T, HID, 0, 16 * q, lane, w0, w1);
    mma16816(z3, a2[q], w0, w1);
  }
}

// ---- Inference on the fifth-generation tensor cores (tcgen05). A CTA of 128
// threads scores 128 candidates: each layer is one 128 x N x K product, issued by
// one thread as K / 16 tcgen05.mma instructions (BF16 operands in shared memory,
// FP32 accumulators in tensor memory), completed on an mbarrier; thread t then
// reads accumulator row t back (tcgen05.ld), adds the bias, applies GELU and
// writes the row's BF16 activations for the next layer's product.
constexpr uint32_t TC_ROWS = 128;     // candidates per CTA: the products' M
constexpr uint32_t TC_THREADS = 128;  // thread t owns row t (tensor-memory lane t)
constexpr uint32_t TC_COLUMNS = 128;  // tensor-memory columns: layer 1 in [0, 64), 2 in [64, 128), 3 in [0, 16)
constexpr uint32_t OUT_N = 16;        // layer 3's N, the smallest with M = 128 (outputs 0-1 real)

// Element offset of (row r, column k) of a BF16 matrix with K columns kept as 8 x 8
// core matrices (8 rows of 16 bytes, 128 contiguous bytes): core matrices along K
// 128 bytes apart, groups of 8 rows (K / 8) * 128 bytes apart. The no-swizzle
// K-major layout of the products' shared-memory descriptors.
__device__ __forceinline__ uint32_t core_offset(uint32_t r, uint32_t k, uint32_t K) {
  return (((r >> 3) * (K >> 3) + (k >> 3)) << 6) + ((r & 7u) << 3) + (k & 7u);
}

// Shared-memory matrix descriptor, no swizzle: start address, the byte distance
// between core matrices along K (leading) and between 8-row groups (stride), and
// the descriptor version (1) in bits 46-47.
__device__ __forceinline__ uint64_t smem_descriptor(const void* start, uint32_t lead_bytes, uint32_t stride_bytes) {
  const uint32_t a = smem_address(start);
  return (uint64_t)((a >> 4) & 0x3FFFu) | ((uint64_t)((lead_bytes >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((stride_bytes >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and
// B (bits 7-9 and 10-12 = 1), both K-major, N / 8 in bits 17-22, M / 16 in 24-28.
constexpr uint32_t mma_descriptor(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// D (+)= A B^T for one 16-deep step; A is M x 16 and B is N x 16, both K-major.
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}
// The barrier's one arrival once every tcgen05.mma this thread issued is complete.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                   smem_address(bar))
               : "memory");
}
// Columns [col, col + 16) of this warp's 32 tensor-memory lanes: lane t's values to thread t.
__device__ __forceinline__ void tc_load16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int e = 0; e < 16; e++) v[e] = __uint_as_float(r[e]);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// Makes this thread's shared-memory writes visible to the tensor cores' reads.
__device__ __forceinline__ void async_proxy_fence() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Eight BF16 values from v[0..8) into 16 bytes of shared memory.
__device__ __forceinline__ void store8(__nv_bfloat16* dst, const float* v) {
  *reinterpret_cast<uint4*>(dst) = make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
}

// Copies rows [0, rows_in) of a packed [rows][K] BF16 matrix into the core-matrix
// layout, rows [rows_in, rows) as zeros. All threads take part.
__device__ __forceinline__ void stage_weights(__nv_bfloat16* dst, const __nv_bfloat16* __restrict__ src,
                                              uint32_t rows, uint32_t rows_in, uint32_t K) {
  for (uint32_t i = threadIdx.x; i < rows * K / 8; i += blockDim.x) {
    const uint32_t r = i / (K / 8), k = (i % (K / 8)) * 8;
    const uint4 v = r < rows_in ? *reinterpret_cast<const uint4*>(src + (size_t)r * K + k) : make_uint4(0, 0, 0, 0);
    *reinterpret_cast<uint4*>(dst + core_offset(r, k, K)) = v;
  }
}

// Waits for the products committed to `bar` (phase `parity`); false on every
// thread if any gave up (DEVICE_ERROR_MMA_WAIT is then set).
__device__ __forceinline__ bool tc_layer_done(uint64_t* bar, uint32_t parity, uint32_t* __restrict__ error) {
  const bool ok = mbar_wait_bounded(bar, parity);
  const bool failed = __syncthreads_or(!ok);
  if (failed && threadIdx.x == 0) atomicOr(error, DEVICE_ERROR_MMA_WAIT);
  tc_fence_after();
  return !failed;
}

// Bias, then GELU, of 16 accumulator columns [c0, c0 + 16) of layer `bias`, as
// BF16 row t of the next layer's A (K = HID).
__device__ __forceinline__ void tc_hidden(uint32_t taddr, const float* __restrict__ bias, uint32_t c0,
                                          __nv_bfloat16* h, uint32_t t) {
  float v[16];
  tc_load16(taddr, v);
#pragma unroll
  for (int e = 0; e < 16; e++) v[e] = gelu(v[e] + bias[c0 + e]);
  store8(h + core_offset(t, c0, HID), v);
  store8(h + core_offset(t, c0 + 8, HID), v + 8);
}

// P(children survive) for each candidate: softmax of the two logits.
__global__ void __launch_bounds__(TC_THREADS) mlp_predict_kernel(const float* __restrict__ features, uint32_t n,
                                                                 const float* __restrict__ norm,
                                                                 const __nv_bfloat16* __restrict__ packed,
                                                                 const float* __restrict__ master,
                                                                 float* __restrict__ survive,
                                                                 uint32_t* __restrict__ error) {
  __shared__ __align__(128) __nv_bfloat16 s_x[TC_ROWS * IN_PAD];
  __shared__ __align__(128) __nv_bfloat16 s_h[TC_ROWS * HID];  // layer 1's activations, then layer 2's
  __shared__ __align__(128) __nv_bfloat16 s_w1[HID * IN_PAD];
  __shared__ __align__(128) __nv_bfloat16 s_w2[HID * HID];
  __shared__ __align__(128) __nv_bfloat16 s_w3[OUT_N * HID];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  const uint32_t t = threadIdx.x, warp = t >> 5;
  const uint32_t row = blockIdx.x * TC_ROWS + t;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_address(&s_tmem)),
                 "r"(TC_COLUMNS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (t == 0) mbar_init(&s_bar, 1);
  {  // row t's normalized features (then zeros) as BF16
    float x[IN_PAD];
#pragma unroll
    for (uint32_t c = 0; c < IN_PAD; c++)
      x[c] = row < n && c < IN ? (features[(size_t)row * IN + c] - norm[c]) * norm[IN + c] : 0.0f;
    store8(s_x + core_offset(t, 0, IN_PAD), x);
    store8(s_x + core_offset(t, 8, IN_PAD), x + 8);
  }
  stage_weights(s_w1, packed + P_W1T, HID, HID, IN_PAD);
  stage_weights(s_w2, packed + P_W2T, HID, HID, HID);
  stage_weights(s_w3, packed + P_W3T, OUT_N, OUT_PAD, HID);
  async_proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t lanes = (warp * 32u) << 16;  // this warp's tensor-memory lanes
  // Each 16-deep step takes the next two core matrices along K: 256 bytes on.
  constexpr uint32_t STEP = 128;  // elements
  bool ok = true;
  if (t == 0) {
    tc_mma(tmem, smem_descriptor(s_x, 128, 2 * 128), smem_descriptor(s_w1, 128, 2 * 128),
           mma_descriptor(TC_ROWS, HID), false);
    tc_commit(&s_bar);
  }
  ok = tc_layer_done(&s_bar, 0, error);
  if (ok) {
#pragma unroll
    for (uint32_t c = 0; c < HID; c += 16) tc_hidden(tmem + lanes + c, master + OFF_B1, c, s_h, t);
    async_proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (t == 0) {
#pragma unroll
      for (uint32_t q = 0; q < HID / 16; q++)
        tc_mma(tmem + HID, smem_descriptor(s_h + q * STEP, 128, 8 * 128), smem_descriptor(s_w2 + q * STEP, 128, 8 * 128),
               mma_descriptor(TC_ROWS, HID), q > 0);
      tc_commit(&s_bar);
    }
    ok = tc_layer_done(&s_bar, 1, error);
  }
  if (ok) {
#pragma unroll
    for (uint32_t c = 0; c < HID; c += 16) tc_hidden(tmem + lanes + HID + c, master + OFF_B2, c, s_h, t);
    async_proxy_fence();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (t == 0) {
#pragma unroll
      for (uint32_t q = 0; q < HID / 16; q++)
        tc_mma(tmem, smem_descriptor(s_h + q * STEP, 128, 8 * 128), smem_descriptor(s_w3 + q * STEP, 128, 8 * 128),
               mma_descriptor(TC_ROWS, OUT_N), q > 0);
      tc_commit(&s_bar);
    }
    ok = tc_layer_done(&s_bar, 0, error);
  }
  if (ok) {
    float z[16];
    tc_load16(tmem + lanes, z);
    if (row < n) survive[row] = 1.0f / (1.0f + expf((z[0] + master[OFF_B3]) - (z[1] + master[OFF_B3 + 1])));
  } else {
    mbar_wait_bounded(&s_bar, 0);  // a product still in flight after a give-up: one more bounded wait
    mbar_wait_bounded(&s_bar, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_COLUMNS) : "memory");
}

// Forward and backward over `batch` samples order[first..first+batch): adds the
// gradients of the mean cross-entropy, each sample weighted by its class's
// weight (class_weight.x for label 0, .y for 1), to grads (master layout) and
// the unweighted cross-entropy's sum to loss.
__global__ void __launch_bounds__(MLP_THREADS) mlp_train_kernel(
    const float* __restrict__ features, const uint8_t* __restrict__ labels, const uint32_t* __restrict__ order,
    uint32_t first, uint32_t batch, float2 class_weight, const float* __restrict__ norm,
    const __nv_bfloat16* __restrict__ packed, const float* __restrict__ master, float* __restrict__ grads,
    float* __restrict__ loss) {
  // Transposed copies for the weight gradients: [feature][sample of the CTA].
  __shared__ __align__(16) __nv_bfloat16 s_xt[IN_PAD][ROWS];
  __shared__ __align__(16) __nv_bfloat16 s_a1t[HID][ROWS];
  __shared__ __align__(16) __nv_bfloat16 s_a2t[HID][ROWS];
  __shared__ __align__(16) __nv_bfloat16 s_d1t[HID][ROWS];
  __shared__ __align__(16) __nv_bfloat16 s_d2t[HID][ROWS];
  __shared__ __align__(16) __nv_bfloat16 s_d3t[OUT_PAD][ROWS];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t g = lane >> 2, t = lane & 3u;
  const uint32_t end = first + batch;
  const uint32_t w_first = first + blockIdx.x * ROWS + warp * 16;
  const float inv_batch = 1.0f / (float)batch;
  const uint32_t r0 = warp * 16 + g, r1 = r0 + 8;  // this thread's rows within the CTA

  uint32_t ax[4];
  float x[8];
  load_input(features, order, w_first, end, norm, lane, ax, x);
  float z1[8][4], z2[8][4], z3[4];
  forward16(ax, packed, master, lane, z1, z2, z3);

  // Softmax cross-entropy: the lanes with t = 0 hold logits 0-1 of rows g, g + 8.
  float d3[4] = {0.f, 0.f, 0.f, 0.f};
  if (t == 0) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const uint32_t r = w_first + g + 8 * h;
      if (r < end) {
        const float y = labels[order[r]] ? 1.0f : 0.0f;
        const float wy = (y > 0.5f ? class_weight.y : class_weight.x) * inv_batch;
        const float m = fmaxf(z3[2 * h], z3[2 * h + 1]);
        const float e0 = expf(z3[2 * h] - m), e1 = expf(z3[2 * h + 1] - m);
        const float p1 = e1 / (e0 + e1);
        atomicAdd(loss, -logf(fmaxf(y > 0.5f ? p1 : 1.0f - p1, 1e-30f)));
        d3[2 * h] = ((1.0f - p1) - (1.0f - y)) * wy;
        d3[2 * h + 1] = (p1 - y) * wy;
      }
    }
  }
  // dA2 = dZ3 W3^T (dZ3 as a 16-deep A fragment: columns 0-7 from d3, 8-15 zero).
  uint32_t ad3[4] = {pack2(d3[0], d3[1]), pack2(d3[2], d3[3]), 0u, 0u};
  float dz2[8][4];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    dz2[j][0] = dz2[j][1] = dz2[j][2] = dz2[j][3] = 0.0f;
    uint32_t w0, w1;
    load_b(packed + P_W3B, OUT_K, 8 * j, 0, lane, w0, w1);
    mma16816(dz2[j], ad3, w0, w1);
#pragma unroll
    for (int e = 0; e < 4; e++) dz2[j][e] *= gelu_grad(z2[j][e]);
  }
  // dA1 = dZ2 W2^T.
  uint32_t ad2[4][4];
#pragma unroll
  for (int q = 0; q < 4; q++) to_a(dz2[2 * q], dz2[2 * q + 1], ad2[q]);
  float dz1[8][4];
#pragma unroll
  for (int j = 0; j < 8; j++) {
    dz1[j][0] = dz1[j][1] = dz1[j][2] = dz1[j][3] = 0.0f;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      uint32_t w0, w1;
      load_b(packed + P_W2B, HID, 8 * j, 16 * q, lane, w0, w1);
      mma16816(dz1[j], ad2[q], w0, w1);
    }
#pragma unroll
    for (int e = 0; e < 4; e++) dz1[j][e] *= gelu_grad(z1[j][e]);
  }

  // Transposed copies: element (row, column c) of a C tile j sits at [8j + c][row].
#pragma unroll
  for (int q = 0; q < 2; q++)
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const uint32_t c = 8 * q + 2 * t + e;
      s_xt[c][r0] = __float2bfloat16_rn(x[4 * q + e]);
      s_xt[c][r1] = __float2bfloat16_rn(x[4 * q + 2 + e]);
    }
#pragma unroll
  for (int j = 0; j < 8; j++)
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const uint32_t c = 8 * j + 2 * t + e;
      s_a1t[c][r0] = __float2bfloat16_rn(gelu(z1[j][e]));
      s_a1t[c][r1] = __float2bfloat16_rn(gelu(z1[j][2 + e]));
      s_a2t[c][r0] = __float2bfloat16_rn(gelu(z2[j][e]));
      s_a2t[c][r1] = __float2bfloat16_rn(gelu(z2[j][2 + e]));
      s_d1t[c][r0] = __float2bfloat16_rn(dz1[j][e]);
      s_d1t[c][r1] = __float2bfloat16_rn(dz1[j][2 + e]);
      s_d2t[c][r0] = __float2bfloat16_rn(dz2[j][e]);
      s_d2t[c][r1] = __float2bfloat16_rn(dz2[j][2 + e]);
    }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    s_d3t[2 * t + e][r0] = __float2bfloat16_rn(d3[e]);
    s_d3t[2 * t + e][r1] = __float2bfloat16_rn(d3[2 + e]);
  }

  // Bias gradients: column sums of dZ over this warp's 16 rows, then over the CTA
  // by atomics (lanes 0-3 hold the warp's sums after the butterfly).
  auto column_sums = [&](const float (&d)[4], float& s0, float& s1) {
    s0 = d[0] + d[2];
    s1 = d[1] + d[3];
#pragma unroll
    for (int o = 4; o < 32; o <<= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
  };
#pragma unroll
  for (int j = 0; j < 8; j++) {
    float s0, s1;
    column_sums(dz1[j], s0, s1);
    if (g == 0) {
      atomicAdd(&grads[OFF_B1 + 8 * j + 2 * t], s0);
      atomicAdd(&grads[OFF_B1 + 8 * j + 2 * t + 1], s1);
    }
    column_sums(dz2[j], s0, s1);
    if (g == 0) {
      atomicAdd(&grads[OFF_B2 + 8 * j + 2 * t], s0);
      atomicAdd(&grads[OFF_B2 + 8 * j + 2 * t + 1], s1);
    }
  }
  {
    float s0, s1;
    column_sums(d3, s0, s1);
    if (g == 0 && t == 0) {
      atomicAdd(&grads[OFF_B3], s0);
      atomicAdd(&grads[OFF_B3 + 1], s1);
    }
  }
  __syncthreads();

  // Weight gradients over the CTA's 64 samples: rows of W are input features
  // (the A operand is the transposed activation), columns outputs (the B operand,
  // [n][k] = the transposed dZ). A fragments of a [m][k] row-major BF16 matrix:
  auto load_a = [&](const __nv_bfloat16* m, uint32_t K, uint32_t m0, uint32_t k0, uint32_t (&a)[4]) {
    const __nv_bfloat16* p0 = m + (size_t)(m0 + g) * K + k0 + 2 * t;
    const __nv_bfloat16* p1 = p0 + 8 * K;
    a[0] = *reinterpret_cast<const uint32_t*>(p0);
    a[1] = *reinterpret_cast<const uint32_t*>(p1);
    a[2] = *reinterpret_cast<const uint32_t*>(p0 + 8);
    a[3] = *reinterpret_cast<const uint32_t*>(p1 + 8);
  };
  // dW2: warp w takes input rows 16w..16w+15, all 64 outputs.
  {
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      uint32_t a[4];
      load_a(&s_a1t[0][0], ROWS, 16 * warp, 16 * kk, a);
#pragma unroll
      for (int j = 0; j < 8; j++) {
        uint32_t w0, w1;
        load_b(&s_d2t[0][0], ROWS, 8 * j, 16 * kk, lane, w0, w1);
        mma16816(acc[j], a, w0, w1);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const uint32_t in0 = 16 * warp + g, out = 8 * j + 2 * t;
      atomicAdd(&grads[OFF_W2 + in0 * HID + out], acc[j][0]);
      atomicAdd(&grads[OFF_W2 + in0 * HID + out + 1], acc[j][1]);
      atomicAdd(&grads[OFF_W2 + (in0 + 8) * HID + out], acc[j][2]);
      atomicAdd(&grads[OFF_W2 + (in0 + 8) * HID + out + 1], acc[j][3]);
    }
  }
  // dW1: one 16-row tile of inputs (12 real); warp w takes outputs 16w..16w+15.
  {
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      uint32_t a[4];
      load_a(&s_xt[0][0], ROWS, 0, 16 * kk, a);
#pragma unroll
      for (int j = 0; j < 2; j++) {
        uint32_t w0, w1;
        load_b(&s_d1t[0][0], ROWS, 16 * warp + 8 * j, 16 * kk, lane, w0, w1);
        mma16816(acc[j], a, w0, w1);
      }
    }
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const uint32_t out = 16 * warp + 8 * j + 2 * t;
      if (g < IN) {
        atomicAdd(&grads[OFF_W1 + g * HID + out], acc[j][0]);
        atomicAdd(&grads[OFF_W1 + g * HID + out + 1], acc[j][1]);
      }
      if (g + 8 < IN) {
        atomicAdd(&grads[OFF_W1 + (g + 8) * HID + out], acc[j][2]);
        atomicAdd(&grads[OFF_W1 + (g + 8) * HID + out + 1], acc[j][3]);
      }
    }
  }
  // dW3: warp w takes input rows 16w..16w+15; the 8-wide output tile (2 real).
  {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      uint32_t a[4];
      load_a(&s_a2t[0][0], ROWS, 16 * warp, 16 * kk, a);
      uint32_t w0, w1;
      load_b(&s_d3t[0][0], ROWS, 0, 16 * kk, lane, w0, w1);
      mma16816(acc, a, w0, w1);
    }
    if (t == 0) {
      const uint32_t in0 = 16 * warp + g;
      atomicAdd(&grads[OFF_W3 + in0 * OUT], acc[0]);
      atomicAdd(&grads[OFF_W3 + in0 * OUT + 1], acc[1]);
      atomicAdd(&grads[OFF_W3 + (in0 + 8) * OUT], acc[2]);
      atomicAdd(&grads[OFF_W3 + (in0 + 8) * OUT + 1], acc[3]);
    }
  }
}

// AdamW on the FP32 master weights (biases without weight decay); clears the
// gradient for the next step.
__global__ void mlp_adamw_kernel(float* __restrict__ master, float* __restrict__ grads, float2* __restrict__ moments,
                                 float lr, float weight_decay, float bc1, float bc2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= PARAMS) return;
  const float g = grads[i];
  grads[i] = 0.0f;
  float2 m = moments[i];
  m.x = 0.9f * m.x + 0.1f * g;
  m.y = 0.999f * m.y + 0.001f * g * g;
  moments[i] = m;
  const bool bias = (i >= OFF_B1 && i < OFF_W2) || (i >= OFF_B2 && i < OFF_W3) || i >= OFF_B3;
  float w = master[i];
  if (!bias) w -= lr * weight_decay * w;
  w -= lr * (m.x / bc1) / (sqrtf(m.y / bc2) + 1e-8f);
  master[i] = w;
}

// The BF16 layouts of the master weights.
__global__ void mlp_pack_kernel(const float* __restrict__ master, __nv_bfloat16* __restrict__ packed) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= PACKED) return;
  float v = 0.0f;
  if (i < P_W2T) {
    const uint32_t n = (i - P_W1T) / IN_PAD, k = (i - P_W1T) % IN_PAD;
    v = k < IN ? master[OFF_W1 + k * HID + n] : 0.0f;
  } else if (i < P_W3T) {
    const uint32_t n = (i - P_W2T) / HID, k = (i - P_W2T) % HID;
    v = master[OFF_W2 + k * HID + n];
  } else if (i < P_W2B) {
    const uint32_t n = (i - P_W3T) / HID, k = (i - P_W3T) % HID;
    v = n < OUT ? master[OFF_W3 + k * OUT + n] : 0.0f;
  } else if (i < P_W3B) {
    const uint32_t n = (i - P_W2B) / HID, k = (i - P_W2B) % HID;  // n: input, k: output
    v = master[OFF_W2 + n * HID + k];
  } else {
    const uint32_t n = (i - P_W3B) / OUT_K, k = (i - P_W3B) % OUT_K;  // n: input, k: output
    v = k < OUT ? master[OFF_W3 + n * OUT + k] : 0.0f;
  }
  packed[i] = __float2bfloat16_rn(v);
}

}  // namespace
}  // namespace dg

using namespace dg;

struct dg_densify_mlp {
  dg_context* ctx;
  dg_buffer *master = nullptr, *grads = nullptr, *moments = nullptr, *packed = nullptr, *norm = nullptr,
            *loss = nullptr;
  std::vector<float> norm_host;  // mean[12], 1/std[12]
  uint32_t steps = 0;
};

namespace dg {

dg_status mlp_predict_launch(dg_densify_mlp* m, const float* features, uint32_t n, float* survive) {
  if (n == 0) return DG_OK;
  DG_LAUNCH(m->ctx, "mlp_predict",
            mlp_predict_kernel<<<ceil_div(n, TC_ROWS), TC_THREADS, 0, m->ctx->stream>>>(
                features, n, typed<float>(m->norm), typed<__nv_bfloat16>(m->packed), typed<float>(m->master),
                survive, m->ctx->device_error));
  return DG_OK;
}

static dg_status pack(dg_densify_mlp* m) {
  DG_LAUNCH(m->ctx, "mlp_pack",
            mlp_pack_kernel<<<ceil_div(PACKED, 256), 256, 0, m->ctx->stream>>>(typed<float>(m->master),
                                                                               typed<__nv_bfloat16>(m->packed)));
  return DG_OK;
}

}  // namespace dg

extern "C" {

dg_status dg_densify_mlp_create(dg_context* ctx, uint32_t seed, dg_densify_mlp** out) {
  DG_REQUIRE(ctx && out, "NULL argument");
  auto* m = new dg_densify_mlp();
  m->ctx = ctx;
  dg_status st = alloc_buffer(ctx, PARAMS * 4, &m->master);
  if (st == DG_OK) st = alloc_buffer(ctx, PARAMS * 4, &m->grads);
  if (st == DG_OK) st = alloc_buffer(ctx, PARAMS * 8, &m->moments);
  if (st == DG_OK) st = alloc_buffer(ctx, PACKED * 2, &m->packed);
  if (st == DG_OK) st = alloc_buffer(ctx, 2 * IN * 4, &m->norm);
  if (st == DG_OK) st = alloc_buffer(ctx, 16, &m->loss);
  if (st != DG_OK) {
    dg_densify_mlp_destroy(m);
    return st;
  }
  // He-style initialization from a seeded generator; biases zero; identity normalization.
  std::mt19937 gen(seed);
  std::vector<float> w(PARAMS, 0.0f);
  auto fill = [&](uint32_t off, uint32_t fan_in, uint32_t count) {
    std::normal_distribution<float> d(0.0f, std::sqrt(2.0f / (float)fan_in));
    for (uint32_t k = 0; k < count; k++) w[off + k] = d(gen);
  };
  fill(OFF_W1, IN, IN * HID);
  fill(OFF_W2, HID, HID * HID);
  fill(OFF_W3, HID, HID * OUT);
  m->norm_host.assign(2 * IN, 0.0f);
  for (uint32_t k = 0; k < IN; k++) m->norm_host[IN + k] = 1.0f;
  st = write_async(ctx, m->master->ptr, w.data(), PARAMS * 4);
  if (st == DG_OK) st = write_async(ctx, m->norm->ptr, m->norm_host.data(), 2 * IN * 4);
  if (st == DG_OK) st = pack(m);
  if (st != DG_OK) {
    dg_densify_mlp_destroy(m);
    return st;
  }
  *out = m;
  return DG_OK;
}

// Trains on count labelled samples (features[count][12], labels 0/1, host arrays):
// the input normalization is set from the samples' mean and standard deviation,
// then `epochs` shuffled passes of minibatches of `batch` with AdamW. With
// balance_classes, each class's samples weigh count / (2 * its size), so both
// classes count equally. mean_loss receives each epoch's mean cross-entropy
// (room for `epochs` values; may be NULL).
dg_status dg_densify_mlp_train(dg_densify_mlp* m, const float* features, const uint8_t* labels, uint32_t count,
                               uint32_t epochs, uint32_t batch, float lr, float weight_decay, int32_t balance_classes,
                               uint32_t seed, double* mean_loss) {
  DG_REQUIRE(m && features && labels, "NULL argument");
  DG_REQUIRE(count > 0 && epochs > 0 && batch > 0, "nothing to train on");
  dg_context* ctx = m->ctx;
  // Normalization from the samples (double sums).
  std::vector<double> mean(IN, 0.0), var(IN, 0.0);
  for (uint32_t i = 0; i < count; i++)
    for (uint32_t k = 0; k < IN; k++) mean[k] += features[(size_t)i * IN + k];
  for (uint32_t k = 0; k < IN; k++) mean[k] /= count;
  for (uint32_t i = 0; i < count; i++)
    for (uint32_t k = 0; k < IN; k++) {
      const double d = features[(size_t)i * IN + k] - mean[k];
      var[k] += d * d;
    }
  for (uint32_t k = 0; k < IN; k++) {
    m->norm_host[k] = (float)mean[k];
    m->norm_host[IN + k] = (float)(1.0 / std::sqrt(var[k] / count + 1e-12));
  }
  DG_TRY(write_async(ctx, m->norm->ptr, m->norm_host.data(), 2 * IN * 4));
  uint64_t positives = 0;
  for (uint32_t i = 0; i < count; i++) positives += labels[i] != 0;
  float2 class_weight = make_float2(1.0f, 1.0f);
  if (balance_classes && positives > 0 && positives < count) {
    class_weight.x = (float)((double)count / (2.0 * (double)(count - positives)));
    class_weight.y = (float)((double)count / (2.0 * (double)positives));
  }
  dg_buffer *f = nullptr, *l = nullptr, *order = nullptr;
  DG_TRY(alloc_buffer(ctx, (size_t)count * IN * 4, &f));
  DG_TRY(alloc_buffer(ctx, count, &l));
  DG_TRY(alloc_buffer(ctx, (size_t)count * 4, &order));
  DG_CUDA(cudaMemcpyAsync(f->ptr, features, (size_t)count * IN * 4, cudaMemcpyHostToDevice, ctx->stream));
  DG_CUDA(cudaMemcpyAsync(l->ptr, labels, count, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<uint32_t> perm(count);
  std::iota(perm.begin(), perm.end(), 0u);
  std::mt19937 gen(seed);
  dg_status st = DG_OK;
  for (uint32_t e = 0; e < epochs && st == DG_OK; e++) {
    std::shuffle(perm.begin(), perm.end(), gen);
    DG_CUDA(cudaMemcpyAsync(order->ptr, perm.data(), (size_t)count * 4, cudaMemcpyHostToDevice, ctx->stream));
    DG_CUDA(cudaMemsetAsync(m->loss->ptr, 0, 4, ctx->stream));
    for (uint32_t first = 0; first < count; first += batch) {
      const uint32_t n = std::min(batch, count - first);
      m->steps++;
      const float bc1 = 1.0f - std::pow(0.9f, (float)m->steps), bc2 = 1.0f - std::pow(0.999f, (float)m->steps);
      DG_LAUNCH(ctx, "mlp_train",
                mlp_train_kernel<<<ceil_div(n, ROWS), MLP_THREADS, 0, ctx->stream>>>(
                    typed<float>(f), typed<uint8_t>(l), typed<uint32_t>(order), first, n, class_weight,
                    typed<float>(m->norm),
                    typed<__nv_bfloat16>(m->packed), typed<float>(m->master), typed<float>(m->grads),
                    typed<float>(m->loss)));
      DG_LAUNCH(ctx, "mlp_adamw",
                mlp_adamw_kernel<<<ceil_div(PARAMS, 256), 256, 0, ctx->stream>>>(
                    typed<float>(m->master), typed<float>(m->grads), typed<float2>(m->moments), lr, weight_decay, bc1,
                    bc2));
      st = pack(m);
      if (st != DG_OK) break;
    }
    if (mean_loss) {
      float sum = 0.0f;
      DG_CUDA(cudaMemcpyAsync(&sum, m->loss->ptr, 4, cudaMemcpyDeviceToHost, ctx->stream));
      DG_CUDA(cudaStreamSynchronize(ctx->stream));
      mean_loss[e] = sum / count;
    }
  }
  DG_CUDA(cudaStreamSynchronize(ctx->stream));
  free_buffer(f);
  free_buffer(l);
  free_buffer(order);
  return st;
}

// The gradient of the mean cross-entropy over count samples (host arrays) at the
// current weights and normalization, in the master layout; nothing is updated.
dg_status dg_densify_mlp_gradient(dg_densify_mlp* m, const float* features, const uint8_t* labels, uint32_t count,
                                  float* gradient) {
  DG_REQUIRE(m && features && labels && gradient, "NULL argument");
  DG_REQUIRE(count > 0, "no samples");
  dg_context* ctx = m->ctx;
  dg_buffer *f = nullptr, *l = nullptr, *order = nullptr;
  DG_TRY(alloc_buffer(ctx, (size_t)count * IN * 4, &f));
  dg_status st = alloc_buffer(ctx, count, &l);
  if (st == DG_OK) st = alloc_buffer(ctx, (size_t)count * 4, &order);
  if (st == DG_OK) {
    std::vector<uint32_t> identity(count);
    std::iota(identity.begin(), identity.end(), 0u);
    DG_CUDA(cudaMemcpyAsync(f->ptr, features, (size_t)count * IN * 4, cudaMemcpyHostToDevice, ctx->stream));
    DG_CUDA(cudaMemcpyAsync(l->ptr, labels, count, cudaMemcpyHostToDevice, ctx->stream));
    DG_CUDA(cudaMemcpyAsync(order->ptr, identity.data(), (size_t)count * 4, cudaMemcpyHostToDevice, ctx->stream));
    DG_CUDA(cudaMemsetAsync(m->grads->ptr, 0, PARAMS * 4, ctx->stream));
    DG_LAUNCH(ctx, "mlp_train",
              mlp_train_kernel<<<ceil_div(count, ROWS), MLP_THREADS, 0, ctx->stream>>>(
                  typed<float>(f), typed<uint8_t>(l), typed<uint32_t>(order), 0, count, make_float2(1.0f, 1.0f),
                  typed<float>(m->norm), typed<__nv_bfloat16>(m->packed), typed<float>(m->master),
                  typed<float>(m->grads), typed<float>(m->loss)));
    DG_CUDA(cudaMemcpyAsync(gradient, m->grads->ptr, PARAMS * 4, cudaMemcpyDeviceToHost, ctx->stream));
    DG_CUDA(cudaMemsetAsync(m->grads->ptr, 0, PARAMS * 4, ctx->stream));
    DG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  free_buffer(f);
  free_buffer(l);
  free_buffer(order);
  return st;
}

// survive[i] = P(the children of candidate i survive), features[count][12] and
// survive[count] on the device.
dg_status dg_densify_mlp_predict(dg_densify_mlp* m, dg_buffer* features, uint32_t count, dg_buffer* survive) {
  DG_REQUIRE(m && features && survive, "NULL argument");
  DG_REQUIRE(features->bytes >= (uint64_t)count * IN * 4 && survive->bytes >= (uint64_t)count * 4,
             "buffers smaller than count samples");
  return mlp_predict_launch(m, typed<float>(features), count, typed<float>(survive));
}

// The model as DG_MLP_PARAMS master weights followed by the 24 normalization
// values (mean, then 1/std of each feature).
dg_status dg_densify_mlp_get_weights(dg_densify_mlp* m, float* out) {
  DG_REQUIRE(m && out, "NULL argument");
  DG_CUDA(cudaMemcpyAsync(out, m->master->ptr, PARAMS * 4, cudaMemcpyDeviceToHost, m->ctx->stream));
  DG_CUDA(cudaStreamSynchronize(m->ctx->stream));
  std::memcpy(out + PARAMS, m->norm_host.data(), 2 * IN * 4);
  return DG_OK;
}

dg_status dg_densify_mlp_set_weights(dg_densify_mlp* m, const float* in) {
  DG_REQUIRE(m && in, "NULL argument");
  m->norm_host.assign(in + PARAMS, in + PARAMS + 2 * IN);
  DG_TRY(write_async(m->ctx, m->master->ptr, in, PARAMS * 4));
  DG_TRY(write_async(m->ctx, m->norm->ptr, m->norm_host.data(), 2 * IN * 4));
  return pack(m);
}

dg_status dg_densify_mlp_destroy(dg_densify_mlp* m) {
  if (!m) return DG_OK;
  for (dg_buffer* b : {m->master, m->grads, m->moments, m->packed, m->norm, m->loss}) free_buffer(b);
  delete m;
  return DG_OK;
}

}  // extern "C"
