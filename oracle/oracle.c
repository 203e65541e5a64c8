/*
 * The oracle: a single-precision CPU restatement of the reference's 3D Gaussian
 * Splatting training path, for TESTS ONLY.
 *
 * This file is test infrastructure. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it, and only as the checker or the timed
 * CPU baseline. The library under diorama_gb300/ never links or calls it.
 *
 * Each function follows one WGSL entry point of the reference, statement by
 * statement and in the same order of float operations, so that a GPU kernel
 * written with the same order produces the same bits. Where WGSL leaves an order
 * open (matrix products, dot products), this file fixes it: sums run from index
 * 0 upwards, and every product is rounded before it is added (no fused
 * multiply-add unless fmaf is written out). Compile with -ffp-contract=off.
 *
 * The exponential used by the blend is dg_exp_ref below (Cody-Waite argument
 * reduction plus a degree-7 Taylor polynomial), which the CUDA blend kernels
 * restate in the same way, so forward images agree bit for bit.
 *
 * Parity of this restatement itself is pinned against the reference's own
 * float64 PyTorch oracles (reference/backward_reference.py and
 * reference/loss_reference.py) through the committed fixtures in tests/golden.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define TILE 16u
#define FPG 16u  /* floats per Gaussian, src/gaussians.ts:32 */
#define FPS 12u  /* floats per splat, src/gaussians.ts:33 */
#define SHF 45u  /* SH rest floats, src/gaussians.ts:36 */
#define SLOTS 61u /* Adam moment slots, src/trainer.ts:17 */

/* Camera as 36 floats: view (16, column-major), proj (16), viewport (2), pad (2). */
#define CAM_VIEW(c, col, row) ((c)[(col) * 4 + (row)])
#define CAM_PROJ(c, col, row) ((c)[16 + (col) * 4 + (row)])
#define CAM_VP(c, k) ((c)[32 + (k)])

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------- math */

/* e^x by Cody-Waite reduction x = n ln2 + r, |r| <= ln2/2, then e^r from its
 * Taylor series to degree 7 by Horner's rule, then scaling by 2^n through the
 * exponent bits. Results below the smallest normal float are returned as 0. */
float dg_exp_ref(float x) {
  if (x < -87.0f) return 0.0f;
  if (x > 88.0f) return INFINITY;
  float n = rintf(x * 1.44269504088896341f);
  float r = fmaf(n, -0.693145751953125f, x);
  r = fmaf(n, -1.428606820309417232e-6f, r);
  float p = 1.98412698412698413e-4f;           /* 1/7! */
  p = fmaf(p, r, 1.38888888888888889e-3f);    /* 1/6! */
  p = fmaf(p, r, 8.33333333333333333e-3f);    /* 1/5! */
  p = fmaf(p, r, 4.16666666666666667e-2f);    /* 1/4! */
  p = fmaf(p, r, 1.66666666666666667e-1f);    /* 1/3! */
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  int32_t e = (int32_t)n + 127;
  union { uint32_t u; float f; } s;
  s.u = (uint32_t)e << 23;
  return p * s.f;
}

static float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

/* WGSL max/min on the values this path meets (no NaN): plain comparisons. */
static float maxf(float a, float b) { return a > b ? a : b; }
static float minf(float a, float b) { return a < b ? a : b; }

/* Rotation matrix of quaternion (w,x,y,z), normalized first, as columns r[col][row]:
 * src/shaders/gaussianMath.wgsl:13-25. */
static void rotation_matrix(const float raw[4], float r[3][3], float q_out[4], float* len_out) {
  float dot = raw[0] * raw[0];
  dot = dot + raw[1] * raw[1];
  dot = dot + raw[2] * raw[2];
  dot = dot + raw[3] * raw[3];
  float len = sqrtf(dot);
  float qw = raw[0] / len, qx = raw[1] / len, qy = raw[2] / len, qz = raw[3] / len;
  r[0][0] = 1.0f - 2.0f * (qy * qy + qz * qz);
  r[0][1] = 2.0f * (qx * qy + qw * qz);
  r[0][2] = 2.0f * (qx * qz - qw * qy);
  r[1][0] = 2.0f * (qx * qy - qw * qz);
  r[1][1] = 1.0f - 2.0f * (qx * qx + qz * qz);
  r[1][2] = 2.0f * (qy * qz + qw * qx);
  r[2][0] = 2.0f * (qx * qz + qw * qy);
  r[2][1] = 2.0f * (qy * qz - qw * qx);
  r[2][2] = 1.0f - 2.0f * (qx * qx + qy * qy);
  if (q_out) { q_out[0] = qw; q_out[1] = qx; q_out[2] = qy; q_out[3] = qz; }
  if (len_out) *len_out = len;
}

static const float SH_C1 = 0.4886025119029199f;
static const float SH_C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                               -1.0925484305920792f, 0.5462742152789498f};
static const float SH_C3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                               0.3731763325901154f, -0.4570457994644658f, 1.445305721320277f,
                               -0.5900435899266435f};

/* src/shaders/gaussianMath.wgsl:30-44 */
static void sh_basis(const float d[3], float b[15]) {
  float x = d[0], y = d[1], z = d[2];
  float xx = x * x, yy = y * y, zz = z * z;
  b[0] = -SH_C1 * y;
  b[1] = SH_C1 * z;
  b[2] = -SH_C1 * x;
  b[3] = SH_C2[0] * x * y;
  b[4] = SH_C2[1] * y * z;
  b[5] = SH_C2[2] * (2.0f * zz - xx - yy);
  b[6] = SH_C2[3] * x * z;
  b[7] = SH_C2[4] * (xx - yy);
  b[8] = SH_C3[0] * y * (3.0f * xx - yy);
  b[9] = SH_C3[1] * x * y * z;
  b[10] = SH_C3[2] * y * (4.0f * zz - xx - yy);
  b[11] = SH_C3[3] * z * (2.0f * zz - 3.0f * xx - 3.0f * yy);
  b[12] = SH_C3[4] * x * (4.0f * zz - xx - yy);
  b[13] = SH_C3[5] * z * (xx - yy);
  b[14] = SH_C3[6] * x * (xx - 3.0f * yy);
}

/* src/shaders/gaussianMath.wgsl:47-71, as g[k][axis]. */
static void sh_basis_gradient(const float d[3], float g[15][3]) {
  float x = d[0], y = d[1], z = d[2];
  float xx = x * x, yy = y * y, zz = z * z;
  const float v[15][3] = {
      {0.0f, -SH_C1, 0.0f},
      {0.0f, 0.0f, SH_C1},
      {-SH_C1, 0.0f, 0.0f},
      {SH_C2[0] * y, SH_C2[0] * x, SH_C2[0] * 0.0f},
      {SH_C2[1] * 0.0f, SH_C2[1] * z, SH_C2[1] * y},
      {SH_C2[2] * (-2.0f * x), SH_C2[2] * (-2.0f * y), SH_C2[2] * (4.0f * z)},
      {SH_C2[3] * z, SH_C2[3] * 0.0f, SH_C2[3] * x},
      {SH_C2[4] * (2.0f * x), SH_C2[4] * (-2.0f * y), SH_C2[4] * 0.0f},
      {SH_C3[0] * (6.0f * x * y), SH_C3[0] * (3.0f * xx - 3.0f * yy), SH_C3[0] * 0.0f},
      {SH_C3[1] * (y * z), SH_C3[1] * (x * z), SH_C3[1] * (x * y)},
      {SH_C3[2] * (-2.0f * x * y), SH_C3[2] * (4.0f * zz - xx - 3.0f * yy), SH_C3[2] * (8.0f * y * z)},
      {SH_C3[3] * (-6.0f * x * z), SH_C3[3] * (-6.0f * y * z), SH_C3[3] * (6.0f * zz - 3.0f * xx - 3.0f * yy)},
      {SH_C3[4] * (4.0f * zz - 3.0f * xx - yy), SH_C3[4] * (-2.0f * x * y), SH_C3[4] * (8.0f * x * z)},
      {SH_C3[5] * (2.0f * x * z), SH_C3[5] * (-2.0f * y * z), SH_C3[5] * (xx - yy)},
      {SH_C3[6] * (3.0f * xx - 3.0f * yy), SH_C3[6] * (-6.0f * x * y), SH_C3[6] * 0.0f},
  };
  memcpy(g, v, sizeof(v));
}

static uint32_t sh_count(uint32_t degree) { return (degree + 1u) * (degree + 1u) - 1u; }

/* ------------------------------------------------------------ preprocess */

/* Shared by the forward and backward: the view-space center and the 2D covariance.
 * Products run in the fixed order of this file's header comment. */
typedef struct {
  float t[3], depth;
  float r[3][3], q[4], qlen;
  float m[3][3], cov3d[3][3];
  float focal[2], limit[2], tx, ty;
  float jw[3][2]; /* columns of J W */
  float w[3][3];  /* columns of W */
  float a, b, c, det;
} Projection;

static void project(const float* cam, const float* g, Projection* p) {
  const float pos[3] = {g[0], g[1], g[2]};
  for (int row = 0; row < 3; row++) {
    float v = CAM_VIEW(cam, 0, row) * pos[0];
    v = v + CAM_VIEW(cam, 1, row) * pos[1];
    v = v + CAM_VIEW(cam, 2, row) * pos[2];
    v = v + CAM_VIEW(cam, 3, row) * 1.0f;
    p->t[row] = v;
  }
  p->depth = -p->t[2];
  rotation_matrix(g + 8, p->r, p->q, &p->qlen);
  for (int col = 0; col < 3; col++)
    for (int row = 0; row < 3; row++) p->m[col][row] = p->r[col][row] * g[4 + col];
  /* cov3d = M Mᵀ: element (row, col) = Σ_k m[k][row] m[k][col]. */
  for (int col = 0; col < 3; col++)
    for (int row = 0; row < 3; row++) {
      float v = p->m[0][row] * p->m[0][col];
      v = v + p->m[1][row] * p->m[1][col];
      v = v + p->m[2][row] * p->m[2][col];
      p->cov3d[col][row] = v;
    }
  p->focal[0] = CAM_PROJ(cam, 0, 0) * CAM_VP(cam, 0) * 0.5f;
  p->focal[1] = CAM_PROJ(cam, 1, 1) * CAM_VP(cam, 1) * 0.5f;
  p->limit[0] = 1.3f * CAM_VP(cam, 0) * 0.5f / p->focal[0];
  p->limit[1] = 1.3f * CAM_VP(cam, 1) * 0.5f / p->focal[1];
  float depth = p->depth;
  p->tx = clampf(p->t[0] / depth, -p->limit[0], p->limit[0]) * depth;
  p->ty = clampf(p->t[1] / depth, -p->limit[1], p->limit[1]) * depth;
  float j[3][2];
  j[0][0] = p->focal[0] / depth;
  j[0][1] = 0.0f;
  j[1][0] = 0.0f;
  j[1][1] = -p->focal[1] / depth;
  j[2][0] = p->focal[0] * p->tx / (depth * depth);
  j[2][1] = -p->focal[1] * p->ty / (depth * depth);
  for (int col = 0; col < 3; col++)
    for (int row = 0; row < 3; row++) p->w[col][row] = CAM_VIEW(cam, col, row);
  /* jw = J W: column col = Σ_k j[k] * W[k][col] where W[k][col] = w[col][k]. */
  for (int col = 0; col < 3; col++)
    for (int row = 0; row < 2; row++) {
      float v = j[0][row] * p->w[col][0];
      v = v + j[1][row] * p->w[col][1];
      v = v + j[2][row] * p->w[col][2];
      p->jw[col][row] = v;
    }
  /* T1 = jw * cov3d (mat3x2): column col = Σ_k jw[k] * cov3d[col][k]. */
  float t1[3][2];
  for (int col = 0; col < 3; col++)
    for (int row = 0; row < 2; row++) {
      float v = p->jw[0][row] * p->cov3d[col][0];
      v = v + p->jw[1][row] * p->cov3d[col][1];
      v = v + p->jw[2][row] * p->cov3d[col][2];
      t1[col][row] = v;
    }
  /* cov = T1 * jwᵀ (mat2x2): element (row, col) = Σ_k t1[k][row] * jw[k][col]. */
  float cov[2][2];
  for (int col = 0; col < 2; col++)
    for (int row = 0; row < 2; row++) {
      float v = t1[0][row] * p->jw[0][col];
      v = v + t1[1][row] * p->jw[1][col];
      v = v + t1[2][row] * p->jw[2][col];
      cov[col][row] = v;
    }
  p->a = cov[0][0] + 0.3f;
  p->b = cov[0][1];
  p->c = cov[1][1] + 0.3f;
  p->det = p->a * p->c - p->b * p->b;
}

static void camera_position(const float* cam, float out[3]) {
  for (int col = 0; col < 3; col++) {
    float v = CAM_VIEW(cam, col, 0) * CAM_VIEW(cam, 3, 0);
    v = v + CAM_VIEW(cam, col, 1) * CAM_VIEW(cam, 3, 1);
    v = v + CAM_VIEW(cam, col, 2) * CAM_VIEW(cam, 3, 2);
    out[col] = -v;
  }
}

static void normalize3(const float v[3], float out[3], float* len_out) {
  float dot = v[0] * v[0];
  dot = dot + v[1] * v[1];
  dot = dot + v[2] * v[2];
  float len = sqrtf(dot);
  out[0] = v[0] / len;
  out[1] = v[1] / len;
  out[2] = v[2] / len;
  if (len_out) *len_out = len;
}

/* src/shaders/preprocess.wgsl:21-88. splats_out gets FPS floats per Gaussian. */
void or_preprocess(const float* cam, const float* gaussians, const float* sh, uint32_t count,
                   uint32_t sh_degree, float* splats) {
  const float vpx = CAM_VP(cam, 0), vpy = CAM_VP(cam, 1);
  float campos[3];
  camera_position(cam, campos);
  uint32_t basis_count = sh_count(sh_degree);
#pragma omp parallel for schedule(static)
  for (int64_t ii = 0; ii < (int64_t)count; ii++) {
    uint32_t i = (uint32_t)ii;
    const float* g = gaussians + (size_t)i * FPG;
    float* s = splats + (size_t)i * FPS;
    memset(s, 0, FPS * sizeof(float));
    s[3] = 0.0f;
    Projection p;
    /* Near cull before anything else, as the WGSL returns before the covariance. */
    {
      float v = CAM_VIEW(cam, 0, 2) * g[0];
      v = v + CAM_VIEW(cam, 1, 2) * g[1];
      v = v + CAM_VIEW(cam, 2, 2) * g[2];
      v = v + CAM_VIEW(cam, 3, 2) * 1.0f;
      if (-v <= 0.2f) continue;
    }
    project(cam, g, &p);
    if (p.det <= 0.0f) continue;
    float mid = 0.5f * (p.a + p.c);
    float lambda = mid + sqrtf(maxf(0.1f, mid * mid - p.det));
    float radius = ceilf(3.0f * sqrtf(lambda));
    float clip[4];
    for (int row = 0; row < 4; row++) {
      float v = CAM_PROJ(cam, 0, row) * p.t[0];
      v = v + CAM_PROJ(cam, 1, row) * p.t[1];
      v = v + CAM_PROJ(cam, 2, row) * p.t[2];
      v = v + CAM_PROJ(cam, 3, row) * 1.0f;
      clip[row] = v;
    }
    float mx = (clip[0] / clip[3] * 0.5f + 0.5f) * vpx;
    float my = (clip[1] / clip[3] * -0.5f + 0.5f) * vpy;
    if (mx + radius < 0.0f || my + radius < 0.0f || mx - radius > vpx || my - radius > vpy) continue;
    float color[3] = {g[12], g[13], g[14]};
    if (basis_count > 0u) {
      float off[3] = {g[0] - campos[0], g[1] - campos[1], g[2] - campos[2]};
      float dir[3], basis[15];
      normalize3(off, dir, NULL);
      sh_basis(dir, basis);
      const float* c = sh + (size_t)i * SHF;
      for (uint32_t k = 0; k < basis_count; k++) {
        color[0] = color[0] + basis[k] * c[k * 3 + 0];
        color[1] = color[1] + basis[k] * c[k * 3 + 1];
        color[2] = color[2] + basis[k] * c[k * 3 + 2];
      }
    }
    for (int k = 0; k < 3; k++) color[k] = maxf(color[k], 0.0f);
    s[0] = mx;
    s[1] = my;
    s[2] = p.depth;
    s[3] = radius;
    s[4] = p.c / p.det;
    s[5] = -p.b / p.det;
    s[6] = p.a / p.det;
    s[7] = 0.0f;
    s[8] = color[0];
    s[9] = color[1];
    s[10] = color[2];
    s[11] = g[3];
  }
}

/* ----------------------------------------------------------- tile stage */

/* src/shaders/common.wgsl:31-42 */
static void tile_grid(const float* cam, uint32_t tiles[2]) {
  tiles[0] = ((uint32_t)CAM_VP(cam, 0) + TILE - 1u) / TILE;
  tiles[1] = ((uint32_t)CAM_VP(cam, 1) + TILE - 1u) / TILE;
}

static void tile_rect(const float* s, const uint32_t tiles[2], uint32_t rect[4]) {
  for (int k = 0; k < 2; k++) {
    float lo = clampf(floorf((s[k] - s[3]) / 16.0f), 0.0f, (float)tiles[k]);
    float hi = clampf(floorf((s[k] + s[3]) / 16.0f) + 1.0f, 0.0f, (float)tiles[k]);
    rect[k] = (uint32_t)lo;
    rect[2 + k] = (uint32_t)hi;
  }
}

/* src/shaders/tiles.wgsl:24-35 */
void or_count_tiles(const float* cam, const float* splats, uint32_t count, uint32_t* out) {
  uint32_t tiles[2];
  tile_grid(cam, tiles);
  for (uint32_t i = 0; i < count; i++) {
    const float* s = splats + (size_t)i * FPS;
    uint32_t touched = 0;
    if (s[3] > 0.0f) {
      uint32_t rect[4];
      tile_rect(s, tiles, rect);
      touched = (rect[2] - rect[0]) * (rect[3] - rect[1]);
    }
    out[i] = touched;
  }
}

/* Exclusive prefix sum in place, returning the total: src/shaders/prefixSum.wgsl:31-91
 * (the sequential form src/checks/depthSort.ts:65-69 checks against). */
uint32_t or_exclusive_scan(uint32_t* data, uint32_t n) {
  uint32_t sum = 0;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t v = data[i];
    data[i] = sum;
    sum += v;
  }
  return sum;
}

/* src/shaders/tiles.wgsl:37-60. keys are (tile << 32) | depth bits. */
void or_duplicate(const float* cam, const float* splats, const uint32_t* offsets, uint32_t count,
                  uint32_t capacity, uint64_t* keys, uint32_t* values) {
  uint32_t tiles[2];
  tile_grid(cam, tiles);
  for (uint32_t i = 0; i < count; i++) {
    const float* s = splats + (size_t)i * FPS;
    if (s[3] == 0.0f) continue;
    uint32_t rect[4];
    tile_rect(s, tiles, rect);
    uint32_t depth_bits;
    memcpy(&depth_bits, &s[2], 4);
    uint32_t slot = offsets[i];
    for (uint32_t y = rect[1]; y < rect[3]; y++)
      for (uint32_t x = rect[0]; x < rect[2]; x++) {
        if (slot < capacity) {
          keys[slot] = ((uint64_t)(y * tiles[0] + x) << 32) | depth_bits;
          values[slot] = i;
        }
        slot++;
      }
  }
}

/* Stable LSD radix sort with 8-bit digits and the reference's pass plan:
 * 4 passes over the low word, then 2·ceil(high_bits/16) over the high word
 * (src/radixSort.ts:101-104 and src/shaders/radixSort.wgsl). high_bits = 0 sorts
 * 32-bit keys held in the low word. */
void or_radix_sort(uint64_t* keys, uint32_t* values, uint32_t n, uint32_t high_bits) {
  uint64_t* k2 = (uint64_t*)malloc((size_t)(n ? n : 1) * 8);
  uint32_t* v2 = (uint32_t*)malloc((size_t)(n ? n : 1) * 4);
  uint32_t passes = 4 + 2 * ((high_bits + 15) / 16);
  uint64_t *ki = keys, *ko = k2;
  uint32_t *vi = values, *vo = v2;
  for (uint32_t pass = 0; pass < passes; pass++) {
    uint32_t shift = pass < 4 ? pass * 8 : 32 + (pass - 4) * 8;
    uint32_t hist[256] = {0};
    for (uint32_t i = 0; i < n; i++) hist[(ki[i] >> shift) & 0xff]++;
    uint32_t sum = 0;
    for (int d = 0; d < 256; d++) {
      uint32_t h = hist[d];
      hist[d] = sum;
      sum += h;
    }
    for (uint32_t i = 0; i < n; i++) {
      uint32_t d = (ki[i] >> shift) & 0xff;
      ko[hist[d]] = ki[i];
      vo[hist[d]] = vi[i];
      hist[d]++;
    }
    uint64_t* tk = ki; ki = ko; ko = tk;
    uint32_t* tv = vi; vi = vo; vo = tv;
  }
  if (ki != keys) {
    memcpy(keys, ki, (size_t)n * 8);
    memcpy(values, vi, (size_t)n * 4);
  }
  free(k2);
  free(v2);
}

/* src/shaders/tiles.wgsl:65-84; ranges must start zeroed (tileRasterizer.ts:141). */
void or_find_ranges(const uint64_t* keys, uint32_t pair_count, uint32_t* ranges) {
  for (uint32_t i = 0; i < pair_count; i++) {
    uint32_t tile = (uint32_t)(keys[i] >> 32);
    if (i == 0) {
      ranges[2 * tile] = 0;
    } else {
      uint32_t prev = (uint32_t)(keys[i - 1] >> 32);
      if (tile != prev) {
        ranges[2 * prev + 1] = i;
        ranges[2 * tile] = i;
      }
    }
    if (i == pair_count - 1) ranges[2 * tile + 1] = pair_count;
  }
}

/* ------------------------------------------------------------- blending */

static uint8_t to_unorm8(float v) {
  float c = clampf(v, 0.0f, 1.0f);
  return (uint8_t)rintf(c * 255.0f);
}

/* power = -0.5 (a dx^2 + c dy^2) - b dx dy (src/shaders/rasterize.wgsl:68) as
 * dx (A dx - b dy) + (C dy) dy, A = -0.5 a and C = -0.5 c (exact scalings), with
 * two fused multiply-adds: the kernels' sequence (WGSL leaves contraction to the
 * implementation), so both round alike. */
static float blend_power(const float* s, float dx, float dy) {
  const float A = -0.5f * s[4], C = -0.5f * s[6];
  const float t = fmaf(A, dx, -(s[5] * dy));
  return fmaf(t, dx, (C * dy) * dy);
}

/* src/shaders/rasterize.wgsl:32-100. pixel_color is vec4 per pixel, rgba8 may be NULL.
 * The colour accumulates as c (alpha T) + colour, one fused multiply-add per
 * channel, as the kernels do. */
void or_rasterize(const float* cam, const float* bg, const float* splats, const uint32_t* pair_splats,
                  const uint32_t* ranges, float* pixel_color, uint32_t* pixel_last, uint8_t* rgba8) {
  uint32_t tiles[2];
  tile_grid(cam, tiles);
  const uint32_t width = (uint32_t)CAM_VP(cam, 0), height = (uint32_t)CAM_VP(cam, 1);
  const float vpx = CAM_VP(cam, 0), vpy = CAM_VP(cam, 1);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t tt = 0; tt < (int64_t)tiles[0] * tiles[1]; tt++) {
    uint32_t tile = (uint32_t)tt;
    uint32_t tx = tile % tiles[0], ty = tile / tiles[0];
    uint32_t start = ranges[2 * tile], end = ranges[2 * tile + 1];
    for (uint32_t ly = 0; ly < TILE; ly++)
      for (uint32_t lx = 0; lx < TILE; lx++) {
        uint32_t px = tx * TILE + lx, py = ty * TILE + ly;
        if (!((float)px < vpx && (float)py < vpy)) continue;
        float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
        float T = 1.0f, r = 0.0f, g = 0.0f, b = 0.0f;
        uint32_t visited = 0, last = 0;
        for (uint32_t k = start; k < end; k++) {
          const float* s = splats + (size_t)pair_splats[k] * FPS;
          visited++;
          float dx = cx - s[0], dy = cy - s[1];
          float power = blend_power(s, dx, dy);
          if (power > 0.0f) continue;
          float alpha = minf(0.99f, s[11] * dg_exp_ref(power));
          if (alpha < 1.0f / 255.0f) continue;
          float remaining = T * (1.0f - alpha);
          if (remaining < 0.0001f) break;
          const float w = alpha * T;
          r = fmaf(s[8], w, r);
          g = fmaf(s[9], w, g);
          b = fmaf(s[10], w, b);
          T = remaining;
          last = visited;
        }
        size_t p = (size_t)py * width + px;
        float fr = r + T * bg[0], fg = g + T * bg[1], fb = b + T * bg[2];
        pixel_color[4 * p + 0] = fr;
        pixel_color[4 * p + 1] = fg;
        pixel_color[4 * p + 2] = fb;
        pixel_color[4 * p + 3] = T;
        pixel_last[p] = last;
        if (rgba8) {
          rgba8[4 * p + 0] = to_unorm8(fr);
          rgba8[4 * p + 1] = to_unorm8(fg);
          rgba8[4 * p + 2] = to_unorm8(fb);
          rgba8[4 * p + 3] = 255;
        }
      }
  }
  (void)height;
}

/* src/shaders/rasterizeBackward.wgsl:50-163. The 256 pixels' shares of each splat
 * are summed per tile, columns first then the column sums, into a per-pair record;
 * the pair records are then added to splat_grads in sorted pair order, so the
 * result does not depend on the thread count. splat_grads (9 per splat) is
 * overwritten. */
void or_rasterize_backward(const float* cam, const float* bg, const float* splats, uint32_t count,
                           const uint32_t* pair_splats, const uint32_t* ranges, uint32_t pair_count,
                           const float* pixel_color, const uint32_t* pixel_last, const float* pixel_grads,
                           float* splat_grads) {
  uint32_t tiles[2];
  tile_grid(cam, tiles);
  const uint32_t width = (uint32_t)CAM_VP(cam, 0);
  const float vpx = CAM_VP(cam, 0), vpy = CAM_VP(cam, 1);
  float* pair_grads = (float*)calloc((size_t)(pair_count ? pair_count : 1) * 9, sizeof(float));
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t tt = 0; tt < (int64_t)tiles[0] * tiles[1]; tt++) {
    uint32_t tile = (uint32_t)tt;
    uint32_t tx = tile % tiles[0], ty = tile / tiles[0];
    uint32_t start = ranges[2 * tile], end = ranges[2 * tile + 1];
    if (end <= start) continue;
    uint32_t n = end - start;
    /* Per pixel state walking back to front. */
    float T[256], Tf[256], behind[256][3], na[256], nc[256][3], pg[256][3], bgg[256];
    uint32_t last[256];
    int inside[256];
    float cxs[256], cys[256];
    for (uint32_t t = 0; t < 256; t++) {
      uint32_t lx = t % TILE, ly = t / TILE;
      uint32_t px = tx * TILE + lx, py = ty * TILE + ly;
      inside[t] = (float)px < vpx && (float)py < vpy;
      cxs[t] = (float)px + 0.5f;
      cys[t] = (float)py + 0.5f;
      Tf[t] = 0.0f;
      last[t] = 0;
      pg[t][0] = pg[t][1] = pg[t][2] = 0.0f;
      if (inside[t]) {
        size_t p = (size_t)py * width + px;
        Tf[t] = pixel_color[4 * p + 3];
        last[t] = pixel_last[p];
        pg[t][0] = pixel_grads[4 * p + 0];
        pg[t][1] = pixel_grads[4 * p + 1];
        pg[t][2] = pixel_grads[4 * p + 2];
      }
      bgg[t] = bg[0] * pg[t][0];
      bgg[t] = bgg[t] + bg[1] * pg[t][1];
      bgg[t] = bgg[t] + bg[2] * pg[t][2];
      T[t] = Tf[t];
      behind[t][0] = behind[t][1] = behind[t][2] = 0.0f;
      na[t] = 0.0f;
      nc[t][0] = nc[t][1] = nc[t][2] = 0.0f;
    }
    for (uint32_t jj = n; jj > 0; jj--) {
      uint32_t j = jj - 1; /* position within the tile's list */
      const float* s = splats + (size_t)pair_splats[start + j] * FPS;
      float share[256][9];
      for (uint32_t t = 0; t < 256; t++) {
        for (int v = 0; v < 9; v++) share[t][v] = 0.0f;
        if (!(inside[t] && j < last[t])) continue;
        float dx = cxs[t] - s[0], dy = cys[t] - s[1];
        float power = blend_power(s, dx, dy);
        if (!(power <= 0.0f)) continue;
        float G = dg_exp_ref(power);
        float alpha = minf(0.99f, s[11] * G);
        if (!(alpha >= 1.0f / 255.0f)) continue;
        T[t] = T[t] / (1.0f - alpha);
        for (int k = 0; k < 3; k++) behind[t][k] = na[t] * nc[t][k] + (1.0f - na[t]) * behind[t][k];
        na[t] = alpha;
        nc[t][0] = s[8];
        nc[t][1] = s[9];
        nc[t][2] = s[10];
        float dotv = (s[8] - behind[t][0]) * pg[t][0];
        dotv = dotv + (s[9] - behind[t][1]) * pg[t][1];
        dotv = dotv + (s[10] - behind[t][2]) * pg[t][2];
        float alpha_grad = T[t] * dotv - Tf[t] / (1.0f - alpha) * bgg[t];
        float power_grad = alpha_grad * s[11] * G;
        share[t][0] = power_grad * (s[4] * dx + s[5] * dy);
        share[t][1] = power_grad * (s[5] * dx + s[6] * dy);
        share[t][2] = power_grad * (-0.5f * dx * dx);
        share[t][3] = power_grad * (-dx * dy);
        share[t][4] = power_grad * (-0.5f * dy * dy);
        share[t][5] = alpha_grad * G;
        share[t][6] = alpha * T[t] * pg[t][0];
        share[t][7] = alpha * T[t] * pg[t][1];
        share[t][8] = alpha * T[t] * pg[t][2];
      }
      float* out = pair_grads + (size_t)(start + j) * 9;
      for (int v = 0; v < 9; v++) {
        float cols[16];
        for (uint32_t col = 0; col < 16; col++) {
          float sum = 0.0f;
          for (uint32_t row = 0; row < 16; row++) sum += share[row * 16 + col][v];
          cols[col] = sum;
        }
        float total = 0.0f;
        for (uint32_t col = 0; col < 16; col++) total += cols[col];
        out[v] = total;
      }
    }
  }
  memset(splat_grads, 0, (size_t)count * 9 * sizeof(float));
  for (uint32_t k = 0; k < pair_count; k++) {
    float* g = splat_grads + (size_t)pair_splats[k] * 9;
    const float* pgk = pair_grads + (size_t)k * 9;
    for (int v = 0; v < 9; v++) g[v] += pgk[v];
  }
  free(pair_grads);
}

/* src/shaders/preprocessBackward.wgsl:28-181. gaussian_grads gets 16 floats per
 * Gaussian (slots 7 and 15 zero), sh_grads 45. */
void or_preprocess_backward(const float* cam, const float* gaussians, const float* sh, uint32_t count,
                            uint32_t sh_degree, const float* splats, const float* splat_grads,
                            float* gaussian_grads, float* sh_grads) {
  float campos[3];
  camera_position(cam, campos);
  uint32_t basis_count = sh_count(sh_degree);
  const float vp[2] = {CAM_VP(cam, 0), CAM_VP(cam, 1)};
#pragma omp parallel for schedule(static)
  for (int64_t ii = 0; ii < (int64_t)count; ii++) {
    uint32_t i = (uint32_t)ii;
    float* gg = gaussian_grads + (size_t)i * FPG;
    float* sg = sh_grads + (size_t)i * SHF;
    memset(gg, 0, FPG * sizeof(float));
    memset(sg, 0, SHF * sizeof(float));
    if (splats[(size_t)i * FPS + 3] == 0.0f) continue;
    const float* grad = splat_grads + (size_t)i * 9;
    const float* g = gaussians + (size_t)i * FPG;
    Projection p;
    project(cam, g, &p);
    const float depth = p.depth;
    float ratio[2] = {p.t[0] / depth, p.t[1] / depth};
    float freev[2] = {fabsf(ratio[0]) > p.limit[0] ? 0.0f : 1.0f, fabsf(ratio[1]) > p.limit[1] ? 0.0f : 1.0f};
    float depth2 = depth * depth, depth3 = depth2 * depth;
    float a = p.a, b = p.b, c = p.c, det = p.det;
    /* 1. conic -> 2D covariance */
    float det2 = det * det;
    float a_grad = (-c * c * grad[2] + b * c * grad[3] - b * b * grad[4]) / det2;
    float b_grad = (2.0f * b * c * grad[2] - (det + 2.0f * b * b) * grad[3] + 2.0f * a * b * grad[4]) / det2;
    float c_grad = (-b * b * grad[2] + a * b * grad[3] - a * a * grad[4]) / det2;
    float G2[2][2] = {{a_grad, 0.5f * b_grad}, {0.5f * b_grad, c_grad}}; /* columns */
    /* 2. cov3d_grad = jwᵀ G jw (3x3); j_grad = 2 G jw cov3d wᵀ (mat3x2). */
    float Gjw[3][2]; /* G * jw: column col = Σ_k G[k] * jw[col][k] */
    for (int col = 0; col < 3; col++)
      for (int row = 0; row < 2; row++) {
        float v = G2[0][row] * p.jw[col][0];
        v = v + G2[1][row] * p.jw[col][1];
        Gjw[col][row] = v;
      }
    float cov3d_grad[3][3]; /* (jwᵀ (G jw))(row, col) = Σ_k jw[row][k] * Gjw[col][k] */
    for (int col = 0; col < 3; col++)
      for (int row = 0; row < 3; row++) {
        float v = p.jw[row][0] * Gjw[col][0];
        v = v + p.jw[row][1] * Gjw[col][1];
        cov3d_grad[col][row] = v;
      }
    float t2[3][2]; /* 2 G jw */
    for (int col = 0; col < 3; col++)
      for (int row = 0; row < 2; row++) t2[col][row] = 2.0f * Gjw[col][row];
    float t3[3][2]; /* (2 G jw) cov3d */
    for (int col = 0; col < 3; col++)
      for (int row = 0; row < 2; row++) {
        float v = t2[0][row] * p.cov3d[col][0];
        v = v + t2[1][row] * p.cov3d[col][1];
        v = v + t2[2][row] * p.cov3d[col][2];
        t3[col][row] = v;
      }
    float jg[3][2]; /* t3 wᵀ: column col = Σ_k t3[k] * wᵀ[col][k] = Σ_k t3[k] * w[k][col] */
    for (int col = 0; col < 3; col++)
      for (int row = 0; row < 2; row++) {
        float v = t3[0][row] * p.w[0][col];
        v = v + t3[1][row] * p.w[1][col];
        v = v + t3[2][row] * p.w[2][col];
        jg[col][row] = v;
      }
    /* 3. J moves with t */
    float tg[3];
    tg[0] = jg[2][0] * freev[0] * p.focal[0] / depth2;
    tg[1] = jg[2][1] * freev[1] * -p.focal[1] / depth2;
    tg[2] = 0.0f;
    float depth_grad = jg[0][0] * (-p.focal[0] / depth2) + jg[1][1] * (p.focal[1] / depth2) +
                       jg[2][0] * (-(1.0f + freev[0]) * p.focal[0] * p.tx / depth3) +
                       jg[2][1] * ((1.0f + freev[1]) * p.focal[1] * p.ty / depth3);
    tg[2] = tg[2] - depth_grad;
    /* 4. the 2D center */
    float clip[4];
    for (int row = 0; row < 4; row++) {
      float v = CAM_PROJ(cam, 0, row) * p.t[0];
      v = v + CAM_PROJ(cam, 1, row) * p.t[1];
      v = v + CAM_PROJ(cam, 2, row) * p.t[2];
      v = v + CAM_PROJ(cam, 3, row) * 1.0f;
      clip[row] = v;
    }
    float ndc_grad[2] = {grad[0] * 0.5f * vp[0], grad[1] * -0.5f * vp[1]};
    float ndc_dot = ndc_grad[0] * clip[0];
    ndc_dot = ndc_dot + ndc_grad[1] * clip[1];
    float clip_grad[4] = {ndc_grad[0] / clip[3], ndc_grad[1] / clip[3], 0.0f, -ndc_dot / (clip[3] * clip[3])};
    /* (projᵀ clip_grad)_col = Σ_k proj[col][k] * clip_grad[k] */
    for (int col = 0; col < 3; col++) {
      float v = CAM_PROJ(cam, col, 0) * clip_grad[0];
      v = v + CAM_PROJ(cam, col, 1) * clip_grad[1];
      v = v + CAM_PROJ(cam, col, 2) * clip_grad[2];
      v = v + CAM_PROJ(cam, col, 3) * clip_grad[3];
      tg[col] = tg[col] + v;
    }
    /* 5. colour */
    float off[3] = {g[0] - campos[0], g[1] - campos[1], g[2] - campos[2]};
    float dir[3], dist, basis[15], bgrad[15][3];
    normalize3(off, dir, &dist);
    sh_basis(dir, basis);
    const float* coef = sh + (size_t)i * SHF;
    float raw_color[3] = {g[12], g[13], g[14]};
    for (uint32_t k = 0; k < basis_count; k++)
      for (int ch = 0; ch < 3; ch++) raw_color[ch] = raw_color[ch] + basis[k] * coef[k * 3 + ch];
    float raw_grad[3];
    for (int ch = 0; ch < 3; ch++) raw_grad[ch] = raw_color[ch] < 0.0f ? 0.0f : grad[6 + ch];
    float dgrad[3] = {0.0f, 0.0f, 0.0f};
    sh_basis_gradient(dir, bgrad);
    for (uint32_t k = 0; k < basis_count; k++) {
      for (int ch = 0; ch < 3; ch++) sg[k * 3 + ch] = basis[k] * raw_grad[ch];
      float d = coef[k * 3] * raw_grad[0];
      d = d + coef[k * 3 + 1] * raw_grad[1];
      d = d + coef[k * 3 + 2] * raw_grad[2];
      for (int ax = 0; ax < 3; ax++) dgrad[ax] = dgrad[ax] + bgrad[k][ax] * d;
    }
    float dd = dir[0] * dgrad[0];
    dd = dd + dir[1] * dgrad[1];
    dd = dd + dir[2] * dgrad[2];
    float cpg[3];
    for (int ax = 0; ax < 3; ax++) cpg[ax] = (dgrad[ax] - dir[ax] * dd) / dist;
    /* 6. position: Wᵀ t_grad */
    float pos_grad[3];
    for (int col = 0; col < 3; col++) {
      float v = p.w[col][0] * tg[0];
      v = v + p.w[col][1] * tg[1];
      v = v + p.w[col][2] * tg[2];
      pos_grad[col] = v + cpg[col];
    }
    /* 7. scale and rotation: m_grad = 2 cov3d_grad m */
    float mg[3][3];
    for (int col = 0; col < 3; col++)
      for (int row = 0; row < 3; row++) {
        float v = 2.0f * cov3d_grad[0][row] * p.m[col][0];
        v = v + 2.0f * cov3d_grad[1][row] * p.m[col][1];
        v = v + 2.0f * cov3d_grad[2][row] * p.m[col][2];
        mg[col][row] = v;
      }
    float scale_grad[3];
    for (int k = 0; k < 3; k++) {
      float v = mg[k][0] * p.r[k][0];
      v = v + mg[k][1] * p.r[k][1];
      v = v + mg[k][2] * p.r[k][2];
      scale_grad[k] = v;
    }
    float rg[3][3];
    for (int col = 0; col < 3; col++)
      for (int row = 0; row < 3; row++) rg[col][row] = mg[col][row] * g[4 + col];
    float qw = p.q[0], qx = p.q[1], qy = p.q[2], qz = p.q[3];
    float g00 = rg[0][0], g01 = rg[1][0], g02 = rg[2][0];
    float g10 = rg[0][1], g11 = rg[1][1], g12 = rg[2][1];
    float g20 = rg[0][2], g21 = rg[1][2], g22 = rg[2][2];
    float qg[4];
    qg[0] = 2.0f * (-qz * g01 + qy * g02 + qz * g10 - qx * g12 - qy * g20 + qx * g21);
    qg[1] = 2.0f * (qy * g01 + qz * g02 + qy * g10 - 2.0f * qx * g11 - qw * g12 + qz * g20 + qw * g21 - 2.0f * qx * g22);
    qg[2] = 2.0f * (-2.0f * qy * g00 + qx * g01 + qw * g02 + qx * g10 + qz * g12 - qw * g20 + qz * g21 - 2.0f * qy * g22);
    qg[3] = 2.0f * (-2.0f * qz * g00 - qw * g01 + qx * g02 + qw * g10 - 2.0f * qz * g11 + qy * g12 + qx * g20 + qy * g21);
    float qd = p.q[0] * qg[0];
    qd = qd + p.q[1] * qg[1];
    qd = qd + p.q[2] * qg[2];
    qd = qd + p.q[3] * qg[3];
    gg[0] = pos_grad[0];
    gg[1] = pos_grad[1];
    gg[2] = pos_grad[2];
    gg[3] = grad[5];
    gg[4] = scale_grad[0];
    gg[5] = scale_grad[1];
    gg[6] = scale_grad[2];
    for (int k = 0; k < 4; k++) gg[8 + k] = (qg[k] - p.q[k] * qd) / p.qlen;
    gg[12] = raw_grad[0];
    gg[13] = raw_grad[1];
    gg[14] = raw_grad[2];
  }
}

/* ------------------------------------------------------------------ loss */

/* src/trainingLoss.ts:7-11: the 11-tap window, weights for offsets 0..5, computed in
 * double and stored as float. */
static void window_weights(float w[6]) {
  double raw[6], total;
  for (int k = 0; k < 6; k++) raw[k] = exp(-(double)(k * k) / (2 * 1.5 * 1.5));
  total = raw[0] + 2 * (raw[1] + raw[2] + raw[3] + raw[4] + raw[5]);
  for (int k = 0; k < 6; k++) w[k] = (float)(raw[k] / total);
}

/* One direction of the separable blur over `maps` planar float maps of w*h*3
 * (pixel-major, rgb): src/shaders/loss.wgsl:68-84. Each tap is one fused
 * multiply-add (written out as fmaf, which the WGSL's `sum + w * v` permits):
 * the GPU's blurs run two sums per packed FMA instruction. */
static void blur(const float* in, float* out, int maps, int w, int h, int horizontal, const float wt[6]) {
  size_t n = (size_t)w * h;
  for (int m = 0; m < maps; m++) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++)
      for (int x = 0; x < w; x++)
        for (int ch = 0; ch < 3; ch++) {
          float sum = 0.0f;
          for (int k = -5; k <= 5; k++) {
            int ax = horizontal ? x + k : x, ay = horizontal ? y : y + k;
            if (ax >= 0 && ay >= 0 && ax < w && ay < h)
              sum = fmaf(wt[k < 0 ? -k : k], in[(m * n + (size_t)ay * w + ax) * 3 + ch], sum);
          }
          out[(m * n + (size_t)y * w + x) * 3 + ch] = sum;
        }
  }
}

/* src/shaders/loss.wgsl:53-121 and src/trainingLoss.ts:74-125. rendered is vec4 per
 * pixel (rgb used), target rgba8. Writes pixel_grads (vec4) and pixel_loss, returns
 * Σ pixel_loss + λ summed in double as the TypeScript read() does. */
double or_loss(const float* rendered, const uint8_t* target, int w, int h, float* pixel_grads, float* pixel_loss) {
  const float LAMBDA = 0.2f, C1 = 0.0001f, C2 = 0.0009f;
  size_t n = (size_t)w * h;
  float wt[6];
  window_weights(wt);
  float* mom = (float*)malloc(n * 15 * sizeof(float));
  float* tmp = (float*)malloc(n * 15 * sizeof(float));
  float* blr = (float*)malloc(n * 15 * sizeof(float));
  float* par = (float*)malloc(n * 12 * sizeof(float));
  for (size_t p = 0; p < n; p++)
    for (int ch = 0; ch < 3; ch++) {
      float x = rendered[4 * p + ch], y = (float)target[4 * p + ch] / 255.0f;
      mom[(0 * n + p) * 3 + ch] = x;
      mom[(1 * n + p) * 3 + ch] = y;
      mom[(2 * n + p) * 3 + ch] = x * x;
      mom[(3 * n + p) * 3 + ch] = y * y;
      mom[(4 * n + p) * 3 + ch] = x * y;
    }
  blur(mom, tmp, 5, w, h, 1, wt);
  blur(tmp, blr, 5, w, h, 0, wt);
  for (size_t p = 0; p < n; p++)
    for (int ch = 0; ch < 3; ch++) {
      float mx = blr[(0 * n + p) * 3 + ch], my = blr[(1 * n + p) * 3 + ch];
      float vx = blr[(2 * n + p) * 3 + ch] - mx * mx;
      float vy = blr[(3 * n + p) * 3 + ch] - my * my;
      float cxy = blr[(4 * n + p) * 3 + ch] - mx * my;
      float a1 = 2.0f * mx * my + C1, a2 = 2.0f * cxy + C2;
      float b1 = mx * mx + my * my + C1, b2 = vx + vy + C2;
      float s = a1 * a2 / (b1 * b2);
      par[(0 * n + p) * 3 + ch] = s * (2.0f * my / a1 - 2.0f * my / a2 - 2.0f * mx / b1 + 2.0f * mx / b2);
      par[(1 * n + p) * 3 + ch] = -s / b2;
      par[(2 * n + p) * 3 + ch] = 2.0f * s / a2;
      par[(3 * n + p) * 3 + ch] = s;
    }
  blur(par, tmp, 3, w, h, 1, wt);
  blur(tmp, blr, 3, w, h, 0, wt);
  float scale = 1.0f / (float)(3u * (uint32_t)n);
  double total = 0.0;
  for (size_t p = 0; p < n; p++) {
    float lsum = 0.0f;
    for (int ch = 0; ch < 3; ch++) {
      float x = rendered[4 * p + ch], y = (float)target[4 * p + ch] / 255.0f;
      float sg = blr[(0 * n + p) * 3 + ch] + 2.0f * x * blr[(1 * n + p) * 3 + ch] + y * blr[(2 * n + p) * 3 + ch];
      float sign = x - y > 0.0f ? 1.0f : (x - y < 0.0f ? -1.0f : 0.0f);
      pixel_grads[4 * p + ch] = ((1.0f - LAMBDA) * sign - LAMBDA * sg) * scale;
      float l = (1.0f - LAMBDA) * fabsf(x - y) - LAMBDA * par[(3 * n + p) * 3 + ch];
      lsum = lsum + l;
    }
    pixel_grads[4 * p + 3] = 0.0f;
    pixel_loss[p] = lsum * scale;
    total += (double)pixel_loss[p];
  }
  free(mom);
  free(tmp);
  free(blr);
  free(par);
  return total + (double)LAMBDA;
}

/* src/metrics.ts:20-51: mean SSIM of two vec4 images (rgb used), evaluated in double
 * like the TypeScript (which holds its maps in Float32Array). */
double or_ssim(const float* a, const float* b, int w, int h) {
  size_t n = (size_t)w * h;
  float wt[11];
  {
    double raw[11], sum = 0;
    for (int k = 0; k < 11; k++) { raw[k] = exp(-((k - 5) * (k - 5)) / (2 * 1.5 * 1.5)); sum += raw[k]; }
    for (int k = 0; k < 11; k++) wt[k] = (float)(raw[k] / sum);
  }
  float* maps = (float*)malloc(n * 5 * sizeof(float));
  float* scratch = (float*)malloc(n * sizeof(float));
  double total = 0;
  for (int ch = 0; ch < 3; ch++) {
    for (size_t p = 0; p < n; p++) {
      double x = a[4 * p + ch], y = b[4 * p + ch];
      maps[0 * n + p] = (float)x;
      maps[1 * n + p] = (float)y;
      maps[2 * n + p] = (float)(x * x);
      maps[3 * n + p] = (float)(y * y);
      maps[4 * n + p] = (float)(x * y);
    }
    for (int m = 0; m < 5; m++) {
      float* map = maps + m * n;
      for (int dir = 0; dir < 2; dir++) {
        float* src = dir == 0 ? map : scratch;
        float* dst = dir == 0 ? scratch : map;
        for (int y = 0; y < h; y++)
          for (int x = 0; x < w; x++) {
            double sum = 0;
            for (int k = -5; k <= 5; k++) {
              int sx = dir == 0 ? x + k : x, sy = dir == 0 ? y : y + k;
              if (sx >= 0 && sx < w && sy >= 0 && sy < h) sum += (double)wt[k + 5] * src[(size_t)sy * w + sx];
            }
            dst[(size_t)y * w + x] = (float)sum;
          }
      }
    }
    for (size_t p = 0; p < n; p++) {
      double mx = maps[p], my = maps[n + p];
      double vx = maps[2 * n + p] - mx * mx, vy = maps[3 * n + p] - my * my, cxy = maps[4 * n + p] - mx * my;
      total += ((2 * mx * my + 0.0001) * (2 * cxy + 0.0009)) / ((mx * mx + my * my + 0.0001) * (vx + vy + 0.0009));
    }
  }
  free(maps);
  free(scratch);
  return total / (3.0 * n);
}

/* src/metrics.ts:5-14 */
double or_psnr(const float* a, const float* b, size_t pixels) {
  double se = 0;
  for (size_t p = 0; p < pixels; p++)
    for (int ch = 0; ch < 3; ch++) {
      double d = (double)a[4 * p + ch] - (double)b[4 * p + ch];
      se += d * d;
    }
  return 10.0 * log10(1.0 / (se / (3.0 * pixels)));
}

/* ------------------------------------------------------------ optimizer */

static float sigmoidf_ref(float x) { return 1.0f / (1.0f + expf(-x)); }

/* adam_params: bc1, bc2, lr position, opacity, scale, rotation, color, sh, viewport x, y. */
static float adam_update(float value, float grad, float* m, float lr, float bc1, float bc2) {
  float m0 = 0.9f * m[0] + 0.1f * grad;
  float m1 = 0.999f * m[1] + 0.001f * grad * grad;
  m[0] = m0;
  m[1] = m1;
  return value - lr * (m0 / bc1) / (sqrtf(m1 / bc2) + 1e-15f);
}

static const float SH_C0 = 0.28209479177387814f;

/* src/shaders/adam.wgsl:60-71 */
static void activate_one(const float* params, float* out) {
  for (int k = 0; k < 3; k++) {
    out[k] = params[k];
    out[4 + k] = expf(params[4 + k]);
    out[12 + k] = 0.5f + SH_C0 * params[12 + k];
  }
  out[3] = sigmoidf_ref(params[3]);
  for (int k = 8; k < 12; k++) out[k] = params[k];
}

void or_activate(const float* params, uint32_t count, float* gaussians) {
  for (uint32_t i = 0; i < count; i++) activate_one(params + (size_t)i * FPG, gaussians + (size_t)i * FPG);
}

/* src/shaders/adam.wgsl:80-107 */
void or_adam_step(const float* ap, float* params, float* sh, float* moments, const float* ggrad, const float* sgrad,
                  float* gaussians, uint32_t count) {
  const float bc1 = ap[0], bc2 = ap[1];
#pragma omp parallel for schedule(static)
  for (int64_t ii = 0; ii < (int64_t)count; ii++) {
    uint32_t i = (uint32_t)ii;
    float* p = params + (size_t)i * FPG;
    const float* g = ggrad + (size_t)i * FPG;
    float* m = moments + (size_t)i * SLOTS * 2;
    for (int k = 0; k < 3; k++) {
      p[k] = adam_update(p[k], g[k], m + 2 * k, ap[2], bc1, bc2);
      float sgr = g[4 + k] * expf(p[4 + k]);
      p[4 + k] = adam_update(p[4 + k], sgr, m + 2 * (4 + k), ap[4], bc1, bc2);
      float cg = g[12 + k] * SH_C0;
      p[12 + k] = adam_update(p[12 + k], cg, m + 2 * (12 + k), ap[6], bc1, bc2);
    }
    float op = sigmoidf_ref(p[3]);
    float og = g[3] * op * (1.0f - op);
    p[3] = adam_update(p[3], og, m + 2 * 3, ap[3], bc1, bc2);
    for (int k = 8; k < 12; k++) p[k] = adam_update(p[k], g[k], m + 2 * k, ap[5], bc1, bc2);
    for (uint32_t k = 0; k < SHF; k++) {
      size_t s = (size_t)i * SHF + k;
      sh[s] = adam_update(sh[s], sgrad[s], m + 2 * (FPG + k), ap[7], bc1, bc2);
    }
    activate_one(p, gaussians + (size_t)i * FPG);
  }
}

/* src/shaders/adam.wgsl:112-121 */
void or_reset_opacity(float* params, float* moments, float* gaussians, uint32_t count) {
  const float RESET = -4.59511985013459f;
  for (uint32_t i = 0; i < count; i++) {
    float* p = params + (size_t)i * FPG;
    p[3] = minf(p[3], RESET);
    moments[(size_t)i * SLOTS * 2 + 6] = 0.0f;
    moments[(size_t)i * SLOTS * 2 + 7] = 0.0f;
    activate_one(p, gaussians + (size_t)i * FPG);
  }
}

/* src/shaders/adam.wgsl:126-134 */
void or_accumulate_stats(const float* splats, const float* splat_grads, float vpx, float vpy, float* stats,
                         uint32_t count) {
  for (uint32_t i = 0; i < count; i++) {
    float radius = splats[(size_t)i * FPS + 3];
    if (radius == 0.0f) continue;
    float gx = splat_grads[(size_t)i * 9] * vpx * 0.5f, gy = splat_grads[(size_t)i * 9 + 1] * vpy * 0.5f;
    float len = sqrtf(gx * gx + gy * gy);
    float* s = stats + (size_t)i * 4;
    s[0] = s[0] + len;
    s[1] = s[1] + 1.0f;
    s[2] = maxf(s[2], radius);
    s[3] = 0.0f;
  }
}

/* --------------------------------------------------------------- densify */

/* dp: grad threshold, clone max size, min opacity, max size (0 = off); seed. */
static uint32_t densify_action(const float* params, const float* stats, uint32_t i, const float* dp) {
  const float* p = params + (size_t)i * FPG;
  const float* s = stats + (size_t)i * 4;
  float grad = s[1] > 0.0f ? s[0] / s[1] : 0.0f;
  float size = expf(maxf(p[4], maxf(p[5], p[6])));
  float opacity = sigmoidf_ref(p[3]);
#define REMOVED(o, sz) ((o) < dp[2] || (dp[3] > 0.0f && (sz) > dp[3]))
  if (grad >= dp[0]) {
    if (size <= dp[1]) return REMOVED(opacity, size) ? 0u : 2u;
    return REMOVED(opacity, size / 1.6f) ? 0u : 3u;
  }
  return REMOVED(opacity, size) ? 0u : 1u;
#undef REMOVED
}

/* src/shaders/densify.wgsl:96-107: per-Gaussian output counts and the tally
 * [dropped, kept, cloned, split]. */
void or_densify_count(const float* params, const float* stats, uint32_t count, const float* dp, uint32_t* outputs,
                      uint32_t tally[4]) {
  tally[0] = tally[1] = tally[2] = tally[3] = 0;
  for (uint32_t i = 0; i < count; i++) {
    uint32_t a = densify_action(params, stats, i, dp);
    outputs[i] = a == 0 ? 0u : (a >= 2 ? 2u : 1u);
    tally[a]++;
  }
}

/* src/shaders/densify.wgsl:112-118 */
uint32_t or_pcg(uint32_t v) {
  uint32_t state = v * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

static float unit_of(uint32_t h) { return ((float)(h >> 8u) + 0.5f) / 16777216.0f; }

/* src/shaders/densify.wgsl:148-180. outputs holds the scanned offsets. */
void or_densify_scatter(const float* params, const float* stats, const float* sh, const float* moments,
                        const uint32_t* outputs, uint32_t count, const float* dp, uint32_t seed, float* new_params,
                        float* new_sh, float* new_moments) {
  for (uint32_t i = 0; i < count; i++) {
    uint32_t a = densify_action(params, stats, i, dp);
    uint32_t o = outputs[i];
    const float* p = params + (size_t)i * FPG;
#define COPY(dst, keep)                                                                          \
  do {                                                                                           \
    memcpy(new_params + (size_t)(dst) * FPG, p, FPG * 4);                                        \
    memcpy(new_sh + (size_t)(dst) * SHF, sh + (size_t)i * SHF, SHF * 4);                         \
    if (keep)                                                                                    \
      memcpy(new_moments + (size_t)(dst) * SLOTS * 2, moments + (size_t)i * SLOTS * 2, SLOTS * 8); \
    else                                                                                         \
      memset(new_moments + (size_t)(dst) * SLOTS * 2, 0, SLOTS * 8);                             \
  } while (0)
    if (a == 1 || a == 2) COPY(o, 1);
    if (a == 2) {
      COPY(o + 1, 0);
      new_params[(size_t)(o + 1) * FPG + 7] = 1.0f;
      new_params[(size_t)(o + 1) * FPG + 15] = (float)seed;
    }
    if (a == 3) {
      float r[3][3];
      rotation_matrix(p + 8, r, NULL, NULL);
      for (uint32_t c = 0; c < 2; c++) {
        uint32_t child = o + c;
        COPY(child, 0);
        uint32_t h1 = or_pcg(seed ^ or_pcg(2u * i + c));
        uint32_t h2 = or_pcg(h1), h3 = or_pcg(h2), h4 = or_pcg(h3);
        float r1 = sqrtf(-2.0f * logf(unit_of(h1)));
        float r2 = sqrtf(-2.0f * logf(unit_of(h3)));
        const float tau = 6.283185307179586f;
        float nrm[3] = {r1 * cosf(tau * unit_of(h2)), r1 * sinf(tau * unit_of(h2)), r2 * cosf(tau * unit_of(h4))};
        float sv[3] = {expf(p[4]) * nrm[0], expf(p[5]) * nrm[1], expf(p[6]) * nrm[2]};
        for (int row = 0; row < 3; row++) {
          float v = r[0][row] * sv[0];
          v = v + r[1][row] * sv[1];
          v = v + r[2][row] * sv[2];
          new_params[(size_t)child * FPG + row] = p[row] + v;
          /* WGSL folds log(SPLIT_SHRINK) of the abstract constant 1.6 at full precision. */
          new_params[(size_t)child * FPG + 4 + row] = p[4 + row] - 0.470003629245735553f;
        }
        new_params[(size_t)child * FPG + 7] = 2.0f;
        new_params[(size_t)child * FPG + 15] = (float)seed;
      }
    }
#undef COPY
  }
}

/* ------------------------------------------------------------------ misc */

/* src/random.ts:3-12: returns the next value and advances *state. */
double or_mulberry32_next(uint32_t* state) {
  *state = *state + 0x6d2b79f5u;
  uint32_t t = *state;
  t = (t ^ (t >> 15)) * (t | 1u);
  t ^= t + (t ^ (t >> 7)) * (t | 61u);
  return (double)((t ^ (t >> 14)) >> 0) / 4294967296.0;
}

/* The whole forward frame as the reference's TileRasterizer.encode records it, for
 * tests and the CPU baseline. Buffers are caller-owned; keys/values need `capacity`
 * entries, ranges tiles*2. Returns the pair total (which may exceed capacity). */
uint32_t or_render_frame(const float* cam, const float* bg, const float* gaussians, const float* sh, uint32_t count,
                         uint32_t sh_degree, uint32_t capacity, float* splats, uint32_t* offsets, uint64_t* keys,
                         uint32_t* values, uint32_t* ranges, float* pixel_color, uint32_t* pixel_last,
                         uint8_t* rgba8) {
  uint32_t tiles[2];
  tile_grid(cam, tiles);
  or_preprocess(cam, gaussians, sh, count, sh_degree, splats);
  or_count_tiles(cam, splats, count, offsets);
  uint32_t total = or_exclusive_scan(offsets, count);
  or_duplicate(cam, splats, offsets, count, capacity, keys, values);
  uint32_t pairs = total < capacity ? total : capacity;
  or_radix_sort(keys, values, pairs, 16);
  memset(ranges, 0, (size_t)tiles[0] * tiles[1] * 8);
  or_find_ranges(keys, pairs, ranges);
  or_rasterize(cam, bg, splats, values, ranges, pixel_color, pixel_last, rgba8);
  return total;
}

/* src/shaders/nearestNeighbors.wgsl:13-44, by brute force as the reference does:
 * for each point (points: n × 4 floats, xyz + padding) the mean of the squared
 * distances to its 3 nearest other points. d = q - p per component, then
 * d.x² + d.y² + d.z² summed from x; the three smallest kept with the WGSL's strict
 * comparisons, starting from 3.4e38. */
static float neighbor_distance2_of(const float* points, uint32_t n, uint32_t i) {
  const float* me = points + (size_t)i * 4;
  float b0 = 3.4e38f, b1 = 3.4e38f, b2 = 3.4e38f;
  for (uint32_t j = 0; j < n; j++) {
    if (j == i) continue;
    const float* q = points + (size_t)j * 4;
    const float dx = q[0] - me[0], dy = q[1] - me[1], dz = q[2] - me[2];
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < b2) {
      if (d2 < b1) {
        b2 = b1;
        if (d2 < b0) {
          b1 = b0;
          b0 = d2;
        } else {
          b1 = d2;
        }
      } else {
        b2 = d2;
      }
    }
  }
  return (b0 + b1 + b2) / 3.0f;
}

void or_mean_neighbor_distance2(const float* points, uint32_t n, float* out) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < (int64_t)n; i++) out[i] = neighbor_distance2_of(points, n, (uint32_t)i);
}

/* The same for the m points listed in `which` only (out[k] for point which[k]). */
void or_mean_neighbor_distance2_of(const float* points, uint32_t n, const uint32_t* which, uint32_t m, float* out) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t k = 0; k < (int64_t)m; k++) out[k] = neighbor_distance2_of(points, n, which[k]);
}

/* src/loadDataset.ts:99-121: the starting raw Gaussians. The arithmetic there is
 * JavaScript's float64, rounded to float32 by the Float32Array stores. */
void or_initial_gaussians(const float* positions, const uint8_t* colors, const float* distance2, uint32_t n,
                          float* params) {
  const double sh_c0 = 0.28209479177387814;
  const float opacity_logit = (float)log(0.1 / 0.9);
  for (uint32_t i = 0; i < n; i++) {
    float* g = params + (size_t)i * FPG;
    memset(g, 0, FPG * sizeof(float));
    const double d2 = (double)distance2[i];
    const double log_scale = 0.5 * log(d2 > 1e-7 ? d2 : 1e-7);
    for (int k = 0; k < 3; k++) {
      g[k] = positions[(size_t)i * 3 + k];
      g[4 + k] = (float)log_scale;
      g[12 + k] = (float)(((double)colors[(size_t)i * 3 + k] / 255.0 - 0.5) / sh_c0);
    }
    g[3] = opacity_logit;
    g[8] = 1.0f;
  }
}
