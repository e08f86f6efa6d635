/*
 * ref_binning.c -- CPU restatement of the reference CUDA rasterizer's binning (TEST
 * INFRASTRUCTURE ONLY: tests/ and the CPU baseline may load it; the product never does).
 *
 * Restates, in IEEE single precision with no contraction (build with -ffp-contract=off):
 *   preprocessCUDA          cuda_rasterizer/forward.cu:126-203
 *     computeCov3D          cuda_rasterizer/forward.cu:65-122 (covariance part)
 *     computeCov2D          cuda_rasterizer/forward.cu:21-60
 *     in_frustum            cuda_rasterizer/auxiliary.h:144-169
 *     ndc2Pix (double)      cuda_rasterizer/auxiliary.h:46-49
 *     getRect               cuda_rasterizer/auxiliary.h:51-61 (BLOCK_X = BLOCK_Y = 8, config.h)
 *     transformPoint4x3/4x4 cuda_rasterizer/auxiliary.h:63-82
 *   focal lengths           cuda_rasterizer/rasterizer_impl.cu:205-206
 *   inclusive scan          cuda_rasterizer/rasterizer_impl.cu:244
 *   getGaussianTileKeys     cuda_rasterizer/rasterizer_impl.cu:82-124
 *   sort of the keys        cuda_rasterizer/rasterizer_impl.cu:287 (unique keys: any sort agrees)
 *   getPerTileRanges        cuda_rasterizer/rasterizer_impl.cu:127-152 (empty tiles stay {0,0})
 *
 * The reference's glm dependency is absent; its column-major mat3 products are restated from the
 * maths as (A*B)[i][j] = A[0][j]*B[i][0] + A[1][j]*B[i][1] + A[2][j]*B[i][2], summed left to
 * right, which is also how the project's glm stand-in (oracle/ref_shim) computes them when the
 * reference sources themselves are compiled.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float c[3][3]; } gm3; /* c[col][row] */

static gm3 gm_mul(const gm3 *a, const gm3 *b) {
  gm3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      float t0 = a->c[0][j] * b->c[i][0];
      float t1 = a->c[1][j] * b->c[i][1];
      float t2 = a->c[2][j] * b->c[i][2];
      float s = t0 + t1;
      r.c[i][j] = s + t2;
    }
  return r;
}

static gm3 gm_t(const gm3 *a) {
  gm3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.c[i][j] = a->c[j][i];
  return r;
}

static gm3 gm_make(float a, float b, float c, float d, float e, float f, float g, float h, float k) {
  gm3 r;
  r.c[0][0] = a; r.c[0][1] = b; r.c[0][2] = c;
  r.c[1][0] = d; r.c[1][1] = e; r.c[1][2] = f;
  r.c[2][0] = g; r.c[2][1] = h; r.c[2][2] = k;
  return r;
}

/* matrix[r]*x + matrix[4+r]*y + matrix[8+r]*z + matrix[12+r], left to right. */
static float tp_row(const float *m, int r, float x, float y, float z) {
  float a = m[r] * x;
  float b = m[4 + r] * y;
  float c = m[8 + r] * z;
  float s = a + b;
  s = s + c;
  return s + m[12 + r];
}

static float ndc2pix(float v, int S) { return (float)((((double)v + 1.0) * S - 1.0) * 0.5); }

/* (int) of a float as the GPU converts it: truncate toward zero, saturate, NaN -> 0. */
static int f2i(float x) {
  if (x != x) return 0;
  if (x >= 2147483647.0f) return 2147483647;
  if (x <= -2147483648.0f) return (-2147483647 - 1);
  return (int)x;
}

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

static void get_rect(float px, float py, int r, int gx, int gy, int *x0, int *y0, int *x1, int *y1) {
  float rf = (float)r;
  *x0 = imin(gx, imax(0, f2i((px - rf) / 8.0f)));
  *y0 = imin(gy, imax(0, f2i((py - rf) / 8.0f)));
  float tx = px + rf; tx = tx + 8.0f; tx = tx - 1.0f;
  float ty = py + rf; ty = ty + 8.0f; ty = ty - 1.0f;
  *x1 = imin(gx, imax(0, f2i(tx / 8.0f)));
  *y1 = imin(gy, imax(0, f2i(ty / 8.0f)));
}

/* One Gaussian of preprocessCUDA. Writes radius, point_image, tiles_touched and the rect. */
static void preprocess_one(int idx, float n_std, const float *means, const float *scales,
                           const float *rots, const float *view, const float *proj, int W, int H,
                           float tan_fovx, float tan_fovy, float focal_x, float focal_y, int gx,
                           int gy, int32_t *radii, float *means2d, uint32_t *touched, int *rect) {
  radii[idx] = 0;
  touched[idx] = 0;
  rect[4 * idx] = rect[4 * idx + 1] = rect[4 * idx + 2] = rect[4 * idx + 3] = 0;
  const float px = means[3 * idx], py = means[3 * idx + 1], pz = means[3 * idx + 2];
  const float vz = tp_row(view, 2, px, py, pz);
  if (vz <= 0.2f) return;
  const float hx = tp_row(proj, 0, px, py, pz);
  const float hy = tp_row(proj, 1, px, py, pz);
  const float hw = tp_row(proj, 3, px, py, pz);
  const float p_w = 1.0f / (hw + 0.0000001f);
  const float projx = hx * p_w, projy = hy * p_w;

  /* computeCov3D */
  const float sx = 1.0f * scales[3 * idx], sy = 1.0f * scales[3 * idx + 1],
              sz = 1.0f * scales[3 * idx + 2];
  const float r = rots[4 * idx], x = rots[4 * idx + 1], y = rots[4 * idx + 2], z = rots[4 * idx + 3];
  gm3 S = gm_make(sx, 0.f, 0.f, 0.f, sy, 0.f, 0.f, 0.f, sz);
  float yy = y * y, zz = z * z, xx = x * x, xy = x * y, xz = x * z, yz = y * z;
  float rz = r * z, ry = r * y, rx = r * x;
  gm3 R = gm_make(1.f - 2.f * (yy + zz), 2.f * (xy - rz), 2.f * (xz + ry),
                  2.f * (xy + rz), 1.f - 2.f * (xx + zz), 2.f * (yz - rx),
                  2.f * (xz - ry), 2.f * (yz + rx), 1.f - 2.f * (xx + yy));
  gm3 M = gm_mul(&S, &R);
  gm3 Mt = gm_t(&M);
  gm3 Sig = gm_mul(&Mt, &M);
  const float c0 = Sig.c[0][0], c1 = Sig.c[0][1], c2 = Sig.c[0][2], c3 = Sig.c[1][1],
              c4 = Sig.c[1][2], c5 = Sig.c[2][2];

  /* computeCov2D */
  float tx = tp_row(view, 0, px, py, pz);
  float ty = tp_row(view, 1, px, py, pz);
  const float tz = vz;
  const float limx = 1.3f * tan_fovx, limy = 1.3f * tan_fovy;
  const float txtz = tx / tz, tytz = ty / tz;
  tx = fminf(limx, fmaxf(-limx, txtz)) * tz;
  ty = fminf(limy, fmaxf(-limy, tytz)) * tz;
  const float tz2 = tz * tz;
  gm3 J = gm_make(focal_x / tz, 0.0f, -((focal_x * tx) / tz2), 0.0f, focal_y / tz,
                  -((focal_y * ty) / tz2), 0.f, 0.f, 0.f);
  gm3 Wm = gm_make(view[0], view[4], view[8], view[1], view[5], view[9], view[2], view[6], view[10]);
  gm3 T = gm_mul(&Wm, &J);
  gm3 Vrk = gm_make(c0, c1, c2, c1, c3, c4, c2, c4, c5);
  gm3 Tt = gm_t(&T), Vt = gm_t(&Vrk);
  gm3 tmp = gm_mul(&Tt, &Vt);
  gm3 cov = gm_mul(&tmp, &T);
  const float ca = cov.c[0][0] + 0.3f, cb = cov.c[0][1], cc = cov.c[1][1] + 0.3f;

  const float det = ca * cc - cb * cb;
  if (det == 0.0f) return;
  const float mid = 0.5f * (ca + cc);
  const float disc = sqrtf(fmaxf(0.1f, mid * mid - det));
  const float l1 = mid + disc, l2 = mid - disc;
  const float radius = ceilf(n_std * sqrtf(fmaxf(l1, l2)));
  const float pix_x = ndc2pix(projx, W), pix_y = ndc2pix(projy, H);
  const int ir = f2i(radius);
  int x0, y0, x1, y1;
  get_rect(pix_x, pix_y, ir, gx, gy, &x0, &y0, &x1, &y1);
  const uint32_t area = (uint32_t)(x1 - x0) * (uint32_t)(y1 - y0);
  if (area == 0) return;
  radii[idx] = ir;
  means2d[2 * idx] = pix_x;
  means2d[2 * idx + 1] = pix_y;
  touched[idx] = area;
  rect[4 * idx] = x0; rect[4 * idx + 1] = y0; rect[4 * idx + 2] = x1; rect[4 * idx + 3] = y1;
}

static int cmp_u64(const void *a, const void *b) {
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/*
 * Full reference binning. tiles_touched receives the inclusive prefix sum (as the reference leaves
 * it after its in-place scan). keys must hold `key_capacity` entries; ranges 2*T uint32.
 * Returns the key count K (or -1 if K > key_capacity; -2 on allocation failure).
 */
int64_t ref_binning(int P, int H, int W, float n_std, const float *means, const float *scales,
                    const float *rots, const float *view, const float *proj, float tan_fovx,
                    float tan_fovy, int32_t *radii, float *means2d, uint32_t *tiles_touched,
                    uint64_t *keys, int64_t key_capacity, uint32_t *ranges) {
  const int gx = (W + 7) / 8, gy = (H + 7) / 8;
  const int64_t T = (int64_t)gx * gy;
  const float focal_y = (float)H / (2.0f * tan_fovy);
  const float focal_x = (float)W / (2.0f * tan_fovx);
  int *rect = (int *)malloc(sizeof(int) * 4 * (size_t)(P > 0 ? P : 1));
  if (!rect) return -2;
  for (int i = 0; i < P; ++i)
    preprocess_one(i, n_std, means, scales, rots, view, proj, W, H, tan_fovx, tan_fovy, focal_x,
                   focal_y, gx, gy, radii, means2d, tiles_touched, rect);
  uint64_t acc = 0;
  for (int i = 0; i < P; ++i) {
    acc += tiles_touched[i];
    tiles_touched[i] = (uint32_t)acc;
  }
  memset(ranges, 0, sizeof(uint32_t) * 2 * (size_t)T);
  if ((int64_t)acc > key_capacity) {
    free(rect);
    return -1;
  }
  int64_t off = 0;
  for (int g = 0; g < P; ++g) {
    if (radii[g] <= 0) continue;
    for (int y = rect[4 * g + 1]; y < rect[4 * g + 3]; ++y)
      for (int x = rect[4 * g]; x < rect[4 * g + 2]; ++x)
        keys[off++] = ((uint64_t)(uint32_t)(y * gx + x) << 32) | (uint64_t)(uint32_t)g;
  }
  free(rect);
  qsort(keys, (size_t)off, sizeof(uint64_t), cmp_u64);
  for (int64_t i = 0; i < off; ++i) {
    const uint32_t t = (uint32_t)(keys[i] >> 32);
    if (i == 0) ranges[2 * t] = 0;
    else {
      const uint32_t pt = (uint32_t)(keys[i - 1] >> 32);
      if (t != pt) {
        ranges[2 * pt + 1] = (uint32_t)i;
        ranges[2 * t] = (uint32_t)i;
      }
    }
    if (i == off - 1) ranges[2 * t + 1] = (uint32_t)off;
  }
  return off;
}
