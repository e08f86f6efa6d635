// fe_footprint.cuh -- float32 screen footprint and ray-invariant record of one (Gaussian,
// camera) pair, shared by the image preprocess (preprocess.cu) and the pixel-list renderer
// (pixlist.cu).
//
//   M = U^T R^T (a = M rays_cam), Y = cof(M), det M = U00 U11 U22 (R is a rotation).
//   Camera-frame covariance: Sc = Yh^T Yh with Yh = Y / det M = M^-T (entries of order sigma).
//   The k-sigma ellipsoid's outline is the conic whose dual is C = k2 Sc - p p^T (p: camera-frame
//   mean, k2 = k^2). Its vertical tangents x = (c02 +- sqrt(D)) / c22 use
//     D = c02^2 - c00 c22 = k2 (|pz Yh0 - px Yh2|^2 - k2 |Yh0 x Yh2|^2)
//   (Yh0, Yh2: columns of Yh), where the p^4 terms cancel analytically; likewise for y.
#pragma once

#include "fe_common.cuh"

namespace fe {

struct CamTerms {
  float M[9];
  float Y[9];
  float detM;
  V3<float> pc;
};

// U: upper-triangular precision factor (row-major, lower entries ignored); R: row-major camera
// rotation (rays_world = rays_cam @ R); t: camera centre.
__device__ __forceinline__ CamTerms camera_terms(const float* mean, const float* prec,
                                                 const float* R, const float* t) {
  CamTerms ct;
  const float U00 = prec[0], U01 = prec[1], U02 = prec[2], U11 = prec[4], U12 = prec[5],
              U22 = prec[8];
  const V3<float> p = v3(mean[0] - t[0], mean[1] - t[1], mean[2] - t[2]);
  ct.pc = matvec(R, p);
  // M[i][j] = sum_{k<=i} U[k][i] R[j][k]
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    ct.M[0 * 3 + j] = U00 * R[j * 3 + 0];
    ct.M[1 * 3 + j] = U01 * R[j * 3 + 0] + U11 * R[j * 3 + 1];
    ct.M[2 * 3 + j] = U02 * R[j * 3 + 0] + U12 * R[j * 3 + 1] + U22 * R[j * 3 + 2];
  }
  cofactor3(ct.M, ct.Y);
  ct.detM = U00 * U11 * U22;
  return ct;
}

// k^2 of the cut-off: density threshold (FE_CULL_EPS) or fixed number of standard deviations.
__device__ __forceinline__ float cutoff_k2(float logw, int cull_mode, float cull_param) {
  if (cull_mode == FE_CULL_EPS) {
    const float eps = cull_param > 0.f ? cull_param : kDefaultCullEps;
    return 2.f * (logw - logf(eps));
  }
  const float k = cull_param > 0.f ? cull_param : 3.f;
  return k * k;
}

enum { kFootBounded = 0, kFootFull = 1 };

// Pixel-space bounding box [ulo, uhi] x [vlo, vhi] of the k-sigma ellipsoid's projection
// (k2 > 0). kFootFull when the projection is unbounded (the camera inside the ellipsoid or the
// ellipsoid reaching the camera plane) or not finite.
__device__ __forceinline__ int screen_bounds(const CamTerms& ct, float k2, float fx, float fy,
                                             float cx, float cy, float& ulo, float& uhi,
                                             float& vlo, float& vhi) {
  const V3<float>& pc = ct.pc;
  if (!(ct.detM != 0.f) || !isfinite(ct.detM)) return kFootFull;
  const float inv = 1.f / ct.detM;
  float Yh[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) Yh[q] = ct.Y[q] * inv;
  // Columns c of Yh: Yh[0*3+c], Yh[1*3+c], Yh[2*3+c].
  auto col = [&](int c) { return v3(Yh[c], Yh[3 + c], Yh[6 + c]); };
  const V3<float> y0 = col(0), y1 = col(1), y2 = col(2);
  const float s02 = dot(y0, y2), s12 = dot(y1, y2), s22 = dot(y2, y2);
  const float c22 = k2 * s22 - pc.z * pc.z;
  if (!(c22 < 0.f)) return kFootFull;
  const V3<float> ex = pc.z * y0 - pc.x * y2, ey = pc.z * y1 - pc.y * y2;
  const V3<float> xx = cross(y0, y2), xy = cross(y1, y2);
  const float dx = fmaxf(k2 * (dot(ex, ex) - k2 * dot(xx, xx)), 0.f);
  const float dy = fmaxf(k2 * (dot(ey, ey) - k2 * dot(xy, xy)), 0.f);
  const float c02 = k2 * s02 - pc.x * pc.z, c12 = k2 * s12 - pc.y * pc.z;
  const float sx = sqrtf(dx), sy = sqrtf(dy);
  const float xa = (c02 + sx) / c22, xb = (c02 - sx) / c22;
  const float ya = (c12 + sy) / c22, yb = (c12 - sy) / c22;
  ulo = fmaf(fx, fminf(xa, xb), cx);
  uhi = fmaf(fx, fmaxf(xa, xb), cx);
  vlo = fmaf(fy, fminf(ya, yb), cy);
  vhi = fmaf(fy, fmaxf(ya, yb), cy);
  if (!(isfinite(ulo) && isfinite(uhi) && isfinite(vlo) && isfinite(vhi))) return kFootFull;
  return kFootBounded;
}

// Ray-invariant record around an expansion centre: the projected mean clamped to
// [ucl, uch] x [vcl, vch], or (uc_def, vc_def) when the projection is unbounded.
__device__ __forceinline__ void make_record(const CamTerms& ct, float logw, float fx, float fy,
                                            float cx, float cy, float uc_def, float vc_def,
                                            float ucl, float uch, float vcl, float vch,
                                            GaussRec& rec) {
  const V3<float>& pc = ct.pc;
  float uc = uc_def, vc = vc_def;
  if (fabsf(pc.z) > 1e-6f * sqrtf(dot(pc, pc))) {
    const float u0 = fmaf(fx, pc.x / pc.z, cx), v0 = fmaf(fy, pc.y / pc.z, cy);
    if (isfinite(u0) && isfinite(v0)) {
      uc = fminf(fmaxf(u0, ucl), uch);
      vc = fminf(fmaxf(v0, vcl), vch);
    }
  }
  const float ifx = 1.f / fx, ify = 1.f / fy;
  const float* M = ct.M;
  const float* Y = ct.Y;
  const V3<float> r0 = v3((uc - cx) * ifx, (vc - cy) * ify, 1.f);
  const V3<float> a0 = matvec(M, r0), b = matvec(M, pc);
  const V3<float> c0 = cross(r0, pc);
  const V3<float> y0 = matvec(Y, c0);
  const V3<float> y1 = matvec(Y, v3(0.f, -pc.z * ifx, pc.y * ifx));
  const V3<float> y2 = matvec(Y, v3(pc.z * ify, 0.f, -pc.x * ify));
  rec.a0[0] = a0.x; rec.a0[1] = a0.y; rec.a0[2] = a0.z;
  rec.a1[0] = M[0] * ifx; rec.a1[1] = M[3] * ifx; rec.a1[2] = M[6] * ifx;
  rec.a2[0] = M[1] * ify; rec.a2[1] = M[4] * ify; rec.a2[2] = M[7] * ify;
  rec.b[0] = b.x; rec.b[1] = b.y; rec.b[2] = b.z;
  rec.y0[0] = y0.x; rec.y0[1] = y0.y; rec.y0[2] = y0.z;
  rec.y1[0] = y1.x; rec.y1[1] = y1.y; rec.y1[2] = y1.z;
  rec.y2[0] = y2.x; rec.y2[1] = y2.y; rec.y2[2] = y2.z;
  rec.uc = uc;
  rec.vc = vc;
  rec.c2 = logw * kLog2e;
}

}  // namespace fe
