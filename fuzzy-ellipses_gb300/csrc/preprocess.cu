// preprocess.cu -- per (Gaussian, view) work: screen footprint in tiles and ray-invariant record.
//
// Two binning rules share the record builder:
//  * preprocess_kernel: the footprint is the exact screen bounding box of the Gaussian's
//    k-sigma ellipsoid as seen through the pinhole (every pixel whose ray line passes within
//    Mahalanobis distance k of the mean), from the dual conic of the ellipsoid. k comes from a
//    density cut-off (FE_CULL_EPS) or is fixed (FE_CULL_NSTD). Float32 throughout, with the
//    conic's discriminant and the record terms in forms free of cancellation.
//  * preprocess_reference_kernel: the reference's binning (cuda_rasterizer/forward.cu:126-203 with
//    computeCov3D :65-122, computeCov2D :21-60 and auxiliary.h:46-61,144-169), restated with
//    explicitly rounded float operations so the compiler cannot contract them, which makes its
//    tile rectangles bit-reproducible (the reference built with -fmad=false computes the same).
#include "fe_footprint.cuh"
#include "fe_kernels.cuh"

namespace fe {

// ------------------------------------------------------------------------------------------
// Record builder, double precision (the legacy-interface records).
// ------------------------------------------------------------------------------------------

// U: upper-triangular precision factor (row-major 3x3, lower entries ignored), precision U U^T.
// R: row-major camera rotation (rays_world = rays_cam @ R). t: camera centre.
struct RecordInputs {
  double m[3];
  double U[9];
  double w;
  double R[9];
  double t[3];
};

__device__ void build_camera_terms(const RecordInputs& in, double M[9], double Y[9],
                                   V3<double>& pc) {
  V3<double> p = v3(in.m[0] - in.t[0], in.m[1] - in.t[1], in.m[2] - in.t[2]);
  pc = matvec(in.R, p);  // camera-frame mean
  // M = U^T R^T:  a = M rays_cam = U^T (rays_cam @ R)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k <= i; ++k) s += in.U[k * 3 + i] * in.R[j * 3 + k];
      M[i * 3 + j] = s;
    }
  cofactor3(M, Y);
}

__device__ void write_record(const RecordInputs& in, const double M[9], const double Y[9],
                             const V3<double>& pc, float fx, float fy, float cx, float cy,
                             int H, int W, GaussRec* out) {
  // Expansion centre: the projected mean when it is finite and near the image, else the image
  // centre. Any centre is exact in real arithmetic; a nearby one keeps the float32 terms small.
  double uc = 0.5 * W, vc = 0.5 * H;
  const double pn = sqrt(dot(pc, pc));
  if (fabs(pc.z) > 1e-6 * pn) {
    double u0 = fx * pc.x / pc.z + cx;
    double v0 = fy * pc.y / pc.z + cy;
    if (isfinite(u0) && isfinite(v0)) {
      uc = fmin(fmax(u0, -1.0 * W), 2.0 * W);
      vc = fmin(fmax(v0, -1.0 * H), 2.0 * H);
    }
  }
  const float ucf = (float)uc, vcf = (float)vc;
  V3<double> r0 = v3(((double)ucf - cx) / fx, ((double)vcf - cy) / fy, 1.0);
  V3<double> a0 = matvec(M, r0);
  V3<double> a1 = v3(M[0] / fx, M[3] / fx, M[6] / fx);
  V3<double> a2 = v3(M[1] / fy, M[4] / fy, M[7] / fy);
  V3<double> b = matvec(M, pc);
  V3<double> c0 = cross(r0, pc);
  V3<double> cxv = v3(0.0, -pc.z / fx, pc.y / fx);
  V3<double> cyv = v3(pc.z / fy, 0.0, -pc.x / fy);
  V3<double> y0 = matvec(Y, c0), y1 = matvec(Y, cxv), y2 = matvec(Y, cyv);
  GaussRec r;
  r.a0[0] = a0.x; r.a0[1] = a0.y; r.a0[2] = a0.z;
  r.a1[0] = a1.x; r.a1[1] = a1.y; r.a1[2] = a1.z;
  r.a2[0] = a2.x; r.a2[1] = a2.y; r.a2[2] = a2.z;
  r.b[0] = b.x; r.b[1] = b.y; r.b[2] = b.z;
  r.y0[0] = y0.x; r.y0[1] = y0.y; r.y0[2] = y0.z;
  r.y1[0] = y1.x; r.y1[1] = y1.y; r.y1[2] = y1.z;
  r.y2[0] = y2.x; r.y2[1] = y2.y; r.y2[2] = y2.z;
  r.uc = ucf;
  r.vc = vcf;
  r.c2 = (float)(in.w * kLog2eD);
  *out = r;
}

__device__ __forceinline__ void load_pose(const float* quat, const float* rotm, const float* trans,
                                          int pose, double R[9], double t[3]) {
  if (rotm) {
    for (int k = 0; k < 9; ++k) R[k] = rotm[9 * pose + k];
  } else {
    quat_to_rot<double>(quat + 4 * pose, R);
  }
  t[0] = trans[3 * pose]; t[1] = trans[3 * pose + 1]; t[2] = trans[3 * pose + 2];
}

// Clamp a floating tile coordinate into [lo, hi] before converting to int.
__device__ __forceinline__ int clamp_tile(float x, int lo, int hi) {
  if (!(x > (float)lo)) return lo;   // also catches NaN
  if (x > (float)hi) return hi;
  return (int)x;
}
__device__ __forceinline__ int clamp_tile(double x, int lo, int hi) {
  if (!(x > lo)) return lo;   // also catches NaN
  if (x > hi) return hi;
  return (int)x;
}

// ------------------------------------------------------------------------------------------
// Exact-projection binning (float32, cancellation-free forms)
// ------------------------------------------------------------------------------------------

// Row form of the footprint ellipse of a bounded record (FootRows), from the record's terms. With
// (du, dv) the pixel offset from the record's expansion centre, the ellipse is
// Q(du, dv) = |y|^2 - k2 |a|^2 <= 0 (the peak's Mahalanobis distance d0 = |y|^2 / |a|^2 at most k),
// a quadratic form Quu du^2 + 2 Quv du dv + Qvv dv^2 + 2 Qu du + 2 Qv dv + Q0. Its centre c solves
// the 2x2 system; along a row the squared half-width is -Q(u_row(dv), dv) / Quu, which is
// -Q(c)/Quu - det/Quu^2 (dv - dv_c)^2; the leftmost and rightmost points lie on the line through c
// where dQ/dv = 0, at c -+ lam (Qvv, -Quv) with lam^2 = -Q(c) / (Qvv det). float32 suffices: the
// |y|^2 terms dominate the quadratic coefficients for a footprint of bounded size, the expansion
// centre is the projected mean (near c), and a rounding of the bound moves it by far less than
// the 0.1 px margin of foot_row_tiles (FP64 would cost the preprocess more than it saves).
__device__ __forceinline__ void foot_rows(const GaussRec& g, float k2, FootRows& f) {
  f.uc = f.vc = f.c1 = f.h2 = f.vl = f.vr = f.pad = 0.f;
  f.hc = __int_as_float(0x7fc00000);  // NaN: the whole rectangle
  auto d = [](const float* a, const float* b) {
    return fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0]));
  };
  const float Quu = d(g.y1, g.y1) - k2 * d(g.a1, g.a1);
  const float Quv = d(g.y1, g.y2) - k2 * d(g.a1, g.a2);
  const float Qvv = d(g.y2, g.y2) - k2 * d(g.a2, g.a2);
  const float Qu = d(g.y0, g.y1) - k2 * d(g.a0, g.a1);
  const float Qv = d(g.y0, g.y2) - k2 * d(g.a0, g.a2);
  const float Q0 = d(g.y0, g.y0) - k2 * d(g.a0, g.a0);
  const float det = fmaf(Quu, Qvv, -Quv * Quv);
  if (!(Quu > 0.f && Qvv > 0.f && det > 0.f)) return;
  const float idet = 1.f / det;
  const float du_c = fmaf(Qv, Quv, -Qu * Qvv) * idet, dv_c = fmaf(Qu, Quv, -Qv * Quu) * idet;
  const float qc = fmaf(Qv, dv_c, fmaf(Qu, du_c, Q0));
  if (!(qc < 0.f)) return;
  const float iq = 1.f / Quu;
  const float lam = sqrtf(-qc * idet / Qvv);
  const float vc = g.vc + dv_c;
  f.uc = g.uc + du_c;
  f.vc = vc;
  f.c1 = -Quv * iq;
  f.hc = -qc * iq;
  f.h2 = -det * iq * iq;
  f.vl = fmaf(lam, Quv, vc);
  f.vr = fmaf(-lam, Quv, vc);
  if (!(isfinite(f.uc) && isfinite(f.vc) && isfinite(f.c1) && isfinite(f.hc) && isfinite(f.h2) &&
        isfinite(f.vl) && isfinite(f.vr)))
    f.hc = __int_as_float(0x7fc00000);
}

// Record and tile footprint of one (Gaussian, view) pair in float32 (fe_footprint.cuh); with
// `foot`, also the footprint's row form (FootRows) when it is bounded.
__device__ __forceinline__ void footprint_and_record(
    const float* mean, const float* prec, float logw, const float* R, const float* t,
    const ViewDev& V, int cull_mode, float cull_param, int tile_w, int tile_h, GaussRec& rec,
    int& tx0, int& ty0, int& tx1, int& ty1, FootRows* foot) {
  const CamTerms ct = camera_terms(mean, prec, R, t);
  const float k2 = cutoff_k2(logw, cull_mode, cull_param);
  tx0 = ty0 = tx1 = ty1 = 0;
  bool bounded = false;
  if (k2 > 0.f) {
    float ulo = 0.f, uhi = 0.f, vlo = 0.f, vhi = 0.f;
    if (screen_bounds(ct, k2, V.fx, V.fy, V.cx, V.cy, ulo, uhi, vlo, vhi) == kFootBounded) {
      // Conservative margin covers the float32 rounding of the bounds (of order 1e-5 px).
      const float margin = 0.02f;
      tx0 = clamp_tile(floorf((ulo - margin) / tile_w), 0, V.gx);
      tx1 = clamp_tile(floorf((uhi + margin) / tile_w) + 1.f, 0, V.gx);
      ty0 = clamp_tile(floorf((vlo - margin) / tile_h), 0, V.gy);
      ty1 = clamp_tile(floorf((vhi + margin) / tile_h) + 1.f, 0, V.gy);
      bounded = true;
    } else {
      tx0 = 0; ty0 = 0; tx1 = V.gx; ty1 = V.gy;
    }
  }
  if (tx1 <= tx0 || ty1 <= ty0) tx0 = ty0 = tx1 = ty1 = 0;
  // Record around the projected mean (image centre when the projection is unbounded).
  make_record(ct, logw, V.fx, V.fy, V.cx, V.cy, 0.5f * V.W, 0.5f * V.H, -1.f * V.W, 2.f * V.W,
              -1.f * V.H, 2.f * V.H, rec);
  if (foot) {
    FootRows f;
    if (bounded && tx1 > tx0) {
      foot_rows(rec, k2, f);
    } else {
      f.uc = f.vc = f.c1 = f.h2 = f.vl = f.vr = f.pad = 0.f;
      f.hc = __int_as_float(0x7fc00000);
    }
    *foot = f;
  }
}

__global__ void __launch_bounds__(64) preprocess_kernel(
    ViewsArg va, int64_t n_rec, const float* __restrict__ means, const float* __restrict__ prec,
    const float* __restrict__ logw, const float* __restrict__ quat, const float* __restrict__ rotm,
    const float* __restrict__ trans, int cull_mode, float cull_param, int tile_w, int tile_h,
    GaussRec* __restrict__ recs, TileRect* __restrict__ rects, FootRows* __restrict__ foot,
    uint32_t* __restrict__ touched, unsigned long long* __restrict__ row_tot, int max_gy,
    Control* __restrict__ ctrl) {
  unsigned long long keys = 0;  // this thread's keys (row_tot != NULL)
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_rec;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int vi = find_view<&ViewDev::rec_base>(va, i);
    const ViewDev& V = view_at(va, vi);
    const int64_t gi = V.gauss_base + (i - V.rec_base);
    float R[9], t[3], m[3], pr[9];
    if (rotm) {
#pragma unroll
      for (int k = 0; k < 9; ++k) R[k] = rotm[9 * V.pose + k];
    } else {
      quat_to_rot<float>(quat + 4 * V.pose, R);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      t[k] = trans[3 * V.pose + k];
      m[k] = means[3 * gi + k];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) pr[k] = prec[9 * gi + k];
    GaussRec rec;
    FootRows f;
    int tx0, ty0, tx1, ty1;
    footprint_and_record(m, pr, logw[gi], R, t, V, cull_mode, cull_param, tile_w, tile_h, rec, tx0,
                         ty0, tx1, ty1, foot ? &f : nullptr);
    recs[i] = rec;
    const TileRect tr{(uint16_t)tx0, (uint16_t)ty0, (uint16_t)tx1, (uint16_t)ty1};
    rects[i] = tr;
    uint32_t n_keys;
    if (foot) {
      foot[i] = f;
      // Keys of every tile row the footprint reaches (its rows' spans differ).
      unsigned long long* rc = row_tot ? row_tot + (int64_t)vi * (max_gy + 1) : nullptr;
      n_keys = 0;
      for (int y = ty0; y < ty1; ++y) {
        int x0, x1;
        foot_row_tiles(f, tr, y, tile_w, tile_h, x0, x1);
        const uint32_t w = (uint32_t)(x1 - x0);
        if (rc && w) atomicAdd(&rc[y], (unsigned long long)w);
        n_keys += w;
      }
    } else {
      // Every row of the rectangle spans its full width.
      const uint32_t w = (uint32_t)(tx1 - tx0);
      n_keys = w * (uint32_t)(ty1 - ty0);
      if (row_tot && w) {
        unsigned long long* rc = row_tot + (int64_t)vi * (max_gy + 1);
        for (int y = ty0; y < ty1; ++y) atomicAdd(&rc[y], (unsigned long long)w);
      }
    }
    touched[i] = n_keys;
    keys += n_keys;
  }
  if (row_tot != nullptr) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) keys += __shfl_xor_sync(0xffffffffu, keys, o);
    if ((threadIdx.x & 31) == 0 && keys) atomicAdd(&ctrl->want_keys, keys);
  }
}

// ------------------------------------------------------------------------------------------
// Reference binning (float32, no contraction)
// ------------------------------------------------------------------------------------------

// glm-style column-major 3x3: c[col][row].
struct GM3 {
  float c[3][3];
};

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

// (A*B)[i][j] = A[0][j]*B[i][0] + A[1][j]*B[i][1] + A[2][j]*B[i][2], summed left to right.
__device__ GM3 gmul(const GM3& A, const GM3& B) {
  GM3 R;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      R.c[i][j] = fa(fa(fm(A.c[0][j], B.c[i][0]), fm(A.c[1][j], B.c[i][1])), fm(A.c[2][j], B.c[i][2]));
  return R;
}

__device__ GM3 gtrans(const GM3& A) {
  GM3 R;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R.c[i][j] = A.c[j][i];
  return R;
}

// Column-major constructor from 9 scalars given column by column.
__device__ GM3 gmake(float a, float b, float c, float d, float e, float f, float g, float h, float k) {
  GM3 R;
  R.c[0][0] = a; R.c[0][1] = b; R.c[0][2] = c;
  R.c[1][0] = d; R.c[1][1] = e; R.c[1][2] = f;
  R.c[2][0] = g; R.c[2][1] = h; R.c[2][2] = k;
  return R;
}

// matrix[0]*p.x + matrix[4]*p.y + matrix[8]*p.z + matrix[12] (auxiliary.h:46-61 neighbours).
__device__ __forceinline__ float tp_row(const float* m, int r, float x, float y, float z) {
  return fa(fa(fa(fm(m[r], x), fm(m[4 + r], y)), fm(m[8 + r], z)), m[12 + r]);
}

// auxiliary.h:46-49, evaluated in double and rounded once to float.
__device__ __forceinline__ float ndc2pix(float v, int S) {
  double t = __dadd_rn((double)v, 1.0);
  t = __dmul_rn(t, (double)S);
  t = __dsub_rn(t, 1.0);
  return (float)__dmul_rn(t, 0.5);
}

// (int) conversion of a float as the GPU performs it (truncate toward zero, saturate, NaN->0).
__device__ __forceinline__ int f2i_trunc(float x) { return __float2int_rz(x); }

// auxiliary.h:51-61 (BLOCK_X = BLOCK_Y = 8).
__device__ __forceinline__ void ref_get_rect(float px, float py, int r, int gx, int gy,
                                             int& x0, int& y0, int& x1, int& y1) {
  const float rf = (float)r;
  x0 = min(gx, max(0, f2i_trunc(__fdiv_rn(fs(px, rf), 8.f))));
  y0 = min(gy, max(0, f2i_trunc(__fdiv_rn(fs(py, rf), 8.f))));
  x1 = min(gx, max(0, f2i_trunc(__fdiv_rn(fs(fa(fa(px, rf), 8.f), 1.f), 8.f))));
  y1 = min(gy, max(0, f2i_trunc(__fdiv_rn(fs(fa(fa(py, rf), 8.f), 1.f), 8.f))));
}

__global__ void preprocess_reference_kernel(
    int P, float n_std, const float* __restrict__ means, const float* __restrict__ scales,
    const float* __restrict__ rots, const float* __restrict__ viewmatrix,
    const float* __restrict__ projmatrix, int W, int H, float tan_fovx, float tan_fovy,
    float focal_x, float focal_y, int gx, int gy, int32_t* __restrict__ radii,
    float* __restrict__ means2d, TileRect* __restrict__ rects, uint32_t* __restrict__ touched) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= P) return;
  radii[idx] = 0;
  touched[idx] = 0;
  rects[idx] = TileRect{0, 0, 0, 0};
  means2d[2 * idx] = 0.f;
  means2d[2 * idx + 1] = 0.f;
  const float px = means[3 * idx], py = means[3 * idx + 1], pz = means[3 * idx + 2];

  // in_frustum (auxiliary.h:144-169): near cull on the view-space depth.
  const float vz = tp_row(viewmatrix, 2, px, py, pz);
  if (vz <= 0.2f) return;
  const float hx = tp_row(projmatrix, 0, px, py, pz);
  const float hy = tp_row(projmatrix, 1, px, py, pz);
  const float hw = tp_row(projmatrix, 3, px, py, pz);
  const float p_w = __fdiv_rn(1.0f, fa(hw, 0.0000001f));
  const float projx = fm(hx, p_w), projy = fm(hy, p_w);

  // computeCov3D (forward.cu:65-122).
  const float sx = fm(1.0f, scales[3 * idx]), sy = fm(1.0f, scales[3 * idx + 1]),
              sz = fm(1.0f, scales[3 * idx + 2]);
  const float r = rots[4 * idx], x = rots[4 * idx + 1], y = rots[4 * idx + 2],
              z = rots[4 * idx + 3];
  GM3 S = gmake(sx, 0.f, 0.f, 0.f, sy, 0.f, 0.f, 0.f, sz);
  GM3 Rm = gmake(fs(1.f, fm(2.f, fa(fm(y, y), fm(z, z)))), fm(2.f, fs(fm(x, y), fm(r, z))),
                 fm(2.f, fa(fm(x, z), fm(r, y))),
                 fm(2.f, fa(fm(x, y), fm(r, z))), fs(1.f, fm(2.f, fa(fm(x, x), fm(z, z)))),
                 fm(2.f, fs(fm(y, z), fm(r, x))),
                 fm(2.f, fs(fm(x, z), fm(r, y))), fm(2.f, fa(fm(y, z), fm(r, x))),
                 fs(1.f, fm(2.f, fa(fm(x, x), fm(y, y)))));
  GM3 Mm = gmul(S, Rm);
  GM3 Sig = gmul(gtrans(Mm), Mm);
  const float cv0 = Sig.c[0][0], cv1 = Sig.c[0][1], cv2 = Sig.c[0][2], cv3 = Sig.c[1][1],
              cv4 = Sig.c[1][2], cv5 = Sig.c[2][2];

  // computeCov2D (forward.cu:21-60).
  float tx = tp_row(viewmatrix, 0, px, py, pz);
  float ty = tp_row(viewmatrix, 1, px, py, pz);
  const float tz = vz;
  const float limx = fm(1.3f, tan_fovx), limy = fm(1.3f, tan_fovy);
  const float txtz = __fdiv_rn(tx, tz), tytz = __fdiv_rn(ty, tz);
  tx = fm(fminf(limx, fmaxf(-limx, txtz)), tz);
  ty = fm(fminf(limy, fmaxf(-limy, tytz)), tz);
  const float tz2 = fm(tz, tz);
  GM3 J = gmake(__fdiv_rn(focal_x, tz), 0.0f, -__fdiv_rn(fm(focal_x, tx), tz2),
                0.0f, __fdiv_rn(focal_y, tz), -__fdiv_rn(fm(focal_y, ty), tz2),
                0.f, 0.f, 0.f);
  GM3 Wm = gmake(viewmatrix[0], viewmatrix[4], viewmatrix[8], viewmatrix[1], viewmatrix[5],
                 viewmatrix[9], viewmatrix[2], viewmatrix[6], viewmatrix[10]);
  GM3 T = gmul(Wm, J);
  GM3 Vrk = gmake(cv0, cv1, cv2, cv1, cv3, cv4, cv2, cv4, cv5);
  GM3 cov = gmul(gmul(gtrans(T), gtrans(Vrk)), T);
  const float ca = fa(cov.c[0][0], 0.3f), cb = cov.c[0][1], cc = fa(cov.c[1][1], 0.3f);

  const float det = fs(fm(ca, cc), fm(cb, cb));
  if (det == 0.0f) return;
  const float mid = fm(0.5f, fa(ca, cc));
  const float disc = __fsqrt_rn(fmaxf(0.1f, fs(fm(mid, mid), det)));
  const float l1 = fa(mid, disc), l2 = fs(mid, disc);
  const float radius = ceilf(fm(n_std, __fsqrt_rn(fmaxf(l1, l2))));
  const float pix_x = ndc2pix(projx, W), pix_y = ndc2pix(projy, H);
  const int ir = f2i_trunc(radius);
  int x0, y0, x1, y1;
  ref_get_rect(pix_x, pix_y, ir, gx, gy, x0, y0, x1, y1);
  const uint32_t area = (uint32_t)(x1 - x0) * (uint32_t)(y1 - y0);
  if (area == 0) return;
  radii[idx] = ir;
  means2d[2 * idx] = pix_x;
  means2d[2 * idx + 1] = pix_y;
  rects[idx] = TileRect{(uint16_t)x0, (uint16_t)y0, (uint16_t)x1, (uint16_t)y1};
  touched[idx] = area;
}

// Records for the legacy interface: precision from (scale, rotation) as the reference's
// computeCov3D defines the covariance (Sigma = R diag(s^2) R^T with R from the unnormalised
// quaternion formula), factorised as U = inv(chol(Sigma))^T; pose given as a rotation matrix.
__global__ void legacy_records_kernel(ViewsArg va, int P, const float* __restrict__ means,
                                      const float* __restrict__ scales,
                                      const float* __restrict__ rots,
                                      const float* __restrict__ logw,
                                      const float* __restrict__ rotm,
                                      const float* __restrict__ trans,
                                      const float* __restrict__ rays,
                                      GaussRec* __restrict__ recs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const ViewDev& V = view_at(va, 0);
  // Pinhole intrinsics recovered from the ray buffer ((u-cx)/fx, (v-cy)/fy, 1): the slope between
  // the first and last pixel of the first row and column, then the offset at pixel (0,0).
  const int H = V.H, W = V.W;
  const double sx = W > 1 ? ((double)rays[3 * (W - 1)] - rays[0]) / (W - 1) : 1.0 / V.fx;
  const double sy = H > 1 ? ((double)rays[3 * (int64_t)(H - 1) * W + 1] - rays[1]) / (H - 1)
                          : 1.0 / V.fy;
  const float fx = (float)(1.0 / sx), fy = (float)(1.0 / sy);
  const float cx = (float)(-(double)rays[0] / sx), cy = (float)(-(double)rays[1] / sy);
  RecordInputs in;
  for (int k = 0; k < 3; ++k) in.m[k] = means[3 * i + k];
  in.w = logw[i];
  const double r = rots[4 * i], x = rots[4 * i + 1], y = rots[4 * i + 2], z = rots[4 * i + 3];
  const double Rq[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y),
                        2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x),
                        2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)};
  const double s[3] = {scales[3 * i], scales[3 * i + 1], scales[3 * i + 2]};
  double S[9];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k) acc += Rq[a * 3 + k] * s[k] * s[k] * Rq[c * 3 + k];
      S[a * 3 + c] = acc;
    }
  // Cholesky S = L L^T, then U = (L^-1)^T.
  const double l00 = sqrt(S[0]);
  const double l10 = S[3] / l00, l20 = S[6] / l00;
  const double l11 = sqrt(S[4] - l10 * l10);
  const double l21 = (S[7] - l20 * l10) / l11;
  const double l22 = sqrt(S[8] - l20 * l20 - l21 * l21);
  const double i00 = 1.0 / l00, i11 = 1.0 / l11, i22 = 1.0 / l22;
  const double i10 = -l10 * i00 / l11;
  const double i21 = -l21 * i11 / l22;
  const double i20 = -(l20 * i00 + l21 * i10) / l22;
  const double U[9] = {i00, i10, i20, 0.0, i11, i21, 0.0, 0.0, i22};
  for (int k = 0; k < 9; ++k) in.U[k] = U[k];
  load_pose(nullptr, rotm, trans, 0, in.R, in.t);
  double M[9], Y[9];
  V3<double> pc;
  build_camera_terms(in, M, Y, pc);
  write_record(in, M, Y, pc, fx, fy, cx, cy, H, W, &recs[i]);
}

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------

void launch_preprocess(const ViewsArg& va, int64_t n_rec, const float* means, const float* prec,
                       const float* logw, const float* quat, const float* rotm,
                       const float* trans, int cull_mode, float cull_param, int tile_w,
                       int tile_h, GaussRec* recs, TileRect* rects, FootRows* foot,
                       uint32_t* touched, unsigned long long* row_tot, int max_gy, Control* ctrl,
                       cudaStream_t st) {
  if (n_rec <= 0) return;
  const int threads = 64;
  const int64_t want = (n_rec + threads - 1) / threads;
  const int blocks = (int)(want < 65535 ? want : 65535);
  preprocess_kernel<<<blocks, threads, 0, st>>>(va, n_rec, means, prec, logw, quat, rotm, trans,
                                                cull_mode, cull_param, tile_w, tile_h, recs,
                                                rects, foot, touched, row_tot, max_gy, ctrl);
}

void launch_preprocess_reference(int P, float n_std, const float* means, const float* scales,
                                 const float* rots, const float* viewmatrix,
                                 const float* projmatrix, int W, int H, float tan_fovx,
                                 float tan_fovy, int gx, int gy, int32_t* radii, float* means2d,
                                 TileRect* rects, uint32_t* touched, cudaStream_t st) {
  if (P <= 0) return;
  // rasterizer_impl.cu:205-206 (float arithmetic on the host).
  const float fx = (float)W / (2.0f * tan_fovx);
  const float fy = (float)H / (2.0f * tan_fovy);
  preprocess_reference_kernel<<<(P + 255) / 256, 256, 0, st>>>(
      P, n_std, means, scales, rots, viewmatrix, projmatrix, W, H, tan_fovx, tan_fovy, fx, fy, gx,
      gy, radii, means2d, rects, touched);
}

void launch_legacy_records(const ViewsArg& va, int P, const float* means, const float* scales,
                           const float* rots, const float* logw, const float* rotm,
                           const float* trans, const float* rays, GaussRec* recs,
                           cudaStream_t st) {
  if (P <= 0) return;
  legacy_records_kernel<<<(P + 127) / 128, 128, 0, st>>>(va, P, means, scales, rots, logw, rotm,
                                                         trans, rays, recs);
}

}  // namespace fe
