// pixlist.cu -- multi-pose pixel-list renderer with optical flow.
//
// Restates baseline/fm_render.py:151-224 (render_func_idx_quattrans and its _flow variant) and
// :130-144 (render_func_quat_cam) with the argument order of their render_func_rays calls fixed
// (they pass the Gaussians where the rays belong). Input rays are the reference's pixel_posei rows
// (x, y, c, pose): the camera ray is (x invF, y invF, c) of pose `pose` (poses: (n_poses, 7) =
// quaternion (4, scalar first), translation (3)); or render_func_quat_cam's pixel_list rows
// (x, y, c) of one pose, whose camera ray is ((x - 0.5) invF, (y - 0.5) aspect invF, c) -- the
// same model with focal lengths 1/invF and 1/(aspect invF) and the pixel offsets shifted.
// Outputs per ray: depth and alpha as render_func_rays computes them (culled at
// the renderer's density cut-off), optionally the softmax-weighted per-Gaussian features
// (fm_render's w applied to a feature table) and the dense weights w (N x rays), and the
// forward / backward optical flow to poses pose+1 / pose-1 (clamped), fm_render.py:186-222.
//
// Work: pixlist_prep_kernel builds, per (pose, Gaussian), the same float32 record and screen
// bound as the image preprocess (fe_footprint.cuh) with focal lengths 1/invF, 1/(aspect invF) and
// the principal point at 0 (pixel offsets (x - shift_x)/c, (y - shift_y)/c). pixlist_kernel gives each ray one thread that tests every Gaussian's
// bound of its pose (a warp of rays of one pose reads the same record: broadcast loads) and
// evaluates only the Gaussians whose k-sigma projection contains the ray.
#include <algorithm>

#include "fe_footprint.cuh"
#include "fe_kernels.cuh"

namespace fe {
namespace {

struct PixRec {
  float ulo, uhi, vlo, vhi;  // pixel-offset bounds of the k-sigma projection
  GaussRec g;
};
static_assert(sizeof(PixRec) == 112, "PixRec layout");

__device__ __forceinline__ void pose_rot(const float* pose, float R[9]) {
  quat_to_rot<float>(pose, R);
}

__global__ void pixlist_prep_kernel(int n, int n_poses, const float* __restrict__ means,
                                    const float* __restrict__ prec,
                                    const float* __restrict__ logw,
                                    const float* __restrict__ poses, float fx, float fy,
                                    int cull_mode, float cull_param, PixRec* __restrict__ recs) {
  const int64_t total = (int64_t)n * n_poses;
  const float L = 4.f * fmaxf(fabsf(fx), fabsf(fy));  // expansion centres within four focal lengths
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / n);
    const int i = (int)(idx - (int64_t)k * n);
    float R[9];
    pose_rot(poses + 7 * k, R);
    const CamTerms ct = camera_terms(means + 3 * (int64_t)i, prec + 9 * (int64_t)i, R,
                                     poses + 7 * k + 4);
    const float lw = logw[i];
    const float k2 = cutoff_k2(lw, cull_mode, cull_param);
    PixRec r;
    r.ulo = INFINITY; r.uhi = -INFINITY; r.vlo = INFINITY; r.vhi = -INFINITY;  // empty
    if (k2 > 0.f) {
      float ulo = 0.f, uhi = 0.f, vlo = 0.f, vhi = 0.f;
      if (screen_bounds(ct, k2, fx, fy, 0.f, 0.f, ulo, uhi, vlo, vhi) == kFootBounded) {
        const float margin = 0.02f;  // covers the float32 rounding of the bounds
        r.ulo = ulo - margin; r.uhi = uhi + margin; r.vlo = vlo - margin; r.vhi = vhi + margin;
      } else {
        r.ulo = -INFINITY; r.uhi = INFINITY; r.vlo = -INFINITY; r.vhi = INFINITY;
      }
    }
    make_record(ct, lw, fx, fy, 0.f, 0.f, 0.f, 0.f, -L, L, -L, L, r.g);
    recs[idx] = r;
  }
}

// Camera-frame point of pose `a` at ray parameter z, seen from pose `b`: pixel offsets (x, y).
__device__ __forceinline__ void reproject(const float* poses, int a, int b, float rx, float ry,
                                          float rz, float z, float inv_f, float& x, float& y) {
  float Ra[9], Rb[9];
  pose_rot(poses + 7 * a, Ra);
  pose_rot(poses + 7 * b, Rb);
  const float* ta = poses + 7 * a + 4;
  const float* tb = poses + 7 * b + 4;
  // world = (ray z) @ Ra + ta;  pt = (world - tb) @ Rb^T
  const float cx = rx * z, cy = ry * z, cz = rz * z;
  float w[3];
  for (int j = 0; j < 3; ++j) w[j] = cx * Ra[0 * 3 + j] + cy * Ra[1 * 3 + j] + cz * Ra[2 * 3 + j] + ta[j];
  float p[3];
  for (int j = 0; j < 3; ++j)
    p[j] = (w[0] - tb[0]) * Rb[j * 3 + 0] + (w[1] - tb[1]) * Rb[j * 3 + 1] + (w[2] - tb[2]) * Rb[j * 3 + 2];
  x = p[0] / (p[2] * inv_f);
  y = p[1] / (p[2] * inv_f);
}

__global__ void __launch_bounds__(128) pixlist_kernel(
    int n, int n_poses, const PixRec* __restrict__ recs, int64_t n_rays,
    const float* __restrict__ rays, PixRayModel rm, float beta2, float beta3,
    const float* __restrict__ poses, const float* __restrict__ feats, int nf,
    float* __restrict__ depth, float* __restrict__ alpha, float* __restrict__ flow_next,
    float* __restrict__ flow_prev, float* __restrict__ out_feats, float* __restrict__ weights) {
  const float nb2 = -beta2 * kLog2e;
  const float kn = -0.5f * kLog2e;
  const float inv_f = rm.inv_f;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n_rays;
       j += (int64_t)gridDim.x * blockDim.x) {
    const float* row = rays + rm.stride * j;
    const float rx = row[0], ry = row[1], rc = row[2];
    int k = 0;
    if (rm.stride == 4) {
      k = (int)row[3];  // astype(int); out-of-range indices clamp, as JAX gathers do
      k = min(max(k, 0), n_poses - 1);
    }
    // The record is evaluated on the unit-depth ray (u/fx, v/fy, 1) with pixel offsets
    // u = (x - shift_x)/c, v = (y - shift_y)/c; the parameter of the input ray
    // ((x - shift_x) inv_f, (y - shift_y) aspect inv_f, c), which the softmax logits, the z > 0
    // mask and the depth use, is z / c.
    const float ic = 1.f / rc;
    const float u = (rx - rm.shift_x) * ic, v = (ry - rm.shift_y) * ic;
    const PixRec* pr = recs + (int64_t)k * n;
    float A = 0.f, m = -1e30f, W = 0.f, Z = 0.f;
    constexpr int kMaxF = 16;
    float F[kMaxF];
#pragma unroll
    for (int q = 0; q < kMaxF; ++q) F[q] = 0.f;
    auto eval = [&](int i) {
      const GaussRec& g = pr[i].g;
      const float du = u - g.uc, dv = v - g.vc;
      float a[3], y[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a[c] = fmaf(g.a2[c], dv, fmaf(g.a1[c], du, g.a0[c]));
        y[c] = fmaf(g.y2[c], dv, fmaf(g.y1[c], du, g.y0[c]));
      }
      const float vsv = fmaf(a[2], a[2], fmaf(a[1], a[1], a[0] * a[0]));
      const float psv = fmaf(a[2], g.b[2], fmaf(a[1], g.b[1], a[0] * g.b[0]));
      const float yy = fmaf(y[2], y[2], fmaf(y[1], y[1], y[0] * y[0]));
      const float qi = 1.f / vsv;
      const float z = psv * qi * ic;  // parameter of the ray (x inv_f, y inv_f, c)
      const float s2 = fmaf(kn * yy, qi, g.c2);
      A += ex2_approx(s2);
      if (z > 0.f) {
        const float l = fmaf(beta3, s2, nb2 * z);
        if (l > m) {
          const float sc = ex2_approx(m - l);
          W *= sc; Z *= sc;
          for (int q = 0; q < nf && q < kMaxF; ++q) F[q] *= sc;
          m = l;
        }
        const float e = ex2_approx(l - m);
        W += e;
        Z = fmaf(e, z, Z);
        for (int q = 0; q < nf && q < kMaxF; ++q) F[q] = fmaf(e, feats[(int64_t)i * nf + q], F[q]);
      }
    };
    // The screen bounds of kBatch Gaussians are loaded together (independent loads in flight),
    // then the Gaussians whose bounds hold the ray are evaluated in index order.
    constexpr int kBatch = 8;
    int i0 = 0;
    for (; i0 + kBatch <= n; i0 += kBatch) {
      float4 bnd[kBatch];
#pragma unroll
      for (int t = 0; t < kBatch; ++t) bnd[t] = *reinterpret_cast<const float4*>(pr + i0 + t);
      unsigned hit = 0;
#pragma unroll
      for (int t = 0; t < kBatch; ++t)
        hit |= (u >= bnd[t].x && u <= bnd[t].y && v >= bnd[t].z && v <= bnd[t].w) ? 1u << t : 0u;
      while (hit) {
        const int t = __ffs(hit) - 1;
        hit &= hit - 1;
        eval(i0 + t);
      }
    }
    for (int i = i0; i < n; ++i) {
      const float4 bnd = *reinterpret_cast<const float4*>(pr + i);
      if (u >= bnd.x && u <= bnd.y && v >= bnd.z && v <= bnd.w) eval(i);
    }
    const float iw = W > 0.f ? 1.f / W : 0.f;
    const float zd = Z * iw;  // parameter of the ray (x inv_f, y inv_f, c)
    depth[j] = zd;
    alpha[j] = -expm1f(-A);
    if (out_feats)
      for (int q = 0; q < nf && q < kMaxF; ++q) out_feats[j * nf + q] = F[q] * iw;
    if (weights) {  // dense softmax weights (rows: Gaussians), a second pass over the Gaussians
      for (int i = 0; i < n; ++i) {
        float wi = 0.f;
        const float4 bnd = *reinterpret_cast<const float4*>(pr + i);
        if (W > 0.f && u >= bnd.x && u <= bnd.y && v >= bnd.z && v <= bnd.w) {
          const GaussRec& g = pr[i].g;
          const float du = u - g.uc, dv = v - g.vc;
          float a[3], y[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            a[c] = fmaf(g.a2[c], dv, fmaf(g.a1[c], du, g.a0[c]));
            y[c] = fmaf(g.y2[c], dv, fmaf(g.y1[c], du, g.y0[c]));
          }
          const float vsv = fmaf(a[2], a[2], fmaf(a[1], a[1], a[0] * a[0]));
          const float psv = fmaf(a[2], g.b[2], fmaf(a[1], g.b[1], a[0] * g.b[0]));
          const float yy = fmaf(y[2], y[2], fmaf(y[1], y[1], y[0] * y[0]));
          const float qi = 1.f / vsv;
          const float z = psv * qi * ic;
          const float s2 = fmaf(kn * yy, qi, g.c2);
          if (z > 0.f) wi = ex2_approx(fmaf(beta3, s2, nb2 * z) - m) * iw;
        }
        weights[(int64_t)i * n_rays + j] = wi;
      }
    }
    if (flow_next || flow_prev) {
      const float rxf = rx * inv_f, ryf = ry * inv_f;
      float x, y;
      if (flow_next) {
        reproject(poses, k, min(k + 1, n_poses - 1), rxf, ryf, rc, zd, inv_f, x, y);
        flow_next[2 * j] = -(x - rx);
        flow_next[2 * j + 1] = -(y - ry);
      }
      if (flow_prev) {
        reproject(poses, k, max(k - 1, 0), rxf, ryf, rc, zd, inv_f, x, y);
        flow_prev[2 * j] = -(x - rx);
        flow_prev[2 * j + 1] = -(y - ry);
      }
    }
  }
}

}  // namespace

size_t pixlist_scratch_bytes(int n, int n_poses) { return sizeof(PixRec) * (size_t)n * n_poses; }

void launch_render_pixels(int n, int n_poses, const float* means, const float* prec,
                          const float* logw, const float* poses, int64_t n_rays, const float* rays,
                          const PixRayModel& rm, float beta2, float beta3, int cull_mode,
                          float cull_param, const float* feats, int nf, float* depth, float* alpha,
                          float* flow_next, float* flow_prev, float* out_feats, float* weights,
                          void* scratch, cudaStream_t st) {
  if (n_rays <= 0) return;
  PixRec* recs = static_cast<PixRec*>(scratch);
  const int64_t total = (int64_t)n * n_poses;
  if (total > 0) {
    const int64_t b = (total + 127) / 128;
    const float fx = 1.f / rm.inv_f, fy = 1.f / (rm.aspect * rm.inv_f);
    pixlist_prep_kernel<<<(unsigned)std::min<int64_t>(b, 152 * 16), 128, 0, st>>>(
        n, n_poses, means, prec, logw, poses, fx, fy, cull_mode, cull_param, recs);
  }
  const int64_t b = (n_rays + 127) / 128;
  pixlist_kernel<<<(unsigned)std::min<int64_t>(b, 152 * 32), 128, 0, st>>>(
      n, n_poses, recs, n_rays, rays, rm, beta2, beta3, poses, feats, nf, depth, alpha,
      flow_next, flow_prev, out_feats, weights);
}

}  // namespace fe
