// adapters.cu -- scene-parameter adapters on the device, with their backward passes.
//
// (1) Precision factor from per-Gaussian scales and rotations. The reference's optimisation loop
//     builds Sigma = R diag(s)^2 R^T (utils/sfs_utils.py:207-213 prec_from_rotscale) and its CUDA
//     rasterizer builds the same Sigma from (scales, rotations) (forward.cu computeCov3D). The
//     renderer takes the upper-triangular factor U with U U^T = Sigma^-1 (fm_render's prec_full,
//     triu read). Here P = Sigma^-1 = R diag(s^-2) R^T and U is P's upper ("reverse") Cholesky
//     factor, in closed form:
//         U22 = sqrt(P22), U12 = P12/U22, U02 = P02/U22, U11 = sqrt(P11 - U12^2),
//         U01 = (P01 - U02 U12)/U11, U00 = sqrt(P00 - U01^2 - U02^2)
//     (prec_from_rotscale itself returns the lower factor cholesky(Sigma^-1), of which fm_render's
//     triu keeps only the diagonal; the factor here is the one the renderer's convention needs.)
//     The backward runs those assignments in reverse, then P = R D R^T, then the rotation formula
//     of quat_to_rot (util_render.py:51-76), all in float64.
// (2) Rigid transforms of points by a pose (t, q) (t first, scalar-first quaternion, as the
//     reference's poses): out = R(q) p + t (transform_points_jittable, sfs_utils.py:171-172) or
//     out = R(q)^T p + t (transform_points_by_inv_jittable, sfs_utils.py:182-184), with the
//     backward to the points and to the pose (block sums, one float64 atomic per block and
//     pose parameter).
#include <algorithm>
#include <cmath>

#include "fe_kernels.cuh"

namespace fe {
namespace {

// R = quat_to_rot(q) and, for the backward, Q (R = I + s Q) and s = 2/|q|^2.
struct Rot {
  double r[9], qm[9], s, n;
  bool ident;
};

__device__ Rot make_rot(const float* qf) {
  Rot o;
  const double w = qf[0], x = qf[1], y = qf[2], z = qf[3];
  o.n = w * w + x * x + y * y + z * z;
  o.ident = !(o.n > 1e-12);
  o.s = o.ident ? 0.0 : 2.0 / o.n;
  const double Q[9] = {-(y * y + z * z), x * y - w * z, x * z + w * y,
                       x * y + w * z, -(x * x + z * z), y * z - w * x,
                       x * z - w * y, y * z + w * x, -(x * x + y * y)};
  for (int i = 0; i < 9; ++i) {
    o.qm[i] = Q[i];
    o.r[i] = (i % 4 == 0 ? 1.0 : 0.0) + o.s * Q[i];
  }
  return o;
}

// dL/dq from dL/dR (row-major 3x3) for R = I + s Q(q), s = 2/|q|^2.
__device__ void rot_vjp(const Rot& R, const float* qf, const double* gR, double* gq) {
  if (R.ident) {
    gq[0] = gq[1] = gq[2] = gq[3] = 0.0;
    return;
  }
  const double w = qf[0], x = qf[1], y = qf[2], z = qf[3];
  // dQ/dw, dQ/dx, dQ/dy, dQ/dz (row-major)
  const double dw[9] = {0, -z, y, z, 0, -x, -y, x, 0};
  const double dx[9] = {0, y, z, y, -2 * x, -w, z, w, -2 * x};
  const double dy[9] = {-2 * y, x, w, x, 0, z, -w, z, -2 * y};
  const double dz[9] = {-2 * z, -w, x, w, -2 * z, y, x, y, 0};
  double gQ = 0.0, aw = 0.0, ax = 0.0, ay = 0.0, az = 0.0;
  for (int i = 0; i < 9; ++i) {
    gQ += gR[i] * R.qm[i];
    aw += gR[i] * dw[i];
    ax += gR[i] * dx[i];
    ay += gR[i] * dy[i];
    az += gR[i] * dz[i];
  }
  // d s / d q_k = -2 s q_k / n
  const double c = -2.0 * R.s / R.n * gQ;
  gq[0] = R.s * aw + c * w;
  gq[1] = R.s * ax + c * x;
  gq[2] = R.s * ay + c * y;
  gq[3] = R.s * az + c * z;
}

__device__ void precision(const Rot& R, const float* sc, double* P, double* d) {
  for (int k = 0; k < 3; ++k) d[k] = 1.0 / ((double)sc[k] * (double)sc[k]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = 0.0;
      for (int k = 0; k < 3; ++k) v += R.r[3 * i + k] * d[k] * R.r[3 * j + k];
      P[3 * i + j] = v;
    }
}

struct Upper {
  double u00, u01, u02, u11, u12, u22;
};

__device__ Upper reverse_cholesky(const double* P) {
  Upper u;
  u.u22 = sqrt(P[8]);
  u.u12 = P[5] / u.u22;
  u.u02 = P[2] / u.u22;
  u.u11 = sqrt(P[4] - u.u12 * u.u12);
  u.u01 = (P[1] - u.u02 * u.u12) / u.u11;
  u.u00 = sqrt(P[0] - u.u01 * u.u01 - u.u02 * u.u02);
  return u;
}

__global__ void prec_from_scale_rot_kernel(int64_t n, const float* __restrict__ scales,
                                           const float* __restrict__ quats,
                                           float* __restrict__ prec) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Rot R = make_rot(quats + 4 * i);
    double P[9], d[3];
    precision(R, scales + 3 * i, P, d);
    const Upper u = reverse_cholesky(P);
    float* o = prec + 9 * i;
    o[0] = (float)u.u00; o[1] = (float)u.u01; o[2] = (float)u.u02;
    o[3] = 0.f;          o[4] = (float)u.u11; o[5] = (float)u.u12;
    o[6] = 0.f;          o[7] = 0.f;          o[8] = (float)u.u22;
  }
}

__global__ void prec_from_scale_rot_bwd_kernel(int64_t n, const float* __restrict__ scales,
                                               const float* __restrict__ quats,
                                               const float* __restrict__ gprec,
                                               float* __restrict__ gscales,
                                               float* __restrict__ gquats) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Rot R = make_rot(quats + 4 * i);
    double P[9], d[3];
    precision(R, scales + 3 * i, P, d);
    const Upper u = reverse_cholesky(P);
    const float* g = gprec + 9 * i;  // strict-lower entries of the output are constant 0
    double g00 = g[0], g01 = g[1], g02 = g[2], g11 = g[4], g12 = g[5], g22 = g[8];
    double p00 = 0, p01 = 0, p02 = 0, p11 = 0, p12 = 0, p22 = 0;  // adjoints of P's upper part
    // U00 = sqrt(P00 - U01^2 - U02^2)
    const double t0 = g00 / (2.0 * u.u00);
    p00 += t0;
    g01 -= 2.0 * u.u01 * t0;
    g02 -= 2.0 * u.u02 * t0;
    // U01 = (P01 - U02 U12) / U11
    const double a = g01 / u.u11;
    g11 -= g01 * u.u01 / u.u11;
    p01 += a;
    g02 -= a * u.u12;
    g12 -= a * u.u02;
    // U11 = sqrt(P11 - U12^2)
    const double t1 = g11 / (2.0 * u.u11);
    p11 += t1;
    g12 -= 2.0 * u.u12 * t1;
    // U02 = P02 / U22, U12 = P12 / U22
    p02 += g02 / u.u22;
    g22 -= g02 * u.u02 / u.u22;
    p12 += g12 / u.u22;
    g22 -= g12 * u.u12 / u.u22;
    // U22 = sqrt(P22)
    p22 += g22 / (2.0 * u.u22);
    // Symmetric adjoint of P (each off-diagonal variable appears at (i,j) and (j,i)).
    const double Pb[9] = {p00, 0.5 * p01, 0.5 * p02, 0.5 * p01, p11, 0.5 * p12,
                          0.5 * p02, 0.5 * p12, p22};
    // P = R D R^T:  dL/dR = 2 Pb R D,  dL/dD_k = (R^T Pb R)_kk
    double gR[9];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        double v = 0.0;
        for (int k = 0; k < 3; ++k) v += Pb[3 * r + k] * R.r[3 * k + c];
        gR[3 * r + c] = 2.0 * v * d[c];
      }
    for (int k = 0; k < 3; ++k) {
      double v = 0.0;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) v += R.r[3 * r + k] * Pb[3 * r + c] * R.r[3 * c + k];
      const double s = scales[3 * i + k];
      gscales[3 * i + k] = (float)(v * (-2.0 / (s * s * s)));
    }
    double gq[4];
    rot_vjp(R, quats + 4 * i, gR, gq);
    for (int k = 0; k < 4; ++k) gquats[4 * i + k] = (float)gq[k];
  }
}

// out = M p + t with M = R (inverse = false) or R^T (inverse = true); pose = [t(3), q(4)].
// The rotation is built in float64 once per thread; the per-point arithmetic is float32, as in
// the reference (jnp.einsum in float32), so the kernel streams at memory speed.
__global__ void transform_points_kernel(int64_t n, const float* __restrict__ points,
                                        const float* __restrict__ pose, int inverse,
                                        float* __restrict__ out) {
  const Rot R = make_rot(pose + 3);
  float M[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) M[3 * r + c] = (float)(inverse ? R.r[3 * c + r] : R.r[3 * r + c]);
  const float t0 = pose[0], t1 = pose[1], t2 = pose[2];
  auto xf = [&](const float* p, float* o) {
    o[0] = fmaf(M[2], p[2], fmaf(M[1], p[1], fmaf(M[0], p[0], t0)));
    o[1] = fmaf(M[5], p[2], fmaf(M[4], p[1], fmaf(M[3], p[0], t1)));
    o[2] = fmaf(M[8], p[2], fmaf(M[7], p[1], fmaf(M[6], p[0], t2)));
  };
  // Groups of four points are three 16-byte words (both buffers are 16-byte aligned).
  const int64_t groups = n >> 2;
  const float4* in4 = reinterpret_cast<const float4*>(points);
  float4* out4 = reinterpret_cast<float4*>(out);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const float4 a = in4[3 * g], b = in4[3 * g + 1], c = in4[3 * g + 2];
    const float p[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
    float o[12];
#pragma unroll
    for (int q = 0; q < 4; ++q) xf(p + 3 * q, o + 3 * q);
    out4[3 * g] = make_float4(o[0], o[1], o[2], o[3]);
    out4[3 * g + 1] = make_float4(o[4], o[5], o[6], o[7]);
    out4[3 * g + 2] = make_float4(o[8], o[9], o[10], o[11]);
  }
  const int64_t tail = groups << 2;
  const int64_t i = tail + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) xf(points + 3 * i, out + 3 * i);
}

// dL/dp = M^T g; dL/dt = sum g; dL/dM = sum g p^T -> dL/dR (transposed when inverse) -> dL/dq.
// Block partial sums of the 12 pose sums go to gacc (float64, zeroed by the caller).
__global__ void transform_points_bwd_kernel(int64_t n, const float* __restrict__ points,
                                            const float* __restrict__ pose, int inverse,
                                            const float* __restrict__ gout,
                                            float* __restrict__ gpoints,
                                            double* __restrict__ gacc) {
  const Rot R = make_rot(pose + 3);
  float M[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) M[3 * r + c] = (float)(inverse ? R.r[3 * c + r] : R.r[3 * r + c]);
  // Per-thread float32 partial sums (a thread sees n / (grid x block) points), then float64.
  float acc[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // dL/dt (3), dL/dM (9)
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float g[3] = {gout[3 * i], gout[3 * i + 1], gout[3 * i + 2]};
    const float p[3] = {points[3 * i], points[3 * i + 1], points[3 * i + 2]};
    if (gpoints)
      for (int c = 0; c < 3; ++c)
        gpoints[3 * i + c] = fmaf(M[6 + c], g[2], fmaf(M[3 + c], g[1], M[c] * g[0]));
    for (int r = 0; r < 3; ++r) {
      acc[r] += g[r];
      for (int c = 0; c < 3; ++c) acc[3 + 3 * r + c] = fmaf(g[r], p[c], acc[3 + 3 * r + c]);
    }
  }
  __shared__ double red[12][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < 12; ++k) {
    double v = (double)acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    double v = 0.0;
    for (int w = 0; w < nw; ++w) v += red[threadIdx.x][w];
    atomicAdd(&gacc[threadIdx.x], v);
  }
}

// Final pose gradient from the accumulated sums: [dL/dt (3), dL/dq (4)].
__global__ void transform_points_pose_grad_kernel(const float* __restrict__ pose, int inverse,
                                                  const double* __restrict__ gacc,
                                                  float* __restrict__ gpose) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const Rot R = make_rot(pose + 3);
  double gR[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) gR[3 * r + c] = inverse ? gacc[3 + 3 * c + r] : gacc[3 + 3 * r + c];
  double gq[4];
  rot_vjp(R, pose + 3, gR, gq);
  for (int k = 0; k < 3; ++k) gpose[k] = (float)gacc[k];
  for (int k = 0; k < 4; ++k) gpose[3 + k] = (float)gq[k];
}

int grid_for_n(int64_t n, int threads) {
  const int64_t b = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

}  // namespace

void launch_prec_from_scale_rot(int64_t n, const float* scales, const float* quats, float* prec,
                                cudaStream_t st) {
  if (n <= 0) return;
  prec_from_scale_rot_kernel<<<grid_for_n(n, 128), 128, 0, st>>>(n, scales, quats, prec);
}

void launch_prec_from_scale_rot_bwd(int64_t n, const float* scales, const float* quats,
                                    const float* gprec, float* gscales, float* gquats,
                                    cudaStream_t st) {
  if (n <= 0) return;
  prec_from_scale_rot_bwd_kernel<<<grid_for_n(n, 128), 128, 0, st>>>(n, scales, quats, gprec,
                                                                      gscales, gquats);
}

void launch_transform_points(int64_t n, const float* points, const float* pose, int inverse,
                             float* out, cudaStream_t st) {
  if (n <= 0) return;
  transform_points_kernel<<<grid_for_n((n + 3) / 4, 256), 256, 0, st>>>(n, points, pose, inverse,
                                                                        out);
}

void launch_transform_points_bwd(int64_t n, const float* points, const float* pose, int inverse,
                                 const float* gout, float* gpoints, float* gpose, double* gacc,
                                 cudaStream_t st) {
  if (n > 0)
    transform_points_bwd_kernel<<<grid_for_n(n, 256), 256, 0, st>>>(n, points, pose, inverse,
                                                                    gout, gpoints, gacc);
  if (gpose) transform_points_pose_grad_kernel<<<1, 32, 0, st>>>(pose, inverse, gacc, gpose);
}

}  // namespace fe
