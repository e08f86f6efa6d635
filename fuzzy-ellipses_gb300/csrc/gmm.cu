// gmm.cu -- log-likelihood of 3-D points under the Gaussian mixture (fm_render.py:231-259).
//
// For points x_j and Gaussians i with precision factor U_i (fm_render's prec_full, upper
// triangle read, Sigma_i^-1 = U_i U_i^T) and mixture weights w = softmax(logw):
//     r_ij = log w_i + log|det U_i| - (|U_i^T (mu_i - x_j)|^2 + 3 log(2 pi)) / 2
//     ll_j = logsumexp_i r_ij
// gmm_prep_kernel folds the per-Gaussian constants (one block: the logsumexp of logw is a global
// reduction); gmm_ll_kernel streams the prepared Gaussians through shared memory while each
// thread keeps an online base-2 logsumexp for its points. Per (point, Gaussian): 3 subtractions,
// 6 FMA for U^T p, 3 for the squared norm, 1 for the log-density, one ex2 (plus the rare
// rescale when the running maximum grows). HBM traffic is only the points and the outputs.
#include <algorithm>

#include "fe_kernels.cuh"

namespace fe {
namespace {

// Prepared Gaussian (12 floats): mu, the six upper-triangle entries of U, and
// c2 = (log w + log|det U| - 1.5 log(2 pi)) log2(e).
struct GmmRec {
  float mx, my, mz;
  float u00, u01, u02, u11, u12, u22;
  float c2;
  float pad0, pad1;
};

constexpr float kHalfLog2Pi3 = 2.7568155996140185f;  // 1.5 ln(2 pi)
constexpr int kGmmThreads = 256;
constexpr int kGmmChunk = 512;  // Gaussians per shared-memory stage
constexpr int kGmmPts = 2;      // points per thread

__global__ void __launch_bounds__(1024) gmm_prep_kernel(int n, const float* __restrict__ means,
                                                        const float* __restrict__ prec,
                                                        const float* __restrict__ logw,
                                                        GmmRec* __restrict__ out) {
  __shared__ float red[32];
  __shared__ float shared_max, shared_lse;
  // logsumexp of logw (two block reductions).
  float m = -INFINITY;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, logw[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) shared_max = v;
  }
  __syncthreads();
  const float mx = shared_max;
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += expf(logw[i] - mx);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) shared_lse = mx + logf(v);
  }
  __syncthreads();
  const float lse = shared_lse;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float* U = prec + 9 * (int64_t)i;
    GmmRec r;
    r.mx = means[3 * (int64_t)i];
    r.my = means[3 * (int64_t)i + 1];
    r.mz = means[3 * (int64_t)i + 2];
    r.u00 = U[0]; r.u01 = U[1]; r.u02 = U[2]; r.u11 = U[4]; r.u12 = U[5]; r.u22 = U[8];
    const float logdet = logf(fabsf(r.u00)) + logf(fabsf(r.u11)) + logf(fabsf(r.u22));
    r.c2 = (logw[i] - lse + logdet - kHalfLog2Pi3) * kLog2e;
    r.pad0 = r.pad1 = 0.f;
    out[i] = r;
  }
}

__global__ void __launch_bounds__(kGmmThreads) gmm_ll_kernel(
    int n, const GmmRec* __restrict__ gs, int64_t n_points, const float* __restrict__ points,
    float* __restrict__ point_ll, float* __restrict__ res, double* __restrict__ total) {
  __shared__ GmmRec sg[kGmmChunk];
  const float kNegHalfLog2e = -0.5f * kLog2e;
  for (int64_t base = (int64_t)blockIdx.x * kGmmThreads * kGmmPts; base < n_points;
       base += (int64_t)gridDim.x * kGmmThreads * kGmmPts) {
    float px[kGmmPts], py[kGmmPts], pz[kGmmPts], m[kGmmPts], acc[kGmmPts];
    int64_t j[kGmmPts];
#pragma unroll
    for (int q = 0; q < kGmmPts; ++q) {
      j[q] = base + threadIdx.x + (int64_t)q * kGmmThreads;
      const bool ok = j[q] < n_points;
      px[q] = ok ? points[3 * j[q]] : 0.f;
      py[q] = ok ? points[3 * j[q] + 1] : 0.f;
      pz[q] = ok ? points[3 * j[q] + 2] : 0.f;
      m[q] = -INFINITY;
      acc[q] = 0.f;
    }
    for (int c0 = 0; c0 < n; c0 += kGmmChunk) {
      const int cn = min(kGmmChunk, n - c0);
      __syncthreads();
      for (int i = threadIdx.x; i < cn; i += kGmmThreads) sg[i] = gs[c0 + i];
      __syncthreads();
      for (int i = 0; i < cn; ++i) {
        const GmmRec g = sg[i];
#pragma unroll
        for (int q = 0; q < kGmmPts; ++q) {
          const float p0 = g.mx - px[q], p1 = g.my - py[q], p2 = g.mz - pz[q];
          const float q0 = g.u00 * p0;
          const float q1 = fmaf(g.u11, p1, g.u01 * p0);
          const float q2 = fmaf(g.u22, p2, fmaf(g.u12, p1, g.u02 * p0));
          const float d = fmaf(q2, q2, fmaf(q1, q1, q0 * q0));
          const float r2 = fmaf(kNegHalfLog2e, d, g.c2);  // log2 of the component density
          if (res && j[q] < n_points) res[(int64_t)(c0 + i) * n_points + j[q]] = r2 * kLn2;
          if (r2 > m[q]) {
            acc[q] = fmaf(acc[q], ex2_approx(m[q] - r2), 1.f);
            m[q] = r2;
          } else if (r2 > -INFINITY) {  // a -inf component adds nothing (and -inf - -inf is NaN)
            acc[q] += ex2_approx(r2 - m[q]);
          } else if (r2 != r2) {
            acc[q] = r2;  // NaN input propagates
          }
        }
      }
    }
    double local = 0.0;
#pragma unroll
    for (int q = 0; q < kGmmPts; ++q) {
      if (j[q] < n_points) {
        const float ll = (m[q] + log2f(acc[q])) * kLn2;
        point_ll[j[q]] = ll;
        local += (double)ll;
      }
    }
    if (total) {
      for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
      if ((threadIdx.x & 31) == 0) atomicAdd(total, local);
    }
  }
}

}  // namespace

size_t gmm_scratch_bytes(int n) { return sizeof(GmmRec) * (size_t)std::max(n, 1); }

void launch_gmm_log_likelihood(int n, const float* means, const float* prec, const float* logw,
                               int64_t n_points, const float* points, float* point_ll,
                               float* res, double* total, void* scratch, cudaStream_t st) {
  if (n <= 0 || n_points <= 0) return;
  GmmRec* gs = static_cast<GmmRec*>(scratch);
  gmm_prep_kernel<<<1, 1024, 0, st>>>(n, means, prec, logw, gs);
  const int64_t per_block = (int64_t)kGmmThreads * kGmmPts;
  const int64_t want = (n_points + per_block - 1) / per_block;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 8));
  gmm_ll_kernel<<<(unsigned)grid, kGmmThreads, 0, st>>>(n, gs, n_points, points, point_ll, res,
                                                        total);
}

}  // namespace fe
