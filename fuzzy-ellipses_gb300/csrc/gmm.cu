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
constexpr int kGmmChunk = 512;  // Gaussians per shared-memory stage (40 KB)
constexpr int kGmmPts = 4;      // points per thread (two packed pairs)

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

// A prepared Gaussian with every field duplicated, so that one 8-byte shared-memory load gives a
// packed f32x2 operand for two points.
struct GmmRec2 {
  f2_t mx, my, mz, u00, u01, u02, u11, u12, u22, c2;
};

// Four points per thread as two packed pairs; Gaussians are consumed in groups of four so that
// the running maximum of each point's logsumexp is updated once per group.
__global__ void __launch_bounds__(kGmmThreads) gmm_ll_kernel(
    int n, const GmmRec* __restrict__ gs, int64_t n_points, const float* __restrict__ points,
    float* __restrict__ point_ll, float* __restrict__ res, double* __restrict__ total) {
  constexpr int kPairs = kGmmPts / 2;
  constexpr int kGroup = 4;
  __shared__ GmmRec2 sg[kGmmChunk];
  const f2_t NH = f2_pack(-0.5f * kLog2e, -0.5f * kLog2e);
  for (int64_t base = (int64_t)blockIdx.x * kGmmThreads * kGmmPts; base < n_points;
       base += (int64_t)gridDim.x * kGmmThreads * kGmmPts) {
    f2_t PX[kPairs], PY[kPairs], PZ[kPairs];
    float m[kGmmPts], acc[kGmmPts];
    int64_t j[kGmmPts];
#pragma unroll
    for (int q = 0; q < kGmmPts; ++q) {
      j[q] = base + threadIdx.x + (int64_t)q * kGmmThreads;
      m[q] = -INFINITY;
      acc[q] = 0.f;
    }
#pragma unroll
    for (int h = 0; h < kPairs; ++h) {
      float c[2][3];
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int q = 2 * h + t;
        const bool ok = j[q] < n_points;
        c[t][0] = ok ? points[3 * j[q]] : 0.f;
        c[t][1] = ok ? points[3 * j[q] + 1] : 0.f;
        c[t][2] = ok ? points[3 * j[q] + 2] : 0.f;
      }
      PX[h] = f2_pack(c[0][0], c[1][0]);
      PY[h] = f2_pack(c[0][1], c[1][1]);
      PZ[h] = f2_pack(c[0][2], c[1][2]);
    }
    for (int c0 = 0; c0 < n; c0 += kGmmChunk) {
      const int cn = min(kGmmChunk, n - c0);
      __syncthreads();
      for (int i = threadIdx.x; i < cn; i += kGmmThreads) {
        const GmmRec g = gs[c0 + i];
        GmmRec2 d;
        d.mx = f2_pack(g.mx, g.mx); d.my = f2_pack(g.my, g.my); d.mz = f2_pack(g.mz, g.mz);
        d.u00 = f2_pack(g.u00, g.u00); d.u01 = f2_pack(g.u01, g.u01);
        d.u02 = f2_pack(g.u02, g.u02); d.u11 = f2_pack(g.u11, g.u11);
        d.u12 = f2_pack(g.u12, g.u12); d.u22 = f2_pack(g.u22, g.u22);
        d.c2 = f2_pack(g.c2, g.c2);
        sg[i] = d;
      }
      __syncthreads();
      for (int i0 = 0; i0 < cn; i0 += kGroup) {
        const int gn = min(kGroup, cn - i0);
        float r[kGroup][kGmmPts];
#pragma unroll
        for (int k = 0; k < kGroup; ++k) {
          if (k < gn) {
            const GmmRec2& g = sg[i0 + k];
#pragma unroll
            for (int h = 0; h < kPairs; ++h) {
              const f2_t p0 = sub2(g.mx, PX[h]), p1 = sub2(g.my, PY[h]), p2 = sub2(g.mz, PZ[h]);
              const f2_t q0 = mul2(g.u00, p0);
              const f2_t q1 = fma2(g.u11, p1, mul2(g.u01, p0));
              const f2_t q2 = fma2(g.u22, p2, fma2(g.u12, p1, mul2(g.u02, p0)));
              const f2_t d = fma2(q2, q2, fma2(q1, q1, mul2(q0, q0)));
              f2_unpack(fma2(NH, d, g.c2), r[k][2 * h], r[k][2 * h + 1]);  // log2 densities
            }
          } else {
#pragma unroll
            for (int q = 0; q < kGmmPts; ++q) r[k][q] = -INFINITY;
          }
        }
#pragma unroll
        for (int q = 0; q < kGmmPts; ++q) {
          if (res && j[q] < n_points)
            for (int k = 0; k < gn; ++k) res[(int64_t)(c0 + i0 + k) * n_points + j[q]] = r[k][q] * kLn2;
          float gmax = r[0][q];
#pragma unroll
          for (int k = 1; k < kGroup; ++k) gmax = fmaxf(gmax, r[k][q]);
          if (gmax > m[q]) {
            acc[q] *= ex2_approx(m[q] - gmax);  // (0 while m is -inf: acc is 0 then)
            m[q] = gmax;
          }
          if (m[q] > -INFINITY) {  // all-(-inf) so far adds nothing (and -inf - -inf is NaN)
#pragma unroll
            for (int k = 0; k < kGroup; ++k) acc[q] += ex2_approx(r[k][q] - m[q]);
          }
          if (gmax != gmax) acc[q] = gmax;  // NaN input propagates
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
