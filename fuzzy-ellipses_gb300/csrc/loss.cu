// loss.cu -- silhouette binary cross-entropy over the renders of a batch.
//
// The shape-from-silhouette loop of the reference (shape_from_silhouette.ipynb cell 12) scores a
// render's alpha against a target silhouette with
//     mean over pixels of -(t log a + (1 - t) log(1 - a)),  a clamped to [3e-8, 1 - 3e-8],
// and differentiates it with jax.grad. Here one kernel evaluates, for many renders laid out
// back to back in one pixel buffer (segment s = pixels [end[s-1], end[s])), every render's mean
// loss and the cotangent dL_s/dalpha of every pixel, which the blend backward consumes.
//
// float32 with the clamp applied to 1 - a rather than to a: 1 - a is exact for a >= 0.5
// (Sterbenz), so max(1 - a, 3e-8) equals 1 - min(a, 1 - 3e-8) evaluated exactly, whereas
// 1 - 3e-8 itself rounds to 1.0 in float32 (which would leave saturated pixels at log(0)).
// The per-render sums accumulate in float64.
#include <algorithm>

#include "fe_kernels.cuh"

namespace fe {
namespace {

constexpr float kClipAlpha = 3e-8f;
constexpr int kPixPerLane = 4;
constexpr int kPixPerWarp = 32 * kPixPerLane;

// Segment of pixel i: the first s with seg_end[s] > i.
__device__ __forceinline__ int segment_of(const int64_t* __restrict__ seg_end, int n_seg,
                                          int64_t i) {
  int lo = 0, hi = n_seg - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (seg_end[mid] > i) hi = mid; else lo = mid + 1;
  }
  return lo;
}

__device__ __forceinline__ double inv_count(const int64_t* __restrict__ seg_end, int s) {
  const int64_t begin = s > 0 ? seg_end[s - 1] : 0;
  return 1.0 / (double)(seg_end[s] - begin);
}

__device__ __forceinline__ float bce_pixel(float a, float t, float* d) {
  const float om = 1.f - a;
  const float ac = fmaxf(a, kClipAlpha);
  const float omc = fmaxf(om, kClipAlpha);
  const bool inside = (a > kClipAlpha) && (om > kClipAlpha);
  *d = inside ? (-t / ac + (1.f - t) / omc) : 0.f;
  return -(t * logf(ac) + (1.f - t) * logf(omc));
}

__global__ void __launch_bounds__(256) silhouette_bce_kernel(
    const float* __restrict__ alpha, const float* __restrict__ target,
    const int64_t* __restrict__ seg_end, int n_seg, int64_t n_pix, float* __restrict__ galpha,
    double* __restrict__ loss) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = warp * kPixPerWarp; base < n_pix; base += n_warps * kPixPerWarp) {
    const int64_t last = min(base + kPixPerWarp, n_pix) - 1;
    const int s0 = segment_of(seg_end, n_seg, base);
    const int s1 = segment_of(seg_end, n_seg, last);
    if (s0 == s1) {
      // The warp's pixels all belong to one render: one float64 sum, one atomic.
      const double inv = inv_count(seg_end, s0);
      double sum = 0.0;
#pragma unroll
      for (int j = 0; j < kPixPerLane; ++j) {
        const int64_t i = base + j * 32 + lane;
        if (i < n_pix) {
          float d;
          sum += (double)bce_pixel(alpha[i], target[i], &d);
          galpha[i] = (float)((double)d * inv);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == 0) atomicAdd(&loss[s0], sum * inv);
    } else {
      // A render boundary inside the warp's pixels: per-pixel segments and atomics.
#pragma unroll
      for (int j = 0; j < kPixPerLane; ++j) {
        const int64_t i = base + j * 32 + lane;
        if (i < n_pix) {
          const int s = segment_of(seg_end, n_seg, i);
          const double inv = inv_count(seg_end, s);
          float d;
          const float term = bce_pixel(alpha[i], target[i], &d);
          galpha[i] = (float)((double)d * inv);
          atomicAdd(&loss[s], (double)term * inv);
        }
      }
    }
  }
}

}  // namespace

void launch_silhouette_bce(const float* alpha, const float* target, const int64_t* seg_end,
                           int n_seg, int64_t n_pix, float* galpha, double* loss,
                           cudaStream_t st) {
  if (n_pix <= 0 || n_seg <= 0) return;
  const int64_t warps = (n_pix + kPixPerWarp - 1) / kPixPerWarp;
  const int64_t blocks = std::min<int64_t>((warps + 7) / 8, 152 * 8);
  silhouette_bce_kernel<<<(unsigned)blocks, 256, 0, st>>>(alpha, target, seg_end, n_seg, n_pix,
                                                         galpha, loss);
}

}  // namespace fe
