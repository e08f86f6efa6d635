// blend_fwd.cu -- per-tile forward blend: depth softmax and alpha in one pass.
//
// One CTA per screen tile, one thread per pixel. The tile's records (TileRec, 64 B each, stored
// contiguously in key order by the gather step) are streamed through a two-stage shared-memory
// ring with 1-D TMA bulk copies (cp.async.bulk ... mbarrier::complete_tx). Per (pixel, Gaussian)
// evaluation, from the tile-local polynomials:
//     vsv = V(du,dv)   psv = P(du,dv)   nq = N(du,dv)          (12 FMA)
//     q = rcp(vsv); z = psv q; s2 = C + nq q                   (z: peak ray parameter,
//                                                               s2: log2 peak density)
//     A += 2^s2                                                (alpha accumulator, all Gaussians)
//     l = beta3 s2 - beta2 log2(e) z, masked to z > 0          (log2 softmax logit)
// and an online max / rescaled sum over groups of 8 Gaussians keeps the softmax in one pass:
//     W = sum 2^(l-m), Z = sum 2^(l-m) z, depth = Z/W, alpha = 1 - exp(-A).
// This is baseline/fm_render.py:11-109 (and the reference kernel gaussianRayRasterizeCUDA,
// cuda_rasterizer/forward.cu:206-423) restricted to the tile's Gaussians.
#include "fe_kernels.cuh"

namespace fe {

namespace {

constexpr int kChunk = 32;   // records per pipeline stage
constexpr int kStages = 2;
constexpr int kGroup = 8;    // records per online-softmax rescale

struct BlendSmem {
  TileRec buf[kStages][kChunk];
  uint64_t full[kStages];
};

__device__ __forceinline__ void null_record(TileRec& r) {
  r.V[0] = 1.f;
#pragma unroll
  for (int k = 1; k < 6; ++k) r.V[k] = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) r.P[k] = 0.f;
#pragma unroll
  for (int k = 0; k < 6; ++k) r.N[k] = 0.f;
  r.C = -INFINITY;
}

__device__ __forceinline__ void issue_chunk(BlendSmem& sm, int stage, const TileRec* src,
                                            int count) {
  const uint32_t bytes = (uint32_t)count * (uint32_t)sizeof(TileRec);
  mbar_arrive_expect_tx(&sm.full[stage], bytes);
  tma_bulk_g2s(&sm.buf[stage][0], src, bytes, &sm.full[stage]);
}

template <int TW, int TH>
__global__ void __launch_bounds__(TW * TH) blend_fwd_kernel(
    ViewsArg va, const TileRec* __restrict__ trec, const uint2* __restrict__ ranges, float nb2,
    float beta3, float* __restrict__ depth, float* __restrict__ alpha, float* __restrict__ stats,
    int64_t stats_stride, Control* __restrict__ ctrl) {
  constexpr int NT = TW * TH;
  static_assert(NT >= kGroup, "tile too small");
  __shared__ __align__(128) BlendSmem sm;

  const int64_t tile = blockIdx.x;
  const int vi = find_view<&ViewDev::tile_base>(va, tile);
  const ViewDev& V = view_at(va, vi);
  const int lt = (int)(tile - V.tile_base);
  const int tx = lt % V.gx, ty = lt / V.gx;
  const int tid = threadIdx.x;
  const int lx = tid % TW, ly = tid / TW;
  const int u = tx * TW + lx, v = ty * TH + ly;
  const bool valid = u < V.W && v < V.H;
  const float du = lx - 0.5f * (TW - 1), dv = ly - 0.5f * (TH - 1);
  const float du2 = du * du, dudv = du * dv, dv2 = dv * dv;

  const uint2 rg = ranges[tile];
  const int n = (int)(rg.y - rg.x);
  float A = 0.f, Wsum = 0.f, Zsum = 0.f, m = -INFINITY;

  if (n > 0) {
    const int nchunks = (n + kChunk - 1) / kChunk;
    const TileRec* src = trec + rg.x;
    if (tid == 0) {
#pragma unroll
      for (int s = 0; s < kStages; ++s) mbar_init(&sm.full[s], 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
      for (int c = 0; c < kStages && c < nchunks; ++c)
        issue_chunk(sm, c, src + c * kChunk, min(kChunk, n - c * kChunk));
    }
    for (int c = 0; c < nchunks; ++c) {
      const int stage = c % kStages;
      const uint32_t parity = (uint32_t)((c / kStages) & 1);
      const int cnt = min(kChunk, n - c * kChunk);
      const int padded = (cnt + kGroup - 1) / kGroup * kGroup;
      // Pad the chunk to whole groups with records that contribute nothing; these slots are
      // disjoint from the bytes the bulk copy writes.
      if (tid < padded - cnt) null_record(sm.buf[stage][cnt + tid]);
      const bool ok = mbar_wait_bounded(&sm.full[stage], parity);
      if (__syncthreads_or(!ok)) {
        // A copy did not land in time: flag it, let every outstanding copy finish (bounded),
        // and leave this tile's outputs at zero.
        if (tid == 0) {
          atomicOr(&ctrl->error, FE_DEVERR_TIMEOUT);
          for (int cc = c; cc < nchunks && cc < c + kStages; ++cc)
            (void)mbar_wait_bounded(&sm.full[cc % kStages], (uint32_t)((cc / kStages) & 1));
        }
        __syncthreads();
        A = 0.f; Wsum = 0.f; Zsum = 0.f; m = -INFINITY;
        break;
      }
      const TileRec* rec = sm.buf[stage];
      for (int j = 0; j < padded; j += kGroup) {
        float lg[kGroup], zg[kGroup];
        float cmax = -INFINITY;
#pragma unroll
        for (int q = 0; q < kGroup; ++q) {
          const TileRec& r = rec[j + q];
          const float vsv = fmaf(r.V[5], dv2, fmaf(r.V[4], dudv, fmaf(r.V[3], du2,
                                 fmaf(r.V[2], dv, fmaf(r.V[1], du, r.V[0])))));
          const float psv = fmaf(r.P[2], dv, fmaf(r.P[1], du, r.P[0]));
          const float nq = fmaf(r.N[5], dv2, fmaf(r.N[4], dudv, fmaf(r.N[3], du2,
                                fmaf(r.N[2], dv, fmaf(r.N[1], du, r.N[0])))));
          const float qi = rcp_approx(vsv);
          const float z = psv * qi;
          const float s2 = fmaf(nq, qi, r.C);
          A += ex2_approx(s2);
          const float l = fmaf(beta3, s2, nb2 * z);
          lg[q] = z > 0.f ? l : -INFINITY;
          zg[q] = z;
          cmax = fmaxf(cmax, lg[q]);
        }
        if (cmax > m) {
          const float sc = ex2_approx(m - cmax);
          Wsum *= sc;
          Zsum *= sc;
          m = cmax;
        }
        if (m > -INFINITY) {
#pragma unroll
          for (int q = 0; q < kGroup; ++q) {
            const float e = ex2_approx(lg[q] - m);
            Wsum += e;
            Zsum = fmaf(e, zg[q], Zsum);
          }
        }
      }
      __syncthreads();
      if (tid == 0 && c + kStages < nchunks) {
        fence_proxy_async_smem();
        issue_chunk(sm, stage, src + (c + kStages) * kChunk,
                    min(kChunk, n - (c + kStages) * kChunk));
      }
    }
  }

  if (valid) {
    const int64_t pix = V.pix_base + (int64_t)v * V.W + u;
    depth[pix] = Wsum > 0.f ? Zsum / Wsum : 0.f;
    alpha[pix] = -expm1f(-A);
    if (stats) {
      stats[pix] = m;
      stats[stats_stride + pix] = Wsum;
      stats[2 * stats_stride + pix] = A;
    }
  }
}

template <int TW, int TH>
void launch_tiles(const ViewsArg& va, int64_t n_tiles, const TileRec* trec, const uint2* ranges,
                  float nb2, float beta3, float* depth, float* alpha, float* stats,
                  int64_t stats_stride, Control* ctrl, cudaStream_t st) {
  blend_fwd_kernel<TW, TH><<<(unsigned)n_tiles, TW * TH, 0, st>>>(
      va, trec, ranges, nb2, beta3, depth, alpha, stats, stats_stride, ctrl);
}

}  // namespace

void launch_blend_fwd(const ViewsArg& va, int tile_w, int tile_h, int64_t n_tiles,
                      const TileRec* trec, const uint2* ranges, float beta2, float beta3,
                      float* depth, float* alpha, float* stats, int64_t stats_stride,
                      Control* ctrl, cudaStream_t st) {
  if (n_tiles <= 0) return;
  const float nb2 = -beta2 * kLog2e;
  if (tile_w == 8 && tile_h == 8)
    launch_tiles<8, 8>(va, n_tiles, trec, ranges, nb2, beta3, depth, alpha, stats, stats_stride,
                       ctrl, st);
  else if (tile_w == 32 && tile_h == 8)
    launch_tiles<32, 8>(va, n_tiles, trec, ranges, nb2, beta3, depth, alpha, stats, stats_stride,
                        ctrl, st);
  else
    launch_tiles<16, 16>(va, n_tiles, trec, ranges, nb2, beta3, depth, alpha, stats,
                         stats_stride, ctrl, st);
}

}  // namespace fe
