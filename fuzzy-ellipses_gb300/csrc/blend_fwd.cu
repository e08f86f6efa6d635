// blend_fwd.cu -- per-tile forward blend: depth softmax and alpha in one pass.
//
// One CTA per screen tile, PX pixels of one row per thread. The tile's records (TileRec, 80 B, stored
// contiguously in key order by the gather step) are streamed through a two-stage shared-memory
// ring with 1-D TMA bulk copies (cp.async.bulk ... mbarrier::complete_tx). Per (pixel, Gaussian)
// evaluation, from the tile-local polynomials:
//     vsv = V(du,dv)   psv = P(du,dv)   nq = N(du-cu,dv-cv)    (polynomials; the row-constant
//                                                               parts are shared by the PX
//                                                               pixels a thread owns)
//     q = rcp(vsv); z = psv q; s2 = C + nq q                   (z: peak ray parameter,
//                                                               s2: log2 peak density)
//     A += 2^s2                                                (alpha accumulator, all Gaussians)
//     l = beta3 s2 - beta2 log2(e) z, masked to z > 0          (log2 softmax logit)
// and an online max / rescaled sum over groups of G Gaussians keeps the softmax in one pass:
//     W = sum 2^(l-m), Z = sum 2^(l-m) z, depth = Z/W, alpha = 1 - exp(-A).
// This is baseline/fm_render.py:11-109 (and the reference kernel gaussianRayRasterizeCUDA,
// cuda_rasterizer/forward.cu:206-423) restricted to the tile's Gaussians.
#include "fe_kernels.cuh"

namespace fe {

namespace {

constexpr int kChunk = 32;   // records per pipeline stage
constexpr int kStages = 2;

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
  r.cu = 0.f;
  r.cv = 0.f;
}

__device__ __forceinline__ void issue_chunk(BlendSmem& sm, int stage, const TileRec* src,
                                            int count) {
  const uint32_t bytes = (uint32_t)count * (uint32_t)sizeof(TileRec);
  mbar_arrive_expect_tx(&sm.full[stage], bytes);
  tma_bulk_g2s(&sm.buf[stage][0], src, bytes, &sm.full[stage]);
}

// Threads per CTA for a tile of TW x TH pixels with PX pixels per thread (PX pixels of one row,
// CW = TW/PX apart), and the number of records per online-softmax group.
template <int TW, int TH, int PX>
struct BlendShape {
  static constexpr int NT = TW * TH / PX;
  static constexpr int CW = TW / PX;
  static constexpr int G = PX >= 4 ? 4 : 8;
  static_assert(TW % PX == 0, "PX must divide the tile width");
};

template <int TW, int TH, int PX>
__global__ void __launch_bounds__(BlendShape<TW, TH, PX>::NT) blend_fwd_kernel(
    ViewsArg va, const TileRec* __restrict__ trec, const uint2* __restrict__ ranges, float nb2,
    float beta3, float* __restrict__ depth, float* __restrict__ alpha, float* __restrict__ stats,
    int64_t stats_stride, Control* __restrict__ ctrl) {
  using Sh = BlendShape<TW, TH, PX>;
  constexpr int G = Sh::G;
  __shared__ __align__(128) BlendSmem sm;

  const int64_t tile = blockIdx.x;
  const int vi = find_view<&ViewDev::tile_base>(va, tile);
  const ViewDev& V = view_at(va, vi);
  const int lt = (int)(tile - V.tile_base);
  const int tx = lt % V.gx, ty = lt / V.gx;
  const int tid = threadIdx.x;
  const int ly = tid / Sh::CW, cx = tid % Sh::CW;
  const float dv = ly - 0.5f * (TH - 1), dv2 = dv * dv;
  float du[PX];
#pragma unroll
  for (int k = 0; k < PX; ++k) du[k] = (cx + k * Sh::CW) - 0.5f * (TW - 1);

  const uint2 rg = ranges[tile];
  const int n = (int)(rg.y - rg.x);
  float A[PX], Wsum[PX], Zsum[PX], m[PX];
#pragma unroll
  for (int k = 0; k < PX; ++k) { A[k] = 0.f; Wsum[k] = 0.f; Zsum[k] = 0.f; m[k] = -INFINITY; }

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
      const int padded = (cnt + G - 1) / G * G;
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
#pragma unroll
        for (int k = 0; k < PX; ++k) { A[k] = 0.f; Wsum[k] = 0.f; Zsum[k] = 0.f; m[k] = -INFINITY; }
        break;
      }
      const float4* rec4 = reinterpret_cast<const float4*>(sm.buf[stage]);
      constexpr int R4 = sizeof(TileRec) / 16;
      for (int j = 0; j < padded; j += G) {
        float lg[G][PX], zg[G][PX];
        float cmax[PX];
#pragma unroll
        for (int k = 0; k < PX; ++k) cmax[k] = -INFINITY;
#pragma unroll
        for (int q = 0; q < G; ++q) {
          const float4 r0 = rec4[R4 * (j + q) + 0], r1 = rec4[R4 * (j + q) + 1];
          const float4 r2 = rec4[R4 * (j + q) + 2], r3 = rec4[R4 * (j + q) + 3];
          const float4 r4 = rec4[R4 * (j + q) + 4];
          // V0..V5 = r0.xyzw r1.xy; P0..P2 = r1.zw r2.x; N0..N5 = r2.yzw r3.xyz; C = r3.w;
          // (cu, cv) = r4.xy. Row-constant parts, shared by the thread's PX pixels of row dv.
          const float bv = fmaf(r1.y, dv2, fmaf(r0.z, dv, r0.x));
          const float cv = fmaf(r1.x, dv, r0.y);
          const float bp = fmaf(r2.x, dv, r1.z);
          const float ev = dv - r4.y;
          const float bn = fmaf(r3.z * ev, ev, fmaf(r2.w, ev, r2.y));
          const float cn = fmaf(r3.y, ev, r2.z);
#pragma unroll
          for (int k = 0; k < PX; ++k) {
            const float vsv = fmaf(fmaf(r0.w, du[k], cv), du[k], bv);
            const float psv = fmaf(r1.w, du[k], bp);
            const float eu = du[k] - r4.x;
            const float nq = fmaf(fmaf(r3.x, eu, cn), eu, bn);
            const float qi = rcp_approx(vsv);
            const float z = psv * qi;
            const float s2 = fmaf(nq, qi, r3.w);
            A[k] += ex2_approx(s2);
            const float l = fmaf(beta3, s2, nb2 * z);
            lg[q][k] = z > 0.f ? l : -INFINITY;
            zg[q][k] = z;
            cmax[k] = fmaxf(cmax[k], lg[q][k]);
          }
        }
#pragma unroll
        for (int k = 0; k < PX; ++k) {
          if (cmax[k] > m[k]) {
            const float sc = ex2_approx(m[k] - cmax[k]);
            Wsum[k] *= sc;
            Zsum[k] *= sc;
            m[k] = cmax[k];
          }
          if (m[k] > -INFINITY) {
#pragma unroll
            for (int q = 0; q < G; ++q) {
              const float e = ex2_approx(lg[q][k] - m[k]);
              Wsum[k] += e;
              Zsum[k] = fmaf(e, zg[q][k], Zsum[k]);
            }
          }
        }
      }
      fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0 && c + kStages < nchunks)
        issue_chunk(sm, stage, src + (c + kStages) * kChunk,
                    min(kChunk, n - (c + kStages) * kChunk));
    }
  }

  const int v = ty * TH + ly;
#pragma unroll
  for (int k = 0; k < PX; ++k) {
    const int u = tx * TW + cx + k * Sh::CW;
    if (u < V.W && v < V.H) {
      const int64_t pix = V.pix_base + (int64_t)v * V.W + u;
      depth[pix] = Wsum[k] > 0.f ? Zsum[k] / Wsum[k] : 0.f;
      alpha[pix] = -expm1f(-A[k]);
      if (stats) {
        stats[pix] = m[k];
        stats[stats_stride + pix] = Wsum[k];
        stats[2 * stats_stride + pix] = A[k];
      }
    }
  }
}

template <int TW, int TH, int PX>
void launch_tiles(const ViewsArg& va, int64_t n_tiles, const TileRec* trec, const uint2* ranges,
                  float nb2, float beta3, float* depth, float* alpha, float* stats,
                  int64_t stats_stride, Control* ctrl, cudaStream_t st) {
  blend_fwd_kernel<TW, TH, PX><<<(unsigned)n_tiles, BlendShape<TW, TH, PX>::NT, 0, st>>>(
      va, trec, ranges, nb2, beta3, depth, alpha, stats, stats_stride, ctrl);
}

}  // namespace

// Pixels per thread: px in {1, 2, 4}; 0 selects the default for the tile shape.
void launch_blend_fwd(const ViewsArg& va, int tile_w, int tile_h, int px, int64_t n_tiles,
                      const TileRec* trec, const uint2* ranges, float beta2, float beta3,
                      float* depth, float* alpha, float* stats, int64_t stats_stride,
                      Control* ctrl, cudaStream_t st) {
  if (n_tiles <= 0) return;
  const float nb2 = -beta2 * kLog2e;
#define FE_BLEND(TW_, TH_, PX_)                                                                 \
  launch_tiles<TW_, TH_, PX_>(va, n_tiles, trec, ranges, nb2, beta3, depth, alpha, stats,     \
                              stats_stride, ctrl, st)
  if (tile_w == 8 && tile_h == 8) {
    if (px == 1) FE_BLEND(8, 8, 1); else FE_BLEND(8, 8, 2);
  } else if (tile_w == 32 && tile_h == 8) {
    if (px == 1) FE_BLEND(32, 8, 1); else if (px == 2) FE_BLEND(32, 8, 2); else FE_BLEND(32, 8, 4);
  } else {
    if (px == 1) FE_BLEND(16, 16, 1); else if (px == 2) FE_BLEND(16, 16, 2); else FE_BLEND(16, 16, 4);
  }
#undef FE_BLEND
}

}  // namespace fe
