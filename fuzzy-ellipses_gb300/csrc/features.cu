// features.cu -- softmax-weighted per-Gaussian features of an image render.
//
// fm_render returns the normalised softmax weights w (N, pixels) next to depth and alpha, "to
// compute color, DINO features, or any other per-Gaussian property" (baseline/fm_render.py:
// 104-109): feature(pixel) = sum_i w_i(pixel) f_i. On the tiled image path the weights never
// exist as a matrix: this pass runs after a forward render and reuses its per-pixel statistics
// (softmax maximum m and normaliser W, base 2), so w_i = 2^(l_i - m) / W for the tile's front
// Gaussians. Persistent warps take tiles from the device counter; each lane owns TW*TH/32 pixels
// of the tile, re-evaluates every key's logit there and accumulates four features at a time
// (the Gaussian index comes from the sorted key, the feature row from global memory). The keys'
// tile records are built 32 at a time, one per lane, into the warp's shared memory.
#include <algorithm>

#include "fe_kernels.cuh"
#include "fe_tilerec.cuh"

namespace fe {
namespace {

constexpr int kFeatWarps = 4;
constexpr int kFeatChunk = 4;

template <int TW, int TH>
__global__ void __launch_bounds__(32 * kFeatWarps) features_kernel(
    ViewsArg va, uint32_t n_tiles, const uint64_t* __restrict__ keys,
    const uint2* __restrict__ ranges, const GaussRec* __restrict__ recs,
    const float* __restrict__ stats, int64_t stride, float nb2, float beta3,
    const float* __restrict__ feats, int nf, float* __restrict__ out, Control* ctrl) {
  constexpr int NPX = TW * TH / 32;  // pixels per lane
  __shared__ TileRec rec_buf[kFeatWarps][32];
  __shared__ uint32_t gid_buf[kFeatWarps][32];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  TileRec* wrec = rec_buf[threadIdx.x >> 5];
  uint32_t* wgid = gid_buf[threadIdx.x >> 5];
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(&ctrl->next_tile, 1u);
    tile = __shfl_sync(full, tile, 0);
    if (tile >= n_tiles) break;
    const int vi = view_of_tile(va, tile);
    const ViewDev& V = view_at(va, vi);
    const int lt = (int)(tile - V.tile_base);
    const int tx = lt % V.gx, ty = lt / V.gx;
    const int xs = min(TW, V.W - tx * TW), ys = min(TH, V.H - ty * TH);
    const uint2 range = ranges[tile];

    float du[NPX], dv[NPX], m[NPX], iw[NPX];
    int64_t pix[NPX];
    bool ok[NPX];
#pragma unroll
    for (int i = 0; i < NPX; ++i) {
      const int q = lane + 32 * i;
      const int ly = q / TW, lx = q - ly * TW;
      ok[i] = lx < xs && ly < ys;
      du[i] = lx - 0.5f * (TW - 1);
      dv[i] = ly - 0.5f * (TH - 1);
      pix[i] = V.pix_base + (int64_t)(ty * TH + ly) * V.W + tx * TW + lx;
      m[i] = ok[i] ? stats[pix[i]] : 0.f;
      const float W = ok[i] ? stats[stride + pix[i]] : 0.f;
      iw[i] = W > 0.f ? 1.f / W : 0.f;
    }
    for (int c0 = 0; c0 < nf; c0 += kFeatChunk) {
      const int cn = min(kFeatChunk, nf - c0);
      float acc[NPX][kFeatChunk];
#pragma unroll
      for (int i = 0; i < NPX; ++i)
#pragma unroll
        for (int j = 0; j < kFeatChunk; ++j) acc[i][j] = 0.f;
      for (uint32_t k0 = range.x; k0 < range.y; k0 += 32) {
        const int nk = (int)min(32u, range.y - k0);
        __syncwarp();  // the previous keys' records are no longer read
        if (lane < nk) {
          const uint32_t g_id = (uint32_t)keys[k0 + lane];
          const GaussRec g = recs[V.rec_base + g_id];
          const float hw = 0.5f * (TW - 1), hh = 0.5f * (TH - 1);
          tile_record(g, tx * TW + hw - g.uc, ty * TH + hh - g.vc, hw, hh, wrec[lane]);
          wgid[lane] = g_id;
        }
        __syncwarp();
        for (int kj = 0; kj < nk; ++kj) {
          const TileRec& tr = wrec[kj];
          const float V0 = tr.V[0], V1 = tr.V[1], V2 = tr.V[2], V3 = tr.V[3], V4 = tr.V[4];
          const float V5 = tr.V[5], P0 = tr.P[0], P1 = tr.P[1], P2 = tr.P[2];
          const float N0 = tr.N[0], N1 = tr.N[1], N2 = tr.N[2], N3 = tr.N[3], N4 = tr.N[4];
          const float N5 = tr.N[5], C = tr.C, cu = tr.cu, cv = tr.cv;
          const uint32_t gid = wgid[kj];
          const float* fr = feats + (int64_t)gid * nf + c0;
          float f[kFeatChunk];
#pragma unroll
          for (int j = 0; j < kFeatChunk; ++j) f[j] = j < cn ? fr[j] : 0.f;
#pragma unroll
          for (int i = 0; i < NPX; ++i) {
            const float u = du[i], v = dv[i];
            const float vsv = fmaf(fmaf(V3, u, fmaf(V4, v, V1)), u, fmaf(fmaf(V5, v, V2), v, V0));
            const float psv = fmaf(P1, u, fmaf(P2, v, P0));
            const float eu = u - cu, ev = v - cv;
            const float nq = fmaf(fmaf(N3, eu, fmaf(N4, ev, N1)), eu, fmaf(fmaf(N5, ev, N2), ev, N0));
            const float qi = rcp_approx(vsv);
            const float z = psv * qi;
            const float s2 = fmaf(nq, qi, C);
            const float l = fmaf(beta3, s2, nb2 * z);
            // (a pixel without front Gaussians has W = 0 and m at the forward's sentinel)
            const float e = (z > 0.f && iw[i] > 0.f) ? ex2_approx(l - m[i]) * iw[i] : 0.f;
#pragma unroll
            for (int j = 0; j < kFeatChunk; ++j) acc[i][j] = fmaf(e, f[j], acc[i][j]);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < NPX; ++i)
        if (ok[i])
          for (int j = 0; j < cn; ++j) out[pix[i] * nf + c0 + j] = acc[i][j];
    }
  }
}

template <int TW, int TH>
void launch_tiles(const ViewsArg& va, int64_t n_tiles, const uint64_t* keys, const uint2* ranges,
                  const GaussRec* recs, const float* stats, int64_t stride, float beta2,
                  float beta3, const float* feats, int nf, float* out, Control* ctrl,
                  cudaStream_t st) {
  constexpr auto kern = features_kernel<TW, TH>;
  const int resident = resident_ctas<kern>(32 * kFeatWarps);
  const int64_t grid =
      std::max<int64_t>(1, std::min<int64_t>((n_tiles + kFeatWarps - 1) / kFeatWarps, resident));
  kern<<<(unsigned)grid, 32 * kFeatWarps, 0, st>>>(va, (uint32_t)n_tiles, keys, ranges, recs,
                                                   stats, stride, -beta2 * kLog2e, beta3, feats,
                                                   nf, out, ctrl);
}

}  // namespace

void launch_features(const ViewsArg& va, int tile_w, int tile_h, int64_t n_tiles,
                     const uint64_t* keys, const uint2* ranges, const GaussRec* recs,
                     const float* stats, int64_t stats_stride, float beta2, float beta3,
                     const float* feats, int nf, float* out, Control* ctrl, cudaStream_t st) {
  if (n_tiles <= 0 || nf <= 0) return;
  if (tile_w == 8 && tile_h == 8)
    launch_tiles<8, 8>(va, n_tiles, keys, ranges, recs, stats, stats_stride, beta2, beta3, feats,
                       nf, out, ctrl, st);
  else if (tile_w == 32 && tile_h == 8)
    launch_tiles<32, 8>(va, n_tiles, keys, ranges, recs, stats, stats_stride, beta2, beta3,
                        feats, nf, out, ctrl, st);
  else
    launch_tiles<16, 16>(va, n_tiles, keys, ranges, recs, stats, stats_stride, beta2, beta3,
                         feats, nf, out, ctrl, st);
}

}  // namespace fe
