// blend_fwd.cu -- per-tile forward blend: depth softmax and alpha in one pass.
//
// Persistent CTAs take screen tiles from a device-side work counter (one launch covers any number
// of uneven renders); each thread owns PX pixels of one tile row. A tile's keys are taken in
// chunks of 2 CH: the chunk's Gaussian records (96 B each) are staged in shared memory by 1-D TMA
// bulk copies (cp.async.bulk, one per record, completing on an mbarrier; every wait bounded)
// while the previous chunk is evaluated, then each thread re-expands its records around
// the tile centre into pair-interleaved TilePairs (two records per 160 B, field by field) in a
// double-buffered shared-memory ring; the Gaussian ids of the chunk after are read one chunk
// ahead of that. No record stream is written to or read from HBM for the forward. Two records
// are evaluated together with packed
// f32x2 arithmetic, so each 16-byte shared load yields two ready operands and every polynomial,
// logit and accumulation step is one instruction for two evaluations. Per (pixel, Gaussian):
//     vsv = V(du,dv)   psv = P(du,dv)   nq = N(du-cu, dv-cv)    (row-constant parts shared by
//                                                                the thread's PX pixels)
//     q = rcp(vsv); z = psv q; s2 = C + nq q                    (z: peak ray parameter,
//                                                                s2: log2 peak density)
//     A += 2^s2                                                 (alpha, all Gaussians)
//     l = beta3 s2 - beta2 log2(e) z, masked to z > 0            (log2 softmax logit; the mask is
//                                                                skipped for pairs whose psv is
//                                                                positive over the whole tile)
// and an online max (updated once per group of records) keeps the softmax in one pass:
//     W = sum 2^(l-m), Z = sum 2^(l-m) z, depth = Z/W, alpha = 1 - exp(-A).
// This is baseline/fm_render.py:11-109 (and the reference kernel gaussianRayRasterizeCUDA,
// cuda_rasterizer/forward.cu:206-423) restricted to the tile's Gaussians.
#include <algorithm>

#include "fe_kernels.cuh"
#include "fe_tilerec.cuh"

namespace fe {

namespace {

template <int CH>
struct BlendSmem {
  TilePair buf[2][CH];      // record pairs: chunk c of a tile in buf[c & 1]
  GaussRec src[2 * CH];     // source records of the next chunk (TMA bulk copies), record r at src[r]
  uint64_t bar;             // completion of the source-record copies, one phase per chunk
  uint32_t tile;
  uint4 entry;              // the work-class list entry of the tile: id, range, view
  uint32_t cls_base[kTileClasses + 1];  // first work index of each tile class (with `order`)
};

// Write a null record into slot `sl` (0 = .x, 1 = .y) of a pair: vsv = 1, psv = 0 (z = 0,
// masked), C = -inf (density 0).
__device__ __forceinline__ void null_slot(TilePair& p, int sl) {
#pragma unroll
  for (int i = 0; i < kRecFields; ++i) {
    float v = 0.f;
    if (i == 0) v = 1.f;
    if (i == 15) v = -INFINITY;
    if (sl == 0) p.f[i].x = v; else p.f[i].y = v;
  }
}

// Threads per CTA for a tile of TW x TH pixels with PX pixels per thread (PX consecutive pixels
// of one row, CW = TW/PX threads per row); GP record pairs per online-softmax group (one max
// update per group).
template <int TW, int TH, int PX, int CH>
struct BlendShape {
  static constexpr int NT = TW * TH / PX;
  // Resident CTAs per SM the register budget is sized for: 20 warps (640 threads) per SM, at
  // most 16 CTAs (one-warp CTAs would otherwise be squeezed into spilling). 20 warps leave the
  // 16x16 kernel 94 registers and no spills; at 24 warps it is held to 80 registers, spills a
  // little and runs about 1.3% slower.
  static constexpr int MIN_CTAS = (640 / NT) < 16 ? (640 / NT) : 16;
  static constexpr int CW = TW / PX;
  static constexpr int GP = PX >= 4 ? 2 : 4;
  static_assert(TW % PX == 0, "PX must divide the tile width");
  static_assert(CH % GP == 0, "groups must tile a chunk");
  static_assert(NT >= GP, "enough threads to pad a chunk");
};

// Initial running max: finite, far below any logit, so logit - max is never inf - inf.
constexpr float kNoLogit = -1e30f;

// Store a thread's PX consecutive pixels of one row (`room` pixels of the row remain from the
// first): one vector store when all PX lie inside the image and the address is aligned to it,
// else one store per pixel inside the image. The outputs may be pinned host memory mapped into
// the device's address space, where whole vectors keep the link's write rate.
template <int PX>
__device__ __forceinline__ void store_pixels(float* dst, const float (&x)[PX], int room) {
  const bool whole =
      room >= PX && (reinterpret_cast<uintptr_t>(dst) & (sizeof(float) * PX - 1)) == 0;
  if (PX == 4 && whole) {
    *reinterpret_cast<float4*>(dst) = make_float4(x[0], x[1], x[2 % PX], x[3 % PX]);
  } else if (PX == 2 && whole) {
    *reinterpret_cast<float2*>(dst) = make_float2(x[0], x[1 % PX]);
  } else {
#pragma unroll
    for (int k = 0; k < PX; ++k)
      if (k < room) dst[k] = x[k];
  }
}

// One group of GP record pairs for the thread's PX pixels: evaluate every logit, raise the running
// maxima once (rescaling W and Z), then accumulate. MASK applies the z > 0 mask to the logits.
template <int PX, int GP, bool MASK>
__device__ __forceinline__ void blend_group(const TilePair* grp, const f2_t (&DU)[PX], f2_t DV,
                                            f2_t DVSQ, f2_t B3, f2_t NB2, f2_t (&A2)[PX],
                                            f2_t (&W2)[PX], f2_t (&Z2)[PX], float (&m)[PX]) {
  f2_t ll[GP][PX], zz[GP][PX];
  float cmax[PX];
#pragma unroll
  for (int k = 0; k < PX; ++k) cmax[k] = -INFINITY;
#pragma unroll
  for (int q = 0; q < GP; ++q) {
    const ulonglong2* rp = reinterpret_cast<const ulonglong2*>(grp + q);
    const ulonglong2 r0 = rp[0], r1 = rp[1], r2 = rp[2], r3 = rp[3], r4 = rp[4];
    const ulonglong2 r5 = rp[5], r6 = rp[6], r7 = rp[7], r8 = rp[8];
    // V0..V5 = r0.x r0.y r1.x r1.y r2.x r2.y; P0..P2 = r3.x r3.y r4.x;
    // N0..N5 = r4.y r5.x r5.y r6.x r6.y r7.x; C = r7.y; cu = r8.x; cv = r8.y.
    // Row-constant parts first, shared by the thread's PX pixels.
    const f2_t bv = fma2(r2.y, DVSQ, fma2(r1.x, DV, r0.x));
    const f2_t cv = fma2(r2.x, DV, r0.y);
    const f2_t bp = fma2(r4.x, DV, r3.x);
    const f2_t ev = sub2(DV, r8.y);
    const f2_t bn = fma2(mul2(r7.x, ev), ev, fma2(r5.y, ev, r4.y));
    const f2_t cn = fma2(r6.y, ev, r5.x);
#pragma unroll
    for (int k = 0; k < PX; ++k) {
      const f2_t vsv = fma2(fma2(r1.y, DU[k], cv), DU[k], bv);
      const f2_t psv = fma2(r3.y, DU[k], bp);
      const f2_t eu = sub2(DU[k], r8.x);
      const f2_t nq = fma2(fma2(r6.x, eu, cn), eu, bn);
      float va, vb;
      f2_unpack(vsv, va, vb);
      const f2_t qi = f2_pack(rcp_approx(va), rcp_approx(vb));
      const f2_t z = mul2(psv, qi);
      const f2_t s2 = fma2(nq, qi, r7.y);
      float sa, sb;
      f2_unpack(s2, sa, sb);
      A2[k] = add2(A2[k], f2_pack(ex2_approx(sa), ex2_approx(sb)));
      f2_t l = fma2(B3, s2, mul2(NB2, z));
      float l0, l1;
      f2_unpack(l, l0, l1);
      if (MASK) {
        float z0, z1;
        f2_unpack(z, z0, z1);
        l0 = z0 > 0.f ? l0 : -INFINITY;
        l1 = z1 > 0.f ? l1 : -INFINITY;
        l = f2_pack(l0, l1);
      }
      ll[q][k] = l;
      zz[q][k] = z;
      cmax[k] = max3f(cmax[k], l0, l1);
    }
  }
#pragma unroll
  for (int k = 0; k < PX; ++k) {
    if (cmax[k] > m[k]) {
      const float sc = ex2_approx(m[k] - cmax[k]);
      const f2_t S = f2_pack(sc, sc);
      W2[k] = mul2(W2[k], S);
      Z2[k] = mul2(Z2[k], S);
      m[k] = cmax[k];
    }
    const f2_t M = f2_pack(m[k], m[k]);
#pragma unroll
    for (int q = 0; q < GP; ++q) {
      float d0, d1;
      f2_unpack(sub2(ll[q][k], M), d0, d1);
      const f2_t e = f2_pack(ex2_approx(d0), ex2_approx(d1));
      W2[k] = add2(W2[k], e);
      Z2[k] = fma2(e, zz[q][k], Z2[k]);
    }
  }
}

template <int TW, int TH, int PX, int CH>
__global__ void __launch_bounds__(BlendShape<TW, TH, PX, CH>::NT,
                                  BlendShape<TW, TH, PX, CH>::MIN_CTAS) blend_fwd_kernel(
    ViewsArg va, uint32_t tile_begin, uint32_t tile_end, uint32_t* __restrict__ counter,
    const uint32_t* __restrict__ order, const uint64_t* __restrict__ keys,
    const GaussRec* __restrict__ recs, const uint2* __restrict__ ranges, float nb2, float beta3,
    float* __restrict__ depth, float* __restrict__ alpha, float* __restrict__ stats,
    int64_t stats_stride, Control* __restrict__ ctrl) {
  using Sh = BlendShape<TW, TH, PX, CH>;
  constexpr int GP = Sh::GP;
  __shared__ __align__(128) BlendSmem<CH> sm;

  const int tid = threadIdx.x;
  const int ly = tid / Sh::CW, cx = tid % Sh::CW;
  const float dv = ly - 0.5f * (TH - 1);
  const f2_t DV = f2_pack(dv, dv), DVSQ = f2_pack(dv * dv, dv * dv);
  const f2_t B3 = f2_pack(beta3, beta3), NB2 = f2_pack(nb2, nb2);
  // The thread's pixels are PX consecutive pixels of its row, so its outputs leave as one vector
  // store per plane.
  f2_t DU[PX];
#pragma unroll
  for (int k = 0; k < PX; ++k) {
    const float du = (cx * PX + k) - 0.5f * (TW - 1);
    DU[k] = f2_pack(du, du);
  }
  const f2_t ZERO2 = f2_pack(0.f, 0.f);

  constexpr int RC = 2 * CH;                     // records per chunk
  constexpr int RPT = (RC + Sh::NT - 1) / Sh::NT;  // records each thread stages and builds
  const float hw = 0.5f * (TW - 1), hh = 0.5f * (TH - 1);
  // Heaviest tiles first: with `order` (the tile-major binning's per-class tile lists over all
  // tiles [0, tile_end), uint4 entries: tile id, first key, end key, view) work index w of class
  // c maps to entry c tile_end + w - cls_base[c], so the tiles taken last, which set the
  // kernel's tail, are the lightest, and a tile's range and view come with its id. The lists are
  // used only when they hold every tile exactly once (their counts sum to tile_end); else tiles
  // go in index order.
  bool use_order = false;
  if (tid == 0) {
    mbar_init(&sm.bar, 1);
    fence_mbar_init();
    if (order && tile_begin == 0) {
      uint32_t b = 0;
      for (int c = 0; c < kTileClasses; ++c) {
        sm.cls_base[c] = b;
        b += ctrl->tile_class[c];
      }
      sm.cls_base[kTileClasses] = b;
      use_order = b == tile_end;
    }
  }
  __syncthreads();
  const bool use_order_all = order && tile_begin == 0 && sm.cls_base[kTileClasses] == tile_end;
  uint32_t phase = 0;  // parity of the next completion of sm.bar

  // Work index of the CTA's first tile: its own index (the grid never exceeds the tiles), so the
  // launch does not start with every CTA contending for the counter; later tiles come from the
  // counter, offset by the grid.
  bool first = true;
  while (true) {
    if (tid == 0) {
      uint32_t w = first ? tile_begin + blockIdx.x
                         : tile_begin + gridDim.x + atomicAdd(counter, 1u);
      if (use_order && w < tile_end) {
        int c = 0;
        while (c + 1 < kTileClasses && w >= sm.cls_base[c + 1]) ++c;
        const uint4 e = reinterpret_cast<const uint4*>(order)[(int64_t)c * tile_end +
                                                              (w - sm.cls_base[c])];
        sm.entry = e;
        w = e.x;
      }
      sm.tile = w;
    }
    first = false;
    __syncthreads();
    const uint32_t tile = sm.tile;
    if (tile >= tile_end) break;
    // With the work-class lists the entry carries the tile's range and view.
    const bool listed = order && tile_begin == 0 && use_order_all;
    const int vi = listed ? (int)sm.entry.w : view_of_tile(va, tile);
    const int gx = view_at(va, vi).gx;
    const int lt = (int)(tile - view_at(va, vi).tile_base);
    const int tx = lt % gx, ty = lt / gx;
    const GaussRec* vrec = recs + view_at(va, vi).rec_base;
    const float tcu = tx * TW + hw, tcv = ty * TH + hh;  // tile centre (pixels)

    const uint2 rg = listed ? make_uint2(sm.entry.y, sm.entry.z) : ranges[tile];
    // m starts finite (kNoLogit) so that logit - m is never (-inf) - (-inf); masked logits are
    // -inf and give weight 0.
    f2_t A2[PX], W2[PX], Z2[PX];
    float m[PX];
#pragma unroll
    for (int k = 0; k < PX; ++k) {
      A2[k] = ZERO2; W2[k] = ZERO2; Z2[k] = ZERO2;
      m[k] = kNoLogit;
    }
    if (rg.y > rg.x) {
      const int nk = (int)(rg.y - rg.x);
      const int nchunks = (nk + RC - 1) / RC;
      const uint64_t* tkeys = keys + rg.x;
      // Chunk c holds the tile's keys [c RC, c RC + RC); thread t stages and builds records
      // t, t + NT, ... of a chunk. The source records of chunk c + 1 arrive by TMA bulk copies
      // (96 B each, completing on sm.bar) while chunk c is evaluated; the Gaussian ids of chunk
      // c + 2 are read one chunk ahead of that. Copies into the staging buffer are issued only
      // after a barrier that every thread reaches after its wait for the previous chunk.
      uint32_t gid_next[RPT];
      auto stage = [&](int c, const uint32_t (&gid)[RPT]) {
        const int cnt = min(RC, nk - c * RC);
        fence_proxy_async_smem();  // this thread's reads of sm.src precede the copies into it
        if (tid == 0) mbar_arrive_expect_tx(&sm.bar, (uint32_t)(cnt * (int)sizeof(GaussRec)));
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
          const int r = tid + q * Sh::NT;
          if (r < cnt) tma_bulk_g2s(&sm.src[r], vrec + gid[q], (uint32_t)sizeof(GaussRec), &sm.bar);
        }
      };
      auto wait_src = [&]() {
        const bool ok = mbar_wait_bounded(&sm.bar, phase);
        phase ^= 1u;
        return ok;
      };
      // A copy that did not land in time: flag it, give the outstanding copies one more bounded
      // wait and stop this CTA; the tile's outputs are left unwritten.
      auto give_up = [&]() {
        if (tid == 0) {
          atomicOr(&ctrl->error, FE_DEVERR_TIMEOUT);
          (void)mbar_wait_bounded(&sm.bar, phase ^ 1u);
        }
      };
      auto load_gids = [&](int c, uint32_t (&gid)[RPT]) {
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
          const int r = tid + q * Sh::NT;
          gid[q] = (r < RC && c * RC + r < nk) ? (uint32_t)tkeys[c * RC + r] : 0u;
        }
      };
      // Build chunk c's record pairs from the staged source records (after the wait every
      // thread sees all of them; each builds its own) and null the slot past the tile's keys
      // that completes the last pair.
      auto build = [&](int c) {
        TilePair* pb = sm.buf[c & 1];
        const int cnt = min(RC, nk - c * RC);
        const int padded = (cnt + 1) & ~1;
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
          const int r = tid + q * Sh::NT;
          if (r < cnt) {
            const GaussRec& g = sm.src[r];
            TileRec t;
            tile_record(g, tcu - g.uc, tcv - g.vc, hw, hh, t);
            const float* f = reinterpret_cast<const float*>(&t);
            float* dst = reinterpret_cast<float*>(&pb[r >> 1]) + (r & 1);
#pragma unroll
            for (int i = 0; i < kRecFields; ++i) dst[2 * i] = f[i];
          } else if (r < padded) {
            null_slot(pb[r >> 1], r & 1);
          }
        }
      };
      {
        // One staging buffer: chunk 1 is copied only once chunk 0 has been built from it.
        uint32_t g0[RPT];
        load_gids(0, g0);
        stage(0, g0);
        load_gids(1, g0);
        const bool ok = wait_src();
        build(0);
        if (__syncthreads_or(!ok)) {
          give_up();
          return;
        }
        if (nchunks > 1) stage(1, g0);
        load_gids(2, gid_next);
      }
      for (int c = 0; c < nchunks; ++c) {
        const int cnt = min(RC, nk - c * RC);
        const int pairs = (cnt + 1) >> 1;
        const TilePair* pb = sm.buf[c & 1];
        int j = 0;
        for (; j + GP <= pairs; j += GP) {
          // Uniform over the CTA: the z > 0 mask is only evaluated for groups holding a record
          // whose psv is not positive over the whole tile (null slots included).
          bool need_mask = false;
#pragma unroll
          for (int q = 0; q < GP; ++q) {
            const float2 fr = pb[j + q].f[18];
            need_mask |= !(fr.x != 0.f && fr.y != 0.f);
          }
          if (need_mask)
            blend_group<PX, GP, true>(&pb[j], DU, DV, DVSQ, B3, NB2, A2, W2, Z2, m);
          else
            blend_group<PX, GP, false>(&pb[j], DU, DV, DVSQ, B3, NB2, A2, W2, Z2, m);
        }
        // The pairs after the last whole group, in groups of two pairs, then one.
        for (; j < pairs;) {
          if (GP > 2 && j + 2 <= pairs) {
            const float2 f0 = pb[j].f[18], f1 = pb[j + 1].f[18];
            if (!(f0.x != 0.f && f0.y != 0.f && f1.x != 0.f && f1.y != 0.f))
              blend_group<PX, 2, true>(&pb[j], DU, DV, DVSQ, B3, NB2, A2, W2, Z2, m);
            else
              blend_group<PX, 2, false>(&pb[j], DU, DV, DVSQ, B3, NB2, A2, W2, Z2, m);
            j += 2;
          } else {
            const float2 f0 = pb[j].f[18];
            if (!(f0.x != 0.f && f0.y != 0.f))
              blend_group<PX, 1, true>(&pb[j], DU, DV, DVSQ, B3, NB2, A2, W2, Z2, m);
            else
              blend_group<PX, 1, false>(&pb[j], DU, DV, DVSQ, B3, NB2, A2, W2, Z2, m);
            j += 1;
          }
        }
        if (c + 1 < nchunks) {
          // Chunk c + 1: wait for its source records, build its pairs (buf[(c + 1) & 1] was last
          // read in chunk c - 1), publish them, then stage chunk c + 2.
          const bool ok = wait_src();
          build(c + 1);
          if (__syncthreads_or(!ok)) {
            give_up();
            return;
          }
          if (c + 2 < nchunks) {
            stage(c + 2, gid_next);
            load_gids(c + 3, gid_next);
          }
        }
      }
    }

    const ViewDev& V = view_at(va, vi);
    const int v = ty * TH + ly;
    const int u0 = tx * TW + cx * PX;
    if (v < V.H) {
      float dep[PX], alp[PX], wsum[PX], asum[PX];
#pragma unroll
      for (int k = 0; k < PX; ++k) {
        float a0, a1, w0, w1, z0, z1;
        f2_unpack(A2[k], a0, a1);
        f2_unpack(W2[k], w0, w1);
        f2_unpack(Z2[k], z0, z1);
        const float A = a0 + a1, W = w0 + w1, Z = z0 + z1;
        dep[k] = W > 0.f ? Z * rcp_approx(W) : 0.f;
        // alpha = 1 - exp(-A): a Taylor polynomial below A = 1/64 (relative error under 1e-9),
        // else from the hardware exp2 (absolute error under 3e-7).
        alp[k] = A < 0.015625f ? A * fmaf(A, fmaf(A, fmaf(A, -1.f / 24.f, 1.f / 6.f), -0.5f), 1.f)
                               : 1.f - ex2_approx(-A * kLog2e);
        wsum[k] = W;
        asum[k] = A;
      }
      const int64_t pix = V.pix_base + (int64_t)v * V.W + u0;
      store_pixels<PX>(depth + pix, dep, V.W - u0);
      store_pixels<PX>(alpha + pix, alp, V.W - u0);
      if (stats) {
        store_pixels<PX>(stats + pix, m, V.W - u0);
        store_pixels<PX>(stats + stats_stride + pix, wsum, V.W - u0);
        store_pixels<PX>(stats + 2 * stats_stride + pix, asum, V.W - u0);
      }
    }
    __syncthreads();  // sm.tile is rewritten next iteration
  }
}

template <int TW, int TH, int PX, int CH>
void launch_tiles(const ViewsArg& va, int64_t tile_begin, int64_t tile_end, uint32_t* counter,
                  const uint32_t* order, const uint64_t* keys, const GaussRec* recs,
                  const uint2* ranges, float nb2, float beta3, float* depth, float* alpha,
                  float* stats, int64_t stats_stride, Control* ctrl, cudaStream_t st) {
  constexpr int NT = BlendShape<TW, TH, PX, CH>::NT;
  constexpr auto kern = blend_fwd_kernel<TW, TH, PX, CH>;
  const int64_t grid = std::min<int64_t>(tile_end - tile_begin, resident_ctas<kern>(NT));
  kern<<<(unsigned)grid, NT, 0, st>>>(va, (uint32_t)tile_begin, (uint32_t)tile_end, counter,
                                      order, keys, recs, ranges, nb2, beta3, depth, alpha, stats,
                                      stats_stride, ctrl);
}

template <int TW, int TH, int PX>
void launch_chunk(int chunk, const ViewsArg& va, int64_t tile_begin, int64_t tile_end,
                  uint32_t* counter, const uint32_t* order, const uint64_t* keys,
                  const GaussRec* recs, const uint2* ranges, float nb2, float beta3, float* depth,
                  float* alpha, float* stats, int64_t stats_stride, Control* ctrl,
                  cudaStream_t st) {
  if (chunk == 8)
    launch_tiles<TW, TH, PX, 8>(va, tile_begin, tile_end, counter, order, keys, recs, ranges, nb2,
                                beta3, depth, alpha, stats, stats_stride, ctrl, st);
  else if (chunk == 16)
    launch_tiles<TW, TH, PX, 16>(va, tile_begin, tile_end, counter, order, keys, recs, ranges,
                                 nb2, beta3, depth, alpha, stats, stats_stride, ctrl, st);
  else
    launch_tiles<TW, TH, PX, 32>(va, tile_begin, tile_end, counter, order, keys, recs, ranges,
                                 nb2, beta3, depth, alpha, stats, stats_stride, ctrl, st);
}

}  // namespace

namespace {

void blend_dispatch(const ViewsArg& va, int tile_w, int tile_h, int px, int chunk,
                    int64_t tile_begin, int64_t tile_end, uint32_t* counter, const uint32_t* order,
                    const uint64_t* keys, const GaussRec* recs, const uint2* ranges, float beta2,
                    float beta3, float* depth, float* alpha, float* stats, int64_t stats_stride,
                    Control* ctrl, cudaStream_t st) {
  if (tile_end <= tile_begin) return;
  const float nb2 = -beta2 * kLog2e;
#define FE_BLEND(TW_, TH_, PX_)                                                                 \
  launch_chunk<TW_, TH_, PX_>(chunk, va, tile_begin, tile_end, counter, order, keys, recs, ranges, \
                              nb2, beta3, depth, alpha, stats, stats_stride, ctrl, st)
  if (tile_w == 8 && tile_h == 8) {
    if (px == 1) FE_BLEND(8, 8, 1); else FE_BLEND(8, 8, 2);
  } else if (tile_w == 32 && tile_h == 8) {
    if (px == 1) FE_BLEND(32, 8, 1); else if (px == 2) FE_BLEND(32, 8, 2); else FE_BLEND(32, 8, 4);
  } else {
    if (px == 1) FE_BLEND(16, 16, 1); else if (px == 2) FE_BLEND(16, 16, 2); else FE_BLEND(16, 16, 4);
  }
#undef FE_BLEND
}

}  // namespace

// Pixels per thread: px in {1, 2, 4} (8x8 tiles: 1, 2); 0 selects the default for the tile.
// Chunk: record pairs per shared-memory stage, 8, 16 or 32; 0 selects 32.
void launch_blend_fwd_band(const ViewsArg& va, int tile_w, int tile_h, int px, int chunk,
                           int64_t tile_begin, int64_t tile_end, uint32_t* counter,
                           const uint64_t* keys, const GaussRec* recs, const uint2* ranges,
                           float beta2, float beta3, float* depth, float* alpha, float* stats,
                           int64_t stats_stride, Control* ctrl, cudaStream_t st) {
  blend_dispatch(va, tile_w, tile_h, px, chunk, tile_begin, tile_end, counter, nullptr, keys, recs,
                 ranges, beta2, beta3, depth, alpha, stats, stats_stride, ctrl, st);
}

void launch_blend_fwd(const ViewsArg& va, int tile_w, int tile_h, int px, int chunk,
                      int64_t n_tiles, const uint32_t* order, const uint64_t* keys,
                      const GaussRec* recs, const uint2* ranges, float beta2, float beta3,
                      float* depth, float* alpha, float* stats, int64_t stats_stride,
                      Control* ctrl, cudaStream_t st) {
  blend_dispatch(va, tile_w, tile_h, px, chunk, 0, n_tiles, &ctrl->next_tile, order, keys, recs,
                 ranges, beta2, beta3, depth, alpha, stats, stats_stride, ctrl, st);
}

}  // namespace fe
