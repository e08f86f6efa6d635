// blend_bwd.cu -- hand-written backward of the fuzzy-metaball render.
//
// The reference has no backward kernel: it differentiates baseline/fm_render.py with jax.grad
// (shape_from_silhouette.ipynb cell 12). This backward recomputes every per-(pixel, Gaussian)
// term from the tile records and the per-pixel statistics saved by the forward (softmax max m,
// normaliser W, density sum A) instead of storing per-pair terms.
//
// Per pixel, with e = 2^(l-m) the unnormalised softmax weight and eA = 2^s2 the peak density:
//   dL/ds = dL/dalpha (1-alpha) eA + beta3 (dL/ddepth / W) e (z - depth)      (s natural log)
//   dL/dz = (dL/ddepth / W) e (1 - beta2 (z - depth))
// Parallelisation is transposed with respect to the forward: persistent warps take tiles from a
// device counter and stage the tile's per-pixel data in shared memory; each (tile, Gaussian) key
// gets one or more lanes that loop over the tile's pixels and accumulate the gradient of its 16
// tile-polynomial coefficients in registers (lanes sharing a key combine by shuffles), map them
// back through the tile re-expansion to record space and add them to the record's accumulator
// (vector reductions). A per-record kernel
// then applies the chain rule of the preprocess (camera transform, cofactors, cross products)
// and accumulates d/dmeans, d/dprec (upper triangle only, as jax.grad through triu gives) and
// d/dlogw over the views of a scene.
#include <algorithm>

#include "fe_kernels.cuh"
#include "fe_tilerec.cuh"

namespace fe {

namespace {

__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b),
               "f"(c), "f"(d)
               : "memory");
}

constexpr int kBwdWarps = 4;

// Per-warp shared-memory slice: the tile's per-pixel data as four planes (depth, -m for the
// softmax max m, dL/ddepth / W, dL/dalpha (1-alpha) ln 2), so that one 64-bit load gives the
// same field of two adjacent pixels for the packed arithmetic. Rows are padded to TW + 2 floats
// (8-byte aligned pairs; lanes of one key reading different rows of the same columns hit
// different banks).
template <int TW, int TH>
struct alignas(16) BwdSlice {
  static constexpr int ROW = TW + 2;
  static_assert((TH * ROW) % 2 == 0 && ROW % 2 == 0, "pairs must stay 8-byte aligned");
  float plane[4][TH * ROW];
};

// Persistent warps: each warp takes a tile from the device counter, stages the tile's pixel data
// in its shared-memory slice and processes the tile's keys in groups of up to 32. A group of n
// keys gets s = 32 / n lanes per key (s a power of two), which split the tile's rows; their
// partial sums are combined with shuffles. Pixels are evaluated in adjacent pairs with packed
// f32x2 arithmetic (one instruction for both pixels; rcp and ex2 per pixel).
template <int TW, int TH>
__global__ void __launch_bounds__(32 * kBwdWarps) blend_bwd_kernel(
    ViewsArg va, uint32_t n_tiles, const uint64_t* __restrict__ keys,
    const uint2* __restrict__ ranges, const GaussRec* __restrict__ recs,
    const float* __restrict__ depth, const float* __restrict__ stats, int64_t stride,
    const float* __restrict__ gdepth, const float* __restrict__ galpha, float nb2, float beta3,
    float beta2, RecGrad* __restrict__ rgrad, Control* ctrl) {
  using Slice = BwdSlice<TW, TH>;
  __shared__ Slice slices[kBwdWarps];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Slice& sl = slices[threadIdx.x >> 5];
  const f2_t B3 = f2_pack(beta3, beta3), NB2 = f2_pack(nb2, nb2);
  const f2_t NEGB2 = f2_pack(-beta2, -beta2), TWO = f2_pack(2.f, 2.f);
  const f2_t B3L = f2_pack(beta3 * kLn2, beta3 * kLn2), FOUR = f2_pack(4.f, 4.f);
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(&ctrl->next_tile, 1u);
    tile = __shfl_sync(full, tile, 0);
    if (tile >= n_tiles) break;
    const uint2 range = ranges[tile];
    if (range.y <= range.x) continue;
    const int vi = view_of_tile(va, tile);
    const ViewDev& V = view_at(va, vi);
    if (V.flags & FE_VIEW_NO_GRAD) continue;
    const int lt = (int)(tile - V.tile_base);
    const int tx = lt % V.gx, ty = lt / V.gx;
    const int xs = min(TW, V.W - tx * TW), ys = min(TH, V.H - ty * TH);

    __syncwarp();  // the previous tile's readers are done with the slice
    // The tile's per-pixel data from the forward's outputs and statistics and the cotangents:
    // depth, -m (softmax max), dL/ddepth / W, dL/dalpha (1 - alpha) ln 2, 1 - alpha = exp(-A).
    for (int q = lane; q < TW * TH; q += 32) {
      const int ly = q / TW, lx = q - ly * TW;
      if (lx < xs && ly < ys) {
        const int64_t pi = V.pix_base + (int64_t)(ty * TH + ly) * V.W + tx * TW + lx;
        const float m = stats[pi], W = stats[stride + pi], A = stats[2 * stride + pi];
        const float gD = gdepth ? gdepth[pi] : 0.f;
        const float gA = galpha ? galpha[pi] : 0.f;
        const int o = ly * Slice::ROW + lx;
        sl.plane[0][o] = depth[pi];
        sl.plane[1][o] = -m;
        sl.plane[2][o] = W > 0.f ? gD * rcp_approx(W) : 0.f;
        sl.plane[3][o] = gA * ex2_approx(-A * kLog2e) * kLn2;
      }
    }
    __syncwarp();

    for (uint32_t base = range.x, step = 0; base < range.y; base += step) {
      // Groups of 32 keys, then the rest; a rest of p + a keys (p a power of two of at least 8,
      // a <= p / 2) runs as p keys and then a, which gives each group more lanes per key: 20
      // keys take 8 + 2 row steps per lane as 16 + 4 instead of 16 as one group (one lane per
      // key). Larger remainders or smaller p would spend more on the extra group's record
      // builds and reductions than they save (16-view backward 0.305 -> 0.289 ms, 256-scene
      // 1.032 -> 0.969 ms).
      int cnt = (int)min(32u, range.y - base);
      if (cnt < 32) {
        const int p2 = 1 << (31 - __clz(cnt));
        if (p2 >= 8 && cnt - p2 <= p2 / 2) cnt = p2;
      }
      step = (uint32_t)cnt;
      int ls = 0;  // log2 of the lanes per key
      while ((cnt << (ls + 1)) <= 32) ++ls;
      const int s = 1 << ls;
      const int kl = lane >> ls, sub = lane & (s - 1);
      const bool active = kl < cnt;
      const uint64_t k = base + (uint32_t)(active ? kl : 0);

      // Coefficient gradients: gV over the basis [1, du, dv, du^2, du dv, dv^2] of vsv, gP over
      // [1, du, dv] of psv, gN over [1, eu, ev, eu^2, eu ev, ev^2] of nq (eu = du - cu,
      // ev = dv - cv). Within a row dv and ev are constant, so the row's polynomials are folded
      // to quadratics in du / eu. Each lane of a pixel pair visits the row's columns
      // du = D0 + 2 i (i = 0 .. n-1, D0 = (du0, du0 + 1)); instead of the moments sum h du^k
      // the pixel loop keeps running sums (S0 = sum h, C1 = sum of S0, C2 = sum of C1), which
      // give sum i h = n S0 - C1 and sum i^2 h = n^2 S0 - (2n+1) C1 + 2 C2. These are linear
      // with coefficients that are the same for every row of the tile, so the rows only add
      // them up (weighted by 1, dv, dv^2 or ev, ev^2) and the basis is formed once per key.
      // h = -dL/dvsv (S), dL/dpsv (Q), dL/dnq (T).
      const int n = (xs + 1) >> 1;  // pair steps per row; for odd xs lane b of the last is off
      f2_t aS0 = 0, aC1 = 0, aC2 = 0, bS0 = 0, bC1 = 0, dS0 = 0;
      f2_t aQ0 = 0, aQ1 = 0, bQ0 = 0;
      f2_t aT0 = 0, aT1 = 0, aT2 = 0, bT0 = 0, bT1 = 0, dT0 = 0;
      f2_t G = 0;
      float cu = 0.f;
      if (active) {
        // The key's tile record, built from its Gaussian record as the forward blend builds it.
        TileRec t;
        {
          const GaussRec g = recs[V.rec_base + (uint32_t)keys[k]];
          const float hw = 0.5f * (TW - 1), hh = 0.5f * (TH - 1);
          tile_record(g, tx * TW + hw - g.uc, ty * TH + hh - g.vc, hw, hh, t);
        }
        const float V0 = t.V[0], V1 = t.V[1], V2 = t.V[2], V3 = t.V[3], V4 = t.V[4], V5 = t.V[5];
        const float P0 = t.P[0], P1 = t.P[1], P2 = t.P[2];
        const float N0 = t.N[0], N1 = t.N[1], N2 = t.N[2], N3 = t.N[3], N4 = t.N[4], N5 = t.N[5];
        const float C = t.C, cvv = t.cv;
        cu = t.cu;
        const f2_t V3p = f2_pack(V3, V3), P1p = f2_pack(P1, P1), N3p = f2_pack(N3, N3);
        const f2_t Cp = f2_pack(C, C), CUp = f2_pack(cu, cu);
        for (int ly = sub; ly < ys; ly += s) {
          const float dv = ly - 0.5f * (TH - 1), dv2 = dv * dv;
          const float ev = dv - cvv, ev2 = ev * ev;
          const float rv0 = fmaf(V5, dv2, fmaf(V2, dv, V0)), rv1 = fmaf(V4, dv, V1);
          const float rp0 = fmaf(P2, dv, P0);
          const float rn0 = fmaf(N5, ev2, fmaf(N2, ev, N0)), rn1 = fmaf(N4, ev, N1);
          const f2_t RV0 = f2_pack(rv0, rv0), RV1 = f2_pack(rv1, rv1), RP0 = f2_pack(rp0, rp0);
          const f2_t RN0 = f2_pack(rn0, rn0), RN1 = f2_pack(rn1, rn1);
          f2_t S0 = 0, C1 = 0, C2 = 0, Q0 = 0, Q1 = 0, T0 = 0, T1 = 0, T2 = 0;
          const int o = ly * Slice::ROW;
          const f2_t* pd = reinterpret_cast<const f2_t*>(&sl.plane[0][o]);
          const f2_t* pm = reinterpret_cast<const f2_t*>(&sl.plane[1][o]);
          const f2_t* pz = reinterpret_cast<const f2_t*>(&sl.plane[2][o]);
          const f2_t* pa = reinterpret_cast<const f2_t*>(&sl.plane[3][o]);
          f2_t du = f2_pack(-0.5f * (TW - 1), 1.f - 0.5f * (TW - 1));
          // One pixel pair. With lane_b_off the pair's second pixel lies past the tile's last
          // column (its plane entries are stale): its four results are replaced by zeros.
          auto step = [&](int j, bool lane_b_off) {
            const f2_t D = pd[j], NM = pm[j], GDW = pz[j], GA = pa[j];
            const f2_t eu = sub2(du, CUp);
            const f2_t vsv = fma2(fma2(V3p, du, RV1), du, RV0);
            const f2_t psv = fma2(P1p, du, RP0);
            const f2_t nq = fma2(fma2(N3p, eu, RN1), eu, RN0);
            float va, vb;
            f2_unpack(vsv, va, vb);
            const f2_t qi = f2_pack(rcp_approx(va), rcp_approx(vb));
            const f2_t z = mul2(psv, qi);
            const f2_t s2 = fma2(nq, qi, Cp);
            float sa, sb;
            f2_unpack(s2, sa, sb);
            const f2_t eA = f2_pack(ex2_approx(sa), ex2_approx(sb));
            const f2_t lm = fma2(B3, s2, fma2(NB2, z, NM));          // logit - m
            float la, lb, za, zb;
            f2_unpack(lm, la, lb);
            f2_unpack(z, za, zb);
            const f2_t e = f2_pack(za > 0.f ? ex2_approx(la) : 0.f, zb > 0.f ? ex2_approx(lb) : 0.f);
            const f2_t we = mul2(GDW, e);                            // dL/ddepth * weight
            const f2_t u = mul2(we, sub2(z, D));
            f2_t gs2 = fma2(B3L, u, mul2(GA, eA));                   // dL/ds2
            const f2_t gz = fma2(NEGB2, u, we);                      // dL/dz
            f2_t gnq = mul2(gs2, qi);
            const f2_t gq = fma2(gs2, nq, mul2(gz, psv));
            f2_t gpsv = mul2(gz, qi);
            f2_t h = mul2(mul2(gq, qi), qi);                         // -dL/dvsv
            if (lane_b_off) {
              float a0, b0;
              f2_unpack(gs2, a0, b0); gs2 = f2_pack(a0, 0.f);
              f2_unpack(gnq, a0, b0); gnq = f2_pack(a0, 0.f);
              f2_unpack(gpsv, a0, b0); gpsv = f2_pack(a0, 0.f);
              f2_unpack(h, a0, b0); h = f2_pack(a0, 0.f);
            }
            G = add2(G, gs2);
            S0 = add2(S0, h); C1 = add2(C1, S0); C2 = add2(C2, C1);
            Q0 = add2(Q0, gpsv); Q1 = add2(Q1, Q0);
            T0 = add2(T0, gnq); T1 = add2(T1, T0); T2 = add2(T2, T1);
          };
          // A full-width row is unrolled completely: its pixel pairs are independent but for the
          // running sums, so the scheduler can interleave them (the loop dominates the kernel).
          if (xs == TW) {
#pragma unroll
            for (int j = 0; j < TW / 2; ++j, du = add2(du, TWO)) step(j, false);
          } else {
            const int pairs = xs >> 1;
#pragma unroll 2
            for (int j = 0; j < pairs; ++j, du = add2(du, TWO)) step(j, false);
            if (xs & 1) step(pairs, true);
          }
          const f2_t DV = f2_pack(dv, dv), DV2 = f2_pack(dv2, dv2);
          const f2_t EV = f2_pack(ev, ev), EV2 = f2_pack(ev2, ev2);
          aS0 = add2(aS0, S0); aC1 = add2(aC1, C1); aC2 = add2(aC2, C2);
          bS0 = fma2(DV, S0, bS0); bC1 = fma2(DV, C1, bC1); dS0 = fma2(DV2, S0, dS0);
          aQ0 = add2(aQ0, Q0); aQ1 = add2(aQ1, Q1); bQ0 = fma2(DV, Q0, bQ0);
          aT0 = add2(aT0, T0); aT1 = add2(aT1, T1); aT2 = add2(aT2, T2);
          bT0 = fma2(EV, T0, bT0); bT1 = fma2(EV, T1, bT1); dT0 = fma2(EV2, T0, dT0);
        }
      }
      // The basis, per lane of the pair, then summed over the pair: with I1 = sum i x and
      // I2 = sum i^2 x, sum x du = D0 x + 2 I1 and sum x du^2 = D0^2 x + 4 D0 I1 + 4 I2
      // (E0 = D0 - cu in place of D0 for eu).
      float gV[6], gP[3], gN[6], gC;
      {
        const float nf = (float)n;
        const f2_t NF = f2_pack(nf, nf), NN = f2_pack(nf * nf, nf * nf);
        const f2_t N21 = f2_pack(2.f * nf + 1.f, 2.f * nf + 1.f);
        const f2_t D0 = f2_pack(-0.5f * (TW - 1), 1.f - 0.5f * (TW - 1));
        const f2_t E0 = sub2(D0, f2_pack(cu, cu));
        auto first = [&](f2_t X0, f2_t X1) { return sub2(mul2(NF, X0), X1); };
        auto second = [&](f2_t X0, f2_t X1, f2_t X2) {
          return fma2(TWO, X2, fma2(NN, X0, mul2(N21, sub2(f2_pack(0.f, 0.f), X1))));
        };
        auto lin = [&](f2_t O, f2_t X0, f2_t I1) { return fma2(O, X0, mul2(TWO, I1)); };
        auto quad = [&](f2_t O, f2_t X0, f2_t I1, f2_t I2) {
          return fma2(O, fma2(O, X0, mul2(FOUR, I1)), mul2(FOUR, I2));
        };
        auto hsum = [](f2_t x) {
          float a, b;
          f2_unpack(x, a, b);
          return a + b;
        };
        const f2_t iS = first(aS0, aC1), iiS = second(aS0, aC1, aC2);
        gV[0] = -hsum(aS0);
        gV[1] = -hsum(lin(D0, aS0, iS));
        gV[2] = -hsum(bS0);
        gV[3] = -hsum(quad(D0, aS0, iS, iiS));
        gV[4] = -hsum(lin(D0, bS0, first(bS0, bC1)));
        gV[5] = -hsum(dS0);
        gP[0] = hsum(aQ0);
        gP[1] = hsum(lin(D0, aQ0, first(aQ0, aQ1)));
        gP[2] = hsum(bQ0);
        const f2_t iT = first(aT0, aT1), iiT = second(aT0, aT1, aT2);
        gN[0] = hsum(aT0);
        gN[1] = hsum(lin(E0, aT0, iT));
        gN[2] = hsum(bT0);
        gN[3] = hsum(quad(E0, aT0, iT, iiT));
        gN[4] = hsum(lin(E0, bT0, first(bT0, bT1)));
        gN[5] = hsum(dT0);
        gC = hsum(G);
      }
      // Combine the s lanes of each key (all lanes take part; idle lanes hold zeros).
      for (int o = 1; o < s; o <<= 1) {
#pragma unroll
        for (int i = 0; i < 6; ++i) gV[i] += __shfl_xor_sync(full, gV[i], o);
#pragma unroll
        for (int i = 0; i < 3; ++i) gP[i] += __shfl_xor_sync(full, gP[i], o);
#pragma unroll
        for (int i = 0; i < 6; ++i) gN[i] += __shfl_xor_sync(full, gN[i], o);
        gC += __shfl_xor_sync(full, gC, o);
      }
      if (!active || sub != 0) continue;
      const uint32_t gid = (uint32_t)keys[k];

      // Back through the tile re-expansion (fe_tilerec.cuh tile_record) to record space.
      const GaussRec g = recs[V.rec_base + gid];
      const float tcx = tx * TW + 0.5f * (TW - 1), tcy = ty * TH + 0.5f * (TH - 1);
      const float du = tcx - g.uc, dv = tcy - g.vc;
      // Same choice of expansion centre as tile_record.
      const bool near = fabsf(du) <= kNearCentre && fabsf(dv) <= kNearCentre;
      const float kn = -0.5f * kLog2e;
      float a0[3], y0[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a0[c] = fmaf(dv, g.a2[c], fmaf(du, g.a1[c], g.a0[c]));
        y0[c] = near ? g.y0[c] : fmaf(dv, g.y2[c], fmaf(du, g.y1[c], g.y0[c]));
      }
      float ga0[3], ga1[3], ga2[3], gb[3], gy0[3], gy1[3], gy2[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ga0[c] = 2.f * (gV[0] * a0[c] + gV[1] * g.a1[c] + gV[2] * g.a2[c]) + gP[0] * g.b[c];
        ga1[c] = 2.f * (gV[1] * a0[c] + gV[3] * g.a1[c] + gV[4] * g.a2[c]) + gP[1] * g.b[c];
        ga2[c] = 2.f * (gV[2] * a0[c] + gV[4] * g.a1[c] + gV[5] * g.a2[c]) + gP[2] * g.b[c];
        gb[c] = gP[0] * a0[c] + gP[1] * g.a1[c] + gP[2] * g.a2[c];
        gy0[c] = 2.f * kn * (gN[0] * y0[c] + gN[1] * g.y1[c] + gN[2] * g.y2[c]);
        gy1[c] = 2.f * kn * (gN[1] * y0[c] + gN[3] * g.y1[c] + gN[4] * g.y2[c]);
        gy2[c] = 2.f * kn * (gN[2] * y0[c] + gN[4] * g.y1[c] + gN[5] * g.y2[c]);
        ga1[c] = fmaf(du, ga0[c], ga1[c]);
        ga2[c] = fmaf(dv, ga0[c], ga2[c]);
        if (!near) {
          gy1[c] = fmaf(du, gy0[c], gy1[c]);
          gy2[c] = fmaf(dv, gy0[c], gy2[c]);
        }
      }
      float* dst = reinterpret_cast<float*>(rgrad + (V.rec_base + gid));
      red_add_v4(dst + 0, ga0[0], ga0[1], ga0[2], ga1[0]);
      red_add_v4(dst + 4, ga1[1], ga1[2], ga2[0], ga2[1]);
      red_add_v4(dst + 8, ga2[2], gb[0], gb[1], gb[2]);
      red_add_v4(dst + 12, gy0[0], gy0[1], gy0[2], gy1[0]);
      red_add_v4(dst + 16, gy1[1], gy1[2], gy2[0], gy2[1]);
      red_add_v4(dst + 20, gy2[2], gC, 0.f, 0.f);
    }
  }
}

// Chain rule of the record builder (preprocess.cu build_camera_terms / write_record), in T:
// float, the precision of the preprocess it differentiates (in double the kernel is FP64-bound
// and adds 4% to a 16-view backward; both pass the float64 and finite-difference gradient tests).
template <typename T>
__global__ void record_vjp_kernel(ViewsArg va, int64_t n_rec, const float* __restrict__ means,
                                  const float* __restrict__ prec, const float* __restrict__ quat,
                                  const float* __restrict__ trans, const GaussRec* __restrict__ recs,
                                  const RecGrad* __restrict__ rgrad, float* __restrict__ gmeans,
                                  float* __restrict__ gprec, float* __restrict__ glogw) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_rec;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int vi = find_view<&ViewDev::rec_base>(va, i);
    const ViewDev& V = view_at(va, vi);
    if (V.flags & FE_VIEW_NO_GRAD) continue;
    const int64_t gi = V.gauss_base + (i - V.rec_base);
    const RecGrad rg = rgrad[i];

    T U[9], R[9];
    for (int k = 0; k < 9; ++k) U[k] = (k == 3 || k == 6 || k == 7) ? T(0) : (T)prec[9 * gi + k];
    quat_to_rot<T>(quat + 4 * V.pose, R);
    const T t[3] = {trans[3 * V.pose], trans[3 * V.pose + 1], trans[3 * V.pose + 2]};
    const V3<T> p = v3<T>(means[3 * gi] - t[0], means[3 * gi + 1] - t[1], means[3 * gi + 2] - t[2]);
    const V3<T> pc = matvec(R, p);
    T M[9], Y[9];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        T s = T(0);
        for (int k = 0; k <= a; ++k) s += U[k * 3 + a] * R[b * 3 + k];
        M[a * 3 + b] = s;
      }
    cofactor3(M, Y);
    const T fx = V.fx, fy = V.fy;
    const V3<T> r0 = v3<T>(((T)recs[i].uc - V.cx) / fx, ((T)recs[i].vc - V.cy) / fy, T(1));
    const V3<T> c0 = cross(r0, pc);
    const V3<T> cxv = v3<T>(T(0), -pc.z / fx, pc.y / fx);
    const V3<T> cyv = v3<T>(pc.z / fy, T(0), -pc.x / fy);

    const V3<T> ga0 = v3<T>(rg.a0[0], rg.a0[1], rg.a0[2]);
    const V3<T> ga1 = v3<T>(rg.a1[0], rg.a1[1], rg.a1[2]);
    const V3<T> ga2 = v3<T>(rg.a2[0], rg.a2[1], rg.a2[2]);
    const V3<T> gb = v3<T>(rg.b[0], rg.b[1], rg.b[2]);
    const V3<T> gy0 = v3<T>(rg.y0[0], rg.y0[1], rg.y0[2]);
    const V3<T> gy1 = v3<T>(rg.y1[0], rg.y1[1], rg.y1[2]);
    const V3<T> gy2 = v3<T>(rg.y2[0], rg.y2[1], rg.y2[2]);

    // a0 = M r0, a1 = M e_x / fx, a2 = M e_y / fy, b = M pc.
    T gM[9];
    const T ga0a[3] = {ga0.x, ga0.y, ga0.z}, ga1a[3] = {ga1.x, ga1.y, ga1.z};
    const T ga2a[3] = {ga2.x, ga2.y, ga2.z}, gba[3] = {gb.x, gb.y, gb.z};
    const T r0a[3] = {r0.x, r0.y, r0.z}, pca[3] = {pc.x, pc.y, pc.z};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) gM[a * 3 + b] = ga0a[a] * r0a[b] + gba[a] * pca[b];
    for (int a = 0; a < 3; ++a) {
      gM[a * 3 + 0] += ga1a[a] / fx;
      gM[a * 3 + 1] += ga2a[a] / fy;
    }
    V3<T> gpc = matTvec(M, gb);
    // y0 = Y c0, y1 = Y cxv, y2 = Y cyv.
    T gY[9];
    const T gy0a[3] = {gy0.x, gy0.y, gy0.z}, gy1a[3] = {gy1.x, gy1.y, gy1.z};
    const T gy2a[3] = {gy2.x, gy2.y, gy2.z};
    const T c0a[3] = {c0.x, c0.y, c0.z}, cxa[3] = {cxv.x, cxv.y, cxv.z};
    const T cya[3] = {cyv.x, cyv.y, cyv.z};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        gY[a * 3 + b] = gy0a[a] * c0a[b] + gy1a[a] * cxa[b] + gy2a[a] * cya[b];
    const V3<T> gc0 = matTvec(Y, gy0), gcx = matTvec(Y, gy1), gcy = matTvec(Y, gy2);
    gpc = gpc + cross(gc0, r0);                  // c0 = r0 x pc
    gpc.y += gcx.z / fx;                         // cxv = (0, -pc.z, pc.y) / fx
    gpc.z -= gcx.y / fx;
    gpc.x -= gcy.z / fy;                         // cyv = (pc.z, 0, -pc.x) / fy
    gpc.z += gcy.x / fy;
    // Y = cof(M).
    const T* m = M;
    const T* gc = gY;
    gM[4] += gc[0] * m[8]; gM[8] += gc[0] * m[4]; gM[5] -= gc[0] * m[7]; gM[7] -= gc[0] * m[5];
    gM[5] += gc[1] * m[6]; gM[6] += gc[1] * m[5]; gM[3] -= gc[1] * m[8]; gM[8] -= gc[1] * m[3];
    gM[3] += gc[2] * m[7]; gM[7] += gc[2] * m[3]; gM[4] -= gc[2] * m[6]; gM[6] -= gc[2] * m[4];
    gM[2] += gc[3] * m[7]; gM[7] += gc[3] * m[2]; gM[1] -= gc[3] * m[8]; gM[8] -= gc[3] * m[1];
    gM[0] += gc[4] * m[8]; gM[8] += gc[4] * m[0]; gM[2] -= gc[4] * m[6]; gM[6] -= gc[4] * m[2];
    gM[1] += gc[5] * m[6]; gM[6] += gc[5] * m[1]; gM[0] -= gc[5] * m[7]; gM[7] -= gc[5] * m[0];
    gM[1] += gc[6] * m[5]; gM[5] += gc[6] * m[1]; gM[2] -= gc[6] * m[4]; gM[4] -= gc[6] * m[2];
    gM[2] += gc[7] * m[3]; gM[3] += gc[7] * m[2]; gM[0] -= gc[7] * m[5]; gM[5] -= gc[7] * m[0];
    gM[0] += gc[8] * m[4]; gM[4] += gc[8] * m[0]; gM[1] -= gc[8] * m[3]; gM[3] -= gc[8] * m[1];
    // M[a][b] = sum_k U[k][a] R[b][k]  ->  dL/dU[k][a] = sum_b gM[a][b] R[b][k]  (k <= a).
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k <= a; ++k) {
        T s = T(0);
        for (int b = 0; b < 3; ++b) s += gM[a * 3 + b] * R[b * 3 + k];
        atomicAdd(&gprec[9 * gi + k * 3 + a], (float)s);
      }
    // pc = R (m - t).
    const V3<T> gm = matTvec(R, gpc);
    atomicAdd(&gmeans[3 * gi + 0], (float)gm.x);
    atomicAdd(&gmeans[3 * gi + 1], (float)gm.y);
    atomicAdd(&gmeans[3 * gi + 2], (float)gm.z);
    atomicAdd(&glogw[gi], rg.w * kLog2e);
  }
}

template <int TW, int TH>
void launch_bwd_tiles(const ViewsArg& va, int64_t n_tiles, const uint64_t* keys,
                      const uint2* ranges, const GaussRec* recs, const float* depth,
                      const float* stats, int64_t stride, const float* gdepth,
                      const float* galpha, float beta2, float beta3, RecGrad* rgrad,
                      Control* ctrl, cudaStream_t st) {
  constexpr auto kern = blend_bwd_kernel<TW, TH>;
  const int resident = resident_ctas<kern>(32 * kBwdWarps);
  const int64_t grid =
      std::max<int64_t>(1, std::min<int64_t>((n_tiles + kBwdWarps - 1) / kBwdWarps, resident));
  kern<<<(unsigned)grid, 32 * kBwdWarps, 0, st>>>(va, (uint32_t)n_tiles, keys, ranges, recs, depth,
                                                  stats, stride, gdepth, galpha, -beta2 * kLog2e,
                                                  beta3, beta2, rgrad, ctrl);
}

}  // namespace


void launch_blend_bwd(const ViewsArg& va, int tile_w, int tile_h, int64_t n_tiles,
                      const uint64_t* keys, const uint2* ranges, const GaussRec* recs,
                      const float* depth, const float* stats, int64_t stats_stride,
                      const float* grad_depth, const float* grad_alpha, float beta2, float beta3,
                      RecGrad* rgrad, Control* ctrl, cudaStream_t st) {
  if (n_tiles <= 0) return;
#define FE_BWD(TW_, TH_)                                                                       \
  launch_bwd_tiles<TW_, TH_>(va, n_tiles, keys, ranges, recs, depth, stats, stats_stride,     \
                             grad_depth, grad_alpha, beta2, beta3, rgrad, ctrl, st)
  if (tile_w == 8 && tile_h == 8)
    FE_BWD(8, 8);
  else if (tile_w == 32 && tile_h == 8)
    FE_BWD(32, 8);
  else
    FE_BWD(16, 16);
#undef FE_BWD
}

void launch_record_vjp(const ViewsArg& va, int64_t n_rec, const float* means, const float* prec,
                       const float* quat, const float* trans, const GaussRec* recs,
                       const RecGrad* rgrad, float* gmeans, float* gprec, float* glogw,
                       cudaStream_t st) {
  if (n_rec <= 0) return;
  const int64_t want = (n_rec + 127) / 128;
  record_vjp_kernel<float><<<(int)(want < 65535 ? want : 65535), 128, 0, st>>>(
      va, n_rec, means, prec, quat, trans, recs, rgrad, gmeans, gprec, glogw);
}

}  // namespace fe
