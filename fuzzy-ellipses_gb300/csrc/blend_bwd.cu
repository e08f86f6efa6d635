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
// Parallelisation is transposed with respect to the forward: one thread per (tile, Gaussian)
// key loops over the tile's pixels and accumulates the gradient of its 16 tile-polynomial
// coefficients in registers (no cross-thread reductions), maps them back through the tile
// re-expansion to record space and adds them to the record's accumulator. A per-record kernel
// then applies the chain rule of the preprocess (camera transform, cofactors, cross products)
// and accumulates d/dmeans, d/dprec (upper triangle only, as jax.grad through triu gives) and
// d/dlogw over the views of a scene.
#include "fe_kernels.cuh"

namespace fe {

namespace {

__global__ void pixel_prep_kernel(ViewsArg va, int64_t n_pix, const float* __restrict__ depth,
                                  const float* __restrict__ stats, int64_t stride,
                                  const float* __restrict__ gdepth,
                                  const float* __restrict__ galpha, float4* __restrict__ pix) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n_pix;
       p += (int64_t)gridDim.x * blockDim.x) {
    const float m = stats[p], W = stats[stride + p], A = stats[2 * stride + p];
    const float gD = gdepth ? gdepth[p] : 0.f;
    const float gA = galpha ? galpha[p] : 0.f;
    pix[p] = make_float4(depth[p], m, W > 0.f ? gD / W : 0.f, gA * expf(-A));
  }
}

__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b),
               "f"(c), "f"(d)
               : "memory");
}

template <int TW, int TH>
__global__ void __launch_bounds__(128) blend_bwd_kernel(
    ViewsArg va, const uint64_t* __restrict__ keys, const Control* __restrict__ ctrl,
    const TilePair* __restrict__ trec, const GaussRec* __restrict__ recs,
    const float4* __restrict__ pix, float nb2, float beta3, float beta2, RecGrad* __restrict__ rgrad) {
  const int64_t K = (int64_t)ctrl->num_keys;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < K;
       k += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t key = keys[k];
    const uint32_t tile = (uint32_t)(key >> 32);
    const uint32_t gid = (uint32_t)key;
    const int vi = find_view<&ViewDev::tile_base>(va, tile);
    const ViewDev& V = view_at(va, vi);
    if (V.flags & FE_VIEW_NO_GRAD) continue;
    const int lt = (int)(tile - V.tile_base);
    const int tx = lt % V.gx, ty = lt / V.gx;
    // Record k lives in slot k%2 of pair k/2 (field i at float offset 2*i + slot).
    const float* tf = reinterpret_cast<const float*>(trec + (k >> 1)) + (k & 1);
    const float V0 = tf[0], V1 = tf[2], V2 = tf[4], V3 = tf[6], V4 = tf[8], V5 = tf[10];
    const float P0 = tf[12], P1 = tf[14], P2 = tf[16];
    const float N0 = tf[18], N1 = tf[20], N2 = tf[22], N3 = tf[24], N4 = tf[26], N5 = tf[28];
    const float C = tf[30], cu = tf[32], cvv = tf[34];

    float gV[6] = {0, 0, 0, 0, 0, 0}, gP[3] = {0, 0, 0}, gN[6] = {0, 0, 0, 0, 0, 0}, gC = 0.f;
    const int xs = min(TW, V.W - tx * TW), ys = min(TH, V.H - ty * TH);
    for (int ly = 0; ly < ys; ++ly) {
      const float dv = ly - 0.5f * (TH - 1), dv2 = dv * dv;
      const float ev = dv - cvv, ev2 = ev * ev;
      const float4* prow = pix + V.pix_base + (int64_t)(ty * TH + ly) * V.W + tx * TW;
      for (int lx = 0; lx < xs; ++lx) {
        const float du = lx - 0.5f * (TW - 1), du2 = du * du, dudv = du * dv;
        const float eu = du - cu, eu2 = eu * eu, euev = eu * ev;
        const float4 px = prow[lx];  // depth, m, gD/W, gA(1-alpha)
        const float vsv = fmaf(V5, dv2, fmaf(V4, dudv, fmaf(V3, du2, fmaf(V2, dv, fmaf(V1, du, V0)))));
        const float psv = fmaf(P2, dv, fmaf(P1, du, P0));
        const float nq = fmaf(N5, ev2, fmaf(N4, euev, fmaf(N3, eu2, fmaf(N2, ev, fmaf(N1, eu, N0)))));
        const float qi = rcp_approx(vsv);
        const float z = psv * qi;
        const float s2 = fmaf(nq, qi, C);
        const float eA = ex2_approx(s2);
        const float l = fmaf(beta3, s2, nb2 * z);
        const float e = z > 0.f ? ex2_approx(l - px.y) : 0.f;
        const float we = px.z * e;                 // dL/ddepth * softmax weight
        const float zd = z - px.x;
        const float gs = fmaf(px.w, eA, beta3 * we * zd);       // dL/ds (natural)
        const float gz = we * fmaf(-beta2, zd, 1.f);            // dL/dz
        const float gs2 = gs * kLn2;                            // dL/ds2
        const float gnq = gs2 * qi;
        const float gq = fmaf(gs2, nq, gz * psv);
        const float gpsv = gz * qi;
        const float gvsv = -gq * qi * qi;
        gC += gs2;
        gV[0] += gvsv; gV[1] = fmaf(gvsv, du, gV[1]); gV[2] = fmaf(gvsv, dv, gV[2]);
        gV[3] = fmaf(gvsv, du2, gV[3]); gV[4] = fmaf(gvsv, dudv, gV[4]); gV[5] = fmaf(gvsv, dv2, gV[5]);
        gP[0] += gpsv; gP[1] = fmaf(gpsv, du, gP[1]); gP[2] = fmaf(gpsv, dv, gP[2]);
        gN[0] += gnq; gN[1] = fmaf(gnq, eu, gN[1]); gN[2] = fmaf(gnq, ev, gN[2]);
        gN[3] = fmaf(gnq, eu2, gN[3]); gN[4] = fmaf(gnq, euev, gN[4]); gN[5] = fmaf(gnq, ev2, gN[5]);
      }
    }

    // Back through the tile re-expansion (binning.cu tile_record) to record space.
    const GaussRec g = recs[V.rec_base + gid];
    const float tcx = tx * TW + 0.5f * (TW - 1), tcy = ty * TH + 0.5f * (TH - 1);
    const float du = tcx - g.uc, dv = tcy - g.vc;
    // Same choice of expansion centre as the gather (binning.cu tile_record).
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

// Chain rule of the record builder (preprocess.cu build_camera_terms / write_record), in double.
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

    double U[9], R[9];
    for (int k = 0; k < 9; ++k) U[k] = (k == 3 || k == 6 || k == 7) ? 0.0 : prec[9 * gi + k];
    quat_to_rot<double>(quat + 4 * V.pose, R);
    const double t[3] = {trans[3 * V.pose], trans[3 * V.pose + 1], trans[3 * V.pose + 2]};
    const V3<double> p = v3(means[3 * gi] - t[0], means[3 * gi + 1] - t[1], means[3 * gi + 2] - t[2]);
    const V3<double> pc = matvec(R, p);
    double M[9], Y[9];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double s = 0.0;
        for (int k = 0; k <= a; ++k) s += U[k * 3 + a] * R[b * 3 + k];
        M[a * 3 + b] = s;
      }
    cofactor3(M, Y);
    const double fx = V.fx, fy = V.fy;
    const V3<double> r0 = v3(((double)recs[i].uc - V.cx) / fx, ((double)recs[i].vc - V.cy) / fy, 1.0);
    const V3<double> c0 = cross(r0, pc);
    const V3<double> cxv = v3(0.0, -pc.z / fx, pc.y / fx);
    const V3<double> cyv = v3(pc.z / fy, 0.0, -pc.x / fy);

    const V3<double> ga0 = v3<double>(rg.a0[0], rg.a0[1], rg.a0[2]);
    const V3<double> ga1 = v3<double>(rg.a1[0], rg.a1[1], rg.a1[2]);
    const V3<double> ga2 = v3<double>(rg.a2[0], rg.a2[1], rg.a2[2]);
    const V3<double> gb = v3<double>(rg.b[0], rg.b[1], rg.b[2]);
    const V3<double> gy0 = v3<double>(rg.y0[0], rg.y0[1], rg.y0[2]);
    const V3<double> gy1 = v3<double>(rg.y1[0], rg.y1[1], rg.y1[2]);
    const V3<double> gy2 = v3<double>(rg.y2[0], rg.y2[1], rg.y2[2]);

    // a0 = M r0, a1 = M e_x / fx, a2 = M e_y / fy, b = M pc.
    double gM[9];
    const double ga0a[3] = {ga0.x, ga0.y, ga0.z}, ga1a[3] = {ga1.x, ga1.y, ga1.z};
    const double ga2a[3] = {ga2.x, ga2.y, ga2.z}, gba[3] = {gb.x, gb.y, gb.z};
    const double r0a[3] = {r0.x, r0.y, r0.z}, pca[3] = {pc.x, pc.y, pc.z};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) gM[a * 3 + b] = ga0a[a] * r0a[b] + gba[a] * pca[b];
    for (int a = 0; a < 3; ++a) {
      gM[a * 3 + 0] += ga1a[a] / fx;
      gM[a * 3 + 1] += ga2a[a] / fy;
    }
    V3<double> gpc = matTvec(M, gb);
    // y0 = Y c0, y1 = Y cxv, y2 = Y cyv.
    double gY[9];
    const double gy0a[3] = {gy0.x, gy0.y, gy0.z}, gy1a[3] = {gy1.x, gy1.y, gy1.z};
    const double gy2a[3] = {gy2.x, gy2.y, gy2.z};
    const double c0a[3] = {c0.x, c0.y, c0.z}, cxa[3] = {cxv.x, cxv.y, cxv.z};
    const double cya[3] = {cyv.x, cyv.y, cyv.z};
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        gY[a * 3 + b] = gy0a[a] * c0a[b] + gy1a[a] * cxa[b] + gy2a[a] * cya[b];
    const V3<double> gc0 = matTvec(Y, gy0), gcx = matTvec(Y, gy1), gcy = matTvec(Y, gy2);
    gpc = gpc + cross(gc0, r0);                  // c0 = r0 x pc
    gpc.y += gcx.z / fx;                         // cxv = (0, -pc.z, pc.y) / fx
    gpc.z -= gcx.y / fx;
    gpc.x -= gcy.z / fy;                         // cyv = (pc.z, 0, -pc.x) / fy
    gpc.z += gcy.x / fy;
    // Y = cof(M).
    const double* m = M;
    const double* gc = gY;
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
        double s = 0.0;
        for (int b = 0; b < 3; ++b) s += gM[a * 3 + b] * R[b * 3 + k];
        atomicAdd(&gprec[9 * gi + k * 3 + a], (float)s);
      }
    // pc = R (m - t).
    const V3<double> gm = matTvec(R, gpc);
    atomicAdd(&gmeans[3 * gi + 0], (float)gm.x);
    atomicAdd(&gmeans[3 * gi + 1], (float)gm.y);
    atomicAdd(&gmeans[3 * gi + 2], (float)gm.z);
    atomicAdd(&glogw[gi], (float)((double)rg.w * kLog2eD));
  }
}

template <int TW, int TH>
void launch_bwd_tiles(const ViewsArg& va, const uint64_t* keys, const Control* ctrl,
                      int64_t capacity, const TilePair* trec, const GaussRec* recs,
                      const float4* pix, float beta2, float beta3, RecGrad* rgrad,
                      cudaStream_t st) {
  const int64_t want = (capacity + 127) / 128;
  const int blocks = (int)(want < 152 * 16 ? (want < 1 ? 1 : want) : 152 * 16);
  blend_bwd_kernel<TW, TH><<<blocks, 128, 0, st>>>(va, keys, ctrl, trec, recs, pix,
                                                   -beta2 * kLog2e, beta3, beta2, rgrad);
}

}  // namespace

void launch_pixel_prep(const ViewsArg& va, int64_t n_pix, const float* depth, const float* stats,
                       int64_t stats_stride, const float* grad_depth, const float* grad_alpha,
                       float4* pix, cudaStream_t st) {
  (void)va;
  if (n_pix <= 0) return;
  const int64_t want = (n_pix + 255) / 256;
  pixel_prep_kernel<<<(int)(want < 8192 ? want : 8192), 256, 0, st>>>(
      va, n_pix, depth, stats, stats_stride, grad_depth, grad_alpha, pix);
}

void launch_blend_bwd(const ViewsArg& va, int tile_w, int tile_h, const uint64_t* keys,
                      const Control* ctrl, int64_t capacity, const TilePair* trec,
                      const GaussRec* recs, const float4* pix, float beta2, float beta3,
                      RecGrad* rgrad, cudaStream_t st) {
  if (tile_w == 8 && tile_h == 8)
    launch_bwd_tiles<8, 8>(va, keys, ctrl, capacity, trec, recs, pix, beta2, beta3, rgrad, st);
  else if (tile_w == 32 && tile_h == 8)
    launch_bwd_tiles<32, 8>(va, keys, ctrl, capacity, trec, recs, pix, beta2, beta3, rgrad, st);
  else
    launch_bwd_tiles<16, 16>(va, keys, ctrl, capacity, trec, recs, pix, beta2, beta3, rgrad, st);
}

void launch_record_vjp(const ViewsArg& va, int64_t n_rec, const float* means, const float* prec,
                       const float* quat, const float* trans, const GaussRec* recs,
                       const RecGrad* rgrad, float* gmeans, float* gprec, float* glogw,
                       cudaStream_t st) {
  if (n_rec <= 0) return;
  const int64_t want = (n_rec + 127) / 128;
  record_vjp_kernel<<<(int)(want < 65535 ? want : 65535), 128, 0, st>>>(
      va, n_rec, means, prec, quat, trans, recs, rgrad, gmeans, gprec, glogw);
}

}  // namespace fe
