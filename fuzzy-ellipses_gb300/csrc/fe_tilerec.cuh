// fe_tilerec.cuh -- a key's tile record: its Gaussian's ray-invariant terms re-expanded around
// the centre of the key's tile (shared by the record gather and the forward blend).
#pragma once

#include "fe_common.cuh"

namespace fe {

// (du, dv): offset of the tile centre from the record's centre (uc, vc), in pixels. The
// Mahalanobis polynomial is expanded at the record's centre when that lies within kNearCentre
// pixels of the tile centre (there it vanishes, up to the rounding of the centre), otherwise at
// the tile centre (where it is large across the whole tile).
__device__ __forceinline__ void tile_record(const GaussRec& g, float du, float dv, float half_w,
                                            float half_h, TileRec& t) {
  float a0[3], y0[3];
  const bool near = fabsf(du) <= kNearCentre && fabsf(dv) <= kNearCentre;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a0[k] = fmaf(dv, g.a2[k], fmaf(du, g.a1[k], g.a0[k]));
    y0[k] = near ? g.y0[k] : fmaf(dv, g.y2[k], fmaf(du, g.y1[k], g.y0[k]));
  }
  auto d3 = [](const float* a, const float* b) { return fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0])); };
  t.V[0] = d3(a0, a0);
  t.V[1] = 2.f * d3(a0, g.a1);
  t.V[2] = 2.f * d3(a0, g.a2);
  t.V[3] = d3(g.a1, g.a1);
  t.V[4] = 2.f * d3(g.a1, g.a2);
  t.V[5] = d3(g.a2, g.a2);
  t.P[0] = d3(a0, g.b);
  t.P[1] = d3(g.a1, g.b);
  t.P[2] = d3(g.a2, g.b);
  const float kn = -0.5f * kLog2e;
  t.N[0] = kn * d3(y0, y0);
  t.N[1] = 2.f * kn * d3(y0, g.y1);
  t.N[2] = 2.f * kn * d3(y0, g.y2);
  t.N[3] = kn * d3(g.y1, g.y1);
  t.N[4] = 2.f * kn * d3(g.y1, g.y2);
  t.N[5] = kn * d3(g.y2, g.y2);
  t.C = g.c2;
  t.cu = near ? -du : 0.f;
  t.cv = near ? -dv : 0.f;
  // psv is affine in the pixel offset: its minimum over the tile is at a corner. Require a
  // relative margin so float32 evaluation cannot flip the sign at any pixel.
  const float span = fabsf(t.P[1]) * half_w + fabsf(t.P[2]) * half_h;
  t.front = (t.P[0] - span > 1e-5f * (fabsf(t.P[0]) + span)) ? 1.f : 0.f;
  t.pad = 0.f;
}

__device__ __forceinline__ void null_tile_record(TileRec& t) {
  float* f = reinterpret_cast<float*>(&t);
#pragma unroll
  for (int i = 0; i < kRecFields; ++i) f[i] = 0.f;
  t.V[0] = 1.f;
  t.C = -INFINITY;
  t.front = 1.f;
}

}  // namespace fe
