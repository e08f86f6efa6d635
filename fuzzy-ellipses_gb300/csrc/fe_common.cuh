// fe_common.cuh -- types, constants and inline-PTX helpers shared by the renderer's kernels.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/fuzzy_ellipses.h"

namespace fe {

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;
constexpr double kLog2eD = 1.4426950408889634;

// Default FE_CULL_EPS density cut-off: a Gaussian whose peak density along a pixel ray is below
// this contributes less than it to that pixel's density sum.
constexpr float kDefaultCullEps = 1e-7f;

// Upper bound on one bounded device wait (globaltimer nanoseconds).
constexpr unsigned long long kWaitLimitNs = 4000000000ull;

// ------------------------------------------------------------------------------------------
// Data layout in HBM
// ------------------------------------------------------------------------------------------

// Per-render (view) table entry, device resident. A batch of renders concatenates:
//   records  (one per (Gaussian, view) pair)   at rec_base
//   tiles    (gx*gy per view)                  at tile_base
//   pixels   (H*W per view)                    at pix_base
struct ViewDev {
  float fx, fy, cx, cy;
  int32_t H, W;
  int32_t gx, gy;         // tiles per row / column
  int32_t n;              // Gaussians of the scene
  int32_t pose;           // index into the pose arrays (quat[4*pose], trans[3*pose])
  uint32_t flags;         // FE_VIEW_* bits
  uint32_t pad;
  int64_t gauss_base;     // first Gaussian of the scene in the input arrays
  int64_t rec_base;       // first record of this view
  int64_t tile_base;      // first global tile id of this view
  int64_t pix_base;       // first output pixel of this view
};

// Ray-invariant terms of one (Gaussian, view) pair, in pixel coordinates around an expansion
// centre (uc, vc). With du = u-uc, dv = v-vc:
//   a(du,dv) = a0 + du*a1 + dv*a2 = L^T (world ray)        -> vsv = |a|^2, psv = a.b
//   y(du,dv) = y0 + du*y1 + dv*y2 = cof(M) (ray x p_cam)   -> |y|^2 = vsv*|b|^2 - psv^2
// so the peak parameter is z = psv/vsv and the Mahalanobis distance of the peak is
// d0 = |y|^2/vsv with no cancellation (Lagrange's identity).
struct __align__(16) GaussRec {
  float a0[3], a1[3], a2[3], b[3];
  float y0[3], y1[3], y2[3];
  float uc, vc;
  float c2;               // logw * log2(e)
};
static_assert(sizeof(GaussRec) == 96, "GaussRec layout");

// Tile-local polynomial form of a record, built per key by the kernels that evaluate it (the
// forward blend stores it pair-interleaved in shared memory, see TilePair; the backward keeps it
// in registers).
// With (du,dv) the pixel offset from the tile centre and (eu,ev) = (du-cu, dv-cv) the offset from
// the expansion centre (cu,cv) of the Mahalanobis term:
//   vsv = V0 + V1 du + V2 dv + V3 du^2 + V4 du dv + V5 dv^2
//   psv = P0 + P1 du + P2 dv
//   nq  = N0 + N1 eu + N2 ev + N3 eu^2 + N4 eu ev + N5 ev^2, scaled by -log2(e)/2
//   s2  = C + nq/vsv  (log2 of the peak density),  z = psv/vsv
// nq vanishes at the Gaussian's projected centre; expanding it there (whenever that centre is
// near the tile) keeps float32 evaluation free of cancellation for Gaussians of sub-pixel size.
struct __align__(16) TileRec {
  float V[6];
  float P[3];
  float N[6];
  float C;
  float cu, cv;
  float front;  // 1 when psv > 0 over the whole tile (no z <= 0 masking needed), else 0
  float pad;
};
static_assert(sizeof(TileRec) == 80, "TileRec layout");

// Keys 2p and 2p+1 of the sorted key list share one TilePair: field i of record 2p is f[i].x and
// of record 2p+1 is f[i].y, so one 16-byte shared-memory load yields two packed f32x2 operands.
// Field order: V0..V5, P0..P2, N0..N5, C, cu, cv, front, pad.
constexpr int kRecFields = 20;
struct __align__(16) TilePair {
  float2 f[kRecFields];
};
static_assert(sizeof(TilePair) == 160, "TilePair layout");

// The Mahalanobis polynomial of a tile record is expanded at the record's centre when that lies
// within this many pixels of the tile centre (in both directions), else at the tile centre.
constexpr float kNearCentre = 64.f;

// Record-space gradient accumulator of one (Gaussian, view) pair: d/d{a0,a1,a2,b,y0,y1,y2,logw}.
struct __align__(16) RecGrad {
  float a0[3], a1[3], a2[3], b[3];
  float y0[3], y1[3], y2[3];
  float w;
  float pad[2];
};
static_assert(sizeof(RecGrad) == 96, "RecGrad layout");

// Screen rectangle of a record in tiles, [x0,x1) x [y0,y1).
struct __align__(8) TileRect {
  uint16_t x0, y0, x1, y1;
};

// Row form of a bounded record's footprint: the ellipse of pixels (u, v) whose rays pass within
// Mahalanobis distance k of the mean. At pixel row v it spans
//     u in [uc + c1 (v - vc) - sqrt(H), uc + c1 (v - vc) + sqrt(H)],  H = hc + h2 (v - vc)^2
// ((uc, vc): the ellipse's centre, hc its squared half-width there, h2 < 0); vl and vr are the
// rows of its leftmost and rightmost points. hc = NaN marks a footprint without this form
// (unbounded or degenerate): every row of its rectangle spans the rectangle's full width.
struct __align__(16) FootRows {
  float uc, vc, c1, hc, h2, vl, vr, pad;
};
static_assert(sizeof(FootRows) == 32, "FootRows layout");

// Tiles [x0, x1) of tile row `row` (tiles tw x th pixels) that the footprint reaches, within its
// rectangle r; x0 == x1 when it reaches none. The row's pixel rows are [row th, row th + th - 1].
// Over that band the footprint's leftmost pixel lies in the band row nearest vl (at vl itself
// when vl is inside the band: the rectangle's left edge), and likewise on the right, since the
// ellipse's left boundary is convex in v and its right boundary concave. The 0.1 px margin covers
// the float32 rounding of the bound; a pixel it could still leave out lies on the cut-off
// boundary, where the Gaussian's density is the cut-off density.
__device__ __forceinline__ void foot_row_tiles(const FootRows& f, const TileRect& r, int row,
                                               int tw, int th, int& x0, int& x1) {
  x0 = r.x0;
  x1 = r.x1;
  if (!(f.hc == f.hc)) return;
  const float va = (float)(row * th), vb = va + (float)(th - 1);
  const float itw = 1.f / (float)tw;  // exact: tile widths are powers of two
  constexpr float kMargin = 0.1f;
  auto half = [&](float v) {
    const float dv = v - f.vc;
    float h;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(h) : "f"(fmaxf(fmaf(f.h2 * dv, dv, f.hc), 0.f)));
    return h;
  };
  if (!(f.vl >= va && f.vl <= vb)) {
    const float v = f.vl < va ? va : vb;
    const float t = floorf((fmaf(f.c1, v - f.vc, f.uc) - half(v) - kMargin) * itw);
    if (t > (float)x0) x0 = t < (float)x1 ? (int)t : x1;
  }
  if (!(f.vr >= va && f.vr <= vb)) {
    const float v = f.vr < va ? va : vb;
    const float t = floorf((fmaf(f.c1, v - f.vc, f.uc) + half(v) + kMargin) * itw) + 1.f;
    if (t < (float)x1) x1 = t > (float)x0 ? (int)t : x0;
  }
}

// Tile work classes of the tile-major binning, heaviest first: class c < kTileClasses - 2 holds
// tiles with 2^(kTileClasses - 2 - c) <= keys < 2^(kTileClasses - 1 - c) (class 0 open-ended),
// class kTileClasses - 2 one key, class kTileClasses - 1 none.
constexpr int kTileClasses = 10;
__host__ __device__ __forceinline__ int tile_class(uint32_t keys) {
  if (keys == 0) return kTileClasses - 1;
  int b = 0;
  while ((keys >> (b + 1)) != 0u && b < 31) ++b;  // floor(log2(keys))
  const int c = (kTileClasses - 2) - b;
  return c < 0 ? 0 : c;
}

// Small device-side control block at the start of every arena.
struct Control {
  unsigned long long num_keys;  // keys produced by the last run (clamped to capacity)
  unsigned long long want_keys; // keys the run needed
  uint32_t error;               // FE_DEVERR_* bits
  uint32_t next_tile;           // work counter of the persistent blend
  uint32_t tile_class[kTileClasses];  // tiles per work class (tile-major binning)
};
static_assert(sizeof(Control) == 64, "Control layout");

// View lookup: the plain single-render path passes its one view by value (so it needs no
// upload and stays capturable); batches pass a device table.
struct ViewsArg {
  const ViewDev* table;
  int32_t count;
  ViewDev one;
  // With a table and the tile-major binning: the view of every tile, written by the emission,
  // so that kernels working per tile look it up with one load instead of a binary search over
  // the views (11 dependent loads for a thousand views). NULL otherwise.
  const uint32_t* tile_view;
};

__device__ __forceinline__ const ViewDev& view_at(const ViewsArg& va, int i) {
  return va.table ? va.table[i] : va.one;
}

// Index of the last entry of a sorted int64 field <= key (views sorted by that field).
template <int64_t ViewDev::*Field>
__device__ __forceinline__ int find_view(const ViewsArg& va, int64_t key) {
  if (va.table == nullptr) return 0;
  int lo = 0, hi = va.count - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (va.table[mid].*Field <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// View of a global tile id.
__device__ __forceinline__ int view_of_tile(const ViewsArg& va, int64_t tile) {
  if (va.table && va.tile_view) return (int)va.tile_view[tile];
  return find_view<&ViewDev::tile_base>(va, tile);
}

// ------------------------------------------------------------------------------------------
// Inline PTX
// ------------------------------------------------------------------------------------------

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Three-input maximum (one instruction on sm_100 and later; NaN inputs are ignored like fmaxf).
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float y;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(a), "f"(b), "f"(c));
  return y;
}

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Make mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arrive on `bar` and raise its expected transaction count by `bytes` (the bytes of TMA copies
// that complete on it; the count may run ahead of or behind the copies).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}

// 1-D TMA bulk copy global -> shared, completion counted on `bar` in bytes.
// Requires 16-byte aligned addresses and a byte count that is a multiple of 16.
__device__ __forceinline__ void tma_bulk_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes,
                                             uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Order this thread's generic-proxy shared-memory accesses before later async-proxy writes.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait on an mbarrier phase. Returns false (and never hangs) if the phase did not
// complete within kWaitLimitNs.
// try_wait that may suspend the thread in hardware for up to `hint_ns` while the phase is
// incomplete (it resumes as soon as the phase completes), so a waiting warp issues little.
__device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, uint32_t parity,
                                                      uint32_t hint_ns) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_timer_ns();
  // Each try suspends for at most 100 us, so the limit is overshot by at most that much.
  while (true) {
    if (mbar_try_wait_suspend(bar, parity, 100000u)) return true;
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  return mbar_wait_bounded(bar, parity, kWaitLimitNs);
}

// Packed float32 pairs (Blackwell add/sub/mul/fma .f32x2): one instruction for two lanes of work.
typedef unsigned long long f2_t;

__device__ __forceinline__ f2_t f2_pack(float lo, float hi) {
  f2_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2_t fma2(f2_t a, f2_t b, f2_t c) {
  f2_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2_t add2(f2_t a, f2_t b) {
  f2_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t sub2(f2_t a, f2_t b) {
  f2_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t mul2(f2_t a, f2_t b) {
  f2_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// ------------------------------------------------------------------------------------------
// Small vector helpers
// ------------------------------------------------------------------------------------------

template <typename T>
struct V3 {
  T x, y, z;
};
template <typename T>
__device__ __forceinline__ V3<T> v3(T x, T y, T z) { return {x, y, z}; }
template <typename T>
__device__ __forceinline__ T dot(const V3<T>& a, const V3<T>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
__device__ __forceinline__ V3<T> cross(const V3<T>& a, const V3<T>& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
__device__ __forceinline__ V3<T> operator+(const V3<T>& a, const V3<T>& b) {
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T>
__device__ __forceinline__ V3<T> operator-(const V3<T>& a, const V3<T>& b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
__device__ __forceinline__ V3<T> operator*(T s, const V3<T>& a) {
  return {s * a.x, s * a.y, s * a.z};
}

// Row-major 3x3 helpers.
template <typename T>
__device__ __forceinline__ V3<T> matvec(const T* m, const V3<T>& v) {
  return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
          m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
template <typename T>
__device__ __forceinline__ V3<T> matTvec(const T* m, const V3<T>& v) {
  return {m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z,
          m[2] * v.x + m[5] * v.y + m[8] * v.z};
}

// Cofactor matrix of a row-major 3x3 matrix (cof(A) = det(A) A^-T).
template <typename T>
__device__ __forceinline__ void cofactor3(const T* a, T* c) {
  c[0] = a[4] * a[8] - a[5] * a[7];
  c[1] = a[5] * a[6] - a[3] * a[8];
  c[2] = a[3] * a[7] - a[4] * a[6];
  c[3] = a[2] * a[7] - a[1] * a[8];
  c[4] = a[0] * a[8] - a[2] * a[6];
  c[5] = a[1] * a[6] - a[0] * a[7];
  c[6] = a[1] * a[5] - a[2] * a[4];
  c[7] = a[2] * a[3] - a[0] * a[5];
  c[8] = a[0] * a[4] - a[1] * a[3];
}

// Scalar-first quaternion to row-major rotation, same formula as baseline/util_render.py:51-76.
template <typename T>
__device__ __forceinline__ void quat_to_rot(const float* q, T* r) {
  T w = q[0], x = q[1], y = q[2], z = q[3];
  T nq = w * w + x * x + y * y + z * z;
  if (!(nq > T(1e-12))) {
    r[0] = 1; r[1] = 0; r[2] = 0; r[3] = 0; r[4] = 1; r[5] = 0; r[6] = 0; r[7] = 0; r[8] = 1;
    return;
  }
  T s = T(2) / nq;
  T X = x * s, Y = y * s, Z = z * s;
  T wX = w * X, wY = w * Y, wZ = w * Z, xX = x * X, xY = x * Y, xZ = x * Z;
  T yY = y * Y, yZ = y * Z, zZ = z * Z;
  r[0] = T(1) - (yY + zZ); r[1] = xY - wZ; r[2] = xZ + wY;
  r[3] = xY + wZ; r[4] = T(1) - (xX + zZ); r[5] = yZ - wX;
  r[6] = xZ - wY; r[7] = yZ + wX; r[8] = T(1) - (xX + yY);
}

// CTAs of kernel `Kern` (with `threads` threads) resident on the current device, queried once per
// (kernel, device); safe to call from several host threads.
template <auto Kern>
inline int resident_ctas(int threads) {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) dev = 0;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, Kern, threads, 0);
    v = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

}  // namespace fe
