// api.cu -- host orchestration and the C ABI (include/fuzzy_ellipses.h).
//
// Replaces the reference's custom-call body RasterizeGaussiansCUDAJAX (rasterize_main.cu:29-114),
// its host pipeline CudaRasterizer::Rasterizer::forwardJAX (rasterizer_impl.cu:174-344) and its
// per-call GpuMemoryPool (rasterizer_impl.h:24-43, rasterizer_impl.cu:47-79). Differences by
// design: scratch comes from a grow-only arena per (device, stream) instead of cudaMalloc/cudaFree
// per call; every stage runs on the caller's stream; the key count stays on the device (capacity
// is planned from the worst case N x tiles when that fits the key budget), so the steady state
// has no host synchronisation; errors are status codes, never exit() or exceptions.
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "fe_kernels.cuh"

namespace fe {
namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(FE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define FE_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Scratch bytes the worst-case key capacity may use before the pipeline falls back to reading
// the exact key count back (one host synchronisation, as the reference always does).
size_t key_budget_bytes() {
  static const size_t v = [] {
    const char* s = std::getenv("FE_KEY_BUDGET_BYTES");
    return s ? (size_t)std::strtoull(s, nullptr, 10) : (size_t)4 << 30;
  }();
  return v;
}

// Bytes of key-proportional scratch per key: the key and its radix-sort twin.
constexpr size_t kBytesPerKey = 2 * sizeof(uint64_t);

int bits_for(int64_t n) {
  int b = 0;
  while (b < 40 && (int64_t(1) << b) < n) ++b;
  return b;
}

// A grow-only device buffer.
struct DevBuf {
  char* ptr = nullptr;
  size_t cap = 0;
  int reserve(size_t bytes, cudaStream_t st) {
    if (bytes <= cap) return FE_OK;
    if (ptr) {
      // Work already enqueued may still use the old buffer.
      FE_CUDA(cudaStreamSynchronize(st));
      FE_CUDA(cudaFree(ptr));
      ptr = nullptr;
      cap = 0;
    }
    const size_t want = align_up(bytes + bytes / 4);
    if (cudaMalloc(&ptr, want) != cudaSuccess) {
      cudaGetLastError();
      ptr = nullptr;
      return fail(FE_ERR_OUT_OF_MEMORY, "scratch arena could not grow to " +
                                            std::to_string(want) + " bytes");
    }
    cap = want;
    return FE_OK;
  }
};

// Sequential carving of a buffer into 256-byte aligned regions.
struct Carver {
  char* base;
  size_t off = 0;
  template <class T>
  T* take(int64_t count) {
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += align_up(sizeof(T) * (size_t)(count > 0 ? count : 0));
    return p;
  }
};

// Per-record scratch (and the control block): sized by records, tiles and pixels.
struct RecSpace {
  Control* ctrl;
  GaussRec* recs;
  TileRect* rects;
  FootRows* foot;  // footprint rows (unless FE_FLAG_RECT_BINNING)
  uint32_t* touched;
  uint32_t* incl;
  unsigned long long* scan_tmp;
  uint2* ranges;
  uint32_t* tile_view;  // tile-major binning of a batch: the view of every tile
  unsigned long long* row_tot;  // tile-major binning: key counts of the tile rows, per view
  uint32_t* order;  // tile-major binning: per work class (kTileClasses lists of n_tiles) the
                    // tiles as uint4 entries (tile id, first key, end key, view)
  RecGrad* rgrad;  // backward only
};

// Key-proportional scratch.
struct KeySpace {
  uint64_t* keys_a;
  uint64_t* keys_b;
  uint32_t* hist;
};

// Zero the control block and the first `rows` row-total entries with one memset (row_tot is
// carved directly after the control block).
inline cudaError_t zero_ctrl_rows(const RecSpace& rs, int64_t rows, cudaStream_t st) {
  const size_t bytes = (size_t)(reinterpret_cast<char*>(rs.row_tot + rows) -
                                reinterpret_cast<char*>(rs.ctrl));
  return cudaMemsetAsync(rs.ctrl, 0, bytes, st);
}

template <class F>
size_t carve_rec(char* base, int64_t n_rec, int64_t n_tiles, int64_t n_pix, bool bwd, F&& out) {
  Carver c{base};
  RecSpace s;
  s.ctrl = c.take<Control>(1);
  // (directly after the control block: one memset clears both; see zero_ctrl_rows)
  s.row_tot = c.take<unsigned long long>(n_tiles + 1);
  s.recs = c.take<GaussRec>(n_rec);
  s.rects = c.take<TileRect>(n_rec);
  s.foot = c.take<FootRows>(n_rec);
  s.touched = c.take<uint32_t>(n_rec);
  s.incl = c.take<uint32_t>(n_rec);
  s.scan_tmp = c.take<unsigned long long>(scan_grid(std::max(n_rec, n_tiles)));
  s.ranges = c.take<uint2>(n_tiles);
  s.tile_view = c.take<uint32_t>(n_tiles);
  s.order = c.take<uint32_t>((int64_t)kTileClasses * n_tiles * 4);  // uint4 entries
  s.rgrad = bwd ? c.take<RecGrad>(n_rec) : nullptr;
  out(s);
  return c.off;
}

template <class F>
size_t carve_keys(char* base, int64_t cap, F&& out) {
  Carver c{base};
  KeySpace s;
  s.keys_a = c.take<uint64_t>(cap);
  s.keys_b = c.take<uint64_t>(cap);
  s.hist = c.take<uint32_t>(int64_t(sort_grid(cap) + 1) * 256);
  out(s);
  return c.off;
}

// Scratch owned by one (device, stream) pair for the plain entry points.
struct Arena {
  DevBuf rec, keys;
  unsigned long long* h_pinned = nullptr;
  int init() {
    if (!h_pinned) FE_CUDA(cudaMallocHost(&h_pinned, 64));
    return FE_OK;
  }
};

std::mutex g_arena_mu;
std::map<std::pair<int, cudaStream_t>, Arena*> g_arenas;

int arena_for(cudaStream_t st, Arena** out) {
  int dev = 0;
  FE_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_arena_mu);
  Arena*& a = g_arenas[{dev, st}];
  if (!a) a = new Arena();
  const int rc = a->init();
  if (rc) return rc;
  *out = a;
  return FE_OK;
}

int check_desc(const fe_render_desc* d) {
  if (!d) return fail(FE_ERR_INVALID_ARGUMENT, "descriptor is NULL");
  if (d->magic != FE_DESC_MAGIC || d->version != FE_DESC_VERSION)
    return fail(FE_ERR_DESCRIPTOR, "descriptor magic/version mismatch");
  if (d->n_gaussians < 0 || d->height < 1 || d->width < 1 || d->height > 65535 * 8 ||
      d->width > 65535 * 8)
    return fail(FE_ERR_INVALID_ARGUMENT, "image size or Gaussian count out of range");
  if (!(d->fx != 0.f) || !(d->fy != 0.f) || !std::isfinite(d->fx) || !std::isfinite(d->fy))
    return fail(FE_ERR_INVALID_ARGUMENT, "focal lengths must be finite and non-zero");
  if (d->cull_mode != FE_CULL_EPS && d->cull_mode != FE_CULL_NSTD)
    return fail(FE_ERR_INVALID_ARGUMENT, "unknown cull mode");
  const bool tile_ok = (d->tile_w == 0 && d->tile_h == 0) || (d->tile_w == 8 && d->tile_h == 8) ||
                       (d->tile_w == 16 && d->tile_h == 16) || (d->tile_w == 32 && d->tile_h == 8);
  if (!tile_ok) return fail(FE_ERR_INVALID_ARGUMENT, "tile shape must be 8x8, 16x16 or 32x8");
  if (d->px_per_thread != 0 && d->px_per_thread != 1 && d->px_per_thread != 2 &&
      d->px_per_thread != 4)
    return fail(FE_ERR_INVALID_ARGUMENT, "px_per_thread must be 0, 1, 2 or 4");
  const uint32_t chunk = (d->flags >> 8) & 0xff;
  if (chunk != 0 && chunk != 8 && chunk != 16 && chunk != 32)
    return fail(FE_ERR_INVALID_ARGUMENT, "blend chunk must be 0, 8, 16 or 32 record pairs");
  return FE_OK;
}

inline void tile_shape(const fe_render_desc* d, int& tw, int& th) {
  tw = d->tile_w ? d->tile_w : 16;
  th = d->tile_h ? d->tile_h : 16;
}

// Shared binning + blend pipeline over a views table. Sizes are host-known; the key count
// lives on the device. When `sync_count` is set the key count is read back after the scan and
// the key scratch sized exactly (used when the worst case exceeds the key budget).
struct Pipeline {
  ViewsArg va;
  int64_t n_rec, n_tiles, n_pix;
  int tile_w, tile_h;
  int px;     // pixels per thread in the blend (0 = default)
  int chunk;  // record pairs per shared-memory stage in the blend (0 = default)
  bool radix;  // FE_FLAG_RADIX_BINNING: emit + sort even where tile-major binning applies
  bool rect_binning;  // FE_FLAG_RECT_BINNING: every tile of each footprint's rectangle
  bool heavy_first;  // FE_FLAG_HEAVY_TILES_FIRST: work-class tile lists for the blend
  int cull_mode;
  float cull_param;
  float beta2, beta3;
  const float *means, *prec, *logw, *quat, *trans;
};

// Tile-major binning filters every view's footprint rectangles once per tile row, in one block
// per row. It is used when every view is at most kMaxRowTiles tiles wide and that filtering is
// cheap: at most 4096 Gaussians per view, or at most 16384 when there are enough row blocks to
// fill the GPU (measured on GB300: faster than emit + sort for 1-64 views of 20-8000 Gaussians,
// slower for one 1280x720 view of 24000); the emit + radix sort path is used otherwise.
constexpr int kRowPlanSmallN = 4096;
constexpr int kRowPlanLargeN = 16384;
constexpr int kRowPlanBlocks = 152;  // row blocks that fill a GB300 (its SM count)

struct RowPlan {
  bool ok = false;
  int max_gy = 0;
  int max_gx = 0;
  int n_views = 0;
};

RowPlan row_plan(const ViewDev* views, int n_views) {
  RowPlan r;
  r.n_views = n_views;
  r.ok = n_views >= 1 && n_views <= 65535;
  int64_t tests = 0, n_rec = 0, rows = 0;
  int max_n = 0;
  for (int i = 0; i < n_views; ++i) {
    const ViewDev& V = views[i];
    if (V.gx > kMaxRowTiles || V.gy > 65535) r.ok = false;
    r.max_gy = std::max(r.max_gy, (int)V.gy);
    r.max_gx = std::max(r.max_gx, (int)V.gx);
    max_n = std::max(max_n, (int)V.n);
    tests += (int64_t)V.gy * V.n;
    rows += V.gy;
    n_rec += V.n;
  }
  if (max_n > kRowPlanLargeN || (max_n > kRowPlanSmallN && rows < kRowPlanBlocks)) r.ok = false;
  if (tests > std::max<int64_t>(INT64_C(1) << 24, 64 * n_rec)) r.ok = false;
  return r;
}

// Footprint rows of the records, or NULL when each footprint's whole rectangle is binned.
inline FootRows* foot_of(const Pipeline& p, const RecSpace& rs) {
  return p.rect_binning ? nullptr : rs.foot;
}

int run_binning(const Pipeline& p, int64_t worst, DevBuf& recbuf, DevBuf& keybuf,
                unsigned long long* h_pinned, bool bwd, cudaStream_t st, RecSpace& rs,
                KeySpace& ks, int64_t& cap, uint64_t*& sorted) {
  size_t rec_bytes = carve_rec(nullptr, p.n_rec, p.n_tiles, p.n_pix, bwd, [](const RecSpace&) {});
  int rc = recbuf.reserve(rec_bytes, st);
  if (rc) return rc;
  carve_rec(recbuf.ptr, p.n_rec, p.n_tiles, p.n_pix, bwd, [&](const RecSpace& s) { rs = s; });

  // `worst`: every record touching every tile of its view.
  const bool exact = worst > 0 && (size_t)worst * kBytesPerKey <= key_budget_bytes();

  // The single-view pipelines describe their view on the host (va.one).
  const RowPlan rp = (p.va.table || p.radix) ? RowPlan{} : row_plan(&p.va.one, 1);
  // The tile-major emission writes every tile's range; the emit + sort path writes only the
  // non-empty ones.
  FE_CUDA(zero_ctrl_rows(rs, rp.ok ? rp.max_gy + 1 : 0, st));
  if (!rp.ok) FE_CUDA(cudaMemsetAsync(rs.ranges, 0, sizeof(uint2) * (size_t)p.n_tiles, st));
  launch_preprocess(p.va, p.n_rec, p.means, p.prec, p.logw, p.quat, nullptr, p.trans, p.cull_mode,
                    p.cull_param, p.tile_w, p.tile_h, rs.recs, rs.rects, foot_of(p, rs),
                    rs.touched, rp.ok ? rs.row_tot : nullptr, rp.max_gy, rs.ctrl, st);
  if (exact) {
    cap = worst;
  } else {
    // Count with an unbounded capacity first, read the count back, then size the keys.
    if (!rp.ok)
      launch_scan(rs.touched, rs.incl, p.n_rec, INT64_C(0xffffffff), rs.scan_tmp, rs.ctrl, st);
    FE_CUDA(cudaMemcpyAsync(h_pinned, &rs.ctrl->want_keys, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st));
    FE_CUDA(cudaStreamSynchronize(st));
    cap = (int64_t)*h_pinned;
    if (cap < 1) cap = 1;
  }
  const size_t key_bytes = carve_keys(nullptr, cap, [](const KeySpace&) {});
  rc = keybuf.reserve(key_bytes, st);
  if (rc) return rc;
  carve_keys(keybuf.ptr, cap, [&](const KeySpace& s) { ks = s; });
  if (exact && !rp.ok) launch_scan(rs.touched, rs.incl, p.n_rec, cap, rs.scan_tmp, rs.ctrl, st);
  if (!rp.ok || !p.heavy_first) rs.order = nullptr;  // the blend takes tiles in index order
  if (rp.ok) {
    launch_tile_binning_emit(p.va, rp.n_views, rp.max_gy, rp.max_gx, rs.rects, foot_of(p, rs),
                             p.tile_w, p.tile_h, rs.row_tot, cap, rs.ctrl, rs.ranges, nullptr,
                             ks.keys_a, rs.order, p.n_tiles, st);
    sorted = ks.keys_a;
  } else {
    launch_emit_keys(p.va, rs.incl, rs.rects, foot_of(p, rs), p.tile_w, p.tile_h, p.n_rec, rs.ctrl,
                     ks.keys_a, cap, st);
    sorted = launch_sort(ks.keys_a, ks.keys_b, bits_for(p.n_tiles), rs.ctrl, cap, ks.hist, st);
    launch_ranges(sorted, rs.ctrl, cap, rs.ranges, st);
  }
  return FE_OK;
}

// Tile count below which a launch defaults to two pixels per blend thread.
constexpr int64_t kPx2Tiles = 3000;

// Pixels per blend thread when the descriptor leaves it at 0: two for small launches (see the
// measurements at single_view_pipeline), else the launcher's default for the tile shape.
int default_px(int px, int tw, int th, int64_t n_tiles) {
  if (px == 0 && !(tw == 8 && th == 8) && n_tiles < kPx2Tiles) return 2;
  return px;
}

Pipeline single_view_pipeline(const fe_render_desc* d, const float* means, const float* prec,
                              const float* logw, const float* quat, const float* trans) {
  Pipeline p{};
  int tw, th;
  tile_shape(d, tw, th);
  ViewDev v{};
  v.fx = d->fx; v.fy = d->fy; v.cx = d->cx; v.cy = d->cy;
  v.H = d->height; v.W = d->width;
  v.gx = (d->width + tw - 1) / tw;
  v.gy = (d->height + th - 1) / th;
  v.n = d->n_gaussians;
  p.va.table = nullptr;
  p.va.count = 1;
  p.va.one = v;
  p.n_rec = d->n_gaussians;
  p.n_tiles = (int64_t)v.gx * v.gy;
  p.n_pix = (int64_t)d->height * d->width;
  p.tile_w = tw;
  p.tile_h = th;
  // A small launch does not fill the GPU, and its heaviest tile sets the blend's duration:
  // below about 3000 tiles, two pixels per thread (twice the threads per tile, half the
  // per-thread work) mostly finish sooner. Device time per forward of 1000 Gaussians, 16x16
  // tiles, 2 vs 4 pixels per thread: single views 320x240 (300 tiles) 33.4 vs 36.8 us, 480x360
  // 38.5 vs 39.1, 560x420 38.4 vs 38.9, 640x480 (1200) 41.6 vs 39.3, 720x540 (1530) 44.5 vs
  // 46.5, 800x600 (1900) 47.9 vs 50.0, 960x720 (2700) 55.7 vs 55.6, 1120x840 (3710) 64.9 vs
  // 61.0, 1280x960 74.0 vs 68.6; batches 8 x 128x128 (512 tiles) 52.9 vs 59.0 us, 4 x 256x256
  // (1024) 50.8 vs 54.9, 16 x 320x240 (4800) 102.0 vs 95.9, 8 x 640x480 134.8 vs 118.4. (The
  // window is not monotonic: 640x480's 1200 tiles fit the four-pixel blend's resident CTAs in
  // one round but not the two-pixel blend's.)
  p.px = default_px((int)d->px_per_thread, tw, th, p.n_tiles);
  p.chunk = (int)(d->flags >> 8) & 0xff;
  p.radix = (d->flags & FE_FLAG_RADIX_BINNING) != 0;
  p.rect_binning = (d->flags & FE_FLAG_RECT_BINNING) != 0;
  p.heavy_first = (d->flags & FE_FLAG_HEAVY_TILES_FIRST) != 0;
  p.cull_mode = d->cull_mode;
  p.cull_param = d->cull_param;
  p.beta2 = d->beta2;
  p.beta3 = d->beta3;
  p.means = means; p.prec = prec; p.logw = logw; p.quat = quat; p.trans = trans;
  return p;
}

}  // namespace

// Error reporting shared with the other host translation units of the library.
int set_last_error(int code, const std::string& msg) { return fail(code, msg); }

}  // namespace fe

using namespace fe;

extern "C" {

const char* fe_version(void) { return "fuzzy_ellipses_gb300 0.1.0 (sm_103a)"; }

const char* fe_last_error_message(void) { return g_last_error.c_str(); }

const char* fe_status_string(int s) {
  switch (s) {
    case FE_OK: return "ok";
    case FE_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FE_ERR_DESCRIPTOR: return "bad descriptor";
    case FE_ERR_CUDA: return "CUDA error";
    case FE_ERR_OUT_OF_MEMORY: return "out of device memory";
    case FE_ERR_CAPACITY: return "key capacity exceeded";
    case FE_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case FE_ERR_UNSUPPORTED: return "unsupported";
    case FE_ERR_SCRATCH_LIMIT: return "request exceeds the fixed scratch size";
    default: return "unknown status";
  }
}

void fe_render_desc_init(fe_render_desc* d, int32_t n, int32_t h, int32_t w, float fx, float fy,
                         float cx, float cy) {
  std::memset(d, 0, sizeof(*d));
  d->magic = FE_DESC_MAGIC;
  d->version = FE_DESC_VERSION;
  d->n_gaussians = n;
  d->height = h;
  d->width = w;
  d->fx = fx; d->fy = fy; d->cx = cx; d->cy = cy;
  d->beta2 = 21.4f;
  d->beta3 = 2.66f;
  d->cull_mode = FE_CULL_EPS;
  d->cull_param = kDefaultCullEps;
  d->tile_w = 16;
  d->tile_h = 16;
}

int fe_render_fwd(const fe_render_desc* d, const float* means, const float* prec,
                  const float* logw, const float* quat, const float* trans, float* depth,
                  float* alpha, float* stats, fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  int rc = check_desc(d);
  if (rc) return rc;
  if (!depth || !alpha || !quat || !trans)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL output or pose pointer");
  const int64_t npix = (int64_t)d->height * d->width;
  if (d->n_gaussians == 0) {
    FE_CUDA(cudaMemsetAsync(depth, 0, sizeof(float) * npix, st));
    FE_CUDA(cudaMemsetAsync(alpha, 0, sizeof(float) * npix, st));
    if (stats) FE_CUDA(cudaMemsetAsync(stats, 0, sizeof(float) * 3 * npix, st));
    return FE_OK;
  }
  if (!means || !prec || !logw) return fail(FE_ERR_INVALID_ARGUMENT, "NULL Gaussian pointer");
  Arena* a = nullptr;
  rc = arena_for(st, &a);
  if (rc) return rc;
  Pipeline p = single_view_pipeline(d, means, prec, logw, quat, trans);
  RecSpace rs;
  KeySpace ks;
  int64_t cap = 0;
  uint64_t* sorted = nullptr;
  rc = run_binning(p, p.n_rec * p.n_tiles, a->rec, a->keys, a->h_pinned, false, st, rs, ks, cap,
                   sorted);
  if (rc) return rc;
  launch_blend_fwd(p.va, p.tile_w, p.tile_h, p.px, p.chunk, p.n_tiles, rs.order, sorted, rs.recs,
                   rs.ranges, p.beta2, p.beta3, depth, alpha, stats, npix, rs.ctrl, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_render_bwd(const fe_render_desc* d, const float* means, const float* prec,
                  const float* logw, const float* quat, const float* trans, const float* depth,
                  const float* alpha, const float* stats, const float* gdepth,
                  const float* galpha, float* gmeans, float* gprec, float* glogw,
                  fe_stream_t stream_) {
  (void)alpha;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  int rc = check_desc(d);
  if (rc) return rc;
  const int64_t n = d->n_gaussians;
  if (n == 0) return FE_OK;
  if (!means || !prec || !logw || !quat || !trans || !depth || !stats || !gmeans || !gprec ||
      !glogw)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL pointer");
  FE_CUDA(cudaMemsetAsync(gmeans, 0, sizeof(float) * 3 * n, st));
  FE_CUDA(cudaMemsetAsync(gprec, 0, sizeof(float) * 9 * n, st));
  FE_CUDA(cudaMemsetAsync(glogw, 0, sizeof(float) * n, st));
  Arena* a = nullptr;
  rc = arena_for(st, &a);
  if (rc) return rc;
  Pipeline p = single_view_pipeline(d, means, prec, logw, quat, trans);
  RecSpace rs;
  KeySpace ks;
  int64_t cap = 0;
  uint64_t* sorted = nullptr;
  rc = run_binning(p, p.n_rec * p.n_tiles, a->rec, a->keys, a->h_pinned, true, st, rs, ks, cap,
                   sorted);
  if (rc) return rc;
  FE_CUDA(cudaMemsetAsync(rs.rgrad, 0, sizeof(RecGrad) * (size_t)p.n_rec, st));
  launch_blend_bwd(p.va, p.tile_w, p.tile_h, p.n_tiles, sorted, rs.ranges, rs.recs, depth,
                   stats, p.n_pix, gdepth, galpha, p.beta2, p.beta3, rs.rgrad, rs.ctrl, st);
  launch_record_vjp(p.va, p.n_rec, means, prec, quat, trans, rs.recs, rs.rgrad, gmeans, gprec,
                    glogw, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_render_features(const fe_render_desc* d, const float* means, const float* prec,
                       const float* logw, const float* quat, const float* trans,
                       const float* stats, const float* features, int32_t n_features,
                       float* out, fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  int rc = check_desc(d);
  if (rc) return rc;
  if (n_features < 1) return fail(FE_ERR_INVALID_ARGUMENT, "n_features must be >= 1");
  if (!stats || !features || !out || !quat || !trans)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL pointer");
  const int64_t npix = (int64_t)d->height * d->width;
  if (d->n_gaussians == 0) {
    FE_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * npix * n_features, st));
    return FE_OK;
  }
  if (!means || !prec || !logw) return fail(FE_ERR_INVALID_ARGUMENT, "NULL Gaussian pointer");
  Arena* a = nullptr;
  rc = arena_for(st, &a);
  if (rc) return rc;
  Pipeline p = single_view_pipeline(d, means, prec, logw, quat, trans);
  RecSpace rs;
  KeySpace ks;
  int64_t cap = 0;
  uint64_t* sorted = nullptr;
  rc = run_binning(p, p.n_rec * p.n_tiles, a->rec, a->keys, a->h_pinned, false, st, rs, ks, cap,
                   sorted);
  if (rc) return rc;
  launch_features(p.va, p.tile_w, p.tile_h, p.n_tiles, sorted, rs.ranges, rs.recs, stats, npix,
                  p.beta2, p.beta3, features, n_features, out, rs.ctrl, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_render_binning(const fe_render_desc* d, const float* means, const float* prec,
                      const float* logw, const float* quat, const float* trans, uint64_t* keys,
                      int64_t key_capacity, uint32_t* ranges, int64_t* h_num_keys,
                      fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  int rc = check_desc(d);
  if (rc) return rc;
  if (!h_num_keys || !ranges || !quat || !trans || key_capacity < 0)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL pointer or negative capacity");
  *h_num_keys = 0;
  Pipeline p = single_view_pipeline(d, means, prec, logw, quat, trans);
  FE_CUDA(cudaMemsetAsync(ranges, 0, sizeof(uint2) * (size_t)p.n_tiles, st));
  if (p.n_rec == 0) return FE_OK;
  if (!means || !prec || !logw) return fail(FE_ERR_INVALID_ARGUMENT, "NULL Gaussian pointer");
  Arena* a = nullptr;
  rc = arena_for(st, &a);
  if (rc) return rc;
  RecSpace rs;
  KeySpace ks;
  int64_t cap = 0;
  uint64_t* sorted = nullptr;
  rc = run_binning(p, p.n_rec * p.n_tiles, a->rec, a->keys, a->h_pinned, false, st, rs, ks, cap,
                   sorted);
  if (rc) return rc;
  FE_CUDA(cudaMemcpyAsync(a->h_pinned, &rs.ctrl->num_keys, sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, st));
  FE_CUDA(cudaStreamSynchronize(st));
  const int64_t K = (int64_t)*a->h_pinned;
  *h_num_keys = K;
  if (K > key_capacity) return fail(FE_ERR_CAPACITY, "key capacity too small");
  if (K > 0 && keys)
    FE_CUDA(cudaMemcpyAsync(keys, sorted, sizeof(uint64_t) * (size_t)K, cudaMemcpyDeviceToDevice, st));
  FE_CUDA(cudaMemcpyAsync(ranges, rs.ranges, sizeof(uint2) * (size_t)p.n_tiles,
                          cudaMemcpyDeviceToDevice, st));
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_silhouette_bce(const float* alpha, const float* target, const int64_t* seg_end,
                      int32_t n_seg, int64_t n_pix, float* galpha, double* loss,
                      fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (n_pix < 0 || n_seg < 0 || (n_pix > 0 && n_seg == 0))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_silhouette_bce: bad pixel or segment count");
  if (n_seg > 0 && (!seg_end || !loss))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_silhouette_bce: NULL segment or loss pointer");
  if (n_pix > 0 && (!alpha || !target || !galpha))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_silhouette_bce: NULL pixel buffer");
  if (n_seg > 0) FE_CUDA(cudaMemsetAsync(loss, 0, sizeof(double) * (size_t)n_seg, st));
  launch_silhouette_bce(alpha, target, seg_end, n_seg, n_pix, galpha, loss, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_gmm_log_likelihood(const float* means, const float* prec, const float* logw, int32_t n,
                          const float* points, int64_t n_points, float* point_ll, float* res,
                          double* total, fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (n < 1 || n_points < 0)
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_gmm_log_likelihood: need n >= 1 and n_points >= 0");
  if (!means || !prec || !logw || (n_points > 0 && (!points || !point_ll)))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_gmm_log_likelihood: NULL argument");
  if (total) FE_CUDA(cudaMemsetAsync(total, 0, sizeof(double), st));
  if (n_points == 0) return FE_OK;
  Arena* a = nullptr;
  int rc = arena_for(st, &a);
  if (rc) return rc;
  // The records' scratch is the front of the arena's record buffer.
  rc = a->rec.reserve(gmm_scratch_bytes(n), st);
  if (rc) return rc;
  launch_gmm_log_likelihood(n, means, prec, logw, n_points, points, point_ll, res, total,
                            a->rec.ptr, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_prec_from_scale_rot(const float* scales, const float* quats, int64_t n, float* prec,
                           fe_stream_t stream_) {
  if (n < 0 || (n > 0 && (!scales || !quats || !prec)))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_prec_from_scale_rot: bad arguments");
  launch_prec_from_scale_rot(n, scales, quats, prec, reinterpret_cast<cudaStream_t>(stream_));
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_prec_from_scale_rot_bwd(const float* scales, const float* quats, int64_t n,
                               const float* grad_prec, float* grad_scales, float* grad_quats,
                               fe_stream_t stream_) {
  if (n < 0 || (n > 0 && (!scales || !quats || !grad_prec || !grad_scales || !grad_quats)))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_prec_from_scale_rot_bwd: bad arguments");
  launch_prec_from_scale_rot_bwd(n, scales, quats, grad_prec, grad_scales, grad_quats,
                                 reinterpret_cast<cudaStream_t>(stream_));
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_transform_points(const float* points, int64_t n, const float* pose, int32_t inverse,
                        float* out, fe_stream_t stream_) {
  if (n < 0 || !pose || (n > 0 && (!points || !out)))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_transform_points: bad arguments");
  if ((reinterpret_cast<uintptr_t>(points) | reinterpret_cast<uintptr_t>(out)) & 15)
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_transform_points: buffers must be 16-byte aligned");
  launch_transform_points(n, points, pose, inverse ? 1 : 0, out,
                          reinterpret_cast<cudaStream_t>(stream_));
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_transform_points_bwd(const float* points, int64_t n, const float* pose, int32_t inverse,
                            const float* grad_out, float* grad_points, float* grad_pose,
                            fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (n < 0 || !pose || (n > 0 && (!points || !grad_out)))
    return fail(FE_ERR_INVALID_ARGUMENT, "fe_transform_points_bwd: bad arguments");
  Arena* a = nullptr;
  int rc = arena_for(st, &a);
  if (rc) return rc;
  rc = a->rec.reserve(12 * sizeof(double), st);
  if (rc) return rc;
  double* gacc = reinterpret_cast<double*>(a->rec.ptr);
  FE_CUDA(cudaMemsetAsync(gacc, 0, 12 * sizeof(double), st));
  launch_transform_points_bwd(n, points, pose, inverse ? 1 : 0, grad_out, grad_points, grad_pose,
                              gacc, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

void fe_pixlist_desc_init(fe_pixlist_desc* d, int32_t n, int32_t n_poses, int64_t n_rays,
                          float inv_f) {
  std::memset(d, 0, sizeof(*d));
  d->magic = FE_DESC_MAGIC;
  d->version = FE_PIXLIST_DESC_VERSION;
  d->n_gaussians = n;
  d->n_poses = n_poses;
  d->n_rays = n_rays;
  d->inv_f = inv_f;
  d->beta2 = 21.4f;
  d->beta3 = 2.66f;
  d->cull_mode = FE_CULL_EPS;
  d->cull_param = kDefaultCullEps;
  d->ray_mode = FE_RAYS_POSE_INDEXED;
  d->aspect = 1.f;
  d->shift_x = 0.5f;
  d->shift_y = 0.5f;
}

int fe_render_pixels(const fe_pixlist_desc* d_in, const float* means, const float* prec,
                     const float* logw, const float* poses, const float* rays,
                     const float* features, float* depth, float* alpha, float* flow_next,
                     float* flow_prev, float* out_features, float* weights,
                     fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (!d_in) return fail(FE_ERR_INVALID_ARGUMENT, "descriptor is NULL");
  if (d_in->magic != FE_DESC_MAGIC || (d_in->version != 1 && d_in->version != 2))
    return fail(FE_ERR_DESCRIPTOR, "pixel-list descriptor magic/version mismatch");
  // A version-1 descriptor is the version-2 layout cut before ray_mode: read only that prefix.
  fe_pixlist_desc dv;
  fe_pixlist_desc_init(&dv, 0, 1, 0, 1.f);
  std::memcpy(&dv, d_in, d_in->version == 1 ? offsetof(fe_pixlist_desc, ray_mode) : sizeof(dv));
  const fe_pixlist_desc* d = &dv;
  const bool cam = d->ray_mode == FE_RAYS_QUAT_CAM;
  if (d->ray_mode != FE_RAYS_POSE_INDEXED && !cam)
    return fail(FE_ERR_INVALID_ARGUMENT, "unknown ray mode");
  if (cam && (!(d->aspect > 0.f) || !std::isfinite(d->aspect) || !std::isfinite(d->shift_x) ||
              !std::isfinite(d->shift_y)))
    return fail(FE_ERR_INVALID_ARGUMENT, "aspect must be finite and positive, shifts finite");
  if (cam && (flow_next || flow_prev))
    return fail(FE_ERR_INVALID_ARGUMENT, "flow needs pose-indexed rays");
  if (d->n_gaussians < 0 || d->n_poses < 1 || d->n_rays < 0)
    return fail(FE_ERR_INVALID_ARGUMENT, "need n_gaussians >= 0, n_poses >= 1, n_rays >= 0");
  if (!(d->inv_f != 0.f) || !std::isfinite(d->inv_f))
    return fail(FE_ERR_INVALID_ARGUMENT, "inv_f must be finite and non-zero");
  if (d->cull_mode != FE_CULL_EPS && d->cull_mode != FE_CULL_NSTD)
    return fail(FE_ERR_INVALID_ARGUMENT, "unknown cull mode");
  if (d->n_features < 0 || d->n_features > 16)
    return fail(FE_ERR_UNSUPPORTED, "n_features must be in [0, 16]");
  if ((d->n_features > 0) != (features != nullptr) || (out_features && d->n_features == 0))
    return fail(FE_ERR_INVALID_ARGUMENT, "features and n_features must be given together");
  if (d->n_rays == 0) return FE_OK;
  if (!poses || !rays || !depth || !alpha ||
      (d->n_gaussians > 0 && (!means || !prec || !logw)))
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  Arena* a = nullptr;
  int rc = arena_for(st, &a);
  if (rc) return rc;
  rc = a->rec.reserve(std::max<size_t>(pixlist_scratch_bytes(d->n_gaussians, d->n_poses), 256),
                      st);
  if (rc) return rc;
  PixRayModel rm;
  rm.inv_f = d->inv_f;
  rm.aspect = cam ? d->aspect : 1.f;
  rm.shift_x = cam ? d->shift_x : 0.f;
  rm.shift_y = cam ? d->shift_y : 0.f;
  rm.stride = cam ? 3 : 4;
  launch_render_pixels(d->n_gaussians, cam ? 1 : d->n_poses, means, prec, logw, poses, d->n_rays,
                       rays, rm, d->beta2, d->beta3, d->cull_mode, d->cull_param, features,
                       d->n_features, depth, alpha, flow_next, flow_prev, out_features, weights,
                       a->rec.ptr, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_selftest_bounded_wait(uint64_t limit_ns, uint32_t* h_status, uint64_t* h_elapsed_ns,
                             fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (!h_status || !h_elapsed_ns) return fail(FE_ERR_INVALID_ARGUMENT, "NULL output");
  if (limit_ns < 1000 || limit_ns > 1000000000ull)
    return fail(FE_ERR_INVALID_ARGUMENT, "limit_ns must be in [1 us, 1 s]");
  Arena* a = nullptr;
  int rc = arena_for(st, &a);
  if (rc) return rc;
  rc = a->rec.reserve(256, st);
  if (rc) return rc;
  uint32_t* status = reinterpret_cast<uint32_t*>(a->rec.ptr);
  unsigned long long* elapsed = reinterpret_cast<unsigned long long*>(a->rec.ptr + 64);
  launch_wait_selftest(limit_ns, status, elapsed, st);
  FE_CUDA(cudaGetLastError());
  FE_CUDA(cudaMemcpyAsync(h_status, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FE_CUDA(cudaMemcpyAsync(h_elapsed_ns, elapsed, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
  FE_CUDA(cudaStreamSynchronize(st));
  return FE_OK;
}

int fe_check_device_status(fe_stream_t stream_, uint32_t* device_error) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  Arena* a = nullptr;
  int rc = arena_for(st, &a);
  if (rc) return rc;
  FE_CUDA(cudaStreamSynchronize(st));
  uint32_t err = 0;
  if (a->rec.ptr) {
    Control* ctrl = reinterpret_cast<Control*>(a->rec.ptr);
    FE_CUDA(cudaMemcpy(&err, &ctrl->error, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    FE_CUDA(cudaMemset(&ctrl->error, 0, sizeof(uint32_t)));
  }
  if (device_error) *device_error = err;
  return FE_OK;
}


// ---------------------------------------------------------------------------------------------
// Reference-compatible binning and the legacy interface
// ---------------------------------------------------------------------------------------------

int fe_reference_binning(int32_t P, int32_t height, int32_t width, float n_std,
                         const float* means, const float* scales, const float* rots,
                         const float* view, const float* proj, float tan_fovx, float tan_fovy,
                         int32_t* radii, float* means2d, uint32_t* tiles_touched, uint64_t* keys,
                         int64_t key_capacity, uint32_t* ranges, int64_t* h_num_keys,
                         fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (P < 0 || height < 1 || width < 1 || !h_num_keys || key_capacity < 0 ||
      key_capacity > INT64_C(0xffffffff))
    return fail(FE_ERR_INVALID_ARGUMENT, "bad size or capacity");
  const int gx = (width + 7) / 8, gy = (height + 7) / 8;
  const int64_t T = (int64_t)gx * gy;
  *h_num_keys = 0;
  if (ranges) FE_CUDA(cudaMemsetAsync(ranges, 0, sizeof(uint2) * (size_t)T, st));
  if (P == 0) return FE_OK;
  if (!means || !scales || !rots || !view || !proj || !radii || !means2d || !tiles_touched ||
      !keys || !ranges)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL pointer");
  Arena* a = nullptr;
  int rc = arena_for(st, &a);
  if (rc) return rc;
  RecSpace rs;
  const size_t rb = carve_rec(nullptr, P, T, 0, false, [](const RecSpace&) {});
  rc = a->rec.reserve(rb, st);
  if (rc) return rc;
  carve_rec(a->rec.ptr, P, T, 0, false, [&](const RecSpace& s_) { rs = s_; });
  FE_CUDA(cudaMemsetAsync(rs.ctrl, 0, sizeof(Control), st));
  launch_preprocess_reference(P, n_std, means, scales, rots, view, proj, width, height, tan_fovx,
                              tan_fovy, gx, gy, radii, means2d, rs.rects, rs.touched, st);
  launch_scan(rs.touched, tiles_touched, P, key_capacity, rs.scan_tmp, rs.ctrl, st);
  FE_CUDA(cudaMemcpyAsync(a->h_pinned, &rs.ctrl->want_keys, sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, st));
  FE_CUDA(cudaStreamSynchronize(st));
  const int64_t K = (int64_t)*a->h_pinned;
  *h_num_keys = K;
  if (K > key_capacity) return fail(FE_ERR_CAPACITY, "key capacity too small");
  if (K == 0) return FE_OK;
  KeySpace ks;
  const size_t kb = carve_keys(nullptr, K, [](const KeySpace&) {});
  rc = a->keys.reserve(kb, st);
  if (rc) return rc;
  carve_keys(a->keys.ptr, K, [&](const KeySpace& s_) { ks = s_; });
  ViewsArg va{};
  va.count = 1;
  va.one.H = height; va.one.W = width; va.one.gx = gx; va.one.gy = gy; va.one.n = P;
  launch_emit_keys(va, tiles_touched, rs.rects, nullptr, 8, 8, P, rs.ctrl, keys, K, st);
  uint64_t* sorted = launch_sort(keys, ks.keys_b, bits_for(T), rs.ctrl, K, ks.hist, st);
  if (sorted != keys)
    FE_CUDA(cudaMemcpyAsync(keys, sorted, sizeof(uint64_t) * (size_t)K, cudaMemcpyDeviceToDevice, st));
  launch_ranges(keys, rs.ctrl, K, reinterpret_cast<uint2*>(ranges), st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

// rasterizer_impl.cu:154-172: the reference's choice of n_std from the Gaussian count.
static float reference_num_stds(int n) {
  if (n <= 1000) return 3.0f;
  if (n <= 5000) return 0.75f;
  if (n <= 100000) return 0.50f;
  return 0.10f;
}

int fe_rasterize_legacy(const fe_legacy_desc* d, const float* means, const float* weights,
                        const float* scales, const float* rots, const float* rays,
                        const float* rot, const float* trans, const float* view,
                        const float* proj, float* out_z, float* out_alpha, fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  if (!d || d->P < 0 || d->image_height < 1 || d->image_width < 1)
    return fail(FE_ERR_INVALID_ARGUMENT, "bad legacy descriptor");
  const int P = d->P, H = d->image_height, W = d->image_width;
  const int gx = (W + 7) / 8, gy = (H + 7) / 8;
  const int64_t T = (int64_t)gx * gy, npix = (int64_t)H * W;
  if (!out_z || !out_alpha) return fail(FE_ERR_INVALID_ARGUMENT, "NULL output");
  if (P == 0) {
    FE_CUDA(cudaMemsetAsync(out_z, 0, sizeof(float) * npix, st));
    FE_CUDA(cudaMemsetAsync(out_alpha, 0, sizeof(float) * npix, st));
    return FE_OK;
  }
  if (!means || !weights || !scales || !rots || !rays || !rot || !trans || !view || !proj)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL input");
  Arena* a = nullptr;
  int rc = arena_for(st, &a);
  if (rc) return rc;
  // Per-record space plus the reference's radii/means2d outputs.
  RecSpace rs;
  Carver extra{nullptr};
  const size_t rb = carve_rec(nullptr, P, T, 0, false, [](const RecSpace&) {});
  extra.off = rb;
  extra.take<int32_t>(P);
  extra.take<float>(2 * (int64_t)P);
  rc = a->rec.reserve(extra.off, st);
  if (rc) return rc;
  carve_rec(a->rec.ptr, P, T, 0, false, [&](const RecSpace& s_) { rs = s_; });
  Carver ex2{a->rec.ptr};
  ex2.off = rb;
  int32_t* radii = ex2.take<int32_t>(P);
  float* means2d = ex2.take<float>(2 * (int64_t)P);

  ViewsArg va{};
  va.count = 1;
  va.one.H = H; va.one.W = W; va.one.gx = gx; va.one.gy = gy; va.one.n = P;
  va.one.fx = 1.f; va.one.fy = 1.f;
  FE_CUDA(cudaMemsetAsync(rs.ctrl, 0, sizeof(Control), st));
  FE_CUDA(cudaMemsetAsync(rs.ranges, 0, sizeof(uint2) * (size_t)T, st));
  launch_preprocess_reference(P, reference_num_stds(P), means, scales, rots, view, proj, W, H,
                              d->tan_fovx, d->tan_fovy, gx, gy, radii, means2d, rs.rects,
                              rs.touched, st);
  launch_legacy_records(va, P, means, scales, rots, weights, rot, trans, rays, rs.recs, st);
  const int64_t worst = (int64_t)P * T;
  int64_t cap;
  if ((size_t)worst * kBytesPerKey <= key_budget_bytes()) {
    cap = worst;
    launch_scan(rs.touched, rs.incl, P, cap, rs.scan_tmp, rs.ctrl, st);
  } else {
    launch_scan(rs.touched, rs.incl, P, INT64_C(0xffffffff), rs.scan_tmp, rs.ctrl, st);
    FE_CUDA(cudaMemcpyAsync(a->h_pinned, &rs.ctrl->want_keys, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st));
    FE_CUDA(cudaStreamSynchronize(st));
    cap = (int64_t)*a->h_pinned;
    if (cap < 1) cap = 1;
  }
  KeySpace ks;
  const size_t kb = carve_keys(nullptr, cap, [](const KeySpace&) {});
  rc = a->keys.reserve(kb, st);
  if (rc) return rc;
  carve_keys(a->keys.ptr, cap, [&](const KeySpace& s_) { ks = s_; });
  launch_emit_keys(va, rs.incl, rs.rects, nullptr, 8, 8, P, rs.ctrl, ks.keys_a, cap, st);
  uint64_t* sorted = launch_sort(ks.keys_a, ks.keys_b, bits_for(T), rs.ctrl, cap, ks.hist, st);
  launch_ranges(sorted, rs.ctrl, cap, rs.ranges, st);
  launch_blend_fwd(va, 8, 8, 0, 0, T, nullptr, sorted, rs.recs, rs.ranges, 21.4f, 2.66f, out_z,
                   out_alpha, nullptr, 0, rs.ctrl, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

// ---------------------------------------------------------------------------------------------
// XLA custom-call targets (api_version 2)
// ---------------------------------------------------------------------------------------------

static void xla_report(XlaCustomCallStatus* status, int rc) {
  if (rc == FE_OK || !status) return;
  using SetFailure = void (*)(XlaCustomCallStatus*, const char*, size_t);
  static SetFailure fn = reinterpret_cast<SetFailure>(dlsym(RTLD_DEFAULT, "XlaCustomCallStatusSetFailure"));
  std::string msg = std::string("fuzzy_ellipses: ") + fe_status_string(rc) + ": " + g_last_error;
  if (fn) fn(status, msg.c_str(), msg.size());
  else std::fprintf(stderr, "%s\n", msg.c_str());
}

void fe_render_fwd_xla(fe_stream_t stream, void** buffers, const char* opaque, size_t opaque_len,
                       XlaCustomCallStatus* status) {
  fe_render_desc d;
  if (opaque_len != sizeof(fe_render_desc)) {
    xla_report(status, fail(FE_ERR_DESCRIPTOR, "opaque has the wrong size"));
    return;
  }
  std::memcpy(&d, opaque, sizeof d);
  float** b = reinterpret_cast<float**>(buffers);
  xla_report(status, fe_render_fwd(&d, b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], stream));
}

void fe_render_bwd_xla(fe_stream_t stream, void** buffers, const char* opaque, size_t opaque_len,
                       XlaCustomCallStatus* status) {
  fe_render_desc d;
  if (opaque_len != sizeof(fe_render_desc)) {
    xla_report(status, fail(FE_ERR_DESCRIPTOR, "opaque has the wrong size"));
    return;
  }
  std::memcpy(&d, opaque, sizeof d);
  float** b = reinterpret_cast<float**>(buffers);
  xla_report(status, fe_render_bwd(&d, b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8], b[9],
                                   b[10], b[11], b[12], stream));
}

void fe_rasterize_legacy_xla(fe_stream_t stream, void** buffers, const char* opaque,
                             size_t opaque_len, XlaCustomCallStatus* status) {
  if (opaque_len != sizeof(fe_legacy_desc)) {
    xla_report(status, fail(FE_ERR_DESCRIPTOR, "opaque has the wrong size"));
    return;
  }
  fe_legacy_desc d;
  std::memcpy(&d, opaque, sizeof d);
  float** b = reinterpret_cast<float**>(buffers);
  xla_report(status, fe_rasterize_legacy(&d, b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8],
                                         b[9], b[10], stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Batches
// ---------------------------------------------------------------------------------------------

struct fe_batch {
  int device = 0;
  fe_render_desc desc{};
  int tile_w = 16, tile_h = 16;
  bool exact = false;  // size key scratch from the device-side count (one readback per run)
  bool keep_binning = false;  // reuse the last forward's binning in the backward
  bool binned = false;        // the scratch holds the binning of the last forward of ...
  const float* binned_for[3] = {nullptr, nullptr, nullptr};  // ... these Gaussian arrays
  int32_t n_views = 0;
  DevBuf tables;  // ViewDev[n_views] | quat[4 n_views] | trans[3 n_views]
  ViewDev* views_d = nullptr;
  float* quat_d = nullptr;
  float* trans_d = nullptr;
  std::vector<ViewDev> views_h;
  std::vector<float> quat_h, trans_h;
  int64_t n_rec = 0, n_tiles = 0, n_pix = 0, cap = 0, worst = 0;
  int64_t n_gauss = 0;  // extent of the concatenated Gaussian arrays the scenes reference
  DevBuf rec, keys;
  RecSpace rs{};
  KeySpace ks{};
  uint64_t* sorted = nullptr;
  unsigned long long* h_pinned = nullptr;
  // fe_batch_fwd_host: device staging of the Gaussians and images, the band plan, and the
  // batch's second compute stream and copy stream with their events (created on first use).
  struct HostBand {
    int64_t t0, t1;  // global tiles [t0, t1): whole tile rows
    int64_t p0, p1;  // the contiguous output pixels [p0, p1) of those rows
  };
  DevBuf io;
  std::vector<HostBand> bands;
  cudaStream_t s_comp = nullptr, s_copy = nullptr;
  cudaEvent_t ev_bin = nullptr, ev_copy = nullptr;
  std::vector<cudaEvent_t> band_ev;
  RowPlan rows;  // tile-major binning plan (rows.ok) or the emit + sort path
};

namespace {

// Fill the host-side plan of a batch (tables, sizes) from scenes and views.
int plan_batch(fe_batch* b, const fe_scene* scenes, int32_t n_scenes, const fe_view* views,
               int32_t n_views) {
  if (n_scenes < 0 || n_views < 1 || !views || (n_scenes > 0 && !scenes))
    return fail(FE_ERR_INVALID_ARGUMENT, "empty batch");
  for (int i = 0; i < n_views; ++i) {
    const fe_view& v = views[i];
    if (v.scene < 0 || v.scene >= n_scenes || v.height < 1 || v.width < 1 || v.pixel_offset < 0 ||
        !(v.fx != 0.f) || !(v.fy != 0.f) || scenes[v.scene].n < 0 || scenes[v.scene].gauss_offset < 0)
      return fail(FE_ERR_INVALID_ARGUMENT, "bad view " + std::to_string(i));
  }
  b->bands.clear();
  b->views_h.assign(n_views, ViewDev{});
  b->quat_h.assign(4 * (size_t)n_views, 0.f);
  b->trans_h.assign(3 * (size_t)n_views, 0.f);
  int64_t rec = 0, tiles = 0, pix_end = 0, worst = 0;
  for (int i = 0; i < n_views; ++i) {
    const fe_view& v = views[i];
    ViewDev& d = b->views_h[i];
    d.fx = v.fx; d.fy = v.fy; d.cx = v.cx; d.cy = v.cy;
    d.H = v.height; d.W = v.width;
    d.gx = (v.width + b->tile_w - 1) / b->tile_w;
    d.gy = (v.height + b->tile_h - 1) / b->tile_h;
    d.n = scenes[v.scene].n;
    d.pose = i;
    d.flags = v.flags;
    d.gauss_base = scenes[v.scene].gauss_offset;
    d.rec_base = rec;
    d.tile_base = tiles;
    d.pix_base = v.pixel_offset;
    rec += d.n;
    tiles += (int64_t)d.gx * d.gy;
    worst += (int64_t)d.n * d.gx * d.gy;
    pix_end = std::max<int64_t>(pix_end, v.pixel_offset + (int64_t)v.height * v.width);
    for (int k = 0; k < 4; ++k) b->quat_h[4 * i + k] = v.quat[k];
    for (int k = 0; k < 3; ++k) b->trans_h[3 * i + k] = v.trans[k];
  }
  if (tiles > INT64_C(0xffffffff)) return fail(FE_ERR_INVALID_ARGUMENT, "too many tiles in one batch");
  b->n_gauss = 0;
  for (int s_ = 0; s_ < n_scenes; ++s_)
    b->n_gauss = std::max<int64_t>(b->n_gauss, scenes[s_].gauss_offset + scenes[s_].n);
  b->n_views = n_views;
  b->n_rec = rec;
  b->n_tiles = tiles;
  b->n_pix = pix_end;
  b->worst = worst;
  b->rows = row_plan(b->views_h.data(), n_views);
  return FE_OK;
}

// Upload the tables and size the scratch (grow-only). Ordered on `st` and synchronised.
int commit_batch(fe_batch* b, cudaStream_t st) {
  Carver c{nullptr};
  c.take<ViewDev>(b->n_views);
  c.take<float>(4 * (int64_t)b->n_views);
  c.take<float>(3 * (int64_t)b->n_views);
  int rc = b->tables.reserve(c.off, st);
  if (rc) return rc;
  Carver t{b->tables.ptr};
  b->views_d = t.take<ViewDev>(b->n_views);
  b->quat_d = t.take<float>(4 * (int64_t)b->n_views);
  b->trans_d = t.take<float>(3 * (int64_t)b->n_views);
  FE_CUDA(cudaMemcpyAsync(b->views_d, b->views_h.data(), sizeof(ViewDev) * b->n_views,
                          cudaMemcpyHostToDevice, st));
  FE_CUDA(cudaMemcpyAsync(b->quat_d, b->quat_h.data(), sizeof(float) * b->quat_h.size(),
                          cudaMemcpyHostToDevice, st));
  FE_CUDA(cudaMemcpyAsync(b->trans_d, b->trans_h.data(), sizeof(float) * b->trans_h.size(),
                          cudaMemcpyHostToDevice, st));
  // (ranges and row totals: sized for the tiles and for the tile-major binning's row slots)
  const int64_t tile_slots =
      std::max<int64_t>(b->n_tiles, (int64_t)b->rows.n_views * (b->rows.max_gy + 1));
  const size_t rb = carve_rec(nullptr, b->n_rec, tile_slots, b->n_pix, true, [](const RecSpace&) {});
  rc = b->rec.reserve(rb, st);
  if (rc) return rc;
  carve_rec(b->rec.ptr, b->n_rec, tile_slots, b->n_pix, true, [&](const RecSpace& s_) { b->rs = s_; });
  if (!b->exact) {
    const int64_t budget_keys = (int64_t)(key_budget_bytes() / kBytesPerKey);
    b->cap = std::max<int64_t>(1, std::min<int64_t>({b->worst, budget_keys, INT64_C(0xffffffff)}));
    const size_t kb = carve_keys(nullptr, b->cap, [](const KeySpace&) {});
    rc = b->keys.reserve(kb, st);
    if (rc) return rc;
    carve_keys(b->keys.ptr, b->cap, [&](const KeySpace& s_) { b->ks = s_; });
  }
  // Host tables may be rewritten right away: a copy from pageable memory returns once its
  // source is staged. Creation uploads on the legacy stream, which does not order the caller's
  // non-blocking streams, so it waits for the upload.
  if (!st) FE_CUDA(cudaStreamSynchronize(st));
  return FE_OK;
}

}  // namespace

extern "C" {

int fe_batch_create(const fe_render_desc* desc, const fe_scene* scenes, int32_t n_scenes,
                    const fe_view* views, int32_t n_views, fe_batch** out) {
  if (!out) return fail(FE_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!desc || desc->magic != FE_DESC_MAGIC || desc->version != FE_DESC_VERSION)
    return fail(FE_ERR_DESCRIPTOR, "descriptor magic/version mismatch");
  fe_render_desc probe = *desc;
  probe.height = 1; probe.width = 1; probe.n_gaussians = 0; probe.fx = 1.f; probe.fy = 1.f;
  int rc = check_desc(&probe);
  if (rc) return rc;
  fe_batch* b = new fe_batch();
  b->desc = *desc;
  b->exact = (desc->flags & FE_FLAG_EXACT_KEYS) != 0;
  b->keep_binning = (desc->flags & FE_FLAG_KEEP_BINNING) != 0;
  tile_shape(desc, b->tile_w, b->tile_h);
  rc = plan_batch(b, scenes, n_scenes, views, n_views);
  if (rc) {
    delete b;
    return rc;
  }
  if (cudaGetDevice(&b->device) != cudaSuccess || cudaMallocHost(&b->h_pinned, 64) != cudaSuccess) {
    cudaGetLastError();
    b->h_pinned = nullptr;
    fe_batch_destroy(b);
    return fail(FE_ERR_CUDA, "batch set-up failed");
  }
  rc = commit_batch(b, nullptr);
  if (rc) {
    fe_batch_destroy(b);
    return rc;
  }
  *out = b;
  return FE_OK;
}

int fe_batch_reset(fe_batch* b, const fe_scene* scenes, int32_t n_scenes, const fe_view* views,
                   int32_t n_views, fe_stream_t stream_) {
  if (!b) return fail(FE_ERR_INVALID_ARGUMENT, "NULL batch");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  // No synchronisation: the new tables reach the device by copies ordered on `st` after the
  // previous run, and buffers that must grow wait for `st` before they are freed.
  b->binned = false;
  int rc = plan_batch(b, scenes, n_scenes, views, n_views);
  if (rc) return rc;
  return commit_batch(b, st);
}

void fe_batch_destroy(fe_batch* b) {
  if (!b) return;
  cudaFree(b->tables.ptr);
  cudaFree(b->rec.ptr);
  cudaFree(b->keys.ptr);
  if (b->h_pinned) cudaFreeHost(b->h_pinned);
  cudaFree(b->io.ptr);
  for (cudaEvent_t e : b->band_ev) cudaEventDestroy(e);
  if (b->ev_bin) cudaEventDestroy(b->ev_bin);
  if (b->ev_copy) cudaEventDestroy(b->ev_copy);
  if (b->s_comp) cudaStreamDestroy(b->s_comp);
  if (b->s_copy) cudaStreamDestroy(b->s_copy);
  delete b;
}

int64_t fe_batch_pixels(const fe_batch* b) { return b ? b->n_pix : 0; }

int64_t fe_batch_scratch_bytes(const fe_batch* b) {
  return b ? (int64_t)(b->tables.cap + b->rec.cap + b->keys.cap) : 0;
}

}  // extern "C"

// Remember which Gaussian arrays the batch's current binning belongs to (FE_FLAG_KEEP_BINNING).
static void note_binning(fe_batch* b, const float* means, const float* prec, const float* logw) {
  b->binned = true;
  b->binned_for[0] = means;
  b->binned_for[1] = prec;
  b->binned_for[2] = logw;
}

static Pipeline batch_pipeline(fe_batch* b, const float* means, const float* prec,
                               const float* logw) {
  Pipeline p{};
  p.va.table = b->views_d;
  p.va.count = b->n_views;
  // (written by the tile-major emission, read from the blend on)
  p.va.tile_view = (b->rows.ok && !(b->desc.flags & FE_FLAG_RADIX_BINNING)) ? b->rs.tile_view
                                                                             : nullptr;
  p.n_rec = b->n_rec;
  p.n_tiles = b->n_tiles;
  p.n_pix = b->n_pix;
  p.tile_w = b->tile_w;
  p.tile_h = b->tile_h;
  p.px = default_px((int)b->desc.px_per_thread, b->tile_w, b->tile_h, p.n_tiles);
  p.chunk = (int)(b->desc.flags >> 8) & 0xff;
  p.radix = (b->desc.flags & FE_FLAG_RADIX_BINNING) != 0;
  p.rect_binning = (b->desc.flags & FE_FLAG_RECT_BINNING) != 0;
  p.heavy_first = (b->desc.flags & FE_FLAG_HEAVY_TILES_FIRST) != 0;
  p.cull_mode = b->desc.cull_mode;
  p.cull_param = b->desc.cull_param;
  p.beta2 = b->desc.beta2;
  p.beta3 = b->desc.beta3;
  p.means = means; p.prec = prec; p.logw = logw; p.quat = b->quat_d; p.trans = b->trans_d;
  return p;
}

// The work-class tile lists of the last binning, when it was tile-major (else NULL).
static const uint32_t* batch_order(const fe_batch* b, const Pipeline& p) {
  return (p.heavy_first && !p.radix && b->rows.ok) ? b->rs.order : nullptr;
}

// Binning of a batch. With exact key sizing the key count is read back after the scan (one
// 8-byte copy and a stream synchronisation) and the key scratch grows to fit it.
static int batch_binning(fe_batch* b, const Pipeline& p, cudaStream_t st, cudaEvent_t* ev) {
  const RecSpace& rs = b->rs;
  const RowPlan rp = p.radix ? RowPlan{} : b->rows;
  FE_CUDA(zero_ctrl_rows(rs, rp.ok ? (int64_t)rp.n_views * (rp.max_gy + 1) : 0, st));
  if (!rp.ok) FE_CUDA(cudaMemsetAsync(rs.ranges, 0, sizeof(uint2) * (size_t)p.n_tiles, st));
  if (ev) FE_CUDA(cudaEventRecord(ev[0], st));
  launch_preprocess(p.va, p.n_rec, p.means, p.prec, p.logw, p.quat, nullptr, p.trans, p.cull_mode,
                    p.cull_param, p.tile_w, p.tile_h, rs.recs, rs.rects, foot_of(p, rs),
                    rs.touched, rp.ok ? rs.row_tot : nullptr, rp.max_gy, rs.ctrl, st);
  if (ev) FE_CUDA(cudaEventRecord(ev[1], st));
  if (b->exact) {
    if (!rp.ok)
      launch_scan(rs.touched, rs.incl, p.n_rec, INT64_C(0xffffffff), rs.scan_tmp, rs.ctrl, st);
    FE_CUDA(cudaMemcpyAsync(b->h_pinned, &rs.ctrl->want_keys, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st));
    FE_CUDA(cudaStreamSynchronize(st));
    const int64_t K = std::max<int64_t>(1, (int64_t)*b->h_pinned);
    if (K > b->cap) {
      const size_t kb = carve_keys(nullptr, K + K / 4, [](const KeySpace&) {});
      int rc = b->keys.reserve(kb, st);
      if (rc) return rc;
      b->cap = K + K / 4;
      carve_keys(b->keys.ptr, b->cap, [&](const KeySpace& s_) { b->ks = s_; });
    }
  } else if (!rp.ok) {
    launch_scan(rs.touched, rs.incl, p.n_rec, b->cap, rs.scan_tmp, rs.ctrl, st);
  }
  if (ev) FE_CUDA(cudaEventRecord(ev[2], st));
  const KeySpace& ks = b->ks;
  if (rp.ok) {
    launch_tile_binning_emit(p.va, rp.n_views, rp.max_gy, rp.max_gx, rs.rects, foot_of(p, rs),
                             p.tile_w, p.tile_h, rs.row_tot, b->cap, rs.ctrl, rs.ranges,
                             rs.tile_view, ks.keys_a, p.heavy_first ? rs.order : nullptr,
                             p.n_tiles, st);
    if (ev) FE_CUDA(cudaEventRecord(ev[3], st));
    b->sorted = ks.keys_a;
    if (ev) FE_CUDA(cudaEventRecord(ev[4], st));
  } else {
    launch_emit_keys(p.va, rs.incl, rs.rects, foot_of(p, rs), p.tile_w, p.tile_h, p.n_rec, rs.ctrl,
                     ks.keys_a, b->cap, st);
    if (ev) FE_CUDA(cudaEventRecord(ev[3], st));
    b->sorted = launch_sort(ks.keys_a, ks.keys_b, bits_for(p.n_tiles), rs.ctrl, b->cap, ks.hist, st);
    if (ev) FE_CUDA(cudaEventRecord(ev[4], st));
    launch_ranges(b->sorted, rs.ctrl, b->cap, rs.ranges, st);
  }
  if (ev) FE_CUDA(cudaEventRecord(ev[5], st));
  return FE_OK;
}

// Bands of whole tile rows for fe_batch_fwd_host: about kHostBandPixels output pixels each (at
// most kMaxHostBands per batch), each covering a contiguous range of output pixels (a band ends
// where the next view's pixels do not follow on).
constexpr int64_t kHostBandPixels = INT64_C(1) << 19;
constexpr int64_t kMaxHostBands = 8;

// Tuning knobs of the host-to-host forward, read once: FE_HOST_BANDS (most bands, default 8) and
// FE_HOST_BAND_STREAMS (1: all bands on the caller's stream; 2, the default: alternate with the
// batch's second stream so one band's tail overlaps the next band's start).
static int64_t host_band_limit() {
  static const int64_t v = [] {
    const char* s = std::getenv("FE_HOST_BANDS");
    const long long x = s ? std::strtoll(s, nullptr, 10) : kMaxHostBands;
    return (int64_t)std::min<long long>(64, std::max<long long>(1, x));
  }();
  return v;
}
static int host_band_streams() {
  static const int v = [] {
    const char* s = std::getenv("FE_HOST_BAND_STREAMS");
    return (s && std::atoi(s) == 1) ? 1 : 2;
  }();
  return v;
}

// FE_HOST_DIRECT=0 makes fe_batch_fwd_host use the banded copies even for pinned outputs.
static bool host_direct_enabled() {
  static const bool v = [] {
    const char* s = std::getenv("FE_HOST_DIRECT");
    return !(s && std::atoi(s) == 0);
  }();
  return v;
}

// The device address of n floats of host memory at h when the whole range is pinned memory
// mapped into the current device's address space (its first and last elements resolve to
// device addresses the same distance apart), else nullptr. Pageable memory gives nullptr.
static const float* mapped_host_floats(const float* h, int64_t n) {
  if (n <= 0) return nullptr;
  cudaPointerAttributes a{}, e{};
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess ||
      cudaPointerGetAttributes(&e, h + (n - 1)) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || e.type != cudaMemoryTypeHost || !a.devicePointer ||
      !e.devicePointer)
    return nullptr;
  const float* d0 = static_cast<const float*>(a.devicePointer);
  return static_cast<const float*>(e.devicePointer) == d0 + (n - 1) ? d0 : nullptr;
}
static float* mapped_host_floats(float* h, int64_t n) {
  return const_cast<float*>(mapped_host_floats(static_cast<const float*>(h), n));
}

static void plan_host_bands(fe_batch* b) {
  b->bands.clear();
  const int64_t k =
      std::min(host_band_limit(), std::max<int64_t>(1, (b->n_pix + kHostBandPixels - 1) / kHostBandPixels));
  const int64_t target = std::max<int64_t>(1, (b->n_tiles + k - 1) / k);
  fe_batch::HostBand cur{0, 0, 0, 0};
  bool open = false;
  for (const ViewDev& V : b->views_h) {
    for (int ty = 0; ty < V.gy; ++ty) {
      const int64_t t = V.tile_base + (int64_t)ty * V.gx;
      const int64_t px = V.pix_base + (int64_t)std::min(ty * b->tile_h, V.H) * V.W;
      if (open && (cur.p1 != px || cur.t1 != t || cur.t1 - cur.t0 >= target)) {
        b->bands.push_back(cur);
        open = false;
      }
      if (!open) {
        cur = {t, t, px, px};
        open = true;
      }
      cur.t1 = t + V.gx;
      cur.p1 = V.pix_base + (int64_t)std::min((ty + 1) * b->tile_h, V.H) * V.W;
    }
  }
  if (open) b->bands.push_back(cur);
}

// Binning and one blend launch over every tile; `heavy_order` lets the blend take the batch's
// heaviest-first tile lists when it has them (else tiles go in index order).
static int batch_forward(fe_batch* b, const float* means, const float* prec, const float* logw,
                         float* depth, float* alpha, float* stats, bool heavy_order,
                         cudaStream_t st) {
  Pipeline p = batch_pipeline(b, means, prec, logw);
  if (p.n_rec > 0 && (!means || !prec || !logw))
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL Gaussian pointer");
  b->binned = false;
  int rc = batch_binning(b, p, st, nullptr);
  if (rc) return rc;
  note_binning(b, means, prec, logw);
  launch_blend_fwd(p.va, p.tile_w, p.tile_h, p.px, p.chunk, p.n_tiles,
                   heavy_order ? batch_order(b, p) : nullptr, b->sorted, b->rs.recs,
                   b->rs.ranges, p.beta2, p.beta3, depth, alpha, stats, p.n_pix, b->rs.ctrl, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

extern "C" {

int fe_batch_fwd(fe_batch* b, const float* means, const float* prec, const float* logw,
                 float* depth, float* alpha, float* stats, fe_stream_t stream_) {
  if (!b || !depth || !alpha) return fail(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  return batch_forward(b, means, prec, logw, depth, alpha, stats, true,
                       reinterpret_cast<cudaStream_t>(stream_));
}

int fe_batch_fwd_host(fe_batch* b, const float* h_means, const float* h_prec,
                      const float* h_logw, float* h_depth, float* h_alpha, fe_stream_t stream_) {
  if (!b || !h_depth || !h_alpha) return fail(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  const int64_t n = b->n_gauss;
  if (n > 0 && (!h_means || !h_prec || !h_logw))
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL Gaussian pointer");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  // Pinned outputs: the blend stores depth and alpha through their device mapping as it
  // renders, in one launch over all tiles, so the images cross the host link while the tiles
  // after them render and no copy follows the last tile. The tiles go in index order: the host
  // link is slower than the blend's output rate, and index order spreads the light and heavy
  // tiles, hence the stores, evenly over the launch (heaviest-first bunches the light tiles'
  // stores at its end). Other outputs: bands of tile rows, each band's images copied back while
  // the next bands render.
  float* dep_map = host_direct_enabled() ? mapped_host_floats(h_depth, b->n_pix) : nullptr;
  float* alp_map = dep_map ? mapped_host_floats(h_alpha, b->n_pix) : nullptr;
  if (dep_map && alp_map) {
    // Pinned inputs are read by the preprocess through their device mapping (one record per
    // thread reads its Gaussian's 13 floats), so no copy precedes the binning.
    const float* m_map = mapped_host_floats(h_means, 3 * n);
    const float* p_map = m_map ? mapped_host_floats(h_prec, 9 * n) : nullptr;
    const float* w_map = p_map ? mapped_host_floats(h_logw, n) : nullptr;
    if (n > 0 && w_map)
      return batch_forward(b, m_map, p_map, w_map, dep_map, alp_map, nullptr, false, st);
    Carver c{nullptr};
    c.take<float>(3 * n); c.take<float>(9 * n); c.take<float>(n);
    int rc = b->io.reserve(c.off, st);
    if (rc) return rc;
    Carver t{b->io.ptr};
    float* m_d = t.take<float>(3 * n);
    float* p_d = t.take<float>(9 * n);
    float* w_d = t.take<float>(n);
    if (n > 0) {
      FE_CUDA(cudaMemcpyAsync(m_d, h_means, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
      FE_CUDA(cudaMemcpyAsync(p_d, h_prec, sizeof(float) * 9 * n, cudaMemcpyHostToDevice, st));
      FE_CUDA(cudaMemcpyAsync(w_d, h_logw, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    }
    return batch_forward(b, m_d, p_d, w_d, dep_map, alp_map, nullptr, false, st);
  }
  if (b->bands.empty()) plan_host_bands(b);
  const int nb = (int)b->bands.size();

  Carver c{nullptr};
  c.take<float>(3 * n); c.take<float>(9 * n); c.take<float>(n);
  c.take<float>(b->n_pix); c.take<float>(b->n_pix); c.take<uint32_t>(nb);
  int rc = b->io.reserve(c.off, st);
  if (rc) return rc;
  Carver t{b->io.ptr};
  float* m_d = t.take<float>(3 * n);
  float* p_d = t.take<float>(9 * n);
  float* w_d = t.take<float>(n);
  float* dep_d = t.take<float>(b->n_pix);
  float* alp_d = t.take<float>(b->n_pix);
  uint32_t* ctr = t.take<uint32_t>(nb);
  if (!b->s_comp) {
    FE_CUDA(cudaStreamCreateWithFlags(&b->s_comp, cudaStreamNonBlocking));
    FE_CUDA(cudaStreamCreateWithFlags(&b->s_copy, cudaStreamNonBlocking));
    FE_CUDA(cudaEventCreateWithFlags(&b->ev_bin, cudaEventDisableTiming));
    FE_CUDA(cudaEventCreateWithFlags(&b->ev_copy, cudaEventDisableTiming));
  }
  while ((int)b->band_ev.size() < nb) {
    cudaEvent_t e;
    FE_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->band_ev.push_back(e);
  }

  if (n > 0) {
    FE_CUDA(cudaMemcpyAsync(m_d, h_means, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    FE_CUDA(cudaMemcpyAsync(p_d, h_prec, sizeof(float) * 9 * n, cudaMemcpyHostToDevice, st));
    FE_CUDA(cudaMemcpyAsync(w_d, h_logw, sizeof(float) * n, cudaMemcpyHostToDevice, st));
  }
  Pipeline p = batch_pipeline(b, m_d, p_d, w_d);
  b->binned = false;
  rc = batch_binning(b, p, st, nullptr);
  if (rc) return rc;
  note_binning(b, m_d, p_d, w_d);
  FE_CUDA(cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * nb, st));
  FE_CUDA(cudaEventRecord(b->ev_bin, st));
  FE_CUDA(cudaStreamWaitEvent(b->s_comp, b->ev_bin, 0));
  // Every band's blend is enqueued before any copy, so copies into pageable memory (which hold
  // the calling thread) cannot delay the renders.
  for (int j = 0; j < nb; ++j) {
    const fe_batch::HostBand& hb = b->bands[j];
    cudaStream_t sj = (host_band_streams() == 2 && (j & 1)) ? b->s_comp : st;
    launch_blend_fwd_band(p.va, p.tile_w, p.tile_h, p.px, p.chunk, hb.t0, hb.t1, ctr + j,
                          b->sorted, b->rs.recs, b->rs.ranges, p.beta2, p.beta3, dep_d, alp_d,
                          nullptr, p.n_pix, b->rs.ctrl, sj);
    FE_CUDA(cudaGetLastError());
    FE_CUDA(cudaEventRecord(b->band_ev[j], sj));
  }
  for (int j = 0; j < nb; ++j) {
    const fe_batch::HostBand& hb = b->bands[j];
    const size_t bytes = sizeof(float) * (size_t)(hb.p1 - hb.p0);
    FE_CUDA(cudaStreamWaitEvent(b->s_copy, b->band_ev[j], 0));
    FE_CUDA(cudaMemcpyAsync(h_depth + hb.p0, dep_d + hb.p0, bytes, cudaMemcpyDeviceToHost,
                            b->s_copy));
    FE_CUDA(cudaMemcpyAsync(h_alpha + hb.p0, alp_d + hb.p0, bytes, cudaMemcpyDeviceToHost,
                            b->s_copy));
  }
  FE_CUDA(cudaEventRecord(b->ev_copy, b->s_copy));
  FE_CUDA(cudaStreamWaitEvent(st, b->ev_copy, 0));
  return FE_OK;
}

int fe_batch_bwd(fe_batch* b, const float* means, const float* prec, const float* logw,
                 const float* depth, const float* alpha, const float* stats, const float* gdepth,
                 const float* galpha, float* gmeans, float* gprec, float* glogw,
                 fe_stream_t stream_) {
  (void)alpha;
  if (!b || !depth || !stats || !gmeans || !gprec || !glogw)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  Pipeline p = batch_pipeline(b, means, prec, logw);
  FE_CUDA(cudaMemsetAsync(gmeans, 0, sizeof(float) * 3 * (size_t)b->n_gauss, st));
  FE_CUDA(cudaMemsetAsync(gprec, 0, sizeof(float) * 9 * (size_t)b->n_gauss, st));
  FE_CUDA(cudaMemsetAsync(glogw, 0, sizeof(float) * (size_t)b->n_gauss, st));
  if (b->keep_binning && b->binned && b->binned_for[0] == means && b->binned_for[1] == prec &&
      b->binned_for[2] == logw) {
    // Reuse the forward's binning; only the blend's tile counter must start again at zero.
    FE_CUDA(cudaMemsetAsync(&b->rs.ctrl->next_tile, 0, sizeof(uint32_t), st));
  } else {
    b->binned = false;
    int rc = batch_binning(b, p, st, nullptr);
    if (rc) return rc;
    note_binning(b, means, prec, logw);
  }
  FE_CUDA(cudaMemsetAsync(b->rs.rgrad, 0, sizeof(RecGrad) * (size_t)p.n_rec, st));
  launch_blend_bwd(p.va, p.tile_w, p.tile_h, p.n_tiles, b->sorted, b->rs.ranges, b->rs.recs,
                   depth, stats, p.n_pix, gdepth, galpha, p.beta2, p.beta3, b->rs.rgrad,
                   b->rs.ctrl, st);
  launch_record_vjp(p.va, p.n_rec, means, prec, p.quat, p.trans, b->rs.recs, b->rs.rgrad, gmeans,
                    gprec, glogw, st);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_batch_status(fe_batch* b, fe_stream_t stream_, int64_t* num_keys, int64_t* want_keys,
                    uint32_t* device_error) {
  if (!b) return fail(FE_ERR_INVALID_ARGUMENT, "NULL batch");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  Control c;
  FE_CUDA(cudaMemcpyAsync(b->h_pinned, b->rs.ctrl, sizeof(unsigned long long) * 3,
                          cudaMemcpyDeviceToHost, st));
  FE_CUDA(cudaStreamSynchronize(st));
  std::memcpy(&c, b->h_pinned, sizeof(unsigned long long) * 3);
  if (num_keys) *num_keys = (int64_t)c.num_keys;
  if (want_keys) *want_keys = (int64_t)c.want_keys;
  if (device_error) *device_error = c.error;
  return FE_OK;
}

}  // extern "C"

namespace fe {
double run_peak(int kind, int iters, float* scratch, cudaStream_t st);
}

extern "C" {

int fe_batch_fwd_timed(fe_batch* b, const float* means, const float* prec, const float* logw,
                       float* depth, float* alpha, float* stats, float* stage_ms,
                       fe_stream_t stream_) {
  if (!b || !depth || !alpha || !stage_ms) return fail(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  Pipeline p = batch_pipeline(b, means, prec, logw);
  cudaEvent_t ev[7];
  for (auto& e : ev) FE_CUDA(cudaEventCreate(&e));
  b->binned = false;
  int rc = batch_binning(b, p, st, ev);
  if (rc) {
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
  }
  note_binning(b, means, prec, logw);
  launch_blend_fwd(p.va, p.tile_w, p.tile_h, p.px, p.chunk, p.n_tiles, batch_order(b, p),
                   b->sorted, b->rs.recs, b->rs.ranges, p.beta2, p.beta3, depth, alpha, stats,
                   p.n_pix, b->rs.ctrl, st);
  FE_CUDA(cudaEventRecord(ev[6], st));
  FE_CUDA(cudaEventSynchronize(ev[6]));
  for (int i = 0; i < 6; ++i) FE_CUDA(cudaEventElapsedTime(&stage_ms[i], ev[i], ev[i + 1]));
  for (auto& e : ev) cudaEventDestroy(e);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

int fe_batch_launch_count(const fe_batch* b) {
  if (!b) return 0;
  const bool radix = (b->desc.flags & FE_FLAG_RADIX_BINNING) != 0;
  // Tile-major binning: preprocess, (row offsets and view bases for many views,) emission, blend.
  if (b->rows.ok && !radix) return b->rows.n_views > kRowBaseViews ? 5 : 3;
  // Emit + sort: preprocess, scan, emission, three kernels per radix pass, ranges, blend.
  const int passes = (bits_for(b->n_tiles) + 7) / 8;
  const int scan = b->n_rec <= 65536 ? 1 : 3;
  return 1 + scan + 1 + 3 * passes + 1 + 1;
}

int fe_bench_peak(int kind, int iters, double* ops_per_second, fe_stream_t stream_) {
  if (!ops_per_second || kind < 0 || kind > 2 || iters < 1)
    return fail(FE_ERR_INVALID_ARGUMENT, "bad peak benchmark request");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  float* scratch = nullptr;
  FE_CUDA(cudaMalloc(&scratch, 1 << 20));
  *ops_per_second = run_peak(kind, iters, scratch, st);
  cudaFree(scratch);
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Forward render with fixed scratch (fe_render_fwd_noalloc)
// ---------------------------------------------------------------------------------------------
// Some callers cannot allocate device memory while a render runs:
//  * an XLA/JAX custom call: XLA's allocator reserves most of the device's memory when the
//    process starts, so a cudaMalloc inside the call can fail although the request is small, and
//    memory taken there is invisible to XLA's buffer planning;
//  * latency-bound loops sharing the device with other streams: cudaFree synchronises the whole
//    device, so an arena that has to grow stalls every stream of the process.
// For them the whole scratch of one single-view forward render (records, keys, tile records,
// sort histograms, tile ranges and the control block) lives in one file-scope device array of
// FE_NOALLOC_SCRATCH_BYTES per device, resolved once per device with cudaGetSymbolAddress.
// Requests whose worst-case scratch (every Gaussian on every tile) does not fit are rejected on
// the host with FE_ERR_SCRATCH_LIMIT before any device work, so the key capacity can never
// overflow on the device. The entry issues kernels and cudaMemsetAsync/cudaMemcpyAsync on the
// caller's stream only; it calls no allocating routine of CUDA or of any library.

namespace fe {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[FE_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
char* g_noalloc_base[kMaxDevices] = {};

// Device address of the fixed scratch on the current device (resolved on the first call).
int noalloc_scratch(char** out) {
  int dev = 0;
  FE_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(FE_ERR_UNSUPPORTED, "device ordinal " + std::to_string(dev) + " above 63");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_base[dev]) {
    void* p = nullptr;
    FE_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_base[dev] = static_cast<char*>(p);
  }
  *out = g_noalloc_base[dev];
  return FE_OK;
}

}  // namespace
}  // namespace fe

extern "C" {

int fe_render_fwd_noalloc(const fe_render_desc* d, const float* means, const float* prec,
                          const float* logw, const float* quat, const float* trans, float* depth,
                          float* alpha, float* stats, uint32_t* device_error,
                          fe_stream_t stream_) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  int rc = check_desc(d);
  if (rc) return rc;
  if (!depth || !alpha || !quat || !trans)
    return fail(FE_ERR_INVALID_ARGUMENT, "NULL output or pose pointer");
  const int64_t npix = (int64_t)d->height * d->width;
  if (d->n_gaussians == 0) {
    FE_CUDA(cudaMemsetAsync(depth, 0, sizeof(float) * npix, st));
    FE_CUDA(cudaMemsetAsync(alpha, 0, sizeof(float) * npix, st));
    if (stats) FE_CUDA(cudaMemsetAsync(stats, 0, sizeof(float) * 3 * npix, st));
    if (device_error) FE_CUDA(cudaMemsetAsync(device_error, 0, sizeof(uint32_t), st));
    return FE_OK;
  }
  if (!means || !prec || !logw) return fail(FE_ERR_INVALID_ARGUMENT, "NULL Gaussian pointer");

  Pipeline p = single_view_pipeline(d, means, prec, logw, quat, trans);
  const int64_t worst = p.n_rec * p.n_tiles;
  const size_t rec_bytes = carve_rec(nullptr, p.n_rec, p.n_tiles, p.n_pix, false,
                                     [](const RecSpace&) {});
  const size_t key_bytes = carve_keys(nullptr, worst, [](const KeySpace&) {});
  if (worst > INT64_C(0xffffffff) || rec_bytes + key_bytes > (size_t)FE_NOALLOC_SCRATCH_BYTES)
    return fail(FE_ERR_SCRATCH_LIMIT,
                "fe_render_fwd_noalloc: " + std::to_string(p.n_rec) + " Gaussians x " +
                    std::to_string(p.n_tiles) + " tiles need " +
                    std::to_string(rec_bytes + key_bytes) +
                    " bytes of worst-case scratch; the fixed scratch holds " +
                    std::to_string((size_t)FE_NOALLOC_SCRATCH_BYTES) + " bytes");

  char* base = nullptr;
  rc = noalloc_scratch(&base);
  if (rc) return rc;
  RecSpace rs;
  KeySpace ks;
  carve_rec(base, p.n_rec, p.n_tiles, p.n_pix, false, [&](const RecSpace& s) { rs = s; });
  carve_keys(base + rec_bytes, worst, [&](const KeySpace& s) { ks = s; });

  // Must start at zero on every call: the control block (key counters, device error word, the
  // blend's tile counter and work-class counts), the row totals of the tile-major binning, and on
  // the emit + sort path the tile ranges (tiles without keys keep an empty range; the tile-major
  // emission writes every tile's range itself).
  const RowPlan rp = p.radix ? RowPlan{} : row_plan(&p.va.one, 1);
  FE_CUDA(zero_ctrl_rows(rs, rp.ok ? rp.max_gy + 1 : 0, st));
  if (!rp.ok) FE_CUDA(cudaMemsetAsync(rs.ranges, 0, sizeof(uint2) * (size_t)p.n_tiles, st));
  launch_preprocess(p.va, p.n_rec, p.means, p.prec, p.logw, p.quat, nullptr, p.trans, p.cull_mode,
                    p.cull_param, p.tile_w, p.tile_h, rs.recs, rs.rects, foot_of(p, rs),
                    rs.touched, rp.ok ? rs.row_tot : nullptr, rp.max_gy, rs.ctrl, st);
  uint64_t* sorted = ks.keys_a;
  if (!rp.ok || !p.heavy_first) rs.order = nullptr;
  if (rp.ok) {
    launch_tile_binning_emit(p.va, rp.n_views, rp.max_gy, rp.max_gx, rs.rects, foot_of(p, rs),
                             p.tile_w, p.tile_h, rs.row_tot, worst, rs.ctrl, rs.ranges, nullptr,
                             ks.keys_a, rs.order, p.n_tiles, st);
  } else {
    launch_scan(rs.touched, rs.incl, p.n_rec, worst, rs.scan_tmp, rs.ctrl, st);
    launch_emit_keys(p.va, rs.incl, rs.rects, foot_of(p, rs), p.tile_w, p.tile_h, p.n_rec, rs.ctrl,
                     ks.keys_a, worst, st);
    sorted = launch_sort(ks.keys_a, ks.keys_b, bits_for(p.n_tiles), rs.ctrl, worst, ks.hist, st);
    launch_ranges(sorted, rs.ctrl, worst, rs.ranges, st);
  }
  launch_blend_fwd(p.va, p.tile_w, p.tile_h, p.px, p.chunk, p.n_tiles, rs.order, sorted, rs.recs,
                   rs.ranges, p.beta2, p.beta3, depth, alpha, stats, npix, rs.ctrl, st);
  if (device_error)
    FE_CUDA(cudaMemcpyAsync(device_error, &rs.ctrl->error, sizeof(uint32_t),
                            cudaMemcpyDeviceToDevice, st));
  FE_CUDA(cudaGetLastError());
  return FE_OK;
}

}  // extern "C"
