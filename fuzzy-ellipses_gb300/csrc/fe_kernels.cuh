// fe_kernels.cuh -- launcher declarations for the renderer's kernels.
#pragma once

#include "fe_common.cuh"

namespace fe {

// preprocess.cu
void launch_preprocess(const ViewsArg& va, int64_t n_rec, const float* means, const float* prec,
                       const float* logw, const float* quat, const float* rotm,
                       const float* trans, int cull_mode, float cull_param, int tile_w,
                       int tile_h, GaussRec* recs, TileRect* rects, FootRows* foot,
                       uint32_t* touched, unsigned long long* row_tot, int max_gy, Control* ctrl,
                       cudaStream_t st);
void launch_preprocess_reference(int P, float n_std, const float* means, const float* scales,
                                 const float* rots, const float* viewmatrix,
                                 const float* projmatrix, int W, int H, float tan_fovx,
                                 float tan_fovy, int gx, int gy, int32_t* radii, float* means2d,
                                 TileRect* rects, uint32_t* touched, cudaStream_t st);
void launch_legacy_records(const ViewsArg& va, int P, const float* means, const float* scales,
                           const float* rots, const float* logw, const float* rotm,
                           const float* trans, const float* rays, GaussRec* recs,
                           cudaStream_t st);

// binning.cu
// Blocks used by the fixed-grid scan / sort kernels.
int scan_grid(int64_t n);
int sort_grid(int64_t key_capacity);
// Inclusive prefix sum of touched[0..n) into incl; total clamped to capacity in ctrl->num_keys,
// the unclamped total in ctrl->want_keys, FE_DEVERR_CAPACITY set on overflow.
// scratch: scan_grid(n) * 8 bytes.
void launch_scan(const uint32_t* touched, uint32_t* incl, int64_t n, int64_t capacity,
                 unsigned long long* scratch, Control* ctrl, cudaStream_t st);
// foot: the records' footprint rows (each row's keys span the tiles the footprint reaches there),
// or NULL (every row of a record's rectangle spans its full width).
void launch_emit_keys(const ViewsArg& va, const uint32_t* incl, const TileRect* rects,
                      const FootRows* foot, int tile_w, int tile_h, int64_t n,
                      const Control* ctrl, uint64_t* keys, int64_t capacity, cudaStream_t st);
// Stable LSD radix sort of keys on bits [32, 32+key_bits); returns the buffer holding the
// result (a or b). hist: 256 * (sort_grid(capacity) + 1) uint32.
uint64_t* launch_sort(uint64_t* a, uint64_t* b, int key_bits, const Control* ctrl,
                      int64_t capacity, uint32_t* hist, cudaStream_t st);
// Tile-major binning for views at most kMaxRowTiles tiles wide. launch_preprocess with row_tot
// (n_views * (max_gy + 1) zeroed entries, view v's at v * (max_gy + 1)) adds each record's keys in
// every tile row to that row's count and the run's key count to ctrl->want_keys; the emit pass
// (one block per tile row of every view) sets ctrl->num_keys = min(want_keys, capacity)
// (FE_DEVERR_CAPACITY past it) and writes the keys of every tile in ascending Gaussian id at their
// place in the sorted order (keys past num_keys dropped) and every tile's range ({0,0} for an
// empty tile, so the ranges need no zeroing). Same keys and ranges as emit + stable sort +
// ranges, with the same `foot` (see launch_emit_keys). For many views the row counts are first
// turned into row offsets and view bases in place (row_tot is consumed). With `order`
// (kTileClasses lists of n_tiles uint4 entries, 16-byte aligned; ctrl's class counts zeroed)
// every tile is also appended to the list of its work class (tile_class of its key count) as
// (tile id, first key, end key, view), which launch_blend_fwd then serves heaviest class first
// without reading the tile's range or view again. With `tile_view` (n_tiles entries) every tile's view index is
// written beside its range (ViewsArg::tile_view).
constexpr int kMaxRowTiles = 1024;
constexpr int kRowBaseViews = 32;  // above this many views the row bases are formed first
void launch_tile_binning_emit(const ViewsArg& va, int n_views, int max_gy, int max_gx,
                              const TileRect* rects, const FootRows* foot, int tile_w, int tile_h,
                              unsigned long long* row_tot, int64_t capacity, Control* ctrl,
                              uint2* ranges, uint32_t* tile_view, uint64_t* keys, uint32_t* order,
                              int64_t n_tiles, cudaStream_t st);
// Tile ranges of the sorted keys (ranges zeroed beforehand; empty tiles keep {0,0}).
void launch_ranges(const uint64_t* keys, const Control* ctrl, int64_t capacity, uint2* ranges,
                   cudaStream_t st);

// blend_fwd.cu
// px: pixels per thread (1, 2 or 4; 0 = default for the tile shape); chunk: record pairs per
// shared-memory stage (8, 16 or 32; 0 = 32). The blend builds each key's tile record itself from
// the sorted keys and the Gaussian records (no gathered record stream). Persistent:
// ctrl->next_tile must be zero. `order`: the tile-major binning's per-class tile lists (heaviest
// tiles are then taken first) or NULL (tiles in index order).
void launch_blend_fwd(const ViewsArg& va, int tile_w, int tile_h, int px, int chunk, int64_t n_tiles,
                      const uint32_t* order, const uint64_t* keys, const GaussRec* recs,
                      const uint2* ranges, float beta2,
                      float beta3, float* depth, float* alpha, float* stats, int64_t stats_stride,
                      Control* ctrl, cudaStream_t st);
// The blend over global tiles [tile_begin, tile_end) only, taking tiles from `counter` (zero at
// launch); bands with their own counters may run concurrently on different streams.
void launch_blend_fwd_band(const ViewsArg& va, int tile_w, int tile_h, int px, int chunk,
                           int64_t tile_begin, int64_t tile_end, uint32_t* counter,
                           const uint64_t* keys, const GaussRec* recs, const uint2* ranges,
                           float beta2, float beta3, float* depth, float* alpha, float* stats,
                           int64_t stats_stride, Control* ctrl, cudaStream_t st);

// blend_bwd.cu
// Tile records are built per key from the Gaussian records (fe_tilerec.cuh), as in the forward;
// each tile's per-pixel terms are formed from depth, the forward's statistics (stats, stride) and
// the cotangents (NULL = zero) when the tile is staged.
void launch_blend_bwd(const ViewsArg& va, int tile_w, int tile_h, int64_t n_tiles,
                      const uint64_t* keys, const uint2* ranges, const GaussRec* recs,
                      const float* depth, const float* stats, int64_t stats_stride,
                      const float* grad_depth, const float* grad_alpha, float beta2, float beta3,
                      RecGrad* rgrad, Control* ctrl, cudaStream_t st);
// Gradients are accumulated (atomically) into gmeans/gprec/glogw, which must be zeroed first.
void launch_record_vjp(const ViewsArg& va, int64_t n_rec, const float* means, const float* prec,
                       const float* quat, const float* trans, const GaussRec* recs,
                       const RecGrad* rgrad, float* gmeans, float* gprec, float* glogw,
                       cudaStream_t st);

// loss.cu
// Silhouette BCE of renders stored back to back (render s = pixels [seg_end[s-1], seg_end[s]),
// seg_end on the device, increasing, seg_end[n_seg-1] == n_pix): adds each render's mean loss to
// loss[s] (float64, zeroed by the caller) and writes dL_s/dalpha to galpha.
void launch_silhouette_bce(const float* alpha, const float* target, const int64_t* seg_end,
                           int n_seg, int64_t n_pix, float* galpha, double* loss,
                           cudaStream_t st);

// gmm.cu
// Log-likelihood of points under the mixture (fm_render.py log_likelihood): point_ll[j] =
// logsumexp_i r_ij; res (n x n_points, row per Gaussian) receives r_ij when non-NULL; total
// (float64, zeroed by the caller) accumulates sum_j point_ll[j] when non-NULL.
// scratch: gmm_scratch_bytes(n) bytes of device memory.
size_t gmm_scratch_bytes(int n);
void launch_gmm_log_likelihood(int n, const float* means, const float* prec, const float* logw,
                               int64_t n_points, const float* points, float* point_ll,
                               float* res, double* total, void* scratch, cudaStream_t st);

// adapters.cu
// Upper precision factor (n,3,3) from scales (n,3) and scalar-first quaternions (n,4), and its
// backward (gradients of the upper-triangle entries to scales and quaternions).
void launch_prec_from_scale_rot(int64_t n, const float* scales, const float* quats, float* prec,
                                cudaStream_t st);
void launch_prec_from_scale_rot_bwd(int64_t n, const float* scales, const float* quats,
                                    const float* gprec, float* gscales, float* gquats,
                                    cudaStream_t st);
// out = R(q) p + t (inverse = 0) or R(q)^T p + t (inverse = 1), pose = [t(3), q(4)]; the backward
// writes dL/dpoints (if non-NULL) and dL/dpose (7, if non-NULL) using gacc (12 doubles, zeroed).
void launch_transform_points(int64_t n, const float* points, const float* pose, int inverse,
                             float* out, cudaStream_t st);
void launch_transform_points_bwd(int64_t n, const float* points, const float* pose, int inverse,
                                 const float* gout, float* gpoints, float* gpose, double* gacc,
                                 cudaStream_t st);

// pixlist.cu
// Pixel-list render (fm_render.py render_func_idx_quattrans[_flow], render_func_quat_cam);
// scratch: pixlist_scratch_bytes(n, n_poses). feats (n x nf, nf <= 16), flows, out_feats and
// weights (n x n_rays) are optional (NULL).
// Ray model: rows of `stride` floats (x, y, c[, pose]); the camera ray is
// ((x - shift_x) inv_f, (y - shift_y) aspect inv_f, c) of pose `pose` (stride 4) or pose 0.
struct PixRayModel {
  float inv_f, aspect, shift_x, shift_y;
  int stride;
};
size_t pixlist_scratch_bytes(int n, int n_poses);
void launch_render_pixels(int n, int n_poses, const float* means, const float* prec,
                          const float* logw, const float* poses, int64_t n_rays, const float* rays,
                          const PixRayModel& rm, float beta2, float beta3, int cull_mode,
                          float cull_param,
                          const float* feats, int nf, float* depth, float* alpha,
                          float* flow_next, float* flow_prev, float* out_feats, float* weights,
                          void* scratch, cudaStream_t st);

// features.cu
// Softmax-weighted features (nf per Gaussian) of an image render from the forward's statistics.
void launch_features(const ViewsArg& va, int tile_w, int tile_h, int64_t n_tiles,
                     const uint64_t* keys, const uint2* ranges, const GaussRec* recs,
                     const float* stats, int64_t stats_stride, float beta2, float beta3,
                     const float* feats, int nf, float* out, Control* ctrl, cudaStream_t st);

// profiling.cu
void launch_wait_selftest(unsigned long long limit_ns, uint32_t* status,
                          unsigned long long* elapsed_ns, cudaStream_t st);

}  // namespace fe
