/*
 * fuzzy_ellipses.h -- C ABI of the GB300-native fuzzy-metaball renderer.
 *
 * Every entry point takes plain pointers, sizes and a CUDA stream, returns an fe_status code
 * (never throws, exits or traps) and enqueues all of its work on the caller's stream.
 * Pointers named "d_*" are device pointers; everything else is host memory.
 *
 * The renderer computes, per pixel of a pinhole camera, the fuzzy-metaball depth (softmax of the
 * ray-Gaussian peak depths) and alpha (1 - exp(-sum of peak densities)) defined by the reference's
 * baseline/fm_render.py:11-126, restricted per screen tile to the Gaussians whose cut-off
 * ellipsoid the tile's rays can reach.
 *
 * Gaussian parameters (per scene of N Gaussians, float32, row-major):
 *   means (N,3); prec (N,3,3) in fm_render's prec_full convention -- only the upper triangle U
 *   is read and the precision is U U^T (baseline/fm_render.py:14,26); logw (N,).
 * Camera pose (fm_render.render_func_quat, baseline/fm_render.py:113-126): world rays are
 *   rays_cam @ quat_to_rot(quat), quat = (w,x,y,z) scalar first, ray origin = trans.
 * Camera rays: rays_cam(u,v) = ((u-cx)/fx, (v-cy)/fy, 1) for integer pixel (u,v), pixel index
 *   v*W + u (baseline/ycb_fmb_rotscale.py:182-189).
 */
#ifndef FUZZY_ELLIPSES_H_
#define FUZZY_ELLIPSES_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st *fe_stream_t;

/* XLA's opaque status object for api_version 2 custom calls. */
typedef struct XlaCustomCallStatus_ XlaCustomCallStatus;

typedef enum fe_status {
  FE_OK = 0,
  FE_ERR_INVALID_ARGUMENT = 1, /* a size, pointer or enum value is out of range */
  FE_ERR_DESCRIPTOR = 2,       /* descriptor has the wrong magic, version or length */
  FE_ERR_CUDA = 3,             /* a CUDA runtime call failed; see fe_last_error_message() */
  FE_ERR_OUT_OF_MEMORY = 4,    /* the scratch arena could not grow */
  FE_ERR_CAPACITY = 5,         /* device-side key count exceeded the planned capacity */
  FE_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait gave up */
  FE_ERR_UNSUPPORTED = 7,
  FE_ERR_SCRATCH_LIMIT = 8     /* request larger than the fixed scratch of the no-alloc entry */
} fe_status;

/* How far a Gaussian's screen footprint reaches (the binning cut-off). */
typedef enum fe_cull_mode {
  /* Cull where the Gaussian's peak density exp(logw - d^2/2) along a pixel ray is below
   * cull_param (default 1e-7): Mahalanobis radius k = sqrt(2*(logw - ln eps)). */
  FE_CULL_EPS = 0,
  /* Fixed radius k = cull_param standard deviations (the reference binning uses 3.0). */
  FE_CULL_NSTD = 1
} fe_cull_mode;

#define FE_DESC_MAGIC 0x31644546u /* "FEd1" */
#define FE_DESC_VERSION 1

/* Flags for fe_render_desc.flags */
#define FE_FLAG_SAVE_STATS 1u /* write per-pixel softmax statistics needed by the backward */
/* Bits 8..15 of flags: record pairs per shared-memory stage of the blend (8, 16 or 32; 0 = 32). */
#define FE_FLAG_CHUNK(pairs) (((uint32_t)(pairs) & 0xffu) << 8)
/* Batches only: size the key scratch from the device-side key count (one 8-byte readback and a
 * stream synchronisation per run) instead of the worst case (views x Gaussians x tiles). */
#define FE_FLAG_EXACT_KEYS 2u
/* Batches only: keep the binning (keys, tile records, ranges) of the last fe_batch_fwd and reuse
 * it in an fe_batch_bwd that gets the same Gaussian pointers with no fe_batch_reset in between,
 * instead of recomputing it. The caller guarantees that the Gaussian data did not change between
 * the two calls. */
#define FE_FLAG_KEEP_BINNING 4u
/* Bin with key emission + radix sort even where the tile-major binning applies (both give the
 * same keys and ranges; the flag exists to compare them). */
#define FE_FLAG_RADIX_BINNING 8u
/* Tile-major binning only: the emission also lists every tile by work class (its key count in
 * log2 buckets) and the blend takes the heaviest tiles first, which shortens the tail of the
 * persistent schedule when each CTA takes a handful of heavy tiles (16 views of 640x480: 206.7 ->
 * 198.5 us per blend) and lengthens it where light tiles dominate or the tiles barely fill the
 * GPU (measured slower on a 1135-view batch of small images and on single views); the
 * autotuner times it on the live batch. */
#define FE_FLAG_HEAVY_TILES_FIRST 0x10000u
/* Bin every Gaussian to all tiles of its footprint's bounding rectangle (the reference
 * rasterizer's rule) instead of, in each tile row, only the tiles its footprint ellipse reaches.
 * The ellipse is the set of pixels whose rays pass within the cut-off's Mahalanobis distance of
 * the mean, so the tiles dropped by default hold only pixels where the Gaussian's density is
 * below the cut-off; on 16 views of 640x480 they are a quarter of the rectangle's keys. */
#define FE_FLAG_RECT_BINNING 0x20000u

/* Render descriptor: everything a render needs besides the Gaussian and pose buffers. It is also
 * the opaque payload of the XLA custom call targets (bit-copied; the size and magic are checked).
 * Replaces RasterizeDescriptor{H,W,P,tan_fovx,tan_fovy} of the reference (rasterize_main.h:14-20,
 * packed by bindings.h:20-29). */
typedef struct fe_render_desc {
  uint32_t magic;      /* FE_DESC_MAGIC */
  uint32_t version;    /* FE_DESC_VERSION */
  int32_t n_gaussians; /* N >= 0 */
  int32_t height;      /* H >= 1 */
  int32_t width;       /* W >= 1 */
  float fx, fy, cx, cy;
  float beta2, beta3;  /* softmax temperature terms (reference default 21.4, 2.66) */
  int32_t cull_mode;   /* fe_cull_mode */
  float cull_param;    /* eps for FE_CULL_EPS, k for FE_CULL_NSTD; <= 0 selects the default */
  int32_t tile_w;      /* screen tile width/height in pixels: 8x8, 16x16 or 32x8; 0 = 16x16 */
  int32_t tile_h;
  uint32_t flags;      /* FE_FLAG_* */
  int32_t px_per_thread; /* blend pixels per thread: 1, 2 or 4 (8x8 tiles: 1 or 2); 0 = default:
                          * 2 for 8x8 tiles and for renders or batches of fewer than 3000 tiles,
                          * else 4 */
} fe_render_desc;

/* Fill d with defaults for an HxW image of n Gaussians. */
void fe_render_desc_init(fe_render_desc *d, int32_t n_gaussians, int32_t height, int32_t width,
                         float fx, float fy, float cx, float cy);

/* Forward render of one camera. Replaces the reference's XLA target body
 * RasterizeGaussiansCUDAJAX (rasterize_main.cu:29-114) and its host orchestration
 * CudaRasterizer::Rasterizer::forwardJAX (cuda_rasterizer/rasterizer_impl.cu:174-344).
 *   d_means (N,3), d_prec (N,3,3), d_logw (N), d_quat (4), d_trans (3): inputs;
 *   d_depth (H,W), d_alpha (H,W): outputs;
 *   d_stats (3,H,W) or NULL: per-pixel (max logit, softmax normaliser, density sum), required
 *     by fe_render_bwd; written when non-NULL.
 * Scratch comes from a per-(device, stream) arena that grows only; the steady state performs no
 * allocation and no host synchronisation. */
int fe_render_fwd(const fe_render_desc *desc, const float *d_means, const float *d_prec,
                  const float *d_logw, const float *d_quat, const float *d_trans, float *d_depth,
                  float *d_alpha, float *d_stats, fe_stream_t stream);

/* Backward of fe_render_fwd: given dL/ddepth and dL/dalpha (H,W) and the forward's outputs and
 * stats, writes dL/dmeans (N,3), dL/dprec (N,3,3; strictly-lower entries are 0, as jax.grad
 * through triu gives) and dL/dlogw (N). No reference counterpart: the reference differentiates
 * baseline/fm_render.py with jax.grad (notebook cell 12). */
int fe_render_bwd(const fe_render_desc *desc, const float *d_means, const float *d_prec,
                  const float *d_logw, const float *d_quat, const float *d_trans,
                  const float *d_depth, const float *d_alpha, const float *d_stats,
                  const float *d_grad_depth, const float *d_grad_alpha, float *d_grad_means,
                  float *d_grad_prec, float *d_grad_logw, fe_stream_t stream);

/* The binning fe_render_fwd performs, exposed for tests and tools: the sorted keys
 * ((tile << 32) | gaussian index, tiles of desc->tile_w x desc->tile_h in row-major order), the
 * per-tile [first, last+1) ranges (T,2; empty tiles {0,0}) and the key count. Synchronises the
 * stream once to return *h_num_keys. Its counterpart in the reference is the key list that
 * forwardJAX builds internally (cuda_rasterizer/rasterizer_impl.cu:269-302). */
int fe_render_binning(const fe_render_desc *desc, const float *d_means, const float *d_prec,
                      const float *d_logw, const float *d_quat, const float *d_trans,
                      uint64_t *d_keys, int64_t key_capacity, uint32_t *d_ranges,
                      int64_t *h_num_keys, fe_stream_t stream);

/* Softmax-weighted per-Gaussian features of an image render: out (H,W,n_features) =
 * sum_i w_i f_i with fm_render's normalised weights w (baseline/fm_render.py:95-109, which returns
 * w "to compute color, DINO features, or any other per-Gaussian property"). d_stats must come
 * from fe_render_fwd with the same descriptor, Gaussians and pose; d_features (n, n_features).
 * Recomputes the binning and evaluates each key's weight per pixel; no weight matrix is formed. */
int fe_render_features(const fe_render_desc *desc, const float *d_means, const float *d_prec,
                       const float *d_logw, const float *d_quat, const float *d_trans,
                       const float *d_stats, const float *d_features, int32_t n_features,
                       float *d_out, fe_stream_t stream);

/* XLA custom-call targets (api_version 2: status-returning), registered under the names
 * "fe_render_fwd" and "fe_render_bwd". opaque = an fe_render_desc.
 * fwd buffers: [means, prec, logw, quat, trans, depth, alpha, stats]
 * bwd buffers: [means, prec, logw, quat, trans, depth, alpha, stats, grad_depth, grad_alpha,
 *               grad_means, grad_prec, grad_logw]
 * Replaces RasterizeGaussiansCUDAJAX (rasterize_main.h:26-30, registered by ext.cpp:23-33). */
void fe_render_fwd_xla(fe_stream_t stream, void **buffers, const char *opaque, size_t opaque_len,
                       XlaCustomCallStatus *status);
void fe_render_bwd_xla(fe_stream_t stream, void **buffers, const char *opaque, size_t opaque_len,
                       XlaCustomCallStatus *status);

/* ---------------------------------------------------------------------------------------------
 * Legacy interface: the reference's own custom-call signature and descriptor.
 * --------------------------------------------------------------------------------------------- */

/* Byte-compatible with the reference's RasterizeDescriptor (rasterize_main.h:14-20). */
typedef struct fe_legacy_desc {
  int32_t image_height;
  int32_t image_width;
  int32_t P;
  float tan_fovx;
  float tan_fovy;
} fe_legacy_desc;

/* Reference-compatible binning (tile keys, sort order, tile ranges bit-exact with the reference
 * CUDA rasterizer's preprocessCUDA + getGaussianTileKeys + thrust sort + getPerTileRanges,
 * cuda_rasterizer/forward.cu:126-203 and rasterizer_impl.cu:82-152,244-302). Inputs are the
 * reference's: means (P,3) in camera frame, scales (P,3), rotations (P,4), viewmatrix and
 * projmatrix (16 floats each, column-major as the reference uses them), tan_fovx/tan_fovy,
 * n_std (rasterizer_impl.cu:154-172 picks it from P). Outputs (device): radii (P), means2d (P,2),
 * tiles_touched (P, inclusive prefix sum as the reference leaves it), keys (capacity entries;
 * the first *h_num_keys are valid and sorted), ranges (T,2) with empty tiles {0,0}.
 * The call synchronises the stream once to return *h_num_keys (as the reference does at
 * rasterizer_impl.cu:248). 8x8 tiles, as the reference's config.h:8-9. */
int fe_reference_binning(int32_t P, int32_t height, int32_t width, float n_std,
                         const float *d_means, const float *d_scales, const float *d_rotations,
                         const float *d_viewmatrix, const float *d_projmatrix, float tan_fovx,
                         float tan_fovy, int32_t *d_radii, float *d_means2d,
                         uint32_t *d_tiles_touched, uint64_t *d_keys, int64_t key_capacity,
                         uint32_t *d_ranges, int64_t *h_num_keys, fe_stream_t stream);

/* The reference's XLA target signature, same buffer order (rasterize_main.cu:54-68):
 * [means3D, weights, scales, rotations, camera_rays, camera_rot, camera_trans, viewmatrix,
 *  projmatrix, out_z, out_alpha], opaque = fe_legacy_desc. Binning follows the reference
 * (fe_reference_binning); depth/alpha are computed with this library's blend from the same keys,
 * using the precision implied by (scales, rotations) and pinhole rays recovered from
 * camera_rays (rays must be of the form ((u-cx)/fx, (v-cy)/fy, 1), as every reference caller
 * passes). api_version 2. */
void fe_rasterize_legacy_xla(fe_stream_t stream, void **buffers, const char *opaque,
                             size_t opaque_len, XlaCustomCallStatus *status);
/* The same as fe_rasterize_legacy_xla with named pointers, for ctypes / torch callers. */
int fe_rasterize_legacy(const fe_legacy_desc *desc, const float *d_means, const float *d_weights,
                        const float *d_scales, const float *d_rotations, const float *d_camera_rays,
                        const float *d_camera_rot, const float *d_camera_trans,
                        const float *d_viewmatrix, const float *d_projmatrix, float *d_out_z,
                        float *d_out_alpha, fe_stream_t stream);

/* ---------------------------------------------------------------------------------------------
 * Batched renders: many scenes and cameras in one launch sequence.
 * --------------------------------------------------------------------------------------------- */

/* One render of a batch: a scene (a slice of the concatenated Gaussian arrays) seen by a camera. */
typedef struct fe_view {
  int32_t scene;          /* index into the scene table */
  int32_t height, width;
  float fx, fy, cx, cy;
  float quat[4];          /* scalar first */
  float trans[3];
  uint32_t flags;         /* FE_VIEW_* */
  int64_t pixel_offset;   /* first pixel of this render in the batch output buffers */
} fe_view;

/* fe_view.flags: the backward skips this view (its cotangents are zero). */
#define FE_VIEW_NO_GRAD 1u

typedef struct fe_scene {
  int64_t gauss_offset;   /* first Gaussian of the scene in the concatenated arrays */
  int32_t n;              /* Gaussians in the scene */
  int32_t reserved;
} fe_scene;

typedef struct fe_batch fe_batch;

/* Plan a batch on the current device: uploads the view/scene tables and reserves scratch for the
 * worst-case key count (so the batch runs with no host synchronisation and can be captured in a
 * CUDA graph). desc supplies beta2/beta3, cull mode/param and tile shape; its size/intrinsics
 * fields are ignored. */
int fe_batch_create(const fe_render_desc *desc, const fe_scene *scenes, int32_t n_scenes,
                    const fe_view *views, int32_t n_views, fe_batch **out);
/* Re-plan an existing batch for new scenes/views, reusing (and only growing) its device buffers.
 * Does not synchronise: the new tables are uploaded on `stream`, ordered after the batch's
 * previous runs, so a batch's runs and resets must be issued on one stream (or ordered by the
 * caller). Buffers that must grow wait for `stream` before the old ones are freed. */
int fe_batch_reset(fe_batch *b, const fe_scene *scenes, int32_t n_scenes, const fe_view *views,
                   int32_t n_views, fe_stream_t stream);
void fe_batch_destroy(fe_batch *b);
/* Total output pixels of the batch (sum of H*W). */
int64_t fe_batch_pixels(const fe_batch *b);
/* Scratch bytes reserved by the batch. */
int64_t fe_batch_scratch_bytes(const fe_batch *b);
/* Forward render of every view. Outputs are indexed by fe_view.pixel_offset. d_stats (3, pixels)
 * or NULL. */
int fe_batch_fwd(fe_batch *b, const float *d_means, const float *d_prec, const float *d_logw,
                 float *d_depth, float *d_alpha, float *d_stats, fe_stream_t stream);
/* fe_batch_fwd from HOST memory to HOST memory: h_means (n,3), h_prec (n,3,3), h_logw (n) and
 * the outputs h_depth, h_alpha. When h_depth and h_alpha are pinned host memory mapped into the
 * device's address space (cudaHostAlloc / cudaHostRegister; every pinned allocation on a
 * unified-addressing system), the blend stores the images through that mapping as it renders,
 * in one launch on `stream`, so they cross the host link while later tiles render and no copy
 * follows the last tile (environment FE_HOST_DIRECT=0 turns this off); pinned inputs are then
 * read by the preprocess through their mapping too, else copied in on `stream`. Otherwise the
 * Gaussians are copied in on `stream` and the blend runs
 * in bands of whole tile rows (alternating between `stream` and a second stream of the batch, so
 * one band's tail overlaps the next band's start) and each band's depth and alpha rows are
 * copied back on a copy stream of the batch as soon as the band is done, so only the last
 * band's copy follows the render; pageable buffers work but the calling thread waits in the
 * copies. Returns once everything is enqueued; synchronising `stream` makes the outputs
 * readable. The outputs are indexed by fe_view.pixel_offset. */
int fe_batch_fwd_host(fe_batch *b, const float *h_means, const float *h_prec, const float *h_logw,
                      float *h_depth, float *h_alpha, fe_stream_t stream);
/* Backward of fe_batch_fwd; gradients are accumulated over all views of a scene. */
int fe_batch_bwd(fe_batch *b, const float *d_means, const float *d_prec, const float *d_logw,
                 const float *d_depth, const float *d_alpha, const float *d_stats,
                 const float *d_grad_depth, const float *d_grad_alpha, float *d_grad_means,
                 float *d_grad_prec, float *d_grad_logw, fe_stream_t stream);
/* Synchronise `stream` and report the last run's key count (clamped to the planned capacity),
 * the count it needed, and its device error word (FE_DEVERR_*). */
int fe_batch_status(fe_batch *b, fe_stream_t stream, int64_t *num_keys, int64_t *want_keys,
                    uint32_t *device_error);

/* ---------------------------------------------------------------------------------------------
 * Diagnostics and measurement
 * --------------------------------------------------------------------------------------------- */

/* fe_batch_fwd with a CUDA event recorded between stages on `stream`; synchronises and writes the
 * six stage durations in milliseconds to stage_ms: preprocess, scan, key emission, sort, tile
 * ranges, blend (the tile-major binning emits keys and ranges in one kernel: its scan, sort and
 * ranges stages are empty). The reference times only its blend, with events
 * (cuda_rasterizer/rasterizer_impl.cu:314-341). */
int fe_batch_fwd_timed(fe_batch *b, const float *d_means, const float *d_prec, const float *d_logw,
                       float *d_depth, float *d_alpha, float *d_stats, float *stage_ms,
                       fe_stream_t stream);
/* Number of kernels one fe_batch_fwd launches. */
int fe_batch_launch_count(const fe_batch *b);
/* ---------------------------------------------------------------------------------------------
 * Continuous-batching render server. No reference counterpart: the reference renders one camera
 * per call (rasterize_main.cu:29-114) and leaves batching and serving to the caller.
 * Requests (one scene of Gaussians, 1..k cameras, optionally per-camera target silhouettes that
 * add the silhouette-BCE loss and its gradients) are queued by fe_server_submit and rendered by
 * `lanes` worker threads, each with its own CUDA stream and batch plan: a free lane takes the
 * queued requests in arrival order while they fit its view and pixel limits and the HBM budget,
 * and renders them as one batch (fe_batch_*), so concurrent requests share launches. Inputs are
 * read from, and outputs written to, the caller's host memory directly; both must stay valid
 * until the request's completion is returned by fe_server_wait.
 * ------------------------------------------------------------------------------------------- */
typedef struct fe_server fe_server;

typedef struct fe_server_config {
  int32_t lanes;             /* worker threads (streams), >= 1 */
  int32_t max_batch_views;   /* cameras per batch */
  int64_t max_batch_pixels;  /* output pixels per batch */
  int64_t hbm_budget_bytes;  /* estimated device bytes of all in-flight batches together */
  fe_render_desc desc;       /* beta2/beta3, cull, tile, px_per_thread, chunk flags; sizes ignored */
} fe_server_config;

typedef struct fe_request {
  int32_t n_gaussians;
  int32_t n_views;
  const float *means;              /* host (N,3) */
  const float *prec;               /* host (N,3,3) upper-triangular factor */
  const float *logw;               /* host (N) */
  const fe_view *views;            /* n_views cameras; scene, flags, pixel_offset are ignored */
  const float *const *targets;     /* NULL: forward only; else n_views host (H,W) silhouettes */
  float *depth;                    /* host output: the renders' depth, back to back */
  float *alpha;                    /* host output: the renders' alpha, back to back */
  float *grad_means;               /* host outputs with targets (may be NULL): dL/dmeans (N,3), */
  float *grad_prec;                /*   dL/dprec (N,3,3), dL/dlogw (N) of the mean BCE over the */
  float *grad_logw;                /*   request's pixels */
  double *loss;                    /* host output with targets: the mean BCE (1 value) */
  uint64_t user_tag;               /* returned in the completion */
} fe_request;

typedef struct fe_completion {
  uint64_t id;                /* from fe_server_submit */
  uint64_t user_tag;
  int32_t status;             /* FE_OK or the failure of the request's batch */
  int32_t n_views;
  double submitted_s, started_s, finished_s;  /* seconds since the server was created */
  char message[160];          /* failure message ("" on success) */
} fe_completion;

typedef struct fe_server_stats {
  int64_t submitted, completed, renders, batches, queued;
  double p50_latency_s, p99_latency_s;  /* over completed requests since the last reset */
  double busy_s;                        /* lane time spent in batches, summed over lanes */
  /* lane time by phase, summed over lanes: 0 upload, 1 plan, 2 forward (with its key-count
   * readback), 3 loss + backward, 4 download (copies into the callers' memory), 5 finish */
  double phase_s[6];
} fe_server_stats;

/* Defaults: 2 lanes, 1024 views and 48 Mi pixels per batch, 16 GiB budget, fe_render_desc_init. */
void fe_server_config_init(fe_server_config *cfg);
/* Starts the lanes on CUDA device `device`. */
int fe_server_create(const fe_server_config *cfg, int device, fe_server **out);
/* Validates and queues a request; *id identifies its completion. FE_ERR_OUT_OF_MEMORY when the
 * request alone exceeds the HBM budget (see fe_request_footprint). Never blocks on the GPU. */
int fe_server_submit(fe_server *s, const fe_request *req, uint64_t *id);
/* Up to `max` completions into `out`, waiting up to timeout_ms for the first; *n_out = count,
 * or -1 once the server is closed and every request has completed and been returned. */
int fe_server_wait(fe_server *s, fe_completion *out, int32_t max, int32_t timeout_ms,
                   int32_t *n_out);
int fe_server_stats_get(fe_server *s, fe_server_stats *out);
void fe_server_stats_reset(fe_server *s);
/* Stop accepting requests, finish the queued ones and stop the lanes (blocks). */
int fe_server_close(fe_server *s);
/* Close (if needed) and free the server; completions not yet returned are dropped. */
void fe_server_destroy(fe_server *s);
/* Estimated device bytes of a request (the admission unit). Host only. */
int64_t fe_request_footprint(const fe_request *req, int32_t tile_w, int32_t tile_h);

/* Pipe-throughput microbenchmark: kind 0 = FP32 FMA, kind 1 = MUFU ex2, kind 2 = packed f32x2
 * FMA (two FMAs per instruction); operations per second.
 * Allocates (and frees) 1 MiB of scratch. No reference counterpart. */
int fe_bench_peak(int kind, int iters, double *ops_per_second, fe_stream_t stream);

/* Forward render of one view that allocates nothing: the same pipeline and results as
 * fe_render_fwd (same arguments), with all scratch in a fixed file-scope device array of
 * FE_NOALLOC_SCRATCH_BYTES per device instead of the per-(device, stream) arena.
 * No counterpart in the reference (whose forwardJAX, rasterizer_impl.cu:174-344, takes scratch
 * from a GpuMemoryPool that calls cudaFree/cudaMalloc whenever a request outgrows it,
 * rasterizer_impl.cu:47-79). For callers that cannot allocate during a call, e.g. an XLA custom
 * call under XLA's preallocating allocator.
 *   Limit: requests whose worst-case scratch (n_gaussians x tiles keys) exceeds
 *     FE_NOALLOC_SCRATCH_BYTES return FE_ERR_SCRATCH_LIMIT before any device work (16 bytes
 *     per Gaussian-tile pair -- the key and its radix-sort twin -- plus small per-Gaussian and
 *     per-tile terms, about 8.3M pairs: 6000 Gaussians on a 640x480 image with 16x16 tiles fit,
 *     7000 do not).
 *   Set-up: the first call on a device resolves the array's address (cudaGetSymbolAddress) and
 *     loads the library's kernels; make it during set-up, before any stream capture begins.
 *   Concurrency: one scratch per device, so calls on one device must not overlap -- issue them
 *     on one stream or order them; overlapping calls race on the scratch.
 *   d_device_error: optional device word receiving the call's device-side error (FE_DEVERR_*),
 *     stream-ordered; NULL to skip. */
#define FE_NOALLOC_SCRATCH_BYTES (128u << 20)
int fe_render_fwd_noalloc(const fe_render_desc *desc, const float *d_means, const float *d_prec,
                          const float *d_logw, const float *d_quat, const float *d_trans,
                          float *d_depth, float *d_alpha, float *d_stats, uint32_t *d_device_error,
                          fe_stream_t stream);

/* Silhouette binary cross-entropy of renders stored back to back in one pixel buffer, the loss
 * of the reference's shape-from-silhouette loop (shape_from_silhouette.ipynb cell 12: mean over
 * pixels of -(t log a + (1-t) log(1-a)) with a clamped to [3e-8, 1-3e-8]), which the reference
 * evaluates in JAX; one kernel here. Render s owns pixels [d_seg_end[s-1], d_seg_end[s])
 * (d_seg_end: n_seg increasing int64 on the device, the last equal to n_pix).
 * Writes d_loss[s] = render s's mean loss (float64, n_seg) and d_galpha = dL_s/dalpha per pixel
 * (zero where the clamp is active), the cotangent fe_render_bwd / fe_batch_bwd take. */
int fe_silhouette_bce(const float *d_alpha, const float *d_target, const int64_t *d_seg_end,
                      int32_t n_seg, int64_t n_pix, float *d_galpha, double *d_loss,
                      fe_stream_t stream);

/* Log-likelihood of 3-D points under the Gaussian mixture: the reference's log_likelihood
 * (baseline/fm_render.py:231-259), which evaluates it in JAX. For Gaussians i (d_means (n,3),
 * d_prec (n,3,3) with only the upper triangle read, Sigma^-1 = U U^T, d_logw (n) unnormalised
 * log weights) and points j (d_points (n_points,3)):
 *   r_ij = log softmax(logw)_i + log|det U_i| - (|U_i^T (mu_i - x_j)|^2 + 3 log(2 pi)) / 2
 * writes d_point_ll[j] = logsumexp_i r_ij, d_res[i * n_points + j] = r_ij when d_res is not NULL
 * (the reference's second output, transposed: n x n_points), and d_total (float64) = sum_j
 * d_point_ll[j] when not NULL (the reference's first output is -d_total / n_points). Uses the
 * per-stream arena for 48 B of scratch per Gaussian. */
int fe_gmm_log_likelihood(const float *d_means, const float *d_prec, const float *d_logw,
                          int32_t n, const float *d_points, int64_t n_points, float *d_point_ll,
                          float *d_res, double *d_total, fe_stream_t stream);

/* Pixel-list render: the reference's render_func_idx_quattrans, render_func_idx_quattrans_flow
 * and render_func_quat_cam (baseline/fm_render.py:130-224, whose render_func_rays calls pass the
 * Gaussians where the rays belong; the intended argument order is used here). Two ray modes:
 *   FE_RAYS_POSE_INDEXED (render_func_idx_quattrans[_flow]): d_rays (n_rays, 4), the reference's
 *     pixel_posei rows (x, y, c, pose); the camera ray is (x inv_f, y inv_f, c) of pose `pose`
 *     (truncated to an integer and clamped to the poses);
 *   FE_RAYS_QUAT_CAM (render_func_quat_cam): d_rays (n_rays, 3), the reference's pixel_list rows
 *     (x, y, c) of the single pose 0; the camera ray is ((x - shift_x) inv_f,
 *     (y - shift_y) aspect inv_f, c) (the reference shifts by 0.5, 0.5); no flow;
 *   d_poses (n_poses, 7): quaternion (4, scalar first) and translation (3) per pose;
 *   d_features (n, n_features) or NULL: per-Gaussian features (n_features <= 16);
 * outputs per ray: d_depth, d_alpha; optional (NULL to skip): d_flow_next / d_flow_prev
 * (n_rays, 2) the flow to poses pose+1 / pose-1 (clamped), d_out_features (n_rays, n_features)
 * the softmax-weighted features, d_weights (n, n_rays) the dense softmax weights (fm_render's w).
 * Gaussians are culled per ray at the renderer's k-sigma screen bound. Uses the per-stream arena
 * (112 B per Gaussian and pose). */
typedef struct fe_pixlist_desc {
  uint32_t magic;      /* FE_DESC_MAGIC */
  uint32_t version;    /* FE_DESC_VERSION */
  int32_t n_gaussians;
  int32_t n_poses;
  int64_t n_rays;
  float inv_f;         /* inverse focal length (the reference's invF) */
  float beta2, beta3;
  int32_t cull_mode;   /* fe_cull_mode */
  float cull_param;
  int32_t n_features;
  /* Version 2 fields (a version-1 descriptor ends before them and renders FE_RAYS_POSE_INDEXED) */
  int32_t ray_mode;    /* fe_ray_mode */
  float aspect;        /* FE_RAYS_QUAT_CAM: y scale of the ray relative to x (1 by default) */
  float shift_x, shift_y; /* FE_RAYS_QUAT_CAM: pixel shift subtracted first (0.5, 0.5 by default) */
} fe_pixlist_desc;

#define FE_PIXLIST_DESC_VERSION 2
typedef enum fe_ray_mode { FE_RAYS_POSE_INDEXED = 0, FE_RAYS_QUAT_CAM = 1 } fe_ray_mode;

void fe_pixlist_desc_init(fe_pixlist_desc *desc, int32_t n, int32_t n_poses, int64_t n_rays,
                          float inv_f);
int fe_render_pixels(const fe_pixlist_desc *desc, const float *d_means, const float *d_prec,
                     const float *d_logw, const float *d_poses, const float *d_rays,
                     const float *d_features, float *d_depth, float *d_alpha, float *d_flow_next,
                     float *d_flow_prev, float *d_out_features, float *d_weights,
                     fe_stream_t stream);

/* Scene-parameter adapters (device kernels, float64 inside).
 * fe_prec_from_scale_rot: the renderer's upper-triangular precision factor U (n,3,3, row-major,
 * zeros below the diagonal; U U^T = Sigma^-1) of Sigma = R(q) diag(s)^2 R(q)^T from scales (n,3)
 * and scalar-first quaternions (n,4) -- the covariance of the reference's prec_from_rotscale
 * (utils/sfs_utils.py:207-213) and CUDA rasterizer (forward.cu computeCov3D). (The reference's
 * prec_from_rotscale returns the lower factor cholesky(Sigma^-1), of which fm_render's triu keeps
 * only the diagonal; this is the factor the renderer's convention needs.)
 * fe_prec_from_scale_rot_bwd: gradients of the upper-triangle entries to scales and quaternions. */
int fe_prec_from_scale_rot(const float *d_scales, const float *d_quats, int64_t n, float *d_prec,
                           fe_stream_t stream);
int fe_prec_from_scale_rot_bwd(const float *d_scales, const float *d_quats, int64_t n,
                               const float *d_grad_prec, float *d_grad_scales,
                               float *d_grad_quats, fe_stream_t stream);
/* Rigid transform of points (n,3) by a pose d_pose = [t(3), q(4)] (scalar-first quaternion, the
 * reference's layout): out = R(q) p + t (inverse = 0; transform_points_jittable,
 * utils/sfs_utils.py:171-172) or R(q)^T p + t (inverse = 1; transform_points_by_inv_jittable,
 * :182-184). The backward writes dL/dpoints (when not NULL) and dL/dpose (7, when not NULL).
 * d_points and d_out must be 16-byte aligned (as every CUDA allocation is). */
int fe_transform_points(const float *d_points, int64_t n, const float *d_pose, int32_t inverse,
                        float *d_out, fe_stream_t stream);
int fe_transform_points_bwd(const float *d_points, int64_t n, const float *d_pose,
                            int32_t inverse, const float *d_grad_out, float *d_grad_points,
                            float *d_grad_pose, fe_stream_t stream);

/* Synchronise `stream` and return the device-side error word of the arena used by calls on that
 * stream (0 = no error; see FE_DEVERR_*), clearing it. */
int fe_check_device_status(fe_stream_t stream, uint32_t *device_error);

#define FE_DEVERR_CAPACITY 1u /* more keys than planned */
#define FE_DEVERR_TIMEOUT 2u  /* a bounded mbarrier wait gave up */

/* Failure-detection self-test (no reference counterpart): one block waits on an mbarrier that
 * nothing arrives at, through the library's bounded mbarrier wait (globaltimer limit), with the
 * limit limit_ns (1 us .. 1 s). Synchronises `stream`; *h_status receives FE_DEVERR_TIMEOUT when
 * the wait gave up (the expected outcome) and *h_elapsed_ns the time the wait took. The context
 * stays usable afterwards. */
int fe_selftest_bounded_wait(uint64_t limit_ns, uint32_t *h_status, uint64_t *h_elapsed_ns,
                             fe_stream_t stream);

/* Message for the most recent error on the calling thread. */
const char *fe_last_error_message(void);
const char *fe_status_string(int status);
/* Library version string. */
const char *fe_version(void);

#ifdef __cplusplus
}
#endif
#endif /* FUZZY_ELLIPSES_H_ */
