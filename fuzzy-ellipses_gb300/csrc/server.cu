// server.cu -- continuous-batching render server (C ABI fe_server_*, include/fuzzy_ellipses.h).
//
// No reference counterpart: the reference renders one camera per call
// (rasterize_main.cu:29-114). Host code only; the lanes drive the batch pipeline of api.cu
// (fe_batch_*) and the silhouette loss of loss.cu.
//
// Life of a request: fe_server_submit validates it, copies its view table and target pointers,
// estimates its device footprint and queues it (no GPU work, no blocking). A lane thread that is
// free takes queued requests in arrival order while they fit its view and pixel limits and the
// HBM budget (the footprints of all in-flight batches), places backward requests first (their
// pixels and Gaussians then form leading ranges), copies the inputs from the callers' host memory
// into its device buffers on its own stream, re-plans its fe_batch, renders, evaluates the
// silhouette loss and the backward for the backward requests, copies every output straight into
// the callers' host memory, synchronises its stream and posts the completions.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fe_kernels.cuh"

namespace fe {
int set_last_error(int code, const std::string& msg);
}  // namespace fe

using fe::set_last_error;

namespace {

struct Request {
  uint64_t id = 0;
  fe_request r{};
  std::vector<fe_view> views;
  std::vector<const float*> targets;
  int64_t pixels = 0;
  int64_t bytes = 0;
  double submitted = 0;
};

// A grow-only device buffer owned by one lane.
struct LaneBuf {
  char* ptr = nullptr;
  size_t cap = 0;
  int reserve(size_t bytes, cudaStream_t st) {
    if (bytes <= cap) return FE_OK;
    if (ptr) {
      cudaStreamSynchronize(st);
      cudaFree(ptr);
      ptr = nullptr;
      cap = 0;
    }
    const size_t want = ((bytes + bytes / 4) + 255) / 256 * 256;
    if (cudaMalloc(&ptr, want) != cudaSuccess) {
      cudaGetLastError();
      return set_last_error(FE_ERR_OUT_OF_MEMORY,
                            "server lane buffer could not grow to " + std::to_string(want));
    }
    cap = want;
    return FE_OK;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

int64_t footprint(const fe_request& r, const fe_view* views, int tile_w, int tile_h) {
  const int64_t n = r.n_gaussians, nv = r.n_views;
  const bool bwd = r.targets != nullptr;
  int64_t pix = 0, tiles = 0;
  for (int i = 0; i < nv; ++i) {
    pix += (int64_t)views[i].height * views[i].width;
    tiles += (int64_t)((views[i].height + tile_h - 1) / tile_h) *
             ((views[i].width + tile_w - 1) / tile_w);
  }
  const int64_t keys = std::min(n * tiles, n * nv * 64);
  const int64_t per_pix = 8 + (bwd ? 36 : 0);
  return 52 * n + nv * n * (96 + 16 + (bwd ? 96 : 0)) + 88 * keys + per_pix * pix;
}

}  // namespace

struct fe_server {
  int device = 0;
  fe_server_config cfg{};
  int tile_w = 16, tile_h = 16;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::deque<fe_completion> done;
  int64_t in_use = 0;
  int running = 0;  // lanes still running
  bool closing = false;
  uint64_t next_id = 1;
  int64_t submitted = 0, completed = 0, renders = 0, batches = 0;
  double busy_s = 0;
  double phase_s[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> latencies;
  std::vector<std::thread> lanes;
  std::mutex close_mu;
  bool joined = false;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

// Take the next batch (blocks); empty when the server is closing and the queue is drained.
std::vector<Request*> take_batch(fe_server* s) {
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    if (!s->queue.empty()) {
      Request* head = s->queue.front();
      if (s->in_use == 0 || s->in_use + head->bytes <= s->cfg.hbm_budget_bytes) break;
    } else if (s->closing) {
      return {};
    }
    s->cv_work.wait(lk);
  }
  std::vector<Request*> batch;
  int64_t views = 0, pixels = 0;
  while (!s->queue.empty()) {
    Request* q = s->queue.front();
    if (!batch.empty() &&
        (views + q->r.n_views > s->cfg.max_batch_views ||
         pixels + q->pixels > s->cfg.max_batch_pixels ||
         s->in_use + q->bytes > s->cfg.hbm_budget_bytes))
      break;
    s->queue.pop_front();
    s->in_use += q->bytes;
    views += q->r.n_views;
    pixels += q->pixels;
    batch.push_back(q);
  }
  return batch;
}

struct Lane {
  fe_server* s;
  cudaStream_t st = nullptr;
  fe_batch* plan = nullptr;
  LaneBuf gauss, pix, tgt, grads, small;
  double phase[6] = {0, 0, 0, 0, 0, 0};
  double mark = 0;
  void tick(int p) {
    const double t = s->now();
    phase[p] += t - mark;
    mark = t;
  }

#define LANE_CUDA(call)                                                              \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return set_last_error(FE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

  int run(std::vector<Request*>& batch) {
    mark = s->now();
    std::stable_partition(batch.begin(), batch.end(),
                          [](const Request* q) { return q->r.targets != nullptr; });
    const int nr = (int)batch.size();
    int n_bwd = 0;
    while (n_bwd < nr && batch[n_bwd]->r.targets) ++n_bwd;

    std::vector<fe_scene> scenes(nr);
    std::vector<fe_view> views;
    std::vector<int64_t> goff(nr + 1, 0), poff(nr + 1, 0);
    for (int k = 0; k < nr; ++k) {
      const Request* q = batch[k];
      scenes[k].gauss_offset = goff[k];
      scenes[k].n = q->r.n_gaussians;
      scenes[k].reserved = 0;
      goff[k + 1] = goff[k] + q->r.n_gaussians;
      int64_t p = poff[k];
      for (const fe_view& v : q->views) {
        fe_view w = v;
        w.scene = k;
        w.flags = k < n_bwd ? 0u : FE_VIEW_NO_GRAD;
        w.pixel_offset = p;
        p += (int64_t)v.height * v.width;
        views.push_back(w);
      }
      poff[k + 1] = p;
    }
    const int64_t G = goff[nr], npx = poff[nr];
    const int64_t pb = poff[n_bwd], gb = goff[n_bwd];

    // Device buffers: Gaussians [means 3G | prec 9G | logw G]; pixels [depth | alpha | stats 3 |
    // galpha]; targets [pb]; grads [3G | 9G | G]; small [seg_end n_bwd (i64) | loss n_bwd (f64)].
    int rc = gauss.reserve(sizeof(float) * (size_t)std::max<int64_t>(13 * G, 1), st);
    if (rc) return rc;
    rc = pix.reserve(sizeof(float) * (size_t)(npx * (n_bwd ? 6 : 2)), st);
    if (rc) return rc;
    float* means = reinterpret_cast<float*>(gauss.ptr);
    float* prec = means + 3 * G;
    float* logw = means + 12 * G;
    float* depth = reinterpret_cast<float*>(pix.ptr);
    float* alpha = depth + npx;
    float* stats = n_bwd ? alpha + npx : nullptr;
    float* galpha = n_bwd ? alpha + 4 * npx : nullptr;
    for (int k = 0; k < nr; ++k) {
      const fe_request& r = batch[k]->r;
      const size_t n = (size_t)r.n_gaussians;
      if (!n) continue;
      LANE_CUDA(cudaMemcpyAsync(means + 3 * goff[k], r.means, 12 * n, cudaMemcpyHostToDevice, st));
      LANE_CUDA(cudaMemcpyAsync(prec + 9 * goff[k], r.prec, 36 * n, cudaMemcpyHostToDevice, st));
      LANE_CUDA(cudaMemcpyAsync(logw + goff[k], r.logw, 4 * n, cudaMemcpyHostToDevice, st));
    }
    tick(0);

    if (!plan) {
      fe_render_desc d = s->cfg.desc;
      d.flags |= FE_FLAG_EXACT_KEYS | FE_FLAG_KEEP_BINNING;  // backward right after forward
      rc = fe_batch_create(&d, scenes.data(), nr, views.data(), (int32_t)views.size(), &plan);
      if (rc) {
        plan = nullptr;
        return rc;
      }
    } else {
      rc = fe_batch_reset(plan, scenes.data(), nr, views.data(), (int32_t)views.size(), st);
      if (rc) return rc;
    }
    tick(1);
    rc = fe_batch_fwd(plan, means, prec, logw, depth, alpha, stats, st);
    if (rc) return rc;
    tick(2);

    double* loss = nullptr;
    if (n_bwd) {
      rc = tgt.reserve(sizeof(float) * (size_t)pb, st);
      if (rc) return rc;
      rc = grads.reserve(sizeof(float) * (size_t)(13 * G), st);
      if (rc) return rc;
      rc = small.reserve(16 * (size_t)n_bwd, st);
      if (rc) return rc;
      float* t = reinterpret_cast<float*>(tgt.ptr);
      for (int k = 0; k < n_bwd; ++k) {
        const Request* q = batch[k];
        int64_t o = poff[k];
        for (int i = 0; i < q->r.n_views; ++i) {
          const int64_t hw = (int64_t)q->views[i].height * q->views[i].width;
          LANE_CUDA(cudaMemcpyAsync(t + o, q->targets[i], sizeof(float) * hw,
                                    cudaMemcpyHostToDevice, st));
          o += hw;
        }
      }
      int64_t* seg_end = reinterpret_cast<int64_t*>(small.ptr);
      loss = reinterpret_cast<double*>(small.ptr + 8 * (size_t)n_bwd);
      LANE_CUDA(cudaMemcpyAsync(seg_end, poff.data() + 1, sizeof(int64_t) * n_bwd,
                                cudaMemcpyHostToDevice, st));
      rc = fe_silhouette_bce(alpha, t, seg_end, n_bwd, pb, galpha, loss, st);
      if (rc) return rc;
      if (npx > pb)
        LANE_CUDA(cudaMemsetAsync(galpha + pb, 0, sizeof(float) * (size_t)(npx - pb), st));
      float* gm = reinterpret_cast<float*>(grads.ptr);
      rc = fe_batch_bwd(plan, means, prec, logw, depth, alpha, stats, nullptr, galpha, gm,
                        gm + 3 * G, gm + 12 * G, st);
      if (rc) return rc;
      tick(3);
    }

    // Outputs straight into the callers' memory.
    for (int k = 0; k < nr; ++k) {
      const fe_request& r = batch[k]->r;
      const size_t np = (size_t)(poff[k + 1] - poff[k]);
      LANE_CUDA(cudaMemcpyAsync(r.depth, depth + poff[k], 4 * np, cudaMemcpyDeviceToHost, st));
      LANE_CUDA(cudaMemcpyAsync(r.alpha, alpha + poff[k], 4 * np, cudaMemcpyDeviceToHost, st));
      if (k < n_bwd) {
        const size_t n = (size_t)r.n_gaussians;
        const float* gm = reinterpret_cast<const float*>(grads.ptr);
        if (n && r.grad_means)
          LANE_CUDA(cudaMemcpyAsync(r.grad_means, gm + 3 * goff[k], 12 * n,
                                    cudaMemcpyDeviceToHost, st));
        if (n && r.grad_prec)
          LANE_CUDA(cudaMemcpyAsync(r.grad_prec, gm + 3 * G + 9 * goff[k], 36 * n,
                                    cudaMemcpyDeviceToHost, st));
        if (n && r.grad_logw)
          LANE_CUDA(cudaMemcpyAsync(r.grad_logw, gm + 12 * G + goff[k], 4 * n,
                                    cudaMemcpyDeviceToHost, st));
        LANE_CUDA(cudaMemcpyAsync(r.loss, loss + k, sizeof(double), cudaMemcpyDeviceToHost, st));
      }
    }
    (void)gb;
    LANE_CUDA(cudaStreamSynchronize(st));
    tick(4);
    int64_t nk = 0, wk = 0;
    uint32_t err = 0;
    rc = fe_batch_status(plan, st, &nk, &wk, &err);
    if (rc) return rc;
    if (err & FE_DEVERR_TIMEOUT)
      return set_last_error(FE_ERR_DEVICE_TIMEOUT, "a bounded device wait gave up");
    if (err & FE_DEVERR_CAPACITY)
      return set_last_error(FE_ERR_CAPACITY, "key capacity exceeded");
    tick(5);
    return FE_OK;
  }
#undef LANE_CUDA

  void main() {
    if (cudaSetDevice(s->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      st = nullptr;
    }
    for (;;) {
      std::vector<Request*> batch = take_batch(s);
      if (batch.empty()) break;
      const double started = s->now();
      int rc = st ? run(batch) : set_last_error(FE_ERR_CUDA, "lane could not create its stream");
      const std::string msg = rc ? std::string(fe_last_error_message()) : std::string();
      if (rc && st) cudaStreamSynchronize(st);  // nothing of a failed batch may still run
      const double finished = s->now();
      {
        std::lock_guard<std::mutex> lk(s->mu);
        for (Request* q : batch) {
          fe_completion c{};
          c.id = q->id;
          c.user_tag = q->r.user_tag;
          c.status = rc;
          c.n_views = q->r.n_views;
          c.submitted_s = q->submitted;
          c.started_s = started;
          c.finished_s = finished;
          std::strncpy(c.message, msg.c_str(), sizeof(c.message) - 1);
          s->done.push_back(c);
          s->in_use -= q->bytes;
          s->latencies.push_back(finished - q->submitted);
          s->completed += 1;
          s->renders += q->r.n_views;
          delete q;
        }
        s->batches += 1;
        s->busy_s += finished - started;
        for (int p = 0; p < 6; ++p) {
          s->phase_s[p] += phase[p];
          phase[p] = 0;
        }
      }
      s->cv_done.notify_all();
      s->cv_work.notify_all();
    }
    if (plan) fe_batch_destroy(plan);
    gauss.release();
    pix.release();
    tgt.release();
    grads.release();
    small.release();
    if (st) cudaStreamDestroy(st);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->running -= 1;
    }
    s->cv_done.notify_all();
  }
};

double quantile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const size_t i = std::min(v.size() - 1, (size_t)(q * (double)v.size()));
  return v[i];
}

}  // namespace

extern "C" {

void fe_server_config_init(fe_server_config* cfg) {
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->lanes = 2;
  cfg->max_batch_views = 1024;
  cfg->max_batch_pixels = INT64_C(48) << 20;
  cfg->hbm_budget_bytes = INT64_C(16) << 30;
  fe_render_desc_init(&cfg->desc, 0, 1, 1, 1.f, 1.f, 0.f, 0.f);
}

int64_t fe_request_footprint(const fe_request* req, int32_t tile_w, int32_t tile_h) {
  if (!req || !req->views || req->n_views < 1 || tile_w < 1 || tile_h < 1) return -1;
  return footprint(*req, req->views, tile_w, tile_h);
}

int fe_server_create(const fe_server_config* cfg, int device, fe_server** out) {
  if (!cfg || !out) return set_last_error(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  if (cfg->lanes < 1 || cfg->lanes > 64 || cfg->max_batch_views < 1 ||
      cfg->max_batch_pixels < 1 || cfg->hbm_budget_bytes < 1)
    return set_last_error(FE_ERR_INVALID_ARGUMENT, "bad server configuration");
  if (cfg->desc.magic != FE_DESC_MAGIC || cfg->desc.version != FE_DESC_VERSION)
    return set_last_error(FE_ERR_DESCRIPTOR, "server descriptor magic/version mismatch");
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || device < 0 || device >= n_dev) {
    cudaGetLastError();
    return set_last_error(FE_ERR_INVALID_ARGUMENT, "no such CUDA device");
  }
  fe_server* s = new fe_server();
  s->device = device;
  s->cfg = *cfg;
  s->tile_w = cfg->desc.tile_w ? cfg->desc.tile_w : 16;
  s->tile_h = cfg->desc.tile_h ? cfg->desc.tile_h : 16;
  s->t0 = std::chrono::steady_clock::now();
  s->running = cfg->lanes;
  for (int i = 0; i < cfg->lanes; ++i)
    s->lanes.emplace_back([s] {
      Lane lane{s};
      lane.main();
    });
  *out = s;
  return FE_OK;
}

int fe_server_submit(fe_server* s, const fe_request* req, uint64_t* id) {
  if (!s || !req || !id) return set_last_error(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  const fe_request& r = *req;
  if (r.n_gaussians < 0 || r.n_views < 1 || !r.views || !r.depth || !r.alpha)
    return set_last_error(FE_ERR_INVALID_ARGUMENT, "request needs views and depth/alpha outputs");
  if (r.n_gaussians > 0 && (!r.means || !r.prec || !r.logw))
    return set_last_error(FE_ERR_INVALID_ARGUMENT, "NULL Gaussian pointer");
  if (r.targets && !r.loss)
    return set_last_error(FE_ERR_INVALID_ARGUMENT, "a backward request needs a loss output");
  for (int i = 0; i < r.n_views; ++i) {
    const fe_view& v = r.views[i];
    if (v.height < 1 || v.width < 1 || !(v.fx != 0.f) || !(v.fy != 0.f) || !std::isfinite(v.fx) ||
        !std::isfinite(v.fy))
      return set_last_error(FE_ERR_INVALID_ARGUMENT, "bad camera " + std::to_string(i));
    if (r.targets && !r.targets[i])
      return set_last_error(FE_ERR_INVALID_ARGUMENT, "NULL target " + std::to_string(i));
  }
  Request* q = new Request();
  q->r = r;
  q->views.assign(r.views, r.views + r.n_views);
  q->r.views = nullptr;
  if (r.targets) {
    q->targets.assign(r.targets, r.targets + r.n_views);
    q->r.targets = q->targets.data();
  }
  for (const fe_view& v : q->views) q->pixels += (int64_t)v.height * v.width;
  q->bytes = footprint(r, q->views.data(), s->tile_w, s->tile_h);
  if (q->bytes > s->cfg.hbm_budget_bytes) {
    const int64_t b = q->bytes;
    delete q;
    return set_last_error(FE_ERR_OUT_OF_MEMORY,
                          "request needs ~" + std::to_string(b) +
                              " device bytes, over the budget " +
                              std::to_string(s->cfg.hbm_budget_bytes));
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->closing) {
      delete q;
      return set_last_error(FE_ERR_INVALID_ARGUMENT, "server is closed");
    }
    q->id = s->next_id++;
    q->submitted = s->now();
    *id = q->id;
    s->queue.push_back(q);
    s->submitted += 1;
  }
  s->cv_work.notify_one();
  return FE_OK;
}

int fe_server_wait(fe_server* s, fe_completion* out, int32_t max, int32_t timeout_ms,
                   int32_t* n_out) {
  if (!s || !out || !n_out || max < 1)
    return set_last_error(FE_ERR_INVALID_ARGUMENT, "bad wait arguments");
  std::unique_lock<std::mutex> lk(s->mu);
  auto finished = [s] { return s->closing && s->running == 0 && s->queue.empty(); };
  s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(0, timeout_ms)),
                      [&] { return !s->done.empty() || finished(); });
  int32_t n = 0;
  while (n < max && !s->done.empty()) {
    out[n++] = s->done.front();
    s->done.pop_front();
  }
  *n_out = (n == 0 && finished()) ? -1 : n;
  return FE_OK;
}

int fe_server_stats_get(fe_server* s, fe_server_stats* out) {
  if (!s || !out) return set_last_error(FE_ERR_INVALID_ARGUMENT, "NULL argument");
  std::vector<double> lat;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->renders = s->renders;
    out->batches = s->batches;
    out->queued = (int64_t)s->queue.size();
    out->busy_s = s->busy_s;
    for (int p = 0; p < 6; ++p) out->phase_s[p] = s->phase_s[p];
    lat = s->latencies;
  }
  out->p50_latency_s = quantile(lat, 0.50);
  out->p99_latency_s = quantile(std::move(lat), 0.99);
  return FE_OK;
}

void fe_server_stats_reset(fe_server* s) {
  if (!s) return;
  std::lock_guard<std::mutex> lk(s->mu);
  s->submitted = s->completed = s->renders = s->batches = 0;
  s->busy_s = 0;
  for (int p = 0; p < 6; ++p) s->phase_s[p] = 0;
  s->latencies.clear();
}

int fe_server_close(fe_server* s) {
  if (!s) return set_last_error(FE_ERR_INVALID_ARGUMENT, "NULL server");
  std::lock_guard<std::mutex> cl(s->close_mu);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->closing = true;
  }
  s->cv_work.notify_all();
  if (!s->joined) {
    for (std::thread& t : s->lanes) t.join();
    s->joined = true;
  }
  s->cv_done.notify_all();
  return FE_OK;
}

void fe_server_destroy(fe_server* s) {
  if (!s) return;
  fe_server_close(s);
  for (Request* q : s->queue) delete q;
  delete s;
}

}  // extern "C"
