"""Continuous-batching render server: a Python front end of the native server (``fe_server_*``).

Requests (a scene of Gaussians plus 1..k cameras; optionally target silhouettes, which turns the
request into forward + backward of the silhouette binary cross-entropy, as the reference's
shape-from-silhouette loop computes with ``jax.grad``, shape_from_silhouette.ipynb cell 12)
arrive at any time through ``submit`` and complete through futures. The batching runs in the
library's own lane threads (no Python, no GIL): each lane has a CUDA stream and a reusable batch
plan; a free lane takes the queued requests in arrival order while they fit its view and pixel
limits and the HBM budget (estimated device bytes of all in-flight batches), renders them as one
batch, evaluates the loss and backward of the backward requests in the same batch, and writes
every output straight into the request's own NumPy arrays. This front end validates requests,
allocates their outputs (one pinned block per request, recycled through torch's pinned-memory
cache once the client drops the result), keeps their arrays alive until completion and resolves
the futures from one collector thread.

A request's results do not depend on which other requests shared its batch beyond float32
rounding (tested to 1e-6).
"""

from __future__ import annotations

import concurrent.futures
import ctypes
import dataclasses
import math
import threading

import numpy as np
import torch

from . import _native as N

__all__ = ["RenderRequest", "RenderResult", "RenderServer", "estimate_footprint",
           "bce_alpha_grad", "bce_terms"]

CLIP_ALPHA = 3e-8


@dataclasses.dataclass
class RenderRequest:
    means: np.ndarray                 # (N, 3) float32
    prec: np.ndarray                  # (N, 3, 3) float32, upper-triangular factor
    logw: np.ndarray                  # (N,) float32
    cameras: list                     # objects with height, width, fx, fy, cx, cy, quat, trans
    targets: list | None = None       # per camera (H, W) silhouettes: forward + BCE backward

    @property
    def backward(self):
        return self.targets is not None

    @property
    def n(self):
        return int(self.means.shape[0])


@dataclasses.dataclass
class RenderResult:
    depth: list
    alpha: list
    loss: float | None
    grad_means: np.ndarray | None
    grad_prec: np.ndarray | None
    grad_logw: np.ndarray | None
    submitted: float
    started: float
    finished: float

    @property
    def latency(self):
        return self.finished - self.submitted


def estimate_footprint(req, tile=16):
    """Upper estimate of a request's device bytes (scene, records, keys, outputs); the same
    formula as the library's admission unit ``fe_request_footprint``."""
    n, views = req.n, len(req.cameras)
    pix = sum(c.height * c.width for c in req.cameras)
    tiles = sum(math.ceil(c.height / tile) * math.ceil(c.width / tile) for c in req.cameras)
    keys = min(n * tiles, n * views * 64)
    per_pix = 8 + (12 + 16 + 8 if req.backward else 0)
    return 52 * n + views * n * (96 + 16 + (96 if req.backward else 0)) + 88 * keys + per_pix * pix


def bce_terms(alpha, target):
    """Per-pixel silhouette BCE -(t log a + (1-t) log(1-a)) with a clamped to [3e-8, 1-3e-8]
    (shape_from_silhouette.ipynb cell 12) and its derivative in alpha (zero where the clamp is
    active), both float64.

    Evaluated in float64: in float32 the upper bound 1-3e-8 rounds to 1.0, so the clamp would
    leave saturated pixels (alpha == 1.0, which the render produces once the summed weight
    exceeds ~17) at log(0) = -inf."""
    a64 = alpha.double()
    t64 = target.double()
    a = a64.clamp(CLIP_ALPHA, 1.0 - CLIP_ALPHA)
    terms = -(t64 * torch.log(a) + (1.0 - t64) * torch.log(1.0 - a))
    inside = (a64 > CLIP_ALPHA) & (a64 < 1.0 - CLIP_ALPHA)
    d = torch.where(inside, -t64 / a + (1.0 - t64) / (1.0 - a), torch.zeros_like(a))
    return terms, d


def bce_alpha_grad(alpha, target, count):
    """Loss sum and float32 gradient of mean-over-``count`` BCE (see ``bce_terms``)."""
    terms, d = bce_terms(alpha, target)
    return terms.sum(), (d / count).float()


def _validate(req):
    """Reject a malformed request at submission, before it can share a batch with others."""
    n = req.n
    if req.means.shape != (n, 3) or np.shape(req.prec) != (n, 3, 3) or np.shape(req.logw) != (n,):
        raise ValueError("means, prec and logw must have shapes (N,3), (N,3,3) and (N,)")
    if not req.cameras:
        raise ValueError("a request needs at least one camera")
    for c in req.cameras:
        if not (int(c.height) >= 1 and int(c.width) >= 1):
            raise ValueError("camera image sizes must be positive")
        if not (math.isfinite(c.fx) and math.isfinite(c.fy) and c.fx != 0 and c.fy != 0):
            raise ValueError("camera focal lengths must be finite and non-zero")
    if req.targets is not None:
        if len(req.targets) != len(req.cameras):
            raise ValueError("one target silhouette per camera")
        for t, c in zip(req.targets, req.cameras):
            if np.shape(t) != (c.height, c.width):
                raise ValueError("target silhouette shape must be (height, width) of its camera")


def _view_table(req):
    """The request's cameras as an ``fe_view`` structured array (scene and flags set per batch)."""
    cams = req.cameras
    v = np.zeros(len(cams), N.VIEW_DTYPE)
    v["height"] = [c.height for c in cams]
    v["width"] = [c.width for c in cams]
    v["fx"] = [c.fx for c in cams]
    v["fy"] = [c.fy for c in cams]
    v["cx"] = [c.cx for c in cams]
    v["cy"] = [c.cy for c in cams]
    v["quat"] = np.asarray([np.asarray(c.quat, np.float32) for c in cams]).reshape(-1, 4)
    v["trans"] = np.asarray([np.asarray(c.trans, np.float32) for c in cams]).reshape(-1, 3)
    if not req.backward:
        v["flags"] = N.FE_VIEW_NO_GRAD
    return v


class RenderServer:
    def __init__(self, device=None, hbm_budget_bytes=16 << 30, max_batch_views=1024,
                 max_batch_pixels=48 << 20, lanes=2, tile=(16, 16), px=0, chunk=0,
                 beta2=21.4, beta3=2.66, cull="eps", cull_param=None):
        dev = torch.device("cuda" if device is None else device)
        if dev.type != "cuda":
            raise ValueError(f"RenderServer needs a CUDA device, got {dev}")
        self.device = dev if dev.index is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.tile = tuple(tile)
        lib = N.load()
        cfg = N.ServerConfig()
        lib.fe_server_config_init(ctypes.byref(cfg))
        cfg.lanes = int(lanes)
        cfg.max_batch_views = int(max_batch_views)
        cfg.max_batch_pixels = int(max_batch_pixels)
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.desc = N.make_desc(0, 1, 1, 1.0, 1.0, 0.0, 0.0, beta2, beta3, cull, cull_param, tile,
                               flags=N.flag_chunk(chunk), px=px)
        h = ctypes.c_void_p()
        N.check(lib.fe_server_create(ctypes.byref(cfg), self.device.index, ctypes.byref(h)))
        self._h = h
        self._lock = threading.Lock()
        self._inflight = {}   # user tag -> (future, request, outputs, keep-alive objects)
        self._tag = 0
        self._closed = False
        self._collector = threading.Thread(target=self._collect, daemon=True)
        self._collector.start()

    # -- submission ------------------------------------------------------------------------------
    def submit(self, req: RenderRequest) -> concurrent.futures.Future:
        _validate(req)
        if self._closed:
            raise RuntimeError("server is closed")
        n = req.n
        views = _view_table(req)
        sizes = (views["height"].astype(np.int64) * views["width"])
        pixels = int(sizes.sum())
        # One pinned block per request: [loss (f64) | depth | alpha | grads] for the outputs, then
        # [means | prec | logw | targets] for the inputs, copied in here on the submitting
        # thread. The lanes' copies from and into it are then asynchronous DMA at full link speed
        # (a copy from pageable memory is staged by the driver and holds the lane), and the block
        # returns to torch's pinned-memory cache once the result arrays are dropped.
        n_out = 2 * pixels + ((2 + 13 * n) if req.backward else 0)
        n_in = 13 * n + (pixels if req.backward else 0)
        block = torch.empty(n_out + n_in, dtype=torch.float32, pin_memory=True).numpy()
        o = 2 if req.backward else 0
        out = {"depth": block[o:o + pixels], "alpha": block[o + pixels:o + 2 * pixels]}
        if req.backward:
            g = o + 2 * pixels
            out.update(loss=block[0:2].view(np.float64),
                       grad_means=block[g:g + 3 * n].reshape(n, 3),
                       grad_prec=block[g + 3 * n:g + 12 * n].reshape(n, 3, 3),
                       grad_logw=block[g + 12 * n:g + 13 * n])
        i = n_out
        means = block[i:i + 3 * n].reshape(n, 3)
        prec = block[i + 3 * n:i + 12 * n].reshape(n, 3, 3)
        logw = block[i + 12 * n:i + 13 * n]
        np.copyto(means, req.means, casting="same_kind")
        np.copyto(prec, req.prec, casting="same_kind")
        np.copyto(logw, req.logw, casting="same_kind")
        keep = [views]
        r = N.Request()
        r.n_gaussians, r.n_views = n, len(req.cameras)
        r.means, r.prec, r.logw = means.ctypes.data, prec.ctypes.data, logw.ctypes.data
        r.views = views.ctypes.data
        r.depth, r.alpha = out["depth"].ctypes.data, out["alpha"].ctypes.data
        if req.backward:
            targets = []
            t0 = i + 13 * n
            for t, hw in zip(req.targets, sizes.tolist()):
                dst = block[t0:t0 + hw]
                np.copyto(dst, np.asarray(t).reshape(-1), casting="same_kind")
                targets.append(dst)
                t0 += hw
            tptr = (ctypes.c_void_p * len(targets))(*[t.ctypes.data for t in targets])
            keep += [tptr]
            r.targets = ctypes.cast(tptr, ctypes.c_void_p)
            r.grad_means = out["grad_means"].ctypes.data
            r.grad_prec = out["grad_prec"].ctypes.data
            r.grad_logw = out["grad_logw"].ctypes.data
            r.loss = out["loss"].ctypes.data
        fut = concurrent.futures.Future()
        with self._lock:
            self._tag += 1
            tag = self._tag
            self._inflight[tag] = (fut, req, out, keep)
        r.user_tag = tag
        rid = ctypes.c_uint64()
        rc = N.load().fe_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid))
        if rc != 0:
            with self._lock:
                self._inflight.pop(tag, None)
            msg = N.load().fe_last_error_message().decode(errors="replace")
            if rc == N.FE_ERR_OUT_OF_MEMORY:
                fut.set_exception(MemoryError(msg))
                return fut
            raise N.FEError(rc, msg)
        return fut

    # -- completions -----------------------------------------------------------------------------
    def _collect(self):
        lib = N.load()
        buf = (N.Completion * 64)()
        count = ctypes.c_int32()
        while True:
            N.check(lib.fe_server_wait(self._h, buf, 64, 200, ctypes.byref(count)))
            if count.value < 0:
                return
            for i in range(count.value):
                c = buf[i]
                with self._lock:
                    fut, req, out, _ = self._inflight.pop(c.user_tag)
                if c.status != 0:
                    fut.set_exception(N.FEError(c.status, c.message.decode(errors="replace")))
                    continue
                d_list, a_list, o = [], [], 0
                for cam in req.cameras:
                    hw = cam.height * cam.width
                    d_list.append(out["depth"][o:o + hw].reshape(cam.height, cam.width))
                    a_list.append(out["alpha"][o:o + hw].reshape(cam.height, cam.width))
                    o += hw
                res = RenderResult(d_list, a_list, None, None, None, None, c.submitted_s,
                                   c.started_s, c.finished_s)
                if req.backward:
                    res.loss = float(out["loss"][0])
                    res.grad_means = out["grad_means"]
                    res.grad_prec = out["grad_prec"]
                    res.grad_logw = out["grad_logw"]
                fut.set_result(res)

    # -- reporting and shutdown ----------------------------------------------------------------
    def stats(self):
        st = N.ServerStats()
        N.check(N.load().fe_server_stats_get(self._h, ctypes.byref(st)))
        return {"submitted": st.submitted, "completed": st.completed, "renders": st.renders,
                "batches": st.batches, "queued": st.queued, "p50_s": st.p50_latency_s,
                "p99_s": st.p99_latency_s, "busy_s": st.busy_s,
                "phase_s": dict(zip(self.PHASES, [round(x, 6) for x in st.phase_s]))}

    PHASES = ("upload", "plan", "forward", "loss_backward", "download", "finish")

    def reset_stats(self):
        """Forget latencies and counters (e.g. after a warm-up)."""
        N.load().fe_server_stats_reset(self._h)

    def close(self):
        if self._closed:
            return
        self._closed = True
        lib = N.load()
        N.check(lib.fe_server_close(self._h))   # finishes the queued requests
        self._collector.join()
        lib.fe_server_destroy(self._h)
        self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
