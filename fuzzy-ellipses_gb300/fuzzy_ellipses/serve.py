"""Continuous-batching render server.

Requests (a scene of Gaussians plus 1..k cameras; optionally target silhouettes, which turns the
request into forward + backward of the silhouette binary cross-entropy, as the reference's
shape-from-silhouette loop computes with ``jax.grad``, shape_from_silhouette.ipynb cell 12)
arrive at any time through ``submit``. The server

* admits a request when its estimated device footprint fits the HBM budget, uploading its scene
  parameters to the device once (they stay resident until the request completes);
* runs ``lanes`` worker threads, each with its own CUDA stream and reusable batch plan
  (``Batch.reset`` grows its scratch only); a free lane takes every admitted request that fits its
  view and pixel limits, in arrival order, and renders them as one batch, so requests that arrive
  while other batches are on the GPU join the next batch and batches overlap on the device;
* returns per-request depth/alpha images (and loss and gradients) through futures and records
  each request's latency (submission to completion).

A request's results do not depend on which other requests shared its batch beyond float32
rounding (tested to 1e-6).
"""

from __future__ import annotations

import collections
import concurrent.futures
import dataclasses
import math
import threading
import time

import numpy as np
import torch

from . import api

__all__ = ["RenderRequest", "RenderResult", "RenderServer", "estimate_footprint",
           "bce_alpha_grad"]

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
    """Upper estimate of a request's device bytes (scene, records, keys, outputs)."""
    n, views = req.n, len(req.cameras)
    pix = sum(c.height * c.width for c in req.cameras)
    tiles = sum(math.ceil(c.height / tile) * math.ceil(c.width / tile) for c in req.cameras)
    keys = min(n * tiles, n * views * 64)
    per_pix = 8 + (12 + 16 + 8 if req.backward else 0)
    return 52 * n + views * n * (96 + 16 + (96 if req.backward else 0)) + 88 * keys + per_pix * pix


def bce_alpha_grad(alpha, target, count):
    """d/dalpha of mean(-(t log a + (1-t) log(1-a))) with a clamped to [3e-8, 1-3e-8]
    (shape_from_silhouette.ipynb cell 12); the gradient is zero where the clamp is active.
    Returns (loss_sum, grad) with the gradient in float32.

    Evaluated in float64: in float32 the upper bound 1-3e-8 rounds to 1.0, so the clamp would
    leave saturated pixels (alpha == 1.0, which the render produces once the summed weight
    exceeds ~17) at log(0) = -inf."""
    a64 = alpha.double()
    t64 = target.double()
    a = a64.clamp(CLIP_ALPHA, 1.0 - CLIP_ALPHA)
    loss = -(t64 * torch.log(a) + (1.0 - t64) * torch.log(1.0 - a)).sum()
    inside = (a64 > CLIP_ALPHA) & (a64 < 1.0 - CLIP_ALPHA)
    g = torch.where(inside, (-t64 / a + (1.0 - t64) / (1.0 - a)) / count,
                    torch.zeros_like(a))
    return loss, g.float()


class _Admitted:
    __slots__ = ("req", "future", "submitted", "bytes", "dev", "ready", "tgt", "host")

    def __init__(self, req, future, submitted, nbytes):
        self.req, self.future, self.submitted, self.bytes = req, future, submitted, nbytes
        self.dev = None
        self.ready = None
        self.tgt = None
        self.host = None  # pinned staging, kept alive until the upload has run


class RenderServer:
    def __init__(self, device=None, hbm_budget_bytes=16 << 30, max_batch_views=1024,
                 max_batch_pixels=48 << 20, lanes=2, tile=(16, 16), px=0, chunk=0,
                 beta2=21.4, beta3=2.66, cull="eps", cull_param=None):
        self.device = (torch.device("cuda", torch.cuda.current_device()) if device is None
                       else torch.device(device))
        self.budget = int(hbm_budget_bytes)
        self.max_views = int(max_batch_views)
        self.max_pixels = int(max_batch_pixels)
        self.cfg = dict(tile=tuple(tile), px=px, chunk=chunk, beta2=beta2, beta3=beta3,
                        cull=cull, cull_param=cull_param)
        self._lock = threading.Condition()
        self._pending = collections.deque()   # waiting for budget
        self._ready = collections.deque()     # admitted, waiting for a lane
        self._in_use = 0
        self._closed = False
        self._upload_stream = torch.cuda.Stream(device=self.device)
        self.latencies = []
        self.completed = 0
        self.renders = 0
        self.batches = 0
        self._lanes = [threading.Thread(target=self._lane, args=(i,), daemon=True)
                       for i in range(lanes)]
        for t in self._lanes:
            t.start()

    # -- submission and admission ------------------------------------------------------------
    def submit(self, req: RenderRequest) -> concurrent.futures.Future:
        fut = concurrent.futures.Future()
        nbytes = estimate_footprint(req, self.cfg["tile"][0])
        item = _Admitted(req, fut, time.perf_counter(), nbytes)
        with self._lock:
            if self._closed:
                raise RuntimeError("server is closed")
            if nbytes > self.budget:
                fut.set_exception(MemoryError(
                    f"request needs ~{nbytes} device bytes, over the budget {self.budget}"))
                return fut
            self._pending.append(item)
            self._admit_locked()
        return fut

    def _admit_locked(self):
        while self._pending and self._in_use + self._pending[0].bytes <= self.budget:
            item = self._pending.popleft()
            self._in_use += item.bytes
            self._upload(item)
            self._ready.append(item)
            self._lock.notify_all()

    def _upload(self, item):
        # Scene parameters (and targets) go to the device once, on the upload stream.
        req = item.req
        with torch.cuda.stream(self._upload_stream):
            host = [torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).pin_memory()
                    for x in (req.means, req.prec, req.logw)]
            item.dev = [h.to(self.device, non_blocking=True) for h in host]
            if req.targets is not None:
                t = np.concatenate([np.asarray(x, np.float32).ravel() for x in req.targets])
                host.append(torch.from_numpy(t).pin_memory())
                item.tgt = host[-1].to(self.device, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self._upload_stream)
        item.ready = ev
        item.host = host

    # -- lanes ---------------------------------------------------------------------------------
    def _take_batch(self):
        with self._lock:
            while not self._ready and not self._closed:
                self._lock.wait()
            if not self._ready:
                return None
            batch, views, pixels = [], 0, 0
            while self._ready:
                r = self._ready[0].req
                nv = len(r.cameras)
                npx = sum(c.height * c.width for c in r.cameras)
                if batch and (views + nv > self.max_views or pixels + npx > self.max_pixels):
                    break
                batch.append(self._ready.popleft())
                views += nv
                pixels += npx
            return batch

    def _lane(self, lane_id):
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream(device=self.device)
        plan = None
        while True:
            items = self._take_batch()
            if items is None:
                break
            started = time.perf_counter()
            try:
                with torch.cuda.stream(stream):
                    plan = self._run(items, plan, stream, started)
            except Exception as e:  # deliver the failure to every request of the batch
                for it in items:
                    if not it.future.done():
                        it.future.set_exception(e)
            with self._lock:
                for it in items:
                    self._in_use -= it.bytes
                self._admit_locked()
        if plan is not None:
            plan.close()

    def _run(self, items, plan, stream, started):
        for it in items:
            stream.wait_event(it.ready)
        scenes, views, off = [], [], 0
        for si, it in enumerate(items):
            scenes.append((off, it.req.n))
            off += it.req.n
            for c in it.req.cameras:
                views.append(dict(scene=si, height=c.height, width=c.width, fx=c.fx, fy=c.fy,
                                  cx=c.cx, cy=c.cy, quat=c.quat, trans=c.trans,
                                  no_grad=not it.req.backward))
        means = torch.cat([it.dev[0] for it in items])
        prec = torch.cat([it.dev[1] for it in items])
        logw = torch.cat([it.dev[2] for it in items])
        cfg = self.cfg
        if plan is None:
            plan = api.Batch(scenes, views, cfg["beta2"], cfg["beta3"], cull=cfg["cull"],
                             cull_param=cfg["cull_param"], tile=cfg["tile"], px=cfg["px"],
                             chunk=cfg["chunk"], exact_keys=True)
        else:
            plan.reset(scenes, views)
        any_bwd = any(it.req.backward for it in items)
        npx = plan.n_pixels
        depth = torch.empty(npx, device=self.device)
        alpha = torch.empty(npx, device=self.device)
        stats = torch.empty(3 * npx, device=self.device) if any_bwd else None
        plan.forward(means, prec, logw, depth, alpha, stats)
        losses = {}
        grads = None
        if any_bwd:
            galpha = torch.zeros(npx, device=self.device)
            vi = 0
            for k, it in enumerate(items):
                nv = len(it.req.cameras)
                if it.req.backward:
                    lo = plan.pixel_offsets[vi]
                    hi = plan.pixel_offsets[vi + nv - 1] + plan.shapes[vi + nv - 1][0] * plan.shapes[vi + nv - 1][1]
                    loss, g = bce_alpha_grad(alpha[lo:hi], it.tgt, hi - lo)
                    galpha[lo:hi] = g
                    losses[k] = loss / (hi - lo)
                vi += nv
            grads = plan.backward(means, prec, logw, depth, alpha, stats, None, galpha)
        # Results to pinned host memory, then complete the futures.
        depth_h = torch.empty(npx, dtype=torch.float32, pin_memory=True)
        alpha_h = torch.empty(npx, dtype=torch.float32, pin_memory=True)
        depth_h.copy_(depth, non_blocking=True)
        alpha_h.copy_(alpha, non_blocking=True)
        if grads is not None:
            grads_h = [torch.empty(g.shape, dtype=torch.float32, pin_memory=True) for g in grads]
            for h, g in zip(grads_h, grads):
                h.copy_(g, non_blocking=True)
            loss_h = {k: v.to("cpu", non_blocking=True) for k, v in losses.items()}
        stream.synchronize()
        finished = time.perf_counter()
        dn, an = depth_h.numpy(), alpha_h.numpy()
        vi, goff = 0, 0
        for k, it in enumerate(items):
            d_list, a_list = [], []
            for c in it.req.cameras:
                lo = plan.pixel_offsets[vi]
                h, w = plan.shapes[vi]
                d_list.append(dn[lo:lo + h * w].reshape(h, w).copy())
                a_list.append(an[lo:lo + h * w].reshape(h, w).copy())
                vi += 1
            n = it.req.n
            res = RenderResult(d_list, a_list, None, None, None, None, it.submitted, started,
                               finished)
            if it.req.backward:
                res.loss = float(loss_h[k])
                res.grad_means = grads_h[0][goff:goff + n].numpy().copy()
                res.grad_prec = grads_h[1][goff:goff + n].numpy().copy()
                res.grad_logw = grads_h[2][goff:goff + n].numpy().copy()
            goff += n
            with self._lock:
                self.latencies.append(res.latency)
                self.completed += 1
                self.renders += len(it.req.cameras)
            it.future.set_result(res)
        with self._lock:
            self.batches += 1
        return plan

    # -- reporting and shutdown ----------------------------------------------------------------
    def stats(self):
        with self._lock:
            lat = sorted(self.latencies)
        q = (lambda p: lat[min(len(lat) - 1, int(p * len(lat)))] if lat else None)
        return {"completed": self.completed, "renders": self.renders, "batches": self.batches,
                "p50_s": q(0.50), "p99_s": q(0.99)}

    def close(self):
        with self._lock:
            self._closed = True
            self._lock.notify_all()
        for t in self._lanes:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
