"""Autotuner for the blend configuration of batched renders.

Three knobs change the work and its mapping onto the GPU:

* ``tile``  -- screen tile of the binning and of one blend work item (8x8, 16x16 or 32x8):
  smaller tiles cull more precisely (fewer evaluations) but produce more keys to emit and
  more tile records to build;
* ``px``    -- pixels of one tile row per thread (1, 2, 4): shares each record's shared-memory
  loads and row-constant polynomial terms across more evaluations, at the cost of registers;
* ``chunk`` -- record pairs per shared-memory stage of the blend's record ring (8, 16, 32);
* ``heavy_first`` -- whether the blend takes the tiles with the most keys first (tried on the
  fastest of the above): it shortens the persistent schedule's tail on batches of a few heavy
  tiles per CTA and costs time where light tiles dominate.

``Autotuner.tune`` times every candidate on the actual batch (median of per-stage CUDA-event
timings of the whole pipeline, not just the blend) and caches the fastest per workload bucket
(mean pixels per view, mean Gaussians per view and number of views, each on a log2 scale) in a
JSON file (``FE_AUTOTUNE_CACHE`` or ``~/.cache/fuzzy_ellipses/autotune.json``).

``target="host"`` tunes the host-to-host call instead (``Batch.forward_host`` into pinned
outputs, which the blend stores into through their device mapping, tiles in index order): the
host link, not the blend, bounds it, and tiles with longer rows (32x8: 128-byte row segments)
use that link better. Its entries are cached under the bucket with a ``_host`` suffix.
"""

from __future__ import annotations

import json
import math
import os
import statistics
import threading

DEFAULT = {"tile": (16, 16), "px": 4, "chunk": 16, "heavy_first": False}

CANDIDATES = [
    ((8, 8), 1, 16), ((8, 8), 2, 8), ((8, 8), 2, 16),
    ((16, 16), 2, 16), ((16, 16), 4, 8), ((16, 16), 4, 16), ((16, 16), 4, 32),
    ((32, 8), 2, 16), ((32, 8), 4, 16), ((32, 8), 4, 32),
]


def bucket(scenes, views):
    """Workload bucket of a batch: log2 classes of pixels per view, Gaussians per view, views."""
    n_of = {i: n for i, (_, n) in enumerate(scenes)}
    pix = sum(int(v["height"]) * int(v["width"]) for v in views) / max(1, len(views))
    gau = sum(n_of[int(v["scene"])] for v in views) / max(1, len(views))
    return (f"p{round(math.log2(max(pix, 1)))}_n{round(math.log2(gau + 1))}"
            f"_v{min(10, int(math.log2(max(1, len(views)))))}")


def _cache_path():
    return os.environ.get("FE_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "fuzzy_ellipses",
                                       "autotune.json"))


class Autotuner:
    def __init__(self, path=None, persist=True):
        self.path = path or _cache_path()
        self.persist = persist
        self._lock = threading.Lock()
        self.table = {}
        if persist and os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.table = json.load(f)
            except (OSError, ValueError):
                self.table = {}

    def lookup(self, scenes, views, target="device"):
        """Cached best configuration for the batch's bucket, or the default."""
        e = self.table.get(bucket(scenes, views) + ("_host" if target == "host" else ""))
        if not e:
            return dict(DEFAULT)
        return {"tile": tuple(e["tile"]), "px": e["px"], "chunk": e["chunk"],
                "heavy_first": bool(e.get("heavy_first", False))}

    def tune(self, scenes, views, means, prec, logw, candidates=CANDIDATES, reps=5,
             target="device", **batch_kw):
        """Time every candidate on this batch; cache and return the fastest configuration.
        ``target="host"`` times the host-to-host call into pinned outputs instead."""
        import torch

        from . import _native as N
        from .api import Batch

        if target == "host":
            host_in = [t.detach().cpu().contiguous().float().pin_memory()
                       for t in (means, prec, logw)]

        def time_device(b):
            depth = torch.empty(b.n_pixels, device=means.device)
            alpha = torch.empty(b.n_pixels, device=means.device)
            b.forward(means, prec, logw, depth, alpha)
            totals, stages = [], []
            for _ in range(reps):
                _, _, ms = b.forward_timed(means, prec, logw, depth, alpha)
                totals.append(sum(ms.values()))
                stages.append(ms)
            return statistics.median(totals), statistics.median(s["blend"] for s in stages)

        def time_host(b):
            # The call's device span on the caller's stream (it joins every stream it uses back
            # into that one), from the C ABI as a host caller makes it.
            lib = N.load()
            out = torch.empty(2 * b.n_pixels, dtype=torch.float32).pin_memory()
            args = (b._h, host_in[0].data_ptr(), host_in[1].data_ptr(), host_in[2].data_ptr(),
                    out.data_ptr(), out.data_ptr() + 4 * b.n_pixels)
            st = torch.cuda.current_stream()
            N.check(lib.fe_batch_fwd_host(*args, st.cuda_stream))
            st.synchronize()
            times = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                N.check(lib.fe_batch_fwd_host(*args, st.cuda_stream))
                e1.record(st)
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            return statistics.median(times), None

        def time_one(tile, px, chunk, heavy_first):
            b = Batch(scenes, views, tile=tile, px=px, chunk=chunk, heavy_first=heavy_first,
                      **batch_kw)
            ms, blend_ms = (time_host if target == "host" else time_device)(b)
            b.close()
            return {"tile": list(tile), "px": px, "chunk": chunk, "heavy_first": heavy_first,
                    "ms": ms, "blend_ms": blend_ms}

        results = [time_one(tile, px, chunk, False) for tile, px, chunk in candidates]
        best = min(results, key=lambda r: r["ms"])
        if target != "host":  # (the host path's direct stores take tiles in index order)
            results.append(time_one(tuple(best["tile"]), best["px"], best["chunk"], True))
            best = min(results, key=lambda r: r["ms"])
        key = bucket(scenes, views) + ("_host" if target == "host" else "")
        with self._lock:
            self.table[key] = {"tile": best["tile"], "px": best["px"], "chunk": best["chunk"],
                               "heavy_first": best["heavy_first"], "ms": best["ms"]}
            if self.persist:
                try:
                    os.makedirs(os.path.dirname(self.path), exist_ok=True)
                    tmp = self.path + ".tmp"
                    with open(tmp, "w") as f:
                        json.dump(self.table, f, indent=1)
                    os.replace(tmp, self.path)
                except OSError:
                    pass
        return {"tile": tuple(best["tile"]), "px": best["px"], "chunk": best["chunk"],
                "heavy_first": best["heavy_first"], "ms": best["ms"], "candidates": results,
                "bucket": key}
