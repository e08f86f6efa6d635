#!/usr/bin/env python
"""Headline benchmark of the GB300 fuzzy-metaball renderer.

Workload (one "step"): forward-render the larger synthetic scene of N = 1000 Gaussians from 16
cameras of 640x480 (fx = fy = 600) spread on a 1.0 m sphere, float32, depth + alpha per pixel.
Metric: ray-Gaussian evaluations per second, counted as E = sum over the (tile, Gaussian) keys of
the pixels in the key's 8x8 tile, with the run's cut-off (peak density 1e-7) -- the algorithmic
work of the render. Renders/s and the per-call drop-in numbers are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on stdout (rank 0). Multi-GPU runs are independent replicas (no collective on the
data path); value is the whole-job aggregate.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fuzzy-ellipses_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Mray-Gaussian evals/s"
WORKLOAD = ("N=1000 Gaussians (means U[-0.3,0.3]^3 m, scales logU[0.005,0.03] m, Haar rotations, "
            "logw N(0,0.5^2)), 16 cameras 640x480 fx=fy=600 on a 1.0 m Fibonacci sphere, fp32, "
            "density cut-off 1e-7 (exact k-sigma screen bounds)")
# Algorithmic cost of one ray-Gaussian evaluation used for the blend roofline: 22 FP32 FMA-pipe
# operations (three 3x3 mat-vec products reduced to quadratic forms, the peak, the log-density,
# the logit and the three accumulations) and 3 MUFU operations (rcp and two ex2).
PER_EVAL_FMA = 22
PER_EVAL_MUFU = 3
# Backward, algorithmic cost of one ray-Gaussian evaluation from the maths of the gradient, in the
# same mat-vec formulation as the forward's 22 (per-pixel constants -- the saved max, 1/W, the
# depth D, gd/W and g_alpha (1 - alpha) -- are formed once per pixel, not per evaluation):
#   recompute without accumulating: a = L r 6, |a|^2 3, a.b 3, z 1, d0 1, s 1, s log2(e) 1,
#     logit 2, shift by the saved max 1                                            = 19
#   chain rule: t = e_w gd/W 1; dL/dl = t (z - D) 2; dL/ds = g_a(1-a) e_d + beta3 dL/dl 2;
#     dL/dz = t - beta2 dL/dl 1; dL/dpsv = dL/dz q + dL/ds z 2;
#     dL/dvsv = -z q (dL/dz + dL/ds z / 2) 4; dL/da = 2 dL/dvsv a + dL/dpsv b 6    = 18
#   per-key accumulations: dL/db += dL/dpsv a 3; dL/dL += dL/da r^T (6 lower entries) 6;
#     sum of dL/ds (log-weight and |b|^2) 1                                        = 10
# = 47 FMA-pipe operations and 3 MUFU (rcp, ex2 of the density, ex2 of the softmax weight).
PER_EVAL_BWD_FMA = 47
PER_EVAL_BWD_MUFU = 3
# What blend_bwd_kernel itself issues per evaluation in its per-pixel loop (polynomials in the
# pixel offset, row-folded; running sums of the coefficient gradients): 32 FMA-pipe operations
# (pixel offsets 2, the three polynomials 5, peak and logit 4, chain rule 12, running sums 9) and
# the same 3 MUFU.
KERNEL_EVAL_BWD_FMA = 32


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-next", action="store_true")
    ap.add_argument("--serve-only", action="store_true",
                    help="run only the served mixed-request workload and print its JSON")
    ap.add_argument("--profile-step", action="store_true",
                    help="build the workload, warm up, run one batched forward step, then one "
                         "forward with statistics and its backward, and exit (the command the "
                         "committed ncu summaries capture)")
    ap.add_argument("--binning", choices=["tiles", "radix"], default="tiles",
                    help="binning of the batched step: tile-major (default) or key emission + "
                         "radix sort (to profile the sort path)")
    ap.add_argument("--blend", default=None,
                    help="with --profile-step: blend configuration TILExTILE/PX/CHUNK[/heavy] "
                         "(e.g. 16x16/4/32/heavy, the one the autotuner picks on the 16-camera "
                         "step); default: the autotuner's untuned default")
    ap.add_argument("--profile-batch3", action="store_true",
                    help="build the 256-scene batch, run its forward twice with the blend the "
                         "autotuner picks there (16x16 tiles, 4 pixels per thread, 32-pair "
                         "chunks) and exit (the batch's ncu launch list)")
    ap.add_argument("--profile-single", type=int, default=0, metavar="CALLS",
                    help="build the workload, then run CALLS plain single-view fe_render_fwd calls "
                         "(camera i mod 16) and exit (the per-call path's ncu capture)")
    ap.add_argument("--profile-host", type=int, default=0, metavar="CALLS",
                    help="build the 16-camera batch with --blend (default 32x8/2/16, the "
                         "autotuner's pick for host outputs there), run CALLS fe_batch_fwd_host "
                         "calls into pinned host outputs and exit (the host-to-host ncu capture)")
    return ap.parse_args()


def blend_cfg(spec):
    """TILExTILE/PX/CHUNK[/heavy] -> the Batch keyword arguments."""
    parts = spec.split("/")
    tw, th = (int(x) for x in parts[0].split("x"))
    return {"tile": (tw, th), "px": int(parts[1]), "chunk": int(parts[2]),
            "heavy_first": len(parts) > 3 and parts[3] == "heavy"}


def job_value(dev_s, units_per_step, steps, world, device):
    """Whole-job throughput of independent replicas (weak scaling): all ranks' units over the
    slowest rank's device time. Returns (value in millions of units per second, that time)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([dev_s], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s = float(t.item())
    return world * units_per_step * steps / dev_s / 1e6, dev_s


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu = gpu_id
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the blend from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "blend_fwd_cfg1.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch_full_workload")
    return None


def build_workload(dev):
    import torch

    from fuzzy_ellipses import synthetic as S
    scene, cams = S.config1(seed=0)
    m = torch.from_numpy(scene.means).to(dev)
    p = torch.from_numpy(scene.prec).to(dev)
    w = torch.from_numpy(scene.logw).to(dev)
    return scene, cams, (m, p, w)


def count_evals(fe, cams, mpw):
    """E = sum over 8x8-tile keys of the pixels in the key's tile, per camera, with every
    Gaussian binned to all tiles of its footprint's bounding rectangle (the reference rasterizer's
    tiling rule). This fixes the metric's unit by the workload; the renderer itself bins to the
    tiles each footprint ellipse reaches, and so evaluates fewer pairs than E counts (reported
    beside it as executed evaluations)."""
    m, p, w = mpw
    per_cam = []
    for c in cams:
        keys, ranges = fe.render_binning(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans,
                                         c.height, c.width, tile=(8, 8), footprint="rect")
        r = ranges.cpu().numpy()
        gx = (c.width + 7) // 8
        t = np.arange(r.shape[0])
        tx, ty = t % gx, t // gx
        pix = np.minimum(8, c.width - 8 * tx) * np.minimum(8, c.height - 8 * ty)
        per_cam.append(int(((r[:, 1] - r[:, 0]) * pix).sum()))
    return per_cam


CPU_SAMPLE_PIXELS = 4096


def cpu_reference(scene, cams, steps, warmup, n_pix=CPU_SAMPLE_PIXELS, seed=0):
    """Time the CPU implementation of the path -- the float64 restatement of fm_render
    (baseline/fm_render.py:11-126) in torch, dense over all Gaussians, on every host core this
    process may use -- on one bounded sample per step: ``n_pix`` random pixels of one camera
    (camera i mod 16 at step i). Both the main line's cpu_baseline and the reference arm use it.

    Returns seconds per step and the host facts (nproc, affinity, threads)."""
    import torch

    from oracle import fm_render_torch as OT
    affinity = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else None
    threads = len(affinity) if affinity else (os.cpu_count() or 1)
    torch.set_num_threads(threads)
    m = torch.from_numpy(scene.means).double()
    p = torch.from_numpy(scene.prec).double()
    w = torch.from_numpy(scene.logw).double()
    rng = np.random.default_rng(seed)
    times = []
    with torch.no_grad():
        for i in range(warmup + steps):
            c = cams[i % len(cams)]
            rays_all = OT.pinhole_rays(c.height, c.width, c.fx, c.fy, c.cx, c.cy)
            pix = torch.from_numpy(rng.choice(c.height * c.width, n_pix, replace=False))
            t0 = time.perf_counter()
            OT.render_func_quat(m, p, w, rays_all[pix], torch.from_numpy(c.quat).double(),
                                torch.from_numpy(c.trans).double(), 21.4, 2.66)
            if i >= warmup:
                times.append(time.perf_counter() - t0)
    return {"s_per_step": statistics.mean(times), "n_pix": n_pix, "n": scene.n,
            "threads": torch.get_num_threads(), "nproc": os.cpu_count(),
            "affinity": (f"{len(affinity)} cpus: {affinity[0]}-{affinity[-1]}" if affinity
                         else "unknown"),
            "impl": "torch float64 restatement of fm_render (oracle/fm_render_torch.py), dense "
                    f"over N={scene.n}, torch.set_num_threads({threads})"}


def cpu_baseline_line(cpu, e_render, n_render_pixels):
    """The cpu_baseline object in the metric's unit: renders/s x evaluations per render."""
    px_s = cpu["n_pix"] / cpu["s_per_step"]
    renders_s = px_s / n_render_pixels
    return {"value": renders_s * e_render / 1e6, "unit": "Mevals/s", "cores": cpu["threads"],
            "kind": "port", "nproc": cpu["nproc"], "affinity": cpu["affinity"],
            "sample": f"{cpu['n_pix']} random pixels of one 640x480 camera per step (camera i "
                      f"mod 16), {cpu['impl']}",
            "renders_per_s": renders_s, "dense_evals_per_s": px_s * cpu["n"]}


def cpu_baseline_child(steps=16, warmup=3):
    """The CPU baseline of the main line: the reference arm itself (same implementation, same
    sample, same conversion), run as a child process so that this process's GPU-side threads do
    not share the host cores with it."""
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT")}
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--impl", "reference",
                        "--steps", str(steps), "--warmup", str(warmup)],
                       capture_output=True, text=True, env=env, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"CPU baseline child failed: {r.stderr[-2000:]}")
    line = json.loads(r.stdout.strip().splitlines()[-1])
    out = dict(line["cpu_baseline"])
    out["run"] = (f"bench.py --impl reference --steps {steps} --warmup {warmup} in a child "
                  "process (the reference arm)")
    return out


def run_reference(args):
    """The reference arm: the CPU implementation of the path (float64 restatement of fm_render,
    torch, all host threads), same workload and metric, bounded per-step sample."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from fuzzy_ellipses import synthetic as S
    from oracle import screen_bounds as SB
    scene, cams = S.config1(seed=0)
    # Evaluations of one tile-binned render (8x8 tiles), from the float64 restatement of the
    # renderer's screen bounds: the unit that converts renders/s into the metric.
    per_cam_evals = [SB.evals_per_render(scene.means, scene.prec, scene.logw, c) for c in cams]
    e_render = float(np.mean(per_cam_evals))
    cpu = cpu_reference(scene, cams, args.steps, args.warmup)
    base = cpu_baseline_line(cpu, e_render, cams[0].height * cams[0].width)
    value = base["value"]
    out = {"metric": METRIC, "value": value, "unit": "Mevals/s", "impl": "reference",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * cpu["s_per_step"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": WORKLOAD,
                      "sample_per_step": f"{cpu['n_pix']} pixels of one camera"},
           "renders_per_s": base["renders_per_s"], "dense_evals_per_s": base["dense_evals_per_s"],
           "cpu_baseline": base,
           "e2e": {"value": value, "unit": "Mevals/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.serve_only:
        import torch

        import fuzzy_ellipses as fe
        print(json.dumps(serve_bench(fe, torch.device("cuda", 0))), flush=True)
        return
    import torch

    import fuzzy_ellipses as fe

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:  # independent replicas; the process group only carries the barriers and timing
        import torch.distributed as dist
        dist.init_process_group("nccl")
    scene, cams, mpw = build_workload(dev)
    m, p, w = mpw
    H, W = cams[0].height, cams[0].width
    npix = H * W
    views = [dict(scene=0, height=c.height, width=c.width, fx=c.fx, fy=c.fy, cx=c.cx, cy=c.cy,
                  quat=c.quat, trans=c.trans) for c in cams]
    if args.profile_batch3:
        profile_batch3(fe, dev)
        return
    if args.profile_host:
        cfg = blend_cfg(args.blend or "32x8/2/16")
        b = fe.Batch([(0, scene.n)], views, tile=cfg["tile"], px=cfg["px"], chunk=cfg["chunk"])
        host_in = [t.cpu().pin_memory() for t in (m, p, w)]
        out = torch.empty(2 * b.n_pixels, dtype=torch.float32).pin_memory()
        for _ in range(args.profile_host):
            b.forward_host(*host_in, out[:b.n_pixels], out[b.n_pixels:])
        assert b.status()["device_error"] == 0
        return
    if args.profile_single:
        out = (torch.empty(H, W, device=dev), torch.empty(H, W, device=dev))
        for i in range(args.profile_single):
            c = cams[i % len(cams)]
            fe.render_forward(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, H, W, out=out)
        torch.cuda.synchronize()
        assert fe.device_status() == 0
        return
    tuned = None
    if args.profile_step:
        cfg = blend_cfg(args.blend) if args.blend else dict(fe.autotune.DEFAULT)
    else:
        tuner = fe.autotune.Autotuner(persist=False)
        tuned = tuner.tune([(0, scene.n)], views, m, p, w, reps=3)
        cfg = {k: tuned[k] for k in ("tile", "px", "chunk", "heavy_first")}
    batch = fe.Batch([(0, scene.n)], views, tile=cfg["tile"], px=cfg["px"], chunk=cfg["chunk"],
                     heavy_first=cfg["heavy_first"],
                     keep_binning=True, binning=args.binning)
    per_cam_evals = count_evals(fe, cams, mpw) if not args.profile_step else [0] * len(cams)
    e_step = float(sum(per_cam_evals))
    depth = torch.empty(batch.n_pixels, device=dev)
    alpha = torch.empty(batch.n_pixels, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    for _ in range(args.warmup):
        batch.forward(m, p, w, depth, alpha)
    # Eager per-step device time (launch by launch from Python), for comparison with the replay.
    eager_ms = _event_ms(lambda: batch.forward(m, p, w, depth, alpha), reps=5, warm=1, calls=1) \
        if not args.profile_step else None
    if args.profile_step:
        batch.forward(m, p, w, depth, alpha)
        torch.cuda.synchronize()
        assert batch.status()["device_error"] == 0
        # then one differentiable step: forward with statistics and the backward
        stats = torch.empty(3 * batch.n_pixels, device=dev)
        batch.forward(m, p, w, depth, alpha, stats)
        gen = torch.Generator(device=dev).manual_seed(1)
        gdep = torch.randn(batch.n_pixels, device=dev, generator=gen) * 1e-3
        galp = torch.randn(batch.n_pixels, device=dev, generator=gen) * 1e-3
        batch.backward(m, p, w, depth, alpha, stats, gdep, galp)
        torch.cuda.synchronize()
        assert batch.status()["device_error"] == 0
        return
    st = batch.status()
    assert st["device_error"] == 0 and st["num_keys"] == st["want_keys"], st

    # The step as one CUDA graph (the batch plan has no host synchronisation in its default
    # worst-case key mode): captured once, replayed every step.
    cap_stream = torch.cuda.Stream(device=dev)
    cap_stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cap_stream):
        batch.forward(m, p, w, depth, alpha)
    torch.cuda.current_stream().wait_stream(cap_stream)
    step_graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(step_graph, stream=cap_stream):
        batch.forward(m, p, w, depth, alpha)
    for _ in range(2):
        step_graph.replay()
    torch.cuda.synchronize()

    # ---- timed region: K batched forward steps, L2 flushed between steps --------------------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    props = torch.cuda.get_device_properties(dev)
    uuid = getattr(props, "uuid", None)
    sampler = ClockSampler(f"GPU-{uuid}" if uuid is not None else str(local))
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        starts[i].record()
        step_graph.replay()
        ends[i].record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    value, dev_s = job_value(sum(step_ms) / 1e3, e_step, args.steps, world, dev)
    renders_s = world * len(cams) * args.steps / dev_s

    if rank != 0:
        return

    # ---- per-stage timings (live events on the launching stream) ---------------------------
    stage_runs = []
    for _ in range(5):
        flush.fill_(1)
        _, _, ms = batch.forward_timed(m, p, w, depth, alpha)
        stage_runs.append(ms)
    stages = {k: statistics.median(r[k] for r in stage_runs) for k in batch.STAGES}
    # FP32 FMA rate: the better of scalar FFMA and packed f32x2 FMA (the blends issue packed
    # operations; both reach the same FMA throughput, about 40 T FMA/s).
    fma_ops = max(fe.bench_peak("fma"), fe.bench_peak("fma2"))
    ex2_ops = fe.bench_peak("ex2")
    peak_evals = min(fma_ops / PER_EVAL_FMA, ex2_ops / PER_EVAL_MUFU)
    blend_evals_per_s = e_step / (stages["blend"] * 1e-3)
    peaks, peak_kind = measured_peaks()
    nk = batch.status()["num_keys"]
    passes = (max(1, int(np.ceil(np.log2(batch_tiles(cams, *cfg["tile"]))))) + 7) // 8
    # The tile-major binning (three launches per forward) writes the keys in order and the tile
    # ranges with them: its scan, sort and ranges stages are empty (event gaps only). The emit +
    # radix sort path moves 16 B per key per sort pass and reads the sorted keys once more for the
    # ranges (8 B per key, 8 B per tile written).
    radix_path = batch.launches_per_forward > 3
    n_tiles_b = batch_tiles(cams, *cfg["tile"])
    hbm = {
        "preprocess": (52 * scene.n + len(cams) * scene.n * (96 + 8 + 4)) / (stages["preprocess"] * 1e-3) / 1e9,
        "emit": (8 * nk + (0 if radix_path else 8 * n_tiles_b)) / (stages["emit"] * 1e-3) / 1e9,
    }
    if radix_path:
        hbm["sort"] = (16 * nk * passes) / (stages["sort"] * 1e-3) / 1e9
        hbm["ranges"] = (8 * nk + 8 * n_tiles_b) / (stages["ranges"] * 1e-3) / 1e9

    # ---- plain per-call drop-in on device-resident inputs ----------------------------------
    outs = [(torch.empty(H, W, device=dev), torch.empty(H, W, device=dev)) for _ in cams]
    for _ in range(3):
        for c, o in zip(cams, outs):
            fe.render_forward(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, H, W, out=o)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(3, args.steps // 2)
    e0.record()
    for _ in range(reps):
        for c, o in zip(cams, outs):
            fe.render_forward(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, H, W, out=o)
    e1.record()
    torch.cuda.synchronize()
    plain_s = e0.elapsed_time(e1) / 1e3 / reps
    plain_renders_s = len(cams) / plain_s

    # ---- end to end: host buffers in, plain C-ABI calls, host buffers out -------------------
    m_h, p_h, w_h = [x.cpu().pin_memory() for x in (m, p, w)]
    poses_h = torch.from_numpy(np.concatenate([np.concatenate([c.quat, c.trans]) for c in cams])
                               .astype(np.float32)).pin_memory()
    out_h = torch.empty((len(cams), 2, H, W), dtype=torch.float32).pin_memory()
    m_d, p_d, w_d = torch.empty_like(m), torch.empty_like(p), torch.empty_like(w)
    poses_d = torch.empty_like(poses_h, device=dev)
    out_d = torch.empty((len(cams), 2, H, W), device=dev)
    h2d = sum(x.numel() * 4 for x in (m_h, p_h, w_h, poses_h))
    d2h = out_h.numel() * 4

    # The per-call C-ABI entry, called through ctypes as a C caller would: one fe_render_fwd per
    # camera with its descriptor built once. The cameras' depth and alpha go back in groups on a
    # second stream, each group as soon as its renders are done, while the next group renders;
    # the last groups are smaller, so that less of the final copy follows the last render.
    # Consecutive calls alternate between two streams (each has its own scratch arena), so one
    # call's small latency-bound kernels overlap the previous call's blend.
    lib = fe._native.load()
    descs = [fe._native.make_desc(scene.n, H, W, c.fx, c.fy, c.cx, c.cy) for c in cams]
    copy_stream = torch.cuda.Stream(device=dev)
    side_stream = torch.cuda.Stream(device=dev)
    group_ends = sorted({min(len(cams), e) for e in (4, 8, 12, 14, len(cams))})
    done_ev = {e: (torch.cuda.Event(), torch.cuda.Event()) for e in group_ends}
    inputs_ev = torch.cuda.Event()

    def e2e_step():
        cs = torch.cuda.current_stream()
        streams = (cs, side_stream)
        for src, dst in ((m_h, m_d), (p_h, p_d), (w_h, w_d), (poses_h, poses_d)):
            dst.copy_(src, non_blocking=True)
        inputs_ev.record(cs)
        side_stream.wait_event(inputs_ev)
        base = poses_d.data_ptr()
        for i in range(len(cams)):
            fe._native.check(lib.fe_render_fwd(
                ctypes.byref(descs[i]), m_d.data_ptr(), p_d.data_ptr(), w_d.data_ptr(),
                base + 28 * i, base + 28 * i + 16, out_d[i, 0].data_ptr(), out_d[i, 1].data_ptr(),
                None, streams[i % 2].cuda_stream))
            if i + 1 in done_ev:
                g0 = max([0] + [e for e in group_ends if e <= i])
                for ev, st in zip(done_ev[i + 1], streams):
                    ev.record(st)
                    copy_stream.wait_event(ev)
                with torch.cuda.stream(copy_stream):
                    out_h[g0:i + 1].copy_(out_d[g0:i + 1], non_blocking=True)
        cs.wait_stream(copy_stream)
        cs.wait_stream(side_stream)
        cs.synchronize()

    for _ in range(3):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_call_s = (time.perf_counter() - t0) / args.steps

    # The same 16 renders through the batch C-ABI (fe_batch_fwd), host buffers in and out.
    out_b = torch.empty(2 * batch.n_pixels, dtype=torch.float32).pin_memory()
    dep_b = torch.empty(batch.n_pixels, device=dev)
    alp_b = torch.empty(batch.n_pixels, device=dev)

    def e2e_serial_step():
        for src, dst in ((m_h, m_d), (p_h, p_d), (w_h, w_d)):
            dst.copy_(src, non_blocking=True)
        batch.forward(m_d, p_d, w_d, dep_b, alp_b)
        out_b[:batch.n_pixels].copy_(dep_b, non_blocking=True)
        out_b[batch.n_pixels:].copy_(alp_b, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    # fe_batch_fwd_host, the C-ABI call: host Gaussians in, the blend storing depth and alpha
    # into the pinned host buffers as it renders; then the stream is synchronised. The same call
    # through the Python wrapper (Batch.forward_host, argument checks included) is timed beside.
    # Its batch is the autotuner's pick for host outputs, where the host link bounds the call.
    tuned_h = fe.autotune.Autotuner(persist=False).tune([(0, scene.n)], views, m, p, w, reps=3,
                                                         target="host")
    batch_h = fe.Batch([(0, scene.n)], views, tile=tuned_h["tile"], px=tuned_h["px"],
                       chunk=tuned_h["chunk"], binning=args.binning)
    lib = fe._native.load()
    host_args = (batch_h._h, m_h.data_ptr(), p_h.data_ptr(), w_h.data_ptr(), out_b.data_ptr(),
                 out_b.data_ptr() + 4 * batch.n_pixels)

    def e2e_batch_step():
        cs = torch.cuda.current_stream()
        fe._native.check(lib.fe_batch_fwd_host(*host_args, cs.cuda_stream))
        cs.synchronize()

    def e2e_wrapper_step():
        batch_h.forward_host(m_h, p_h, w_h, out_b[:batch.n_pixels], out_b[batch.n_pixels:])

    def timed_host(step):
        for _ in range(3):
            step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        return (time.perf_counter() - t0) / args.steps

    e2e_serial_s = timed_host(e2e_serial_step)
    e2e_s = timed_host(e2e_batch_step)
    e2e_wrapper_s = timed_host(e2e_wrapper_step)
    e2e_value = e_step / e2e_s / 1e6
    h2d_batch = sum(x.numel() * 4 for x in (m_h, p_h, w_h))

    # ---- backward of the same step (recompute-based), CUDA events, L2 flushed between ------
    stats = torch.empty(3 * batch.n_pixels, device=dev)
    batch.forward(m, p, w, depth, alpha, stats)
    gen = torch.Generator(device=dev).manual_seed(1)
    gdep = torch.randn(batch.n_pixels, device=dev, generator=gen) * 1e-3
    galp = torch.randn(batch.n_pixels, device=dev, generator=gen) * 1e-3
    for _ in range(3):
        batch.backward(m, p, w, depth, alpha, stats, gdep, galp)
    b_start = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    b_end = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        b_start[i].record()
        batch.backward(m, p, w, depth, alpha, stats, gdep, galp)
        b_end[i].record()
    torch.cuda.synchronize()
    bwd_ms = statistics.median(a.elapsed_time(b) for a, b in zip(b_start, b_end))
    bwd_evals_s = e_step / (bwd_ms * 1e-3)
    bwd_peak = min(fma_ops / PER_EVAL_BWD_FMA, ex2_ops / PER_EVAL_BWD_MUFU)
    backward = {"ms_per_step": bwd_ms, "evals_per_s": bwd_evals_s,
                "roofline": {"bound": "fma+xu", "achieved": bwd_evals_s / 1e9,
                             "peak": bwd_peak / 1e9, "unit": "Gevals/s",
                             "frac": bwd_evals_s / bwd_peak,
                             "per_eval": {"fma_pipe": PER_EVAL_BWD_FMA, "mufu": PER_EVAL_BWD_MUFU,
                                          "basis": "algorithmic (maths of the gradient)"},
                             "kernel_per_eval": {"fma_pipe": KERNEL_EVAL_BWD_FMA,
                                                 "mufu": PER_EVAL_BWD_MUFU},
                             "frac_of_kernel_count": bwd_evals_s / min(
                                 fma_ops / KERNEL_EVAL_BWD_FMA, ex2_ops / PER_EVAL_BWD_MUFU),
                             "scope": "whole backward (per-key recompute and coefficient "
                                      "gradients, record VJP) of the 16-view step, reusing the "
                                      "forward's binning"}}

    # ---- the kernels beyond the render path ------------------------------------------------
    next_rows = None if args.no_next else next_rows_bench(fe, dev, scene, cams, fma_ops, ex2_ops,
                                                          peaks["hbm_gbs"])

    # ---- batched uneven renders (256 scenes) ----------------------------------------------
    config3 = None if args.no_next else config3_bench(fe, dev, max(5, args.steps // 2), fma_ops,
                                                      ex2_ops)

    # ---- served mixed requests vs the plain per-call drop-in ------------------------------
    served = None if args.no_serve else serve_bench(fe, dev)

    # ---- CPU baseline (oracle on the host cores, bounded sample) ---------------------------
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline_child()

    blend_achieved = blend_evals_per_s / 1e9
    # Pairs the blend evaluates: every key's tile (all tiles of these 640x480 views are whole).
    executed = nk * cfg["tile"][0] * cfg["tile"][1]
    out = {
        "metric": METRIC, "value": value, "unit": "Mevals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "step": "batched forward of all 16 cameras",
                   "tile": f"{cfg['tile'][0]}x{cfg['tile'][1]}", "px_per_thread": cfg["px"],
                   "chunk_pairs": cfg["chunk"], "heavy_tiles_first": cfg["heavy_first"],
                   "autotuned": tuned is not None,
                   "binning": "tile-major (keys emitted in sorted order)" if args.binning == "tiles"
                   else "key emission + radix sort",
                   "launch": "CUDA graph replay of the batched forward (captured once)",
                   "eager_ms_per_step": eager_ms,
                   "l2": "flushed between steps (256 MiB write outside the per-step CUDA "
                   "events); step working set ~100 MB < L2",
                   "parallelism": f"replicas x{world}"},
        "renders_per_s": renders_s,
        "evals_per_step": e_step,
        "plain_per_call": {"renders_per_s": plain_renders_s, "ms_per_render": 1e3 * plain_s / len(cams),
                           "mevals_per_s": e_step / plain_s / 1e6},
        "e2e": {"value": e2e_value, "unit": "Mevals/s", "h2d_bytes_per_step": h2d_batch,
                "d2h_bytes_per_step": out_b.numel() * 4,
                "path": "fe_batch_fwd_host C-ABI call (ctypes) over the 16 cameras: pinned "
                        "host Gaussians in (read by the preprocess through their device "
                        "mapping), depth and alpha out to pinned host buffers, which the blend "
                        "stores into through their device mapping as it renders (one launch, "
                        "tiles in index order, no copy before the binning or after the last "
                        "tile); poses part of the batch plan; wall clock per call including the "
                        "final sync",
                "ms_per_step": 1e3 * e2e_s,
                "autotuned": {"tile": f"{tuned_h['tile'][0]}x{tuned_h['tile'][1]}",
                              "px": tuned_h["px"], "chunk": tuned_h["chunk"],
                              "target": "host",
                              "candidates_ms": {f"{c['tile'][0]}x{c['tile'][1]}/px{c['px']}"
                                                f"/ch{c['chunk']}": round(c["ms"], 4)
                                                for c in tuned_h["candidates"]}},
                "python_wrapper": {"value": e_step / e2e_wrapper_s / 1e6,
                                   "ms_per_step": 1e3 * e2e_wrapper_s,
                                   "path": "the same call through Batch.forward_host"},
                "serial": {"value": e_step / e2e_serial_s / 1e6, "ms_per_step": 1e3 * e2e_serial_s,
                           "path": "copy in, fe_batch_fwd, then copy depth and alpha out"}},
        "e2e_per_call": {"value": e_step / e2e_call_s / 1e6, "unit": "Mevals/s",
                         "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                         "path": "fe_render_fwd per camera (the reference's one-camera-per-call "
                                 "pattern) through the C-ABI (ctypes, descriptors built once), "
                                 "consecutive calls alternating between two streams, pinned host "
                                 "buffers; the images copied back in groups (4, 4, 4, 2, 2 "
                                 "cameras) on a third stream while the next group renders",
                         "ms_per_step": 1e3 * e2e_call_s},
        "roofline": {"bound": "fma+xu", "achieved": blend_achieved,
                     "peak": peak_evals / 1e9, "unit": "Gevals/s",
                     "frac": blend_evals_per_s / peak_evals, "traffic": ncu_traffic(),
                     "evals_basis": "E, the metric's unit: 8x8-tile keys of footprint rectangles "
                                    "x tile pixels",
                     "executed_evals_per_launch": executed,
                     "frac_executed": executed / (stages["blend"] * 1e-3) / peak_evals,
                     "kernel": f"blend_fwd_kernel<{cfg['tile'][0]},{cfg['tile'][1]},{cfg['px'] or 4},{cfg['chunk'] or 16}>",
                     "per_eval": {"fma_pipe": PER_EVAL_FMA, "mufu": PER_EVAL_MUFU},
                     "fma_ops_per_s": fma_ops, "mufu_ex2_ops_per_s": ex2_ops,
                     "peak_source": "fe_bench_peak microbenchmarks on this GPU (the better of scalar "
                                    "and packed FP32 FMA, and MUFU ex2)"},
        "stages_ms": stages,
        "stages_note": ("emit + radix sort binning" if radix_path else
                        "tile-major binning: keys and ranges come from the emit stage; scan, "
                        "sort and ranges are empty (the gap between two events)"),
        "stages_hbm_gbs": hbm, "hbm_peak_gbs": peaks.get("hbm_gbs"), "hbm_peak_kind": peak_kind,
        "num_keys": nk,
        "evals_per_camera": per_cam_evals,
        "cpu_baseline": cpu,
        "backward": backward,
        "next_rows": next_rows,
        "batched_uneven_256_scenes": config3,
        "served": served,
        "autotune": tuned and {"bucket": tuned["bucket"],
                               "candidates_ms": {f"{c['tile'][0]}x{c['tile'][1]}/px{c['px']}/ch{c['chunk']}{'/heavy' if c['heavy_first'] else ''}": round(c["ms"], 4)
                                                 for c in tuned["candidates"]}},
        "clocks": clocks,
        "gpu_launches": batch.launches_per_forward * args.steps,
        "wall_s_timed_region": wall,
    }
    print(json.dumps(out), flush=True)


def _silhouette(h, w):
    """Target silhouette for the backward requests: a centred disk."""
    v, u = np.mgrid[0:h, 0:w]
    return (((u - w / 2) ** 2 + (v - h / 2) ** 2) < (0.3 * min(h, w)) ** 2).astype(np.float32)


SERVE_LOAD_FRACTIONS = (0.1, 0.25, 0.5, 0.75, 1.0)


def serve_bench(fe, dev, n_requests=500, seed=0):
    """Served mixed requests (N log-uniform in [20, 2000], 1-32 poses, sides 96-480, 30% with a
    silhouette-BCE backward): saturating arrivals for throughput, then Poisson arrivals swept
    over SERVE_LOAD_FRACTIONS of that rate (renders/s, p50, p99 per rate); the plain per-call
    drop-in on the same 500 requests for comparison -- one fe_render_fwd (forward requests) or
    differentiable render (backward requests) per camera, the silhouette loss and its cotangent
    from the same fused kernel the server uses (fe_silhouette_bce), results and gradients read
    back per request."""
    import threading

    import torch

    from fuzzy_ellipses import serve, synthetic as S
    stream = S.config4_request_stream(n_requests, rate_hz=1.0, seed=seed)
    reqs = []
    for r in stream:
        sc = r["scene"]
        tg = [_silhouette(c.height, c.width) for c in r["cameras"]] if r["backward"] else None
        reqs.append(serve.RenderRequest(sc.means, sc.prec, sc.logw, r["cameras"], tg))
    renders = sum(len(r.cameras) for r in reqs)

    def run(arrival_gaps):
        # A streaming consumer: each result is taken as it completes (latency recorded, one pixel
        # read) and released, so the server's pinned result buffers are recycled.
        lat, done = [], threading.Semaphore(0)
        lock = threading.Lock()

        def consume(fut):
            r = fut.result()
            with lock:
                lat.append(r.latency)
                _ = float(r.alpha[0][0, 0])
            done.release()

        with serve.RenderServer(device=dev, lanes=3) as srv:
            for r in reqs[:4] + [q for q in reqs if q.backward][:4]:
                srv.submit(r).result(timeout=300)
            srv.reset_stats()
            t0 = time.perf_counter()
            for r, gap in zip(reqs, arrival_gaps):
                if gap > 0:
                    time.sleep(gap)
                srv.submit(r).add_done_callback(consume)
            for _ in reqs:
                if not done.acquire(timeout=300):
                    raise RuntimeError("served request did not complete")
            wall = time.perf_counter() - t0
            st = srv.stats()
        lat.sort()
        return {"renders_per_s": renders / wall, "requests_per_s": len(reqs) / wall,
                "p50_ms": 1e3 * lat[len(lat) // 2], "p99_ms": 1e3 * lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                "batches": st["batches"], "wall_s": wall, "lane_busy_s": st["busy_s"],
                "lane_phase_s": st["phase_s"]}

    sat = run([0.0] * len(reqs))
    sweep = []
    rng = np.random.default_rng(seed + 1)
    for frac in SERVE_LOAD_FRACTIONS:
        rate = frac * sat["requests_per_s"]
        r = run(list(rng.exponential(1.0 / rate, size=len(reqs))))
        r.update(load_fraction=frac, arrival_rate_hz=rate)
        sweep.append(r)

    # The plain per-call drop-in on all the same requests.
    def plain(req):
        m, p, w = [torch.from_numpy(x).to(dev) for x in (req.means, req.prec, req.logw)]
        if req.targets is None:
            for c in req.cameras:
                d, a = fe.render_forward(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
                d.cpu(), a.cpu()
            return
        m.requires_grad_(); p.requires_grad_(); w.requires_grad_()
        total = sum(c.height * c.width for c in req.cameras)
        loss = 0.0
        for c, t in zip(req.cameras, req.targets):
            d, a = fe.render(m, p, w, c.fx, c.fy, c.cx, c.cy, c.quat, c.trans, c.height, c.width)
            hw = c.height * c.width
            tt = torch.from_numpy(t).to(dev).reshape(-1)
            seg = torch.full((1,), hw, dtype=torch.int64, device=dev)
            # the request's loss is the mean over all its pixels: weight each camera's mean by
            # its share of the pixels (the server's segment is the whole request)
            lc, ga = fe.silhouette_bce(a.detach().reshape(-1), tt, seg)
            ga.mul_(hw / total)
            loss = loss + lc * (hw / total)
            torch.autograd.backward(a, ga.view(c.height, c.width))
            d.detach().cpu(), a.detach().cpu()
        float(loss)
        m.grad.cpu(), p.grad.cpu(), w.grad.cpu()

    for r in reqs[:3]:
        plain(r)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        plain(r)
    torch.cuda.synchronize()
    pw = time.perf_counter() - t0
    plain_rs = renders / pw
    half = next(r for r in sweep if r["load_fraction"] == 0.5)
    return {"workload": f"{n_requests} requests: N logU[20,2000], 1-32 poses at 0.5 m, side U[96,480], "
                        "30% forward+backward (silhouette BCE), fp32",
            "saturating": sat,
            "poisson_sweep": sweep,
            "poisson_half_load": half,
            "plain_per_call": {"renders_per_s": plain_rs, "wall_s": pw, "requests": len(reqs),
                               "loss": "fe_silhouette_bce per camera (the server's fused kernel)"},
            "plain_per_call_renders_per_s": plain_rs,
            "served_over_plain": sat["renders_per_s"] / plain_rs}


def _event_ms(fn, reps=5, warm=2, calls=10):
    """Median CUDA-event time (ms) per call of fn() on the current stream, timing `calls`
    back-to-back calls between two events so that host launch overhead overlaps device work."""
    import torch
    for _ in range(warm):
        fn()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(calls):
            fn()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b) / calls)
    return statistics.median(ts)


# GMM log-likelihood per (point, Gaussian): 3 subtractions, 6 for U^T p, 3 for the squared norm,
# 1 for the log-density, 2 for the online logsumexp = 15 FMA-pipe operations and 1 ex2.
PER_PAIR_GMM_FMA = 15
PER_PAIR_GMM_MUFU = 1


def next_rows_bench(fe, dev, scene, cams, fma_ops, ex2_ops, hbm_gbs):
    """Throughput of the kernels beyond the render path: GMM log-likelihood, the multi-pose
    pixel-list renderer with flow, and the scene-parameter adapters."""
    import torch
    out = {}
    m, p, w = [torch.from_numpy(x).to(dev) for x in (scene.means, scene.prec, scene.logw)]
    g = torch.Generator(device=dev).manual_seed(0)
    # GMM: 1000 Gaussians, 2^21 points uniform in the scene's box
    pts = (torch.rand((1 << 21, 3), device=dev, generator=g) - 0.5) * 0.6
    ms = _event_ms(lambda: fe.gmm_log_likelihood(m, p, w, pts))
    pairs = pts.shape[0] * scene.n
    peak = min(fma_ops / PER_PAIR_GMM_FMA, ex2_ops / PER_PAIR_GMM_MUFU)
    out["gmm_log_likelihood"] = {
        "workload": f"{scene.n} Gaussians x {pts.shape[0]} points", "ms": ms,
        "pairs_per_s": pairs / (ms * 1e-3),
        "roofline": {"bound": "fma+xu", "achieved": pairs / (ms * 1e-3) / 1e9,
                     "peak": peak / 1e9, "unit": "Gpairs/s", "frac": pairs / (ms * 1e-3) / peak,
                     "per_pair": {"fma_pipe": PER_PAIR_GMM_FMA, "mufu": PER_PAIR_GMM_MUFU}}}
    # Pixel list: every other pixel of the 16 cameras, poses interleaved per camera, with flow
    H, W = cams[0].height, cams[0].width
    v, u = np.mgrid[0:H:2, 0:W:2]
    rays = np.concatenate([np.stack([u.ravel() - cams[0].cx, v.ravel() - cams[0].cy,
                                     np.ones(u.size), np.full(u.size, k)], 1)
                           for k in range(len(cams))]).astype(np.float32)
    poses = np.stack([np.concatenate([c.quat, c.trans]) for c in cams]).astype(np.float32)
    rays_d = torch.from_numpy(rays).to(dev)
    poses_d = torch.from_numpy(poses).to(dev)
    ms = _event_ms(lambda: fe.render_pixels(m, p, w, rays_d, 1.0 / cams[0].fx, poses_d, flow=True))
    out["render_pixels"] = {"workload": f"{len(rays)} rays over {len(cams)} poses "
                                        f"({H}x{W} at stride 2), N={scene.n}, with flow",
                            "ms": ms, "rays_per_s": len(rays) / (ms * 1e-3)}
    # Adapters: precision factors of 2^20 Gaussians; a pose transform of 2^23 points
    n_g = 1 << 20
    sc = torch.exp(torch.empty((n_g, 3), device=dev).uniform_(np.log(0.005), np.log(0.03), generator=g))
    qs = torch.randn((n_g, 4), device=dev, generator=g)
    ms = _event_ms(lambda: fe.adapters.prec_from_scale_rot(sc, qs))
    out["prec_from_scale_rot"] = {"workload": f"{n_g} Gaussians", "ms": ms,
                                  "gaussians_per_s": n_g / (ms * 1e-3),
                                  "hbm_gbs": n_g * (28 + 36) / (ms * 1e-3) / 1e9,
                                  "bound": "float64 arithmetic (FP64 rate)"}
    n_p = 1 << 25
    pp = torch.randn((n_p, 3), device=dev, generator=g)
    pose = torch.tensor([0.01, 0.02, 0.03, 0.9, 0.1, 0.2, 0.3], device=dev)
    ms = _event_ms(lambda: fe.adapters.transform_points(pose, pp))
    gbs = n_p * 24 / (ms * 1e-3) / 1e9
    out["transform_points"] = {"workload": f"{n_p} points", "ms": ms, "hbm_gbs": gbs,
                               "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_gbs,
                                            "unit": "GB/s", "frac": gbs / hbm_gbs}}
    return out


def config3_workload(fe, dev):
    """The 256-scene batch's scenes, views and concatenated Gaussians on `dev`."""
    import torch

    from fuzzy_ellipses import synthetic as S
    items = S.config3(seed=0)
    means, prec, logw, scenes, views = [], [], [], [], []
    off = 0
    for si, (sc, cs) in enumerate(items):
        means.append(sc.means); prec.append(sc.prec); logw.append(sc.logw)
        scenes.append((off, sc.n))
        off += sc.n
        for c in cs:
            views.append(dict(scene=si, height=c.height, width=c.width, fx=c.fx, fy=c.fy,
                              cx=c.cx, cy=c.cy, quat=c.quat, trans=c.trans))
    m, p, w = [torch.from_numpy(np.concatenate(x)).to(dev) for x in (means, prec, logw)]
    return scenes, views, (m, p, w)


def profile_batch3(fe, dev):
    import torch
    scenes, views, (m, p, w) = config3_workload(fe, dev)
    b = fe.Batch(scenes, views, tile=(16, 16), px=4, chunk=32)
    for _ in range(2):
        b.forward(m, p, w)
    torch.cuda.synchronize()
    assert b.status()["device_error"] == 0
    b.close()


def config3_bench(fe, dev, steps, fma_ops, ex2_ops):
    """Batched uneven renders at their stated size: 256 scenes (N logU[8,512]), 1-8 poses each at
    0.5 m, sides {64, 128, 256}; one persistent launch sequence with the autotuned tile shape,
    pixels per thread and record chunk, captured once as a CUDA graph and replayed (L2 flushed
    between replays). Evaluations counted as for the headline (8x8-tile keys x tile pixels)."""
    import torch

    from fuzzy_ellipses import synthetic as S
    items = S.config3(seed=0)
    means, prec, logw, scenes, views, cams = [], [], [], [], [], []
    off = 0
    for si, (sc, cs) in enumerate(items):
        means.append(sc.means); prec.append(sc.prec); logw.append(sc.logw)
        scenes.append((off, sc.n))
        off += sc.n
        for c in cs:
            views.append(dict(scene=si, height=c.height, width=c.width, fx=c.fx, fy=c.fy,
                              cx=c.cx, cy=c.cy, quat=c.quat, trans=c.trans))
            cams.append((si, c))
    m, p, w = [torch.from_numpy(np.concatenate(x)).to(dev) for x in (means, prec, logw)]
    tuner = fe.autotune.Autotuner(persist=False)
    tuned = tuner.tune(scenes, views, m, p, w, reps=3)
    b = fe.Batch(scenes, views, tile=tuned["tile"], px=tuned["px"], chunk=tuned["chunk"],
                 heavy_first=tuned["heavy_first"])
    depth = torch.empty(b.n_pixels, device=dev)
    alpha = torch.empty(b.n_pixels, device=dev)
    e_total = 0
    for si, c in cams:
        sl = slice(scenes[si][0], scenes[si][0] + scenes[si][1])
        e_total += count_evals(fe, [c], (m[sl], p[sl], w[sl]))[0]
    cap = torch.cuda.Stream(device=dev)
    cap.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cap):
        b.forward(m, p, w, depth, alpha)
    torch.cuda.current_stream().wait_stream(cap)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=cap):
        b.forward(m, p, w, depth, alpha)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    st = b.status()
    assert st["device_error"] == 0 and st["num_keys"] == st["want_keys"], st
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for i in range(steps):
        flush.fill_(i & 0xFF)
        ev[i][0].record()
        g.replay()
        ev[i][1].record()
    torch.cuda.synchronize()
    ms = statistics.median(a.elapsed_time(z) for a, z in ev)
    stage_runs = []
    for _ in range(5):
        flush.fill_(1)
        _, _, sm = b.forward_timed(m, p, w, depth, alpha)
        stage_runs.append(sm)
    stages = {k: statistics.median(r[k] for r in stage_runs) for k in b.STAGES}
    peak = min(fma_ops / PER_EVAL_FMA, ex2_ops / PER_EVAL_MUFU)
    blend_evals_s = e_total / (stages["blend"] * 1e-3)
    executed = st["num_keys"] * tuned["tile"][0] * tuned["tile"][1]  # whole tiles (sides 64..256)
    out = {"workload": f"256 scenes (N logU[8,512]), {len(views)} views of 64^2/128^2/256^2, "
                       f"{b.n_pixels} pixels, fp32",
           "launch": "one persistent launch sequence, CUDA graph replay, L2 flushed between",
           "autotuned": {"tile": f"{tuned['tile'][0]}x{tuned['tile'][1]}", "px": tuned["px"],
                         "chunk": tuned["chunk"], "heavy_first": tuned["heavy_first"],
                         "bucket": tuned["bucket"],
                         "candidates_ms": {f"{c['tile'][0]}x{c['tile'][1]}/px{c['px']}/ch{c['chunk']}{'/heavy' if c['heavy_first'] else ''}": round(c["ms"], 4)
                                           for c in tuned["candidates"]}},
           "views": len(views), "ms_per_step": ms, "renders_per_s": len(views) / (ms * 1e-3),
           "evals_per_step": e_total, "mevals_per_s": e_total / (ms * 1e-3) / 1e6,
           "num_keys": st["num_keys"], "stages_ms": stages,
           "gpu_launches_per_step": b.launches_per_forward,
           "blend_roofline": {"bound": "fma+xu", "achieved": blend_evals_s / 1e9,
                              "peak": peak / 1e9, "unit": "Gevals/s",
                              "frac": blend_evals_s / peak,
                              "executed_evals_per_launch": executed,
                              "frac_executed": executed / (stages["blend"] * 1e-3) / peak}}
    b.close()
    return out


def batch_tiles(cams, tw, th):
    return sum(((c.width + tw - 1) // tw) * ((c.height + th - 1) // th) for c in cams)


if __name__ == "__main__":
    main()
