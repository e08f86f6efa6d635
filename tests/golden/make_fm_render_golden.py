"""Generate tests/golden/fm_render_golden.npz by running the reference's own pure-JAX renderer.

The reference's ``baseline/fm_render.py`` and ``baseline/util_render.py`` are imported
UNMODIFIED from the reference checkout, with ``tests/golden/numpy_jax.py`` standing in for JAX
(installed on neither machine) in float64. Every depth, alpha, weight, flow, log-likelihood and
gradient in the fixture file is therefore the reference's own arithmetic, not a restatement.

Usage (this machine only; the reference checkout does not exist where the GPU tests run, which
is why the outputs are committed):

    FE_REFERENCE_DIR=<reference checkout> python tests/golden/make_fm_render_golden.py

The reference location is taken from ``--reference`` or ``FE_REFERENCE_DIR``; the script stops
if neither is given.

Cases (inputs are stored beside the outputs, float32 as the renderer receives them):

* ``cfg0``      the 40-Gaussian, 200x200 camera, every pixel, with the weights of 500 pixels;
* ``cfg1``      the 1000-Gaussian scene, a fixed 2000-pixel sample of each of its 16 cameras;
* ``cfg2``      the 200-Gaussian differentiable step: two full 128x128 views of the model scene,
                and central differences (float64, h = 1e-6) of the silhouette BCE loss of the
                reference's optimisation loop (``shape_from_silhouette.ipynb`` cell 12) over
                four views, on 48 parameters: means, upper and strictly-lower precision entries
                (the latter must come out zero, as ``jax.grad`` through ``triu`` gives) and
                log-weights;
* ``behind``, ``straddle``, ``subpixel``, ``tiny*``: the edge scenes of the GPU render tests;
* ``gmm``       ``log_likelihood`` (``fm_render.py:231-259``);
* ``pix``       ``render_func_idx_quattrans`` and ``render_func_idx_quattrans_flow``
                (``fm_render.py:151-224``);
* ``cam``       ``render_func_quat_cam`` (``fm_render.py:130-144``).

The three pixel-list functions call ``render_func_rays`` with the Gaussians where the rays belong
(``fm_render.py:142-144,162-164,181-183``); they cannot run as written. For those cases only, the
module's ``render_func_rays`` name is rebound, while they run, to a function that passes its
arguments on in the order ``render_func_rays`` declares. Nothing else is changed.
"""

from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "fuzzy-ellipses_gb300"))

from fuzzy_ellipses import synthetic as S  # noqa: E402
from tests.golden import numpy_jax  # noqa: E402

OUT = os.path.join(HERE, "fm_render_golden.npz")
BETA2, BETA3 = 21.4, 2.66
CLIP_ALPHA = 3e-8


def import_reference(ref_dir):
    if not os.path.isfile(os.path.join(ref_dir, "baseline", "fm_render.py")):
        raise SystemExit(f"{ref_dir} has no baseline/fm_render.py")
    numpy_jax.install()
    sys.path.insert(0, ref_dir)
    for name in ("baseline.fm_render", "baseline.util_render", "baseline"):
        sys.modules.pop(name, None)
    fm = importlib.import_module("baseline.fm_render")
    assert fm.__file__.startswith(os.path.abspath(ref_dir)), fm.__file__
    return fm


def pinhole_rays(h, w, fx, fy, cx, cy):
    """Camera-frame rays [(u-cx)/fx, (v-cy)/fy, 1], pixel index v*W+u (the reference scripts'
    construction, ``baseline/ycb_fmb_rotscale.py:182-189``)."""
    u, v = np.meshgrid(np.arange(w, dtype=np.float64), np.arange(h, dtype=np.float64))
    return np.stack([(u.ravel() - cx) / fx, (v.ravel() - cy) / fy, np.ones(h * w)], 1)


def f64(x):
    return np.asarray(x, dtype=np.float64).view(numpy_jax.JArray)


def render(fm, means, prec, logw, rays, quat, trans):
    d, a, _, w = fm.render_func_quat(f64(means), f64(prec), f64(logw), f64(rays), f64(quat),
                                     f64(trans), BETA2, BETA3)
    return np.asarray(d), np.asarray(a), np.asarray(w)


def put_scene(out, key, scene):
    out[f"{key}_means"] = scene.means.astype(np.float32)
    out[f"{key}_prec"] = scene.prec.astype(np.float32)
    out[f"{key}_logw"] = scene.logw.astype(np.float32)


def put_cam(out, key, cam):
    out[f"{key}_cam"] = np.array([cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy],
                                 np.float64)
    out[f"{key}_quat"] = np.asarray(cam.quat, np.float32)
    out[f"{key}_trans"] = np.asarray(cam.trans, np.float32)


def full_view(fm, out, key, scene, cam):
    put_scene(out, key, scene)
    put_cam(out, key, cam)
    rays = pinhole_rays(cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy)
    d, a, w = render(fm, scene.means, scene.prec, scene.logw, rays, cam.quat, cam.trans)
    out[f"{key}_depth"] = d.reshape(cam.height, cam.width)
    out[f"{key}_alpha"] = a.reshape(cam.height, cam.width)
    return w


def bce(alpha, target):
    """The silhouette loss of the reference's optimisation loop (notebook cell 12)."""
    a = np.clip(alpha, CLIP_ALPHA, 1 - CLIP_ALPHA)
    return float((-(target * np.log(a) + (1 - target) * np.log(1 - a))).mean())


def case_cfg0(fm, out):
    scene, cams = S.config0(seed=0)
    w = full_view(fm, out, "cfg0", scene, cams[0])
    pix = np.random.default_rng(100).choice(w.shape[1], 500, replace=False)
    out["cfg0_wpix"] = pix.astype(np.int32)
    out["cfg0_w"] = w[:, pix]


def case_cfg1(fm, out):
    scene, cams = S.config1(seed=0)
    put_scene(out, "cfg1", scene)
    rng = np.random.default_rng(101)
    pix, ds, as_ = [], [], []
    for cam in cams:
        p = np.sort(rng.choice(cam.height * cam.width, 2000, replace=False))
        rays = pinhole_rays(cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy)[p]
        d, a, _ = render(fm, scene.means, scene.prec, scene.logw, rays, cam.quat, cam.trans)
        pix.append(p)
        ds.append(d)
        as_.append(a)
    out["cfg1_cams"] = np.array([[c.height, c.width, c.fx, c.fy, c.cx, c.cy] for c in cams])
    out["cfg1_quats"] = np.stack([c.quat for c in cams]).astype(np.float32)
    out["cfg1_trans"] = np.stack([c.trans for c in cams]).astype(np.float32)
    out["cfg1_pix"] = np.stack(pix).astype(np.int32)
    out["cfg1_depth"] = np.stack(ds)
    out["cfg1_alpha"] = np.stack(as_)


def case_cfg2(fm, out):
    gt, model, cams = S.config2(seed=0)
    put_scene(out, "cfg2", model)
    put_scene(out, "cfg2gt", gt)
    out["cfg2_cams"] = np.array([[c.height, c.width, c.fx, c.fy, c.cx, c.cy] for c in cams])
    out["cfg2_quats"] = np.stack([c.quat for c in cams]).astype(np.float32)
    out["cfg2_trans"] = np.stack([c.trans for c in cams]).astype(np.float32)
    # Two full views of the model scene.
    for vi in (0, 11):
        c = cams[vi]
        rays = pinhole_rays(c.height, c.width, c.fx, c.fy, c.cx, c.cy)
        d, a, _ = render(fm, model.means, model.prec, model.logw, rays, c.quat, c.trans)
        out[f"cfg2_v{vi}_depth"] = d.reshape(c.height, c.width)
        out[f"cfg2_v{vi}_alpha"] = a.reshape(c.height, c.width)
    # Silhouette targets of every view: alpha > 0.5 of the ground-truth scene.
    targets = []
    for c in cams:
        rays = pinhole_rays(c.height, c.width, c.fx, c.fy, c.cx, c.cy)
        _, a, _ = render(fm, gt.means, gt.prec, gt.logw, rays, c.quat, c.trans)
        targets.append((a > 0.5).reshape(c.height, c.width))
    out["cfg2_targets"] = np.stack(targets).astype(np.uint8)
    # Central differences of the mean BCE over four views.
    views = [0, 5, 10, 15]
    out["cfg2_fd_views"] = np.array(views, np.int32)
    rays_v = [pinhole_rays(cams[v].height, cams[v].width, cams[v].fx, cams[v].fy, cams[v].cx,
                           cams[v].cy) for v in views]

    def loss(means, prec, logw):
        tot = 0.0
        for v, rays in zip(views, rays_v):
            _, a, _ = render(fm, means, prec, logw, rays, cams[v].quat, cams[v].trans)
            tot += bce(a, targets[v].ravel().astype(np.float64))
        return tot / len(views)

    m0 = model.means.astype(np.float64)
    p0 = model.prec.astype(np.float64)
    w0 = model.logw.astype(np.float64)
    out["cfg2_fd_loss"] = np.array(loss(m0, p0, w0))
    rng = np.random.default_rng(102)
    upper = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    lower = [(1, 0), (2, 0), (2, 1)]
    # params: (kind, gaussian, i, j); kind 0 mean[g, i], 1 prec[g, i, j], 2 logw[g]
    params = []
    for k in range(48):
        kind = (0, 1, 1, 2)[k % 4]
        g = int(rng.integers(model.n))
        if kind == 0:
            params.append((0, g, int(rng.integers(3)), 0))
        elif kind == 1:
            i, j = (lower[int(rng.integers(3))] if k % 12 == 1 else upper[int(rng.integers(6))])
            params.append((1, g, i, j))
        else:
            params.append((2, g, 0, 0))
    fd = []
    for kind, g, i, j in params:
        vals = []
        h = 1e-6 * (max(1.0, abs(p0[g, i, j])) if kind == 1 else 1.0)
        for sgn in (1.0, -1.0):
            m, p, w = m0.copy(), p0.copy(), w0.copy()
            if kind == 0:
                m[g, i] += sgn * h
            elif kind == 1:
                p[g, i, j] += sgn * h
            else:
                w[g] += sgn * h
            vals.append(loss(m, p, w))
        fd.append((vals[0] - vals[1]) / (2 * h))
    out["cfg2_fd_params"] = np.array(params, np.int32)
    out["cfg2_fd_grad"] = np.array(fd)


def case_edges(fm, out):
    # One Gaussian in front, one behind the camera whose ray line passes close to it.
    quat, trans = np.array([1, 0, 0, 0], np.float32), np.zeros(3, np.float32)
    prec = np.stack([np.triu(np.eye(3) / 0.02)] * 2).astype(np.float32)
    sc = S.Scene(np.array([[0.01, -0.02, 0.5], [0.0, 0.0, -0.4]], np.float32), prec,
                 np.array([0.2, -1.0], np.float32))
    full_view(fm, out, "behind", sc, S.Camera(40, 48, 60.0, 60.0, 24.0, 20.0, quat, trans))
    # A Gaussian straddling the camera plane.
    sc = S.Scene(np.array([[0.3, 0.0, 0.02], [0.0, 0.0, 0.6]], np.float32),
                 np.stack([np.triu(np.eye(3) / 0.1), np.triu(np.eye(3) / 0.05)]).astype(np.float32),
                 np.array([0.0, 0.5], np.float32))
    full_view(fm, out, "straddle", sc, S.Camera(32, 32, 32.0, 32.0, 16.0, 16.0, quat, trans))
    # Sub-pixel Gaussians.
    rng = np.random.default_rng(11)
    sc = S.random_gaussians(80, 0.1, rng, scale_lo=0.002, scale_hi=0.006)
    q, t = S.look_at(0.5 * S.random_unit_vectors(1, rng)[0])
    full_view(fm, out, "subpixel", sc, S.Camera(64, 64, 64.0, 64.0, 32.0, 32.0, q, t))
    # Tiny and ragged images.
    scene, cams = S.config0(seed=4)
    c = cams[0]
    for (h, w) in [(1, 1), (3, 17), (37, 23), (64, 1)]:
        f = float(max(h, w)) + 1.0
        full_view(fm, out, f"tiny{h}x{w}", scene, S.Camera(h, w, f, f, w / 2, h / 2, c.quat, c.trans))


def case_gmm(fm, out):
    rng = np.random.default_rng(103)
    scene = S.random_gaussians(40, 0.1, rng)
    pts = rng.uniform(-0.15, 0.15, size=(600, 3))
    pts[:100] = scene.means[rng.integers(40, size=100)] + rng.normal(0, 0.01, size=(100, 3))
    put_scene(out, "gmm", scene)
    out["gmm_points"] = pts.astype(np.float32)
    ll, res = fm.log_likelihood((f64(scene.means), f64(scene.prec), f64(scene.logw)),
                                f64(pts.astype(np.float32)))
    out["gmm_ll"] = np.array(float(ll))
    out["gmm_res"] = np.asarray(res)


class _ArgumentOrderFixed:
    """While active, ``fm.render_func_rays`` takes (means, prec_full, weights_log, rays, b2, b3),
    the order the reference's pixel-list functions pass, and calls the original in its declared
    order (rays first)."""

    def __init__(self, fm):
        self.fm = fm
        self.orig = fm.render_func_rays

    def __enter__(self):
        orig = self.orig

        def fixed(means, prec_full, weights_log, camera_starts_rays, beta_2, beta_3):
            return orig(camera_starts_rays, means, prec_full, weights_log, beta_2, beta_3)

        self.fm.render_func_rays = fixed

    def __exit__(self, *exc):
        self.fm.render_func_rays = self.orig


def case_pixel_lists(fm, out):
    rng = np.random.default_rng(104)
    scene = S.random_gaussians(60, 0.1, rng)
    put_scene(out, "pix", scene)
    n_pose, inv_f = 4, 1.0 / 80.0
    poses = []
    for d in S.random_unit_vectors(n_pose, rng):
        q, t = S.look_at(0.5 * d)
        poses.append(np.concatenate([q, t]))
    poses = np.array(poses, np.float32)
    n_rays = 900
    # pixel coordinates relative to the principal point (the reference's rays are
    # [x invF, y invF, 1] per pose), pose index in the last column
    pp = np.stack([rng.uniform(-40, 40, n_rays), rng.uniform(-40, 40, n_rays), np.ones(n_rays),
                   rng.integers(0, n_pose, n_rays)], 1).astype(np.float32)
    out["pix_poses"] = poses
    out["pix_rays"] = pp
    out["pix_invf"] = np.array(inv_f)
    with _ArgumentOrderFixed(fm):
        d, a, _, w = fm.render_func_idx_quattrans(f64(scene.means), f64(scene.prec),
                                                  f64(scene.logw), f64(pp), inv_f, f64(poses),
                                                  BETA2, BETA3)
        d2, a2, _, w2, fp, fmn = fm.render_func_idx_quattrans_flow(
            f64(scene.means), f64(scene.prec), f64(scene.logw), f64(pp), inv_f, f64(poses),
            BETA2, BETA3)
    assert np.array_equal(np.asarray(d), np.asarray(d2))
    out["pix_depth"] = np.asarray(d)
    out["pix_alpha"] = np.asarray(a)
    out["pix_w"] = np.asarray(w)
    out["pix_flowp"] = np.asarray(fp)
    out["pix_flowm"] = np.asarray(fmn)


def case_quat_cam(fm, out):
    rng = np.random.default_rng(105)
    scene = S.random_gaussians(50, 0.1, rng)
    put_scene(out, "cam", scene)
    h, w = 48, 64
    inv_f, aspect = 1.0 / 70.0, 1.1
    q, t = S.look_at(0.5 * S.random_unit_vectors(1, rng)[0])
    # pixel list: (x, y, 1) in pixels relative to the principal point, the shift [0.5, 0.5, 0]
    # applied by render_func_quat_cam itself
    u, v = np.meshgrid(np.arange(w, dtype=np.float64) - w / 2, np.arange(h, dtype=np.float64) - h / 2)
    pl = np.stack([u.ravel(), v.ravel(), np.ones(h * w)], 1).astype(np.float32)
    out["cam_pixels"] = pl
    out["cam_hw"] = np.array([h, w])
    out["cam_invf_aspect"] = np.array([inv_f, aspect])
    out["cam_quat"] = q
    out["cam_trans"] = t
    with _ArgumentOrderFixed(fm):
        d, a, _, _ = fm.render_func_quat_cam(f64(scene.means), f64(scene.prec), f64(scene.logw),
                                             f64(pl), aspect, inv_f, f64(q), f64(t), BETA2, BETA3)
    out["cam_depth"] = np.asarray(d)
    out["cam_alpha"] = np.asarray(a)


CASES = [case_cfg0, case_cfg1, case_cfg2, case_edges, case_gmm, case_pixel_lists, case_quat_cam]


def time_reference(fm, n_pix, n_cams):
    """Throughput of the reference's own ``render_func_quat`` (through the float64 NumPy
    stand-in) on a fixed sample of ``n_pix`` pixels of each of the first ``n_cams`` config-1
    cameras, in the benchmark's unit: the metric's evaluations of the sampled pixels (the
    reference tiling's culled count of each camera, scaled by the sampled fraction of its
    pixels) per second, beside the dense rate (every ray against every Gaussian)."""
    from oracle import screen_bounds as SB

    scene, cams = S.config1(seed=0)
    rng = np.random.default_rng(7)
    metric_evals, dense_evals, seconds = 0.0, 0, 0.0
    for cam in cams[:n_cams]:
        p = np.sort(rng.choice(cam.height * cam.width, n_pix, replace=False))
        rays = pinhole_rays(cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy)[p]
        t0 = time.perf_counter()
        render(fm, scene.means, scene.prec, scene.logw, rays, cam.quat, cam.trans)
        seconds += time.perf_counter() - t0
        metric_evals += SB.evals_per_render(scene.means, scene.prec, scene.logw, cam) * \
            n_pix / (cam.height * cam.width)
        dense_evals += n_pix * scene.n
    try:
        from threadpoolctl import threadpool_info
        threads = max([i.get("num_threads", 1) for i in threadpool_info()] or [1])
    except ImportError:
        threads = None
    print(json.dumps({"impl": "reference fm_render.render_func_quat (float64 NumPy stand-in "
                              "for JAX)",
                      "sample": f"{n_pix} pixels of each of {n_cams} config-1 cameras",
                      "mevals_per_s": metric_evals / seconds / 1e6,
                      "dense_mevals_per_s": dense_evals / seconds / 1e6,
                      "seconds": seconds, "cpu_count": os.cpu_count(),
                      "blas_threads": threads}))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--reference", default=os.environ.get("FE_REFERENCE_DIR"),
                    help="reference checkout (default: $FE_REFERENCE_DIR)")
    ap.add_argument("--out", default=OUT)
    ap.add_argument("--only", nargs="*", help="case names to run (default: all)")
    ap.add_argument("--time", type=int, default=0, metavar="PIXELS",
                    help="time the reference's render_func_quat on PIXELS sampled pixels of "
                         "four config-1 cameras and print one JSON line; write no fixtures")
    args = ap.parse_args()
    if not args.reference:
        raise SystemExit("set FE_REFERENCE_DIR or pass --reference")
    fm = import_reference(os.path.abspath(args.reference))
    if args.time:
        time_reference(fm, args.time, 4)
        return
    out = {}
    for case in CASES:
        if args.only and case.__name__[5:] not in args.only:
            continue
        t0 = time.time()
        case(fm, out)
        print(f"{case.__name__}: {time.time() - t0:.1f} s", flush=True)
    out["meta_reference_files"] = np.array(["baseline/fm_render.py", "baseline/util_render.py"])
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out} ({os.path.getsize(args.out) / 1e6:.2f} MB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
