"""Shared helpers for the parity tests."""

import functools
import os

import numpy as np
import torch

from fuzzy_ellipses import synthetic as S
from oracle import fm_render_np as O

# Outputs of the reference's own baseline/fm_render.py (imported unmodified, float64), made by
# tests/golden/make_fm_render_golden.py; inputs are stored beside them.
GOLDEN_FM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                         "fm_render_golden.npz")


@functools.lru_cache(maxsize=1)
def golden():
    with np.load(GOLDEN_FM) as z:
        return {k: z[k] for k in z.files}


def golden_scene(key):
    g = golden()
    return S.Scene(g[f"{key}_means"], g[f"{key}_prec"], g[f"{key}_logw"])


def golden_camera(key):
    """The camera of a full-view fixture: (Camera, depth (H, W), alpha (H, W))."""
    g = golden()
    h, w, fx, fy, cx, cy = g[f"{key}_cam"]
    cam = S.Camera(int(h), int(w), float(fx), float(fy), float(cx), float(cy), g[f"{key}_quat"],
                   g[f"{key}_trans"])
    return cam, g[f"{key}_depth"], g[f"{key}_alpha"]


def golden_cameras(key):
    """The cameras of a multi-camera fixture (cfg1, cfg2)."""
    g = golden()
    out = []
    for row, q, t in zip(g[f"{key}_cams"], g[f"{key}_quats"], g[f"{key}_trans"]):
        h, w, fx, fy, cx, cy = row
        out.append(S.Camera(int(h), int(w), float(fx), float(fy), float(cx), float(cy), q, t))
    return out


# Full-view fixtures of the edge scenes, in the order the generator writes them.
GOLDEN_VIEWS = ["cfg0", "behind", "straddle", "subpixel", "tiny1x1", "tiny3x17", "tiny37x23",
                "tiny64x1"]

# Stated tolerances (the benchmark spec): absolute alpha, relative depth on pixels where the oracle's
# alpha exceeds DEPTH_MASK_ALPHA (fm_render's depth on near-empty pixels is a softmax over far
# Gaussians that any tile-culled renderer omits by construction).
TOL_ALPHA = 1e-5
TOL_DEPTH_REL = 1e-4
DEPTH_MASK_ALPHA = 1e-3


def to_dev(x, dev):
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def scene_to_dev(scene, dev):
    return to_dev(scene.means, dev), to_dev(scene.prec, dev), to_dev(scene.logw, dev)


def oracle_pixels(scene, cam, pix):
    """Dense float64 oracle on a subset of pixel indices (v*W+u) of a camera."""
    rays = O.pinhole_rays(cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy)[pix]
    d, a, _, _ = O.render_func_quat(scene.means, scene.prec, scene.logw, rays, cam.quat,
                                    cam.trans, 21.4, 2.66)
    return d, a


def floor_dominated(scene, cam, beta2=21.4, beta3=2.66):
    """Pixels where fm_render's depth is set by its +1e-20 weight floor (fm_render.py:93-99).

    fm_render subtracts the max logit over *all* Gaussians, including those behind the camera
    (z <= 0, whose logit -beta2*z is large), before masking them out; where the front Gaussians'
    share of that max falls below the floor, its depth becomes the floor-weighted mean of every z.
    A tile-culled renderer normalises over the front Gaussians instead. Returns a bool (H*W,)."""
    rays = O.pinhole_rays(cam.height, cam.width, cam.fx, cam.fy, cam.cx, cam.cy) @ O.quat_to_rot(cam.quat)
    zs, stds = O.ray_gaussian_terms(rays, np.tile(np.asarray(cam.trans, np.float64), (rays.shape[0], 1)),
                                    scene.means, scene.prec, scene.logw)
    logit = -beta2 * zs + beta3 * stds
    mass = np.where(zs > 0, np.exp(logit - logit.max(0)), 0.0).sum(0)
    return mass < 1e-12


def parity_errors(depth, alpha, d_ref, a_ref, mask_alpha=DEPTH_MASK_ALPHA, exclude=None):
    depth = np.asarray(depth, np.float64).ravel()
    alpha = np.asarray(alpha, np.float64).ravel()
    d_ref = np.asarray(d_ref).ravel()
    a_ref = np.asarray(a_ref).ravel()
    ea = float(np.abs(alpha - a_ref).max()) if alpha.size else 0.0
    m = a_ref > mask_alpha
    if exclude is not None:
        m &= ~np.asarray(exclude).ravel()
    ed = float((np.abs(depth - d_ref)[m] / np.abs(d_ref[m])).max()) if m.any() else 0.0
    return ea, ed


def tile_lists_from_keys(keys, n_tiles):
    keys = keys.cpu().numpy().view(np.uint64)
    tiles = (keys >> np.uint64(32)).astype(np.int64)
    gids = (keys & np.uint64(0xFFFFFFFF)).astype(np.int64)
    lists = [[] for _ in range(n_tiles)]
    for t, g in zip(tiles, gids):
        lists[t].append(g)
    return [np.array(x, np.int64) for x in lists]
