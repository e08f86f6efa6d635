"""CPU float64 restatement of the reference's pure-JAX renderer (TEST INFRASTRUCTURE ONLY).

This module is the depth/alpha oracle. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it, and only as the checker or the timed CPU
baseline; the product path never calls it.

It restates, operation for operation and in float64 NumPy:

* ``render_func_rays``  -- ``baseline/fm_render.py:11-109``
* ``render_func_quat``  -- ``baseline/fm_render.py:113-126``
* ``render_func_quat_cam`` -- ``baseline/fm_render.py:130-144``
* ``render_func_idx_quattrans[_flow]`` -- ``baseline/fm_render.py:151-224``
* ``jax_stable_exp``    -- ``baseline/util_render.py:5-9``
* ``quat_to_rot``       -- ``baseline/util_render.py:51-76``

Details kept exactly as the reference has them:

* ``prec = triu(prec_full)`` and the per-Gaussian transpose to a lower factor (``:14,26``);
* alpha uses every Gaussian with no ``z > 0`` mask (``:89``, the reference's own BUG note at ``:92``);
* the softmax max is taken over *all* Gaussians before the ``z > 0`` mask (``:93-96``);
* ``+1e-20`` is added to every weight (``:96``);
* ``nan_to_num`` on the weights and on ``z`` (``:96,102``).

The reference evaluates ``jax.lax.map`` in batches of 16 (``:79,86``); batching does not change
results, so this restatement evaluates a dense ``[N, pixels]`` block per chunk of pixels.

JAX is not installed on either machine this project runs on. The restatement is pinned against
the reference's own ``fm_render.py``, imported unmodified with a float64 NumPy stand-in for JAX
(``tests/golden/numpy_jax.py``): ``tests/golden/make_fm_render_golden.py`` ran it and committed
its outputs as ``tests/golden/fm_render_golden.npz``, and ``tests/test_oracle.py`` checks this
module against them (agreement to about 1e-13), beside analytic known-answer cases.

A *culled* variant (``render_culled``) evaluates each pixel only over the Gaussians listed for its
tile. It defines the quantity a tile-binned renderer computes, so arithmetic error (kernel vs
culled oracle) and tail error (culled vs dense oracle) can be reported separately.
"""

from __future__ import annotations

import numpy as np

__all__ = [
    "quat_to_rot",
    "jax_stable_exp",
    "render_func_rays",
    "render_func_quat",
    "pinhole_rays",
    "render_pinhole",
    "render_culled",
    "render_func_quat_cam",
    "ray_gaussian_terms",
]


def quat_to_rot(q):
    """Scalar-first quaternion to rotation matrix (``baseline/util_render.py:51-76``)."""
    w, x, y, z = (float(v) for v in np.asarray(q, dtype=np.float64))
    nq = w * w + x * x + y * y + z * z
    if not nq > 1e-12:
        return np.eye(3)
    s = 2.0 / nq
    X, Y, Z = x * s, y * s, z * s
    wX, wY, wZ = w * X, w * Y, w * Z
    xX, xY, xZ = x * X, x * Y, x * Z
    yY, yZ, zZ = y * Y, y * Z, z * Z
    return np.array(
        [
            [1.0 - (yY + zZ), xY - wZ, xZ + wY],
            [xY + wZ, 1.0 - (xX + zZ), yZ - wX],
            [xZ - wY, yZ + wX, 1.0 - (xX + yY)],
        ]
    )


def jax_stable_exp(z, s=1.0, axis=0):
    """``exp(s*z - max(s*z))`` along ``axis`` (``baseline/util_render.py:5-9``)."""
    z = s * z
    z = z - z.max(axis)
    return np.exp(z)


def ray_gaussian_terms(rays, origins, means, prec_full, weights_log):
    """Per (Gaussian, ray) peak parameter ``z`` and log-density ``d2`` (``fm_render.py:23-76``).

    rays, origins: (P, 3); means: (N, 3); prec_full: (N, 3, 3); weights_log: (N,).
    Returns zs, stds of shape (N, P), float64.
    """
    prec = np.triu(np.asarray(prec_full, dtype=np.float64))          # :14
    prc = np.transpose(prec, (0, 2, 1))                               # :26 (lower factor)
    r = np.asarray(rays, dtype=np.float64)
    t = np.asarray(origins, dtype=np.float64)
    m = np.asarray(means, dtype=np.float64)
    w = np.asarray(weights_log, dtype=np.float64)
    p = m[:, None, :] - t[None, :, :]                                 # :39  (N, P, 3)
    projp = np.einsum("nij,npj->npi", prc, p)                         # :42
    lr = np.einsum("nij,pj->npi", prc, r)                             # prc @ r
    vsv = (lr ** 2).sum(-1)                                           # :45
    psv = (projp * lr).sum(-1)                                        # :48
    with np.errstate(divide="ignore", invalid="ignore"):
        res = psv / vsv                                               # :57
    v = r[None, :, :] * res[:, :, None] - p                           # :60
    d0 = (np.einsum("nij,npj->npi", prc, v) ** 2).sum(-1)             # :63
    d2 = -0.5 * d0 + w[:, None]                                       # :66
    return res, d2


def _reduce(zs, stds, beta_2, beta_3):
    """The per-pixel reductions of ``fm_render.py:88-102`` over axis 0 (Gaussians)."""
    est_alpha = 1.0 - np.exp(-np.exp(stds).sum(0))                    # :89
    sig1 = zs > 0                                                     # :93
    with np.errstate(over="ignore", invalid="ignore"):
        w = sig1 * np.nan_to_num(jax_stable_exp(-zs * beta_2 + beta_3 * stds)) + 1e-20  # :96
    w = w / w.sum(0)                                                  # :99
    init_t = (w * np.nan_to_num(zs)).sum(0)                           # :102
    return init_t, est_alpha, w


def render_func_rays(camera_starts_rays, means, prec_full, weights_log, beta_2, beta_3,
                     chunk=4096, return_weights=False):
    """Dense render (``fm_render.py:11-109``). ``camera_starts_rays``: (P, 2, 3) = [ray, origin].

    Returns ``(depth (P,), alpha (P,), None, w (N, P) or None)``; ``w`` is materialised only when
    ``return_weights`` is set (it is N x P).
    """
    csr = np.asarray(camera_starts_rays, dtype=np.float64)
    npix = csr.shape[0]
    depth = np.empty(npix)
    alpha = np.empty(npix)
    ws = [] if return_weights else None
    for s in range(0, npix, chunk):
        e = min(npix, s + chunk)
        zs, stds = ray_gaussian_terms(csr[s:e, 0], csr[s:e, 1], means, prec_full, weights_log)
        d, a, w = _reduce(zs, stds, beta_2, beta_3)
        depth[s:e] = d
        alpha[s:e] = a
        if return_weights:
            ws.append(w)
    return depth, alpha, None, (np.concatenate(ws, axis=1) if return_weights else None)


def render_func_quat(means, prec_full, weights_log, camera_rays, quat, t, beta_2, beta_3,
                     chunk=4096, return_weights=False):
    """``fm_render.py:113-126``: rotate the camera-frame rays by ``quat_to_rot(quat)``."""
    rest = quat_to_rot(quat)
    rays = np.asarray(camera_rays, dtype=np.float64) @ rest            # :117
    trans = np.tile(np.asarray(t, dtype=np.float64)[None], (rays.shape[0], 1))  # :118
    csr = np.stack([rays, trans], 1)                                   # :120
    return render_func_rays(csr, means, prec_full, weights_log, beta_2, beta_3,
                            chunk=chunk, return_weights=return_weights)


def pinhole_rays(height, width, fx, fy, cx, cy):
    """Camera-frame rays ``[(u-cx)/fx, (v-cy)/fy, 1]``, pixel index ``v*W+u``.

    Same construction as ``baseline/ycb_fmb_rotscale.py:182-189`` (meshgrid of ``arange(W)``,
    ``arange(H)``, then ``(pixel - K[:,2]) / diag(K)`` with the last column set to 1).
    """
    u, v = np.meshgrid(np.arange(width, dtype=np.float64), np.arange(height, dtype=np.float64))
    rays = np.stack([(u.ravel() - cx) / fx, (v.ravel() - cy) / fy, np.ones(height * width)], 1)
    return rays


def render_pinhole(means, prec_full, weights_log, height, width, fx, fy, cx, cy, quat, t,
                   beta_2=21.4, beta_3=2.66, chunk=4096):
    """Dense float64 depth and alpha images (H, W) for one pinhole camera."""
    rays = pinhole_rays(height, width, fx, fy, cx, cy)
    d, a, _, _ = render_func_quat(means, prec_full, weights_log, rays, quat, t, beta_2, beta_3,
                                  chunk=chunk)
    return d.reshape(height, width), a.reshape(height, width)


def render_culled(means, prec_full, weights_log, height, width, fx, fy, cx, cy, quat, t,
                  tile_lists, tile_w, tile_h, beta_2=21.4, beta_3=2.66):
    """Per-tile culled float64 render.

    ``tile_lists[tile]`` is the array of Gaussian indices binned to ``tile`` (tile = ty*gx+tx).
    Per pixel, alpha sums over that list only; the depth softmax uses the list's ``z > 0``
    entries with their own max, and depth is 0 where no listed Gaussian has ``z > 0`` -- the
    definition a tile-binned renderer computes. With every Gaussian listed for every tile this
    equals the dense render up to the reference's ``+1e-20`` weight floor.
    """
    rest = quat_to_rot(quat)
    rays_all = pinhole_rays(height, width, fx, fy, cx, cy) @ rest
    t = np.asarray(t, dtype=np.float64)
    depth = np.zeros((height, width))
    alpha = np.zeros((height, width))
    gx = (width + tile_w - 1) // tile_w
    gy = (height + tile_h - 1) // tile_h
    for ty in range(gy):
        for tx in range(gx):
            ids = np.asarray(tile_lists[ty * gx + tx], dtype=np.int64)
            us = np.arange(tx * tile_w, min(width, (tx + 1) * tile_w))
            vs = np.arange(ty * tile_h, min(height, (ty + 1) * tile_h))
            vv, uu = np.meshgrid(vs, us, indexing="ij")
            pix = (vv * width + uu).ravel()
            if ids.size == 0:
                continue
            zs, stds = ray_gaussian_terms(rays_all[pix], np.tile(t, (pix.size, 1)),
                                          np.asarray(means)[ids], np.asarray(prec_full)[ids],
                                          np.asarray(weights_log)[ids])
            a = 1.0 - np.exp(-np.exp(stds).sum(0))
            logit = -zs * beta_2 + beta_3 * stds
            front = zs > 0
            lm = np.where(front, logit, -np.inf)
            mx = lm.max(0)
            has = np.isfinite(mx)
            with np.errstate(invalid="ignore", over="ignore"):
                wgt = np.where(front, np.exp(lm - np.where(has, mx, 0.0)), 0.0)
            wsum = wgt.sum(0)
            with np.errstate(invalid="ignore", divide="ignore"):
                d = np.where(has, (wgt * np.nan_to_num(zs)).sum(0) / np.where(has, wsum, 1.0), 0.0)
            depth.ravel()[pix] = d
            alpha.ravel()[pix] = a
    return depth, alpha


def render_func_quat_cam(means, prec_full, weights_log, pixel_list, aspect, invF, quat, t,
                         beta_2, beta_3, return_weights=False):
    """``fm_render.py:130-144`` (argument order of its render_func_rays call fixed): rays
    ``(pixel_list - [0.5, 0.5, 0]) * [invF, aspect invF, 1]`` rotated by ``quat_to_rot(quat)``."""
    pl = np.asarray(pixel_list, dtype=np.float64)
    rays = (pl - np.array([0.5, 0.5, 0.0])) * np.array([invF, aspect * invF, 1.0])   # :133-135
    return render_func_quat(means, prec_full, weights_log, rays, quat, t, beta_2, beta_3,
                            return_weights=return_weights)                           # :137-144


def _pose_rays(pixel_posei, invF, poses):
    pp = np.asarray(pixel_posei, dtype=np.float64)
    poses = np.asarray(poses, dtype=np.float64)
    rots = np.stack([quat_to_rot(p[:4]) for p in poses])               # :157
    idx = np.clip(pp[:, 3].astype(int), 0, len(poses) - 1)              # astype(int); JAX clamps
    rays = pp[:, :3] * np.array([invF, invF, 1.0])                      # :160
    rw = np.einsum("pi,pij->pj", rays, rots[idx])                       # ray @ rot_mats[idx]
    return pp, poses, rots, idx, rays, rw


def render_func_idx_quattrans(means, prec_full, weights_log, pixel_posei, invF, poses, beta_2,
                              beta_3, return_weights=False):
    """``fm_render.py:151-167`` with the intended argument order of its render_func_rays call."""
    _, poses, _, idx, _, rw = _pose_rays(pixel_posei, invF, poses)
    csr = np.stack([rw, poses[idx, 4:]], 1)
    return render_func_rays(csr, means, prec_full, weights_log, beta_2, beta_3,
                            return_weights=return_weights)


def flow_from_depth(pixel_posei, invF, poses, depth):
    """Per-ray forward / backward flow of ``fm_render.py:186-222`` for given depths."""
    pp, poses, rots, idx, rays, _ = _pose_rays(pixel_posei, invF, poses)
    n = len(poses)
    pt1 = rays * np.asarray(depth, dtype=np.float64)[:, None]
    world = np.einsum("pi,pij->pj", pt1, rots[idx]) + poses[idx, 4:]
    out = []
    for nb in (np.minimum(idx + 1, n - 1), np.maximum(idx - 1, 0)):
        pt2 = np.einsum("pj,pij->pi", world - poses[nb, 4:], rots[nb])   # (world - t) @ R^T
        coord = pt2[:, :2] / (pt2[:, 2:3] * invF)
        out.append(-(coord - pp[:, :2]))
    return out[0], out[1]


def render_func_idx_quattrans_flow(means, prec_full, weights_log, pixel_posei, invF, poses,
                                   beta_2, beta_3, return_weights=False):
    """``fm_render.py:171-224`` (argument order fixed as above)."""
    d, a, nrm, w = render_func_idx_quattrans(means, prec_full, weights_log, pixel_posei, invF,
                                             poses, beta_2, beta_3, return_weights)
    fp, fm = flow_from_depth(pixel_posei, invF, poses, d)
    return d, a, nrm, w, fp, fm
