"""torch float64 restatement of the reference renderer, for gradients (TEST INFRASTRUCTURE ONLY).

Same operations as ``oracle/fm_render_np.py`` (``baseline/fm_render.py:11-126``,
``baseline/util_render.py:5-9,51-76``), written with differentiable torch ops so that torch
autograd in float64 stands in for ``jax.grad`` of ``fm_render`` (JAX is unavailable). Gradients
with respect to the strictly-lower entries of ``prec_full`` come out zero, as ``jax.grad`` through
``jnp.triu`` gives.

Only ``tests/`` may import this module.
"""

from __future__ import annotations

import torch

__all__ = ["quat_to_rot", "render_func_rays", "render_func_quat", "pinhole_rays",
           "render_pinhole", "bce_silhouette_loss"]


def quat_to_rot(q):
    """``baseline/util_render.py:51-76`` (scalar-first)."""
    w, x, y, z = q[0], q[1], q[2], q[3]
    nq = w * w + x * x + y * y + z * z
    s = 2.0 / nq
    X, Y, Z = x * s, y * s, z * s
    wX, wY, wZ = w * X, w * Y, w * Z
    xX, xY, xZ = x * X, x * Y, x * Z
    yY, yZ, zZ = y * Y, y * Z, z * Z
    r1 = torch.stack([
        torch.stack([1.0 - (yY + zZ), xY - wZ, xZ + wY]),
        torch.stack([xY + wZ, 1.0 - (xX + zZ), yZ - wX]),
        torch.stack([xZ - wY, yZ + wX, 1.0 - (xX + yY)]),
    ])
    return torch.where(nq > 1e-12, r1, torch.eye(3, dtype=q.dtype, device=q.device))


def render_func_rays(rays, origins, means, prec_full, weights_log, beta_2, beta_3):
    """``fm_render.py:11-109`` for rays (P,3) with origins (P,3); returns depth (P,), alpha (P,)."""
    prec = torch.triu(prec_full)                                      # :14
    prc = prec.transpose(1, 2)                                        # :26
    p = means[:, None, :] - origins[None, :, :]                       # :39
    projp = torch.einsum("nij,npj->npi", prc, p)                      # :42
    lr = torch.einsum("nij,pj->npi", prc, rays)
    vsv = (lr ** 2).sum(-1)                                           # :45
    psv = (projp * lr).sum(-1)                                        # :48
    res = psv / vsv                                                   # :57
    v = rays[None] * res[..., None] - p                               # :60
    d0 = (torch.einsum("nij,npj->npi", prc, v) ** 2).sum(-1)          # :63
    stds = -0.5 * d0 + weights_log[:, None]                           # :66
    zs = res
    est_alpha = 1.0 - torch.exp(-torch.exp(stds).sum(0))              # :89
    sig1 = (zs > 0).to(zs.dtype)                                      # :93
    logits = -zs * beta_2 + beta_3 * stds
    e = torch.exp(logits - logits.amax(0))                            # util_render.py:5-9
    w = sig1 * torch.nan_to_num(e) + 1e-20                            # :96
    w = w / w.sum(0)                                                  # :99
    init_t = (w * torch.nan_to_num(zs)).sum(0)                        # :102
    return init_t, est_alpha


def render_func_quat(means, prec_full, weights_log, camera_rays, quat, t, beta_2, beta_3):
    """``fm_render.py:113-126``."""
    rest = quat_to_rot(quat)
    rays = camera_rays @ rest
    origins = t[None].expand(rays.shape[0], 3)
    return render_func_rays(rays, origins, means, prec_full, weights_log, beta_2, beta_3)


def pinhole_rays(height, width, fx, fy, cx, cy, dtype=torch.float64, device=None):
    """Camera-frame rays, pixel index v*W+u (``baseline/ycb_fmb_rotscale.py:182-189``)."""
    v, u = torch.meshgrid(torch.arange(height, dtype=dtype, device=device),
                          torch.arange(width, dtype=dtype, device=device), indexing="ij")
    return torch.stack([(u.reshape(-1) - cx) / fx, (v.reshape(-1) - cy) / fy,
                        torch.ones(height * width, dtype=dtype, device=device)], 1)


def render_pinhole(means, prec_full, weights_log, height, width, fx, fy, cx, cy, quat, t,
                   beta_2=21.4, beta_3=2.66):
    rays = pinhole_rays(height, width, fx, fy, cx, cy, dtype=means.dtype, device=means.device)
    d, a = render_func_quat(means, prec_full, weights_log, rays, quat, t, beta_2, beta_3)
    return d.reshape(height, width), a.reshape(height, width)


def bce_silhouette_loss(alpha, target, clip=3e-8):
    """The shape-from-silhouette objective (notebook cell 12): clipped binary cross-entropy, mean."""
    a = torch.clamp(alpha, clip, 1.0 - clip)
    return -(target * torch.log(a) + (1.0 - target) * torch.log(1.0 - a)).mean()
