"""Scene-parameter adapters on the device, differentiable (torch.autograd.Function).

* ``prec_from_scale_rot(scales, quats)``: the renderer's upper precision factor of
  Sigma = R diag(s)^2 R^T (the covariance of the reference's ``prec_from_rotscale``,
  utils/sfs_utils.py:207-213, and of its CUDA rasterizer), so that callers holding the
  reference's (scales, rotations) parameters can use ``render``.
* ``transform_points(pose, points)`` / ``transform_points_by_inv(pose, points)``: the reference's
  ``transform_points_jittable`` / ``transform_points_by_inv_jittable`` (sfs_utils.py:171-184),
  pose = [t(3), q(4)] with a scalar-first quaternion.

Forward and backward are CUDA kernels of the native library (float64 inside).
"""

from __future__ import annotations

import torch

from . import _native as N
from .api import _ptr, _stream

__all__ = ["prec_from_scale_rot", "transform_points", "transform_points_by_inv"]


def _f32(x, shape_tail, name):
    if x.dtype != torch.float32 or not x.is_cuda:
        raise ValueError(f"{name} must be a float32 CUDA tensor")
    if tuple(x.shape[1:]) != shape_tail:
        raise ValueError(f"{name} must have shape (n, {', '.join(map(str, shape_tail))})")
    return x.contiguous()


class _PrecFromScaleRot(torch.autograd.Function):
    @staticmethod
    def forward(ctx, scales, quats):
        scales = _f32(scales, (3,), "scales")
        quats = _f32(quats, (4,), "quats")
        n = scales.shape[0]
        if quats.shape[0] != n:
            raise ValueError("scales and quats must have the same length")
        prec = torch.empty((n, 3, 3), device=scales.device)
        N.check(N.load().fe_prec_from_scale_rot(_ptr(scales), _ptr(quats), n, _ptr(prec),
                                                _stream()))
        ctx.save_for_backward(scales, quats)
        return prec

    @staticmethod
    def backward(ctx, gprec):
        scales, quats = ctx.saved_tensors
        n = scales.shape[0]
        gprec = gprec.contiguous().float()
        gs = torch.empty_like(scales)
        gq = torch.empty_like(quats)
        N.check(N.load().fe_prec_from_scale_rot_bwd(_ptr(scales), _ptr(quats), n, _ptr(gprec),
                                                    _ptr(gs), _ptr(gq), _stream()))
        return gs, gq


class _TransformPoints(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pose, points, inverse):
        points = _f32(points, (3,), "points")
        if pose.dtype != torch.float32 or not pose.is_cuda or pose.numel() != 7:
            raise ValueError("pose must be a float32 CUDA tensor [t(3), q(4)]")
        pose = pose.contiguous().reshape(7)
        out = torch.empty_like(points)
        N.check(N.load().fe_transform_points(_ptr(points), points.shape[0], _ptr(pose),
                                             int(inverse), _ptr(out), _stream()))
        ctx.save_for_backward(pose, points)
        ctx.inverse = int(inverse)
        return out

    @staticmethod
    def backward(ctx, gout):
        pose, points = ctx.saved_tensors
        gout = gout.contiguous().float()
        gp = torch.empty_like(points) if ctx.needs_input_grad[1] else None
        gpose = torch.empty(7, device=pose.device) if ctx.needs_input_grad[0] else None
        N.check(N.load().fe_transform_points_bwd(_ptr(points), points.shape[0], _ptr(pose),
                                                 ctx.inverse, _ptr(gout), _ptr(gp), _ptr(gpose),
                                                 _stream()))
        return gpose, gp, None


def prec_from_scale_rot(scales, quats):
    """Upper precision factor (n,3,3) of Sigma = R(q) diag(s)^2 R(q)^T; differentiable."""
    return _PrecFromScaleRot.apply(scales, quats)


def transform_points(pose, points):
    """R(q) p + t for pose [t(3), q(4)]; differentiable in pose and points."""
    return _TransformPoints.apply(pose, points, False)


def transform_points_by_inv(pose, points):
    """R(q)^T p + t for pose [t(3), q(4)]; differentiable in pose and points."""
    return _TransformPoints.apply(pose, points, True)
