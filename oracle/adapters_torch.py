"""Float64 torch restatements of the scene-parameter adapters (test infrastructure only).

``prec_from_scale_rot`` builds Sigma = R diag(s)^2 R^T as utils/sfs_utils.py:207-213 does and
returns the upper factor U with U U^T = Sigma^-1, computed as J chol(J Sigma^-1 J) J (J the
index reversal) -- a different algorithm from the closed form the kernel uses. The transforms
restate sfs_utils.py:171-184. Autograd through these gives the reference gradients.
"""

from __future__ import annotations

import torch


def quat_to_rot(q):
    w, x, y, z = q.unbind(-1)
    n = (q * q).sum(-1)
    s = 2.0 / n
    X, Y, Z = x * s, y * s, z * s
    R = torch.stack([
        1 - (y * Y + z * Z), x * Y - w * Z, x * Z + w * Y,
        x * Y + w * Z, 1 - (x * X + z * Z), y * Z - w * X,
        x * Z - w * Y, y * Z + w * X, 1 - (x * X + y * Y)], -1)
    return R.reshape(q.shape[:-1] + (3, 3))


def prec_from_scale_rot(scales, quats):
    R = quat_to_rot(quats)
    RS = R * scales[..., None, :]
    cov = RS @ RS.transpose(-1, -2)
    P = torch.linalg.inv(cov)
    Pf = P.flip(-1).flip(-2)
    L = torch.linalg.cholesky(Pf)
    return L.flip(-1).flip(-2)


def transform_points(pose, points):
    return points @ quat_to_rot(pose[3:]).T + pose[:3]


def transform_points_by_inv(pose, points):
    return points @ quat_to_rot(pose[3:]) + pose[:3]
